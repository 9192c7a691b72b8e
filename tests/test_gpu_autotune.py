"""The autotuner picks launch shapes on the run's first steps; launch shapes cannot change results,
so a tuned run equals an untuned one bit for bit."""
import tempfile

import numpy as np
import pytest

import sts_cases as sc

pytestmark = pytest.mark.gpu

FIELDS = ["u", "v", "p", "T", "rho"]


@pytest.mark.parametrize("precision", [0, 2])
def test_tuned_run_equals_untuned(precision, lib_built):
    import sts
    case = sc.config_case("channel_ma2.43", scale=0.25, Nt=40)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        a = sts.Solver(d, fixed_sweeps=False, precision=precision, autotune=True)
        b = sts.Solver(d, fixed_sweeps=False, precision=precision, autotune=False)
        left = a.autotune_result()["steps_left"]
        assert left > 0
        assert a.step(left + 6) == b.step(left + 6) == left + 6
        res = a.autotune_result()
        print(res)
        assert res["steps_left"] == 0
        assert res["ctas_per_sm"] >= 1
        assert res["asm_block"] in ((32, 8), (64, 4), (128, 2))
        for f in FIELDS:
            np.testing.assert_array_equal(a.field(f), b.field(f), err_msg=f)
        np.testing.assert_array_equal(a.sweep_history(), b.sweep_history())
        a.close()
        b.close()


def test_tuned_batch_equals_untuned(lib_built):
    import os
    import sts
    cases = sc.batch_cases(n=3, Nt=40, nx_range=(40, 100))
    with tempfile.TemporaryDirectory() as root:
        dirs = []
        for k, c in enumerate(cases):
            d = os.path.join(root, f"c{k}")
            os.makedirs(d)
            c.write(d)
            dirs.append(d)
        a = sts.Batch(dirs, fixed_sweeps=False, precision=2, autotune=True)
        b = sts.Batch(dirs, fixed_sweeps=False, precision=2, autotune=False)
        left = a.autotune_result()["steps_left"]
        assert left > 0
        assert a.step(left + 4) == b.step(left + 4) == left + 4
        res = a.autotune_result()
        print(res)
        assert res["steps_left"] == 0 and res["asm_block"] in ((32, 8), (64, 4), (128, 2))
        for k in range(len(dirs)):
            for f in FIELDS:
                np.testing.assert_array_equal(a.cases[k].field(f), b.cases[k].field(f), err_msg=f"case {k} {f}")
        a.close()
        b.close()
