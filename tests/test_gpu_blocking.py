"""Temporal blocking of the FP32 correction sweeps: two sweeps per tile load (tiles of the
corrections staged by TMA with a margin of two cells, the first sweep also computed on the margin)
against one sweep per round of the persistent loop.  The stop rule is applied after each sweep to
that sweep's residual, so the loop stops at the same sweep with the same iterate: every field and
every sweep count must be equal bit for bit (the reference sweep loop, SIMPLE_TS_MPI.cpp:3788-4131,
and its stop rule, :4087-4107)."""
import tempfile

import numpy as np
import pytest

import sts_cases as sc

pytestmark = pytest.mark.gpu

FIELDS = ("u", "v", "p", "T", "rho")


@pytest.mark.parametrize("which,scale,steps,warm", [("channel_ma2.43", 0.25, 30, 0), ("channel_ma2.43", 0.25, 30, 4),
                                                    ("rayleigh_benard", 0.0625, 30, 0), ("channel_ma0.1", 0.5, 20, 2),
                                                    ("channel_ma2.43", 1.0, 6, 0)])
@pytest.mark.parametrize("precision", [2, 3])
@pytest.mark.parametrize("use_graph", [True, False], ids=["graph", "launches"])
def test_two_sweeps_per_load_equal_one(which, scale, steps, warm, precision, use_graph, lib_built):
    import sts
    case = sc.config_case(which, scale=scale, Nt=steps)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        runs = []
        for k in (1, 2):
            s = sts.Solver(d, fixed_sweeps=False, use_graph=use_graph, precision=precision, warm_start=warm,
                           autotune=False)
            s.set_sweep_blocking(k)
            assert s.sweep_blocking() == k
            assert s.step(steps) == steps
            runs.append(({f: s.field(f) for f in FIELDS}, s.sweep_history()))
            s.close()
        for f in FIELDS:
            np.testing.assert_array_equal(runs[0][0][f], runs[1][0][f], err_msg=f)
        np.testing.assert_array_equal(runs[0][1], runs[1][1])


def test_blocking_rejected_where_not_available(lib_built):
    import sts
    case = sc.channel_case("c", 40, 8, 0.5, 0.003, 1e-3, 5)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        s = sts.Solver(d, fixed_sweeps=False, precision=0)
        with pytest.raises(sts.StsError):
            s.set_sweep_blocking(2)
        s.close()
