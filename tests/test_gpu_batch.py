"""Batches of independent cases (one launch per kernel and step for all cases, the sweep loops
of all cases in one cooperative launch) give each case exactly the bits it gets alone: against
the oracle for the FP64 path, against single-case runs for the other precision modes."""
import os
import tempfile

import numpy as np
import pytest

import sts_cases as sc

pytestmark = pytest.mark.gpu

FIELDS = ["u", "v", "p", "T", "rho"]


def small_batch(n, Nt, seed=20261204):
    """Uneven channel cases drawn like the 64-case batch, at oracle-friendly sizes, plus a
    periodic Rayleigh-Benard box."""
    cases = sc.batch_cases(n=n, seed=seed, Nt=Nt, nx_range=(40, 120))
    cases.append(sc.rayleigh_benard_case("rb", 32, 16, Nt=Nt))
    return cases


def write_all(cases, root):
    dirs = []
    for k, c in enumerate(cases):
        d = os.path.join(root, f"c{k:02d}")
        os.makedirs(d)
        c.write(d)
        dirs.append(d)
    return dirs


def test_batch_matches_oracle_per_case(lib_built, oracle_built):
    import ora
    import sts
    cases = small_batch(5, Nt=40)
    with tempfile.TemporaryDirectory() as root:
        dirs = write_all(cases, root)
        b = sts.Batch(dirs, fixed_sweeps=False)
        assert b.step(6) == 6
        for k, d in enumerate(dirs):
            o = ora.Oracle(d, fixed_sweeps=False)
            assert o.step(6) == 6
            g = b.cases[k]
            for f in FIELDS:
                np.testing.assert_array_equal(g.field(f), o.field(f), err_msg=f"case {k} {f}")
            np.testing.assert_array_equal(g.sweep_history(), o.sweeps())
            np.testing.assert_array_equal(g.stats(), o.stats())
        b.close()


@pytest.mark.parametrize("precision", [1, 2, 3])
def test_batch_equals_single_runs(precision, lib_built):
    import sts
    cases = small_batch(4, Nt=40, seed=7)
    with tempfile.TemporaryDirectory() as root:
        dirs = write_all(cases, root)
        b = sts.Batch(dirs, fixed_sweeps=False, precision=precision)
        assert b.step(8) == 8
        for k, d in enumerate(dirs):
            s = sts.Solver(d, fixed_sweeps=False, precision=precision)
            assert s.step(8) == 8
            for f in FIELDS:
                np.testing.assert_array_equal(b.cases[k].field(f), s.field(f), err_msg=f"case {k} {f}")
            np.testing.assert_array_equal(b.cases[k].sweep_history(), s.sweep_history())
            s.close()
        b.close()


def test_batch_cases_end_independently(lib_built, oracle_built):
    """A case whose run ends (Nt reached) stays put while the others go on."""
    import ora
    import sts
    cases = small_batch(2, Nt=20)
    cases[0].entered["Nt"] = 3
    with tempfile.TemporaryDirectory() as root:
        dirs = write_all(cases, root)
        b = sts.Batch(dirs, fixed_sweeps=False)
        assert b.step(5) == 5
        assert b.step(2) == 2
        for k, d in enumerate(dirs):
            o = ora.Oracle(d, fixed_sweeps=False)
            o.step(7)
            for f in FIELDS:
                np.testing.assert_array_equal(b.cases[k].field(f), o.field(f), err_msg=f"case {k} {f}")
        assert len(b.cases[0].sweep_history()) == 3
        assert len(b.cases[1].sweep_history()) == 7
        with pytest.raises(sts.StsError):
            b.cases[0].step(1)
        b.close()


def test_batch_fixed_sweeps_matches_oracle(lib_built, oracle_built):
    import ora
    import sts
    cases = small_batch(3, Nt=40, seed=11)
    for c in cases:
        c.entered["N_I_p_c"] = 3
    with tempfile.TemporaryDirectory() as root:
        dirs = write_all(cases, root)
        b = sts.Batch(dirs, fixed_sweeps=True)
        assert b.step(4) == 4
        for k, d in enumerate(dirs):
            o = ora.Oracle(d, fixed_sweeps=True)
            o.step(4)
            for f in FIELDS:
                np.testing.assert_array_equal(b.cases[k].field(f), o.field(f), err_msg=f"case {k} {f}")
        b.close()


def test_batch_launch_mode_equals_graph(lib_built):
    import sts
    cases = small_batch(3, Nt=40, seed=5)
    with tempfile.TemporaryDirectory() as root:
        dirs = write_all(cases, root)
        a = sts.Batch(dirs, fixed_sweeps=False, precision=2, use_graph=True)
        b = sts.Batch(dirs, fixed_sweeps=False, precision=2, use_graph=False)
        assert a.step(6) == b.step(6) == 6
        for k in range(len(dirs)):
            for f in FIELDS:
                np.testing.assert_array_equal(a.cases[k].field(f), b.cases[k].field(f), err_msg=f"case {k} {f}")
        a.close()
        b.close()
