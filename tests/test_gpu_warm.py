"""Warm start of the p-T sweeps (extrapolation in time of p and T): the GPU equals the oracle
with the same warm start bit for bit, the sweep count falls, and the answer stays within the
tolerance-level distance of the reference's (cold-start) run."""
import tempfile

import numpy as np
import pytest

import sts_cases as sc
from conftest import golden_case

pytestmark = pytest.mark.gpu

FIELDS = ["u", "v", "p", "T", "rho"]


@pytest.mark.parametrize("warm", [1, 2])
@pytest.mark.parametrize("name", ["channel_ma2.43_60x12_resid", "rayleigh_benard_32x16_resid",
                                  "channel_circle_120x12_resid"])
def test_warm_start_matches_oracle(name, warm, lib_built, oracle_built):
    import ora
    import sts
    case, fixed = golden_case(name)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        o = ora.Oracle(d, fixed_sweeps=fixed, warm_start=warm)
        for use_graph in (True, False):
            g = sts.Solver(d, fixed_sweeps=fixed, use_graph=use_graph, warm_start=warm)
            assert g.step(10) == 10
            if use_graph:
                assert o.step(10) == 10
            for f in FIELDS:
                np.testing.assert_array_equal(g.field(f), o.field(f), err_msg=f"{f} graph={use_graph}")
            np.testing.assert_array_equal(g.sweep_history(), o.sweeps())
            g.close()


@pytest.mark.parametrize("warm", [2, 4])
def test_warm_start_with_outer_iterations(warm, lib_built, oracle_built):
    """Three outer iterations per step: the warm start belongs to the step's first one; the step
    graph and the launch-by-launch loop both equal to the oracle bit for bit."""
    import ora
    import sts
    case = sc.channel_case("c", 60, 12, 2.43, 0.00283, 2.5e-4, 100)
    case.entered["N_I"] = 3
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        o = ora.Oracle(d, fixed_sweeps=False, warm_start=warm)
        assert o.step(30) == 30
        for use_graph in (True, False):
            g = sts.Solver(d, fixed_sweeps=False, use_graph=use_graph, warm_start=warm)
            assert g.step(30) == 30
            for f in FIELDS:
                np.testing.assert_array_equal(g.field(f), o.field(f), err_msg=f"{f} graph={use_graph}")
            np.testing.assert_array_equal(g.sweep_history(), o.sweeps())
            g.close()


def test_warm_start_cuts_sweeps_within_tolerance(lib_built, oracle_built):
    import ora
    import sts
    case = sc.rayleigh_benard_case("rb", 64, 32, Nt=60)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        cold = ora.Oracle(d, fixed_sweeps=False)
        cold.step(60)
        g = sts.Solver(d, fixed_sweeps=False, warm_start=2, precision=sts.MIXED)
        assert g.step(60) == 60
        hw, hc = g.sweep_history()[10:], cold.sweeps()[10:]
        print("sweeps per step: cold", hc.mean(), "warm", hw.mean())
        assert hw.mean() < 0.75 * hc.mean()
        for f in ("p", "T"):
            e = np.linalg.norm(g.field(f) - cold.field(f)) / np.linalg.norm(cold.field(f))
            print(f, e)
            assert e < 1e-6
        g.close()


def test_batch_warm_start_equals_single(lib_built):
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
        b = sts.Batch(dirs, fixed_sweeps=False, warm_start=2)
        assert b.step(8) == 8
        for k, d in enumerate(dirs):
            s = sts.Solver(d, fixed_sweeps=False, warm_start=2)
            s.step(8)
            for f in FIELDS:
                np.testing.assert_array_equal(b.cases[k].field(f), s.field(f), err_msg=f"case {k} {f}")
            s.close()
        b.close()


def test_bad_warm_start_rejected(lib_built):
    import sts
    case = sc.channel_case("c", 20, 6, 0.2, 0.002, 1e-3, 5)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        with pytest.raises(sts.StsError):
            sts.Solver(d, warm_start=7)


@pytest.mark.parametrize("which,scale,steps", [("channel_ma0.1", 1.0, 40), ("rayleigh_benard", 0.125, 60),
                                               ("channel_ma2.43", 0.25, 40)])
def test_learned_warm_start(which, scale, steps, lib_built, oracle_built):
    """Mode 3 against the oracle's mode 3 (its least-squares sums run in another order, so the
    comparison is to the tolerance level, not bit for bit) and against the cold start."""
    import ora
    import sts
    case = sc.config_case(which, scale=scale, Nt=steps)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        o3 = ora.Oracle(d, fixed_sweeps=False, warm_start=3)
        o3.step(steps)
        cold = ora.Oracle(d, fixed_sweeps=False)
        cold.step(steps)
        g = sts.Solver(d, fixed_sweeps=False, warm_start=3)
        assert g.step(steps) == steps
        hg, ho, hc = g.sweep_history()[10:], o3.sweeps()[10:], cold.sweeps()[10:]
        print(which, "sweeps per step: cold", hc.mean(), "oracle mode 3", ho.mean(), "gpu mode 3", hg.mean())
        assert abs(hg.mean() - ho.mean()) <= 0.3
        assert hg.mean() <= 0.8 * hc.mean()
        for f in ("p", "T", "u"):
            e = np.linalg.norm(g.field(f) - o3.field(f)) / np.linalg.norm(o3.field(f))
            assert e < 1e-6, (f, e)
        g.close()


def test_batch_learned_warm_start_equals_single(lib_built):
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
        b = sts.Batch(dirs, fixed_sweeps=False, warm_start=3, precision=2)
        assert b.step(14) == 14
        for k, d in enumerate(dirs):
            s = sts.Solver(d, fixed_sweeps=False, warm_start=3, precision=2)
            s.step(14)
            for f in FIELDS:
                np.testing.assert_array_equal(b.cases[k].field(f), s.field(f), err_msg=f"case {k} {f}")
            s.close()
        b.close()


@pytest.mark.parametrize("which,scale,steps", [("channel_ma2.43", 0.25, 30), ("rayleigh_benard", 0.125, 30),
                                               ("rayleigh_benard", 0.25, 30), ("channel_ma0.1", 0.5, 30)])
def test_conv_warm_start_matches_oracle(which, scale, steps, lib_built, oracle_built):
    """Mode 4 (the convolutional predictor fitted every step) against the oracle's restatement:
    the FP32 features, strip sums, window sums, Cholesky solve and prediction run in the same
    order on both, so every field and every sweep count agree bit for bit, in graph and launch
    modes, from the steps where the fit is still filling its window to those where it acts.  The
    oracle flags every cell on its own; the library skips the tiles without a source nearby, and
    on the periodic meshes (128 and 64 cells wide) those whose reach wraps around take the
    per-cell test."""
    import ora
    import sts
    case = sc.config_case(which, scale=scale, Nt=steps)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        o = ora.Oracle(d, fixed_sweeps=False, warm_start=4)
        assert o.step(steps) == steps
        for use_graph in (True, False):
            g = sts.Solver(d, fixed_sweeps=False, use_graph=use_graph, warm_start=4)
            assert g.step(steps) == steps
            for f in FIELDS:
                np.testing.assert_array_equal(g.field(f), o.field(f), err_msg=f"{f} graph={use_graph}")
            np.testing.assert_array_equal(g.sweep_history(), o.sweeps())
            g.close()


def test_conv_warm_start_gain(lib_built, oracle_built):
    """What the fitted stencil adds: on the supersonic channel (a front that moves a fraction of
    a cell per step), once its window has seen the front move, it takes fewer sweeps than
    quadratic extrapolation and little more than half the cold start's, it steps faster than the
    cold start at the same precision (device time of steps 41-80), and the fields stay within the
    tolerance-level distance of the cold-start run."""
    import ora
    import sts
    case = sc.config_case("channel_ma2.43", scale=0.5, Nt=80)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        cold = ora.Oracle(d, fixed_sweeps=False)
        cold.step(80)
        runs, rate = {}, {}
        for warm in (0, 2, 4):
            g = sts.Solver(d, fixed_sweeps=False, warm_start=warm, precision=sts.MIXED)
            assert g.step(40) == 40  # autotuning and the predictor's window
            n, ms = g.step_timed(40)
            assert n == 40
            rate[warm] = g.Nx * g.Ny * n / (ms / 1e3)
            runs[warm] = (g.sweep_history()[40:].mean(), {f: g.field(f) for f in ("p", "T")})
            g.close()
        hc = cold.sweeps()[40:80].mean()
        print("sweeps per step: cold", hc, "quadratic", runs[2][0], "stencil", runs[4][0])
        print("cell-steps/s on the FP32-correction path: cold %.3e, quadratic %.3e, stencil %.3e"
              % (rate[0], rate[2], rate[4]))
        assert runs[4][0] < runs[2][0]
        assert runs[4][0] <= 0.55 * hc
        # at equal precision the stencil's start is faster than the cold start, sweeps and predictor
        # together (against quadratic extrapolation it is not, on every case: its kernels cost about
        # what the sweeps it saves cost where the flow is smooth)
        assert rate[4] > rate[0]
        for f in ("p", "T"):
            e = np.linalg.norm(runs[4][1][f] - cold.field(f)) / np.linalg.norm(cold.field(f))
            assert e < 1e-6, (f, e)


def test_batch_conv_warm_start_equals_single(lib_built):
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
        b = sts.Batch(dirs, fixed_sweeps=False, warm_start=4, precision=2)
        assert b.step(16) == 16
        for k, d in enumerate(dirs):
            s = sts.Solver(d, fixed_sweeps=False, warm_start=4, precision=2)
            s.step(16)
            for f in FIELDS:
                np.testing.assert_array_equal(b.cases[k].field(f), s.field(f), err_msg=f"case {k} {f}")
            np.testing.assert_array_equal(b.cases[k].sweep_history(), s.sweep_history())
            s.close()
        b.close()
