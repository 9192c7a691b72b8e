"""GB300 library against the reference (golden dumps) and the CPU oracle: bit-exact FP64."""
import hashlib
import os
import tempfile

import numpy as np
import pytest

import sts_cases as sc
from conftest import golden_case

pytestmark = pytest.mark.gpu

NAMES = ["channel_ma0.1_80x8_resid", "channel_ma0.1_80x8_fixed", "channel_ma2.43_60x12_resid",
         "rayleigh_benard_32x16_resid", "channel_circle_120x12_resid", "channel_ma0.1_400x40_resid_5steps",
         "channel_diagnostics_80x8_resid", "rayleigh_benard_diagnostics_txt_32x16_fixed", "channel_newfiles_80x8_resid",
         "rayleigh_benard_newfiles_txt_32x16_fixed", "shipped_example_5steps"]

ALL_FIELDS = ["u", "v", "p", "T", "rho", "sqrt_T", "rho_u", "rho_v", "Fx", "Fy", "D_ux", "D_uy", "D_vx", "D_vy",
              "DTx", "DTy", "Gamma_xf", "Gamma_yf", "ScT1", "apx", "apy", "bpx", "bpy", "u_pseudo", "v_pseudo",
              "d_p_c_12", "d_p_c_34", "Tw_u", "Tw_v"]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("use_graph", [True, False], ids=["graph", "launches"])
@pytest.mark.parametrize("name", NAMES)
def test_dropin_run_matches_reference_dumps(name, use_graph, lib_built, golden_records):
    """The drop-in run writes the same dumps and logs as the reference binary, byte for byte."""
    import sts
    rec = golden_records[name]
    case, fixed = golden_case(name)
    case.entered["Nt_save_temp_data"] = 1
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        sts.run_case(d, fixed_sweeps=fixed, use_graph=use_graph)
        for f in ("u", "v", "p", "Temper", "vol_inf_fb"):
            assert sha(sc.read_field(d, f, rec["Nx"], rec["Ny"])) == rec["sha256_" + f], f
        lines = open(os.path.join(d, "Iterations_in_loops.txt")).read().split("\n")
        assert [int(l.split()[-1]) for l in lines if l.strip() and not l.startswith("it")] == rec["sweeps"]
        assert open(os.path.join(d, "Tmp.txt")).read() == rec["tmp_txt"]
        # every file the reference wrote: mesh, drag coefficients, pressure control, continuity
        for f, h in rec["files"].items():
            assert os.path.exists(os.path.join(d, f)), f
            from make_golden import file_digest
            assert file_digest(os.path.join(d, f)) == h, f


@pytest.mark.parametrize("name", ["channel_ma2.43_60x12_resid", "rayleigh_benard_32x16_resid",
                                  "channel_circle_120x12_resid", "shipped_example_5steps"])
def test_every_array_matches_oracle_step_by_step(name, lib_built, oracle_built):
    import ora
    import sts
    case, fixed = golden_case(name)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        o = ora.Oracle(d, fixed_sweeps=fixed)
        g = sts.Solver(d, fixed_sweeps=fixed)
        for f in ALL_FIELDS:  # after set-up
            np.testing.assert_array_equal(g.field(f), o.field(f), err_msg=f"setup {f}")
        for k in range(4):
            assert g.step(1) == o.step(1) == 1
            for f in ALL_FIELDS:
                np.testing.assert_array_equal(g.field(f), o.field(f), err_msg=f"step {k + 1} {f}")
            np.testing.assert_array_equal(g.stats(), o.stats())
        g.close()


def ratio_corrected_example(steps, **entered):
    """The shipped example with Pressure_ratio_correct = 1, the inflow pressure corrected
    towards the given mean inflow velocity (p_BC_xb_correction_method = 2) and temperature-jump
    walls.  With the pressure boundary, the ratio correction and the local Kn all on, the
    temperature-jump walls read the pressure that the boundary kernel has just corrected, so the
    jump kernel runs after the boundary kernel instead of beside the wall kernels (the one graph
    order no other case takes)."""
    case = sc.shipped_example(steps)
    case.entered.update(Pressure_ratio_correct=1, p_BC_xb_correction_method=2)
    case.entered.update(entered)
    for body in case.polygons:
        body.jump = 1
    return case


@pytest.mark.parametrize("use_graph", [True, False], ids=["graph", "launches"])
def test_ratio_corrected_jump_walls_match_oracle(use_graph, lib_built, oracle_built):
    import ora
    import sts
    with tempfile.TemporaryDirectory() as d:
        ratio_corrected_example(8).write(d)
        o = ora.Oracle(d, fixed_sweeps=False)
        g = sts.Solver(d, fixed_sweeps=False, use_graph=use_graph)
        for k in range(4):
            assert g.step(2) == o.step(2) == 2
            for f in ALL_FIELDS:
                np.testing.assert_array_equal(g.field(f), o.field(f), err_msg=f"step {2 * k + 2} {f}")
            np.testing.assert_array_equal(g.stats(), o.stats())
        np.testing.assert_array_equal(g.sweep_history(), o.sweeps())
        g.close()


def test_ratio_corrected_jump_walls_in_a_batch(lib_built, oracle_built):
    """The batched graph takes the same order when one of its cases needs it."""
    import ora
    import sts
    cases = [ratio_corrected_example(6), ratio_corrected_example(6, Kn=0.02, p_correction_auto=1),
             ratio_corrected_example(6, correct_p_BC_xb=0, p_BC_xb_correction_method=1),
             sc.channel_case("c", 60, 8, 0.3, 0.002, 1e-3, 6)]
    with tempfile.TemporaryDirectory() as root:
        dirs = []
        for k, c in enumerate(cases):
            dirs.append(os.path.join(root, f"c{k}"))
            os.makedirs(dirs[-1])
            c.write(dirs[-1])
        b = sts.Batch(dirs, fixed_sweeps=False)
        assert b.step(6) == 6
        for k, d in enumerate(dirs):
            o = ora.Oracle(d, fixed_sweeps=False)
            assert o.step(6) == 6
            for f in ("u", "v", "p", "T", "rho"):
                np.testing.assert_array_equal(b.cases[k].field(f), o.field(f), err_msg=f"case {k} {f}")
            np.testing.assert_array_equal(b.cases[k].sweep_history(), o.sweeps())
        b.close()


def test_graph_and_launch_modes_agree(lib_built):
    import sts
    case = sc.channel_case("c", 100, 10, 0.3, 0.002, 1e-3, 40)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        a = sts.Solver(d, fixed_sweeps=False, use_graph=True)
        b = sts.Solver(d, fixed_sweeps=False, use_graph=False)
        assert a.step(17) == b.step(17) == 17
        for f in ("u", "v", "p", "T", "rho"):
            np.testing.assert_array_equal(a.field(f), b.field(f))
        np.testing.assert_array_equal(a.sweep_history(), b.sweep_history())


def test_run_stops_at_Nt(lib_built):
    import sts
    case = sc.channel_case("c", 40, 6, 0.3, 0.002, 1e-3, 7)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        s = sts.Solver(d, fixed_sweeps=False)
        assert s.step(5) == 5
        assert s.step(5) == 2  # Nt = 7 ends the run (SIMPLE_TS_MPI.cpp:4442)
        assert s.step(5) == 0


def test_full_size_channel_matches_oracle(lib_built, oracle_built):
    """The 400x40 channel with the square, 60 steps at the 1e-8 residual tolerance."""
    import ora
    import sts
    case = sc.config_case("channel_ma0.1", Nt=60)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        o = ora.Oracle(d, fixed_sweeps=False)
        g = sts.Solver(d, fixed_sweeps=False)
        assert g.step(60) == o.step(60) == 60
        for f in ("u", "v", "p", "T", "rho"):
            np.testing.assert_array_equal(g.field(f), o.field(f), err_msg=f)
        np.testing.assert_array_equal(g.sweep_history(), o.sweeps())


@pytest.mark.parametrize("which,steps", [("channel_2048", 2), ("channel_ma2.43", 3)])
def test_large_meshes_match_oracle(which, steps, lib_built, oracle_built):
    """Meshes with more 32x8 tiles than resident CTAs (the sweep loop's CTAs take several tiles)."""
    import ora
    import sts
    case = sc.config_case(which, Nt=steps)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        o = ora.Oracle(d, fixed_sweeps=False)
        g = sts.Solver(d, fixed_sweeps=False)
        assert g.step(steps) == o.step(steps) == steps
        for f in ("u", "v", "p", "T", "rho"):
            np.testing.assert_array_equal(g.field(f), o.field(f), err_msg=f)
        np.testing.assert_array_equal(g.sweep_history(), o.sweeps())
        g.close()


@pytest.mark.parametrize("nx,ny", [(12, 40), (30, 29)])
def test_tall_periodic_box_matches_oracle(nx, ny, lib_built, oracle_built):
    """Domains taller than wide: the energy source's upper neighbour row is chosen by comparing
    the row with Nx (the reference's own test), so cells from row Nx - 1 up use their own row
    there; the shared-corner form of the assembly must hand those cells to the per-cell form.
    A periodic box also exercises the wrap in x."""
    import ora
    import sts
    case = sc.rayleigh_benard_case("rb_tall", nx, ny, Kn=0.01, ht=1e-3, Nt=12)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        o = ora.Oracle(d, fixed_sweeps=False)
        g = sts.Solver(d, fixed_sweeps=False)
        assert g.step(12) == o.step(12) == 12
        for f in ("u", "v", "p", "T", "rho"):
            np.testing.assert_array_equal(g.field(f), o.field(f), err_msg=f)
        np.testing.assert_array_equal(g.sweep_history(), o.sweeps())
        g.close()


def test_nonfinite_residual_is_reported(lib_built):
    import sts
    case = sc.channel_case("c", 40, 6, 0.3, 0.002, 1e-3, 10)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        s = sts.Solver(d, fixed_sweeps=False)
        s.step(1)
        T = s.field("T")
        T[3, 10] = np.nan
        s.set_field("T", T)
        with pytest.raises(sts.StsError) as e:
            s.step(1)
        assert e.value.code == sts.STS_ERR_NONFINITE


@pytest.mark.parametrize("memory", ["pageable", "pinned"])
@pytest.mark.parametrize("autotune", [False, True], ids=["fixed_shapes", "autotuned"])
def test_step_exchange_equals_three_calls(memory, autotune, lib_built):
    """sts_step_exchange gives the bits of sts_set_state + sts_step + sts_get_state: over several
    calls of one and of several steps, with separate and with the same input and output buffers,
    from the autotuner's first steps (launched one by one) on, and with no steps at all."""
    import sts
    case = sc.channel_case("c", 80, 10, 0.3, 0.002, 1e-3, 80)
    keep = []

    def bufs(ny, nx):
        if memory == "pinned":
            torch = pytest.importorskip("torch")
            ts = [torch.empty((ny, nx), dtype=torch.float64).pin_memory() for _ in range(4)]
            keep.append(ts)
            return [t.numpy() for t in ts]
        return [np.empty((ny, nx)) for _ in range(4)]

    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        a = sts.Solver(d, fixed_sweeps=False, autotune=autotune)
        b = sts.Solver(d, fixed_sweeps=False, autotune=autotune)
        assert a.step(2) == b.step(2) == 2
        ins, outs = bufs(a.Ny, a.Nx), bufs(a.Ny, a.Nx)
        a.get_state_ptr(*[x.ctypes.data for x in ins])
        for rnd, n in enumerate((3, 1, 4, 0, 1, 5, 1, 4)):
            ins[2] *= 1.0 + 1e-7  # a slightly different state goes in every time
            b_in = [x.copy() for x in ins]
            b_out = [np.empty_like(x) for x in ins]
            b.set_state_ptr(*[x.ctypes.data for x in b_in])
            assert b.step(n) == n
            b.get_state_ptr(*[x.ctypes.data for x in b_out])
            o = ins if rnd % 2 else outs
            assert a.step_exchange_ptr(n, [x.ctypes.data for x in ins], [x.ctypes.data for x in o]) == n
            for f, x, y in zip(("u", "v", "p", "T"), o, b_out):
                np.testing.assert_array_equal(x, y, err_msg=f"{f} round {rnd}")
            for f in ALL_FIELDS:
                np.testing.assert_array_equal(a.field(f), b.field(f), err_msg=f"{f} round {rnd}")
            if o is outs:
                for x, y in zip(ins, outs):
                    x[...] = y
        a.close()
        b.close()


@pytest.mark.parametrize("which", ["channel", "jump_walls", "periodic_box"])
def test_one_step_exchanges_match_oracle(which, lib_built, oracle_built):
    """One step per sts_step_exchange call with pinned buffers: the new state goes out to the host
    beside the flux kernel and the zero-gradient copies of p and T move into the boundary kernel.
    Every array after every step, the statistics and the sweep counts equal the oracle's, and the
    state that comes out is the library's state (the ratio-corrected jump walls write p and T on
    the walls; the periodic box wraps)."""
    torch = pytest.importorskip("torch")
    import ora
    import sts
    if which == "channel":
        case = sc.channel_case("c", 120, 12, 0.5, 0.002, 1e-3, 20)
    elif which == "jump_walls":
        case = ratio_corrected_example(20)
    else:
        case = sc.config_case("rayleigh_benard", scale=0.125, Nt=20)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        o = ora.Oracle(d, fixed_sweeps=False)
        g = sts.Solver(d, fixed_sweeps=False, autotune=False)  # every step in the graph
        assert g.step(2) == o.step(2) == 2
        ts = [torch.empty((g.Ny, g.Nx), dtype=torch.float64).pin_memory() for _ in range(8)]
        ins, outs = [t.numpy() for t in ts[:4]], [t.numpy() for t in ts[4:]]
        g.get_state_ptr(*[x.ctypes.data for x in ins])
        for k in range(6):
            assert g.step_exchange_ptr(1, [x.ctypes.data for x in ins], [x.ctypes.data for x in outs]) == 1
            assert o.step(1) == 1
            for f in ALL_FIELDS:
                np.testing.assert_array_equal(g.field(f), o.field(f), err_msg=f"step {k + 3} {f}")
            for f, x in zip(("u", "v", "p", "T"), outs):
                np.testing.assert_array_equal(x, o.field(f), err_msg=f"state out, step {k + 3} {f}")
            np.testing.assert_array_equal(g.stats(), o.stats())
            ins, outs = outs, ins
        np.testing.assert_array_equal(g.sweep_history(), o.sweeps())
        g.close()


@pytest.mark.parametrize("memory", ["pageable", "pinned"])
def test_state_exchange_equals_field_calls(memory, lib_built):
    """sts_get_state / sts_set_state move the same bytes as four get/set_field calls, and a run
    continued from a state set either way is the same run.  Pinned host buffers take the
    library's direct kernel path, ordinary ones the copy engines."""
    import sts
    case = sc.channel_case("c", 80, 10, 0.3, 0.002, 1e-3, 40)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        a = sts.Solver(d, fixed_sweeps=False)
        b = sts.Solver(d, fixed_sweeps=False)
        assert a.step(12) == b.step(12) == 12
        if memory == "pinned":
            torch = pytest.importorskip("torch")
            pins = [torch.empty((a.Ny, a.Nx), dtype=torch.float64).pin_memory() for _ in range(4)]
            bufs = [t.numpy() for t in pins]
        else:
            bufs = [np.empty((a.Ny, a.Nx)) for _ in range(4)]
        a.get_state_ptr(*[x.ctypes.data for x in bufs])
        for f, x in zip(("u", "v", "p", "T"), bufs):
            np.testing.assert_array_equal(x, a.field(f), err_msg=f)
        bufs[2] *= 1.0 + 1e-6  # perturb p; the same state goes in both ways
        a.set_state_ptr(*[x.ctypes.data for x in bufs])
        for f, x in zip(("u", "v", "p", "T"), bufs):
            b.set_field(f, x)
        assert a.step(5) == b.step(5) == 5
        for f in ("u", "v", "p", "T", "rho"):
            np.testing.assert_array_equal(a.field(f), b.field(f), err_msg=f)
        a.close()
        b.close()
