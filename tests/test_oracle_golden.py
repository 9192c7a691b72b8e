"""The CPU oracle against the golden dumps of the reference solver (tests/golden)."""
import hashlib
import os
import tempfile

import numpy as np
import pytest

import sts_cases as sc
from conftest import GOLDEN, golden_case

NAMES = ["channel_ma0.1_80x8_resid", "channel_ma0.1_80x8_fixed", "channel_ma2.43_60x12_resid",
         "rayleigh_benard_32x16_resid", "channel_circle_120x12_resid", "channel_ma0.1_400x40_resid_5steps",
         "channel_diagnostics_80x8_resid", "rayleigh_benard_diagnostics_txt_32x16_fixed", "channel_newfiles_80x8_resid",
         "rayleigh_benard_newfiles_txt_32x16_fixed", "shipped_example_5steps"]


def file_sha(path):
    from make_golden import file_digest
    return file_digest(path)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference_dumps(name, oracle_built, golden_records):
    import ora
    rec = golden_records[name]
    case, fixed = golden_case(name)
    case.entered["Nt_save_temp_data"] = 1
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        ora.run_cli(d, fixed_sweeps=fixed)
        for f in ("u", "v", "p", "Temper", "vol_inf_fb"):
            a = sc.read_field(d, f, rec["Nx"], rec["Ny"])
            assert sha(a) == rec["sha256_" + f], f
        if rec["arrays"]:
            g = np.load(os.path.join(GOLDEN, name + ".npz"))
            for f in ("u", "v", "p", "Temper"):
                np.testing.assert_array_equal(sc.read_field(d, f, rec["Nx"], rec["Ny"]), g[f])
        assert open(os.path.join(d, "Tmp.txt")).read() == rec["tmp_txt"]
        lines = open(os.path.join(d, "Iterations_in_loops.txt")).read().split("\n")
        sweeps = [int(l.split()[-1]) for l in lines if l.strip() and not l.startswith("it")]
        assert sweeps == rec["sweeps"]
        # every file the reference wrote (mesh, drag-coefficient, pressure-control and
        # continuity outputs included), byte for byte
        for f, h in rec["files"].items():
            assert os.path.exists(os.path.join(d, f)), f
            assert file_sha(os.path.join(d, f)) == h, f


def test_oracle_library_matches_cli(oracle_built, golden_records):
    """The in-process oracle (the checker of the GPU tests) steps exactly like its CLI."""
    import ora
    rec = golden_records["channel_ma2.43_60x12_resid"]
    case, fixed = golden_case(rec["name"])
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        o = ora.Oracle(d, fixed_sweeps=fixed)
        assert o.step(10 ** 6) == rec["steps"]
        o.finish()
        assert list(o.sweeps()) == rec["sweeps"]
        assert sha(o.field("u")) == rec["sha256_u"]
        assert sha(o.field("p")) == rec["sha256_p"]


def test_oracle_conservation_sums_definition(oracle_built):
    """The oracle's conservation sums of a restart state equal the same sums taken with numpy
    (to rounding: numpy sums in another order)."""
    import tempfile
    import numpy as np
    import ora
    import sts_cases as sc
    case = sc.rayleigh_benard_case("rb", 40, 20, Nt=5)
    rng = np.random.default_rng(3)
    Ny, Nx = case.restart["u"].shape
    case.restart["u"] = 0.01 * rng.standard_normal((Ny, Nx))
    case.restart["v"] = 0.01 * rng.standard_normal((Ny, Nx))
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        o = ora.Oracle(d, fixed_sweeps=False)
        got = o.conservation()
        u, v, T, rho = o.field("u"), o.field("v"), o.field("T"), o.field("rho")
        hx, hy = o.field("hx"), o.field("hy")
        fluid = case.restart["vol_inf_fb"] == 0
        A = hy[:, None] * hx[None, :]
        ue = np.concatenate([u[:, 1:], u[:, -1:]], axis=1)
        vn = np.concatenate([v[1:, :], v[-1:, :]], axis=0)
        uc, vc = 0.5 * (u + ue), 0.5 * (v + vn)
        m = rho * A
        want = [m, m * uc, m * vc, m * T / (5.0 / 3.0 - 1.0), m * (uc ** 2 + vc ** 2)]
        want = np.array([x[fluid].sum() for x in want])
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-15)


@pytest.mark.parametrize("ranks", [2, 4])
def test_reference_mpi_build_equals_serial(ranks, oracle_built, golden_records):
    """The reference's own MPI build, run on the minimal shared-memory MPI (oracle/mpishim) with one
    strip of the mesh per rank, writes the serial reference's dumps and logs byte for byte: the
    multi-core CPU baseline is the reference itself."""
    import tempfile
    import sts_cases as sc
    from build_oracle import build_reference_mpi
    from make_golden import digest
    if build_reference_mpi() is None:
        pytest.skip("the reference sources are not present")
    import reference_mpi
    rec = golden_records["channel_ma2.43_60x12_resid"]
    case, _ = golden_case("channel_ma2.43_60x12_resid")
    case.entered["Nt_save_temp_data"] = 1
    with tempfile.TemporaryDirectory() as d:
        reference_mpi.run(case, d, ranks, timeout=300)
        for f in ("u", "v", "p", "Temper"):
            assert digest(sc.read_field(d, f, rec["Nx"], rec["Ny"])) == rec["sha256_" + f], f
        assert open(os.path.join(d, "Tmp.txt")).read() == rec["tmp_txt"]
