"""The drop-in executable run as a process, and the reference's wall-clock stop.

* ``simple_ts_gb300`` (simple-ts_gb300/csrc/sts_main.cpp) is started in a case directory like the
  serial reference binary and must write the reference's dumps and logs byte for byte.
* ``max_time_for_solve`` (EnteredData.txt) ends the reference's run after the first step that ends
  at or after start + max_time_for_solve hours (SIMPLE_TS_MPI.cpp:1799, :2010, :4443); the drop-in
  run obeys it, and its final dumps are the reference's dumps after the same number of steps.
"""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import sts_cases as sc
from conftest import ROOT, golden_case

pytestmark = pytest.mark.gpu

EXE = os.path.join(ROOT, "simple-ts_gb300", "_build", "simple_ts_gb300")


@pytest.mark.parametrize("name", ["channel_ma2.43_60x12_resid", "channel_newfiles_80x8_resid",
                                  "rayleigh_benard_diagnostics_txt_32x16_fixed", "shipped_example_5steps"])
def test_executable_matches_reference(name, lib_built, golden_records):
    from make_golden import digest, file_digest
    rec = golden_records[name]
    case, fixed = golden_case(name)
    case.entered["Nt_save_temp_data"] = 1
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        args = [EXE, d] + ([] if fixed else ["--residual"])
        r = subprocess.run(args, capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        for f in ("u", "v", "p", "Temper", "vol_inf_fb"):
            assert digest(sc.read_field(d, f, rec["Nx"], rec["Ny"])) == rec["sha256_" + f], f
        assert open(os.path.join(d, "Tmp.txt")).read() == rec["tmp_txt"]
        for f, h in rec["files"].items():
            assert file_digest(os.path.join(d, f)) == h, f


def _steps_taken(d, ht):
    return int(round(float(open(os.path.join(d, "it_begin.txt")).read().split()[0]) / ht))


def _oracle_dumps(case, steps):
    """The CPU oracle's drop-in run of `case` for `steps` steps (no time limit): final dumps."""
    import ora
    c = sc.Case(case.name, dict(case.entered), case.polygons, case.circles, case.restart)
    c.entered.update(Nt=steps, max_time_for_solve=1e6, Nt_save_solved_data=steps, Nt_save_temp_data=steps)
    with tempfile.TemporaryDirectory() as d:
        c.write(d)
        ora.run_cli(d, fixed_sweeps=False)
        return {f: sc.read_field(d, f, c.Nx, c.Ny) for f in ("u", "v", "p", "Temper")}


@pytest.mark.parametrize("hours", [0.0, 2e-4])
def test_wallclock_limit_ends_the_run(hours, lib_built, oracle_built):
    """max_time_for_solve = 0 ends the run after its first step (the loop is a do-while);
    0.72 s ends it within about a second, long before Nt.  Either way the final dumps are the
    oracle's after the steps taken."""
    import sts
    ht = 1e-3
    case = sc.channel_case("c", 60, 12, 0.5, 0.003, ht, 10 ** 7)
    case.entered.update(max_time_for_solve=hours)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        sts.run_case(d, fixed_sweeps=False)
        n = _steps_taken(d, ht)
        if hours == 0.0:
            assert n == 1
        assert 1 <= n < 10 ** 7
        want = _oracle_dumps(case, n)
        for f, a in want.items():
            np.testing.assert_array_equal(sc.read_field(d, f, case.Nx, case.Ny), a, err_msg=f)
        # the rewritten EnteredData.txt records the run's time in hours, as the reference's does
        e = sc.read_entered_data(os.path.join(d, "EnteredData.txt"))
        assert 0.0 <= e["max_time_for_solve"] < 0.01
