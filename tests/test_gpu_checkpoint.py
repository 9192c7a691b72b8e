"""Checkpoint dumps written from the writer thread while the steps go on.

The drop-in run's files (every per-save copy included) are compared with the reference's in
test_gpu_parity.py with asynchronous saves (the default); here the asynchronous and the
synchronous paths are compared with each other, file by file, and snapshots taken with
sts_write_outputs_async are checked to hold the state of the call, not of the steps that
followed it.
"""
import os
import tempfile

import numpy as np
import pytest

import sts_cases as sc
from conftest import golden_case

pytestmark = pytest.mark.gpu


def files_of(d):
    from make_golden import file_digest
    return {f: file_digest(os.path.join(d, f)) for f in sorted(os.listdir(d)) if f != "EnteredData.txt"}


@pytest.mark.parametrize("name", ["channel_newfiles_80x8_resid", "rayleigh_benard_newfiles_txt_32x16_fixed",
                                  "channel_diagnostics_80x8_resid"])
def test_async_and_sync_saves_write_the_same_files(name, lib_built):
    import sts
    case, fixed = golden_case(name)
    out = []
    for async_save in (True, False):
        with tempfile.TemporaryDirectory() as d:
            case.write(d)
            sts.run_case(d, fixed_sweeps=fixed, async_save=async_save)
            out.append(files_of(d))
    assert out[0] == out[1]


def test_async_snapshot_holds_the_state_of_the_call(lib_built):
    """Three saves two steps apart, the third one while both snapshot slots may still be
    pending: every per-save file equals the synchronous save at the same step, and the last
    dumps equal the fields read from the solver at that step."""
    import sts
    case = sc.channel_case("c", 120, 12, 0.3, 0.002, 1e-3, 40, square_x=3.0)
    case.entered.update(ToWriteSolvedDataToNewFiles=1)
    got = []
    for mode in ("async", "sync"):
        with tempfile.TemporaryDirectory() as d:
            case.write(d)
            s = sts.Solver(d, fixed_sweeps=False)
            s.step(3)
            for k in range(3):
                if mode == "async":
                    s.write_outputs_async()
                else:
                    s.write_outputs()
                s.step(2)
            if mode == "async":
                s.wait_outputs()
            got.append(files_of(d))
            # a fourth, synchronous save after the waits: the plain dumps hold the current state
            s.write_outputs()
            u = np.fromfile(os.path.join(d, "u.bin"), dtype=np.float64).reshape(s.Ny, s.Nx)
            np.testing.assert_array_equal(u, s.field("u"))
            s.close()
    assert got[0] == got[1]
    assert sum(1 for f in got[0] if f.startswith("u.0.")) == 3


def test_destroy_writes_pending_saves(lib_built):
    import sts
    case = sc.channel_case("c", 60, 8, 0.3, 0.002, 1e-3, 10)
    with tempfile.TemporaryDirectory() as d:
        case.write(d)
        s = sts.Solver(d, fixed_sweeps=False)
        s.step(2)
        ref = s.field("p")
        s.write_outputs_async()
        s.step(3)
        s.close()  # joins the writer thread after the queued save is on disk
        p = np.fromfile(os.path.join(d, "p.bin"), dtype=np.float64).reshape(ref.shape)
        np.testing.assert_array_equal(p, ref)
