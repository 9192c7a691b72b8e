"""sts_pt_sweeps_noalloc, the sweep loop for callers that must not allocate device memory.

Such callers (an application whose device memory is reserved by its own pool, or a
time-critical loop that cannot take the stall of an allocation) give the library their
input and output arrays and nothing else; the scratch lives in a fixed array inside the
library.  This file is collected last so that a run stopping at the first failure has
already run every other test.  It must pass alone in a fresh process and after the rest.
"""
import numpy as np
import pytest

import sts_cases as sc
from test_gpu_sweeps import device_fields, sweep_inputs

pytestmark = pytest.mark.gpu


def _cudart():
    """The CUDA runtime of the toolkit, for the device's memory counters."""
    import ctypes
    import glob
    for path in sorted(glob.glob("/usr/local/cuda/lib64/libcudart.so*")):
        try:
            return ctypes.CDLL(path)
        except OSError:
            pass
    pytest.skip("no CUDA runtime library to read the device memory counters")


def _memory_state(rt, reset_high=False):
    """(free device bytes, bytes the default stream-ordered pool has reserved, the pool's
    high-water mark of bytes in use): what any cudaMalloc or cudaMallocAsync would change."""
    import ctypes
    free, total = ctypes.c_size_t(), ctypes.c_size_t()
    assert rt.cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total)) == 0
    pool = ctypes.c_void_p()
    assert rt.cudaDeviceGetDefaultMemPool(ctypes.byref(pool), 0) == 0
    reserved, used_high = ctypes.c_uint64(), ctypes.c_uint64()
    if reset_high:  # cudaMemPoolAttrUsedMemHigh = 8: setting it to 0 restarts the high-water mark
        assert rt.cudaMemPoolSetAttribute(pool, 8, ctypes.byref(ctypes.c_uint64(0))) == 0
    assert rt.cudaMemPoolGetAttribute(pool, 5, ctypes.byref(reserved)) == 0  # ReservedMemCurrent
    assert rt.cudaMemPoolGetAttribute(pool, 8, ctypes.byref(used_high)) == 0  # UsedMemHigh
    return free.value, reserved.value, used_high.value


def _run(meta, f, p0, T0, max_sweeps, fixed, noalloc):
    import sts
    import torch
    F, pt, Tt, keep = device_fields(meta, f, p0, T0)
    fn = sts.pt_sweeps_noalloc if noalloc else sts.pt_sweeps
    mem = None
    if noalloc:
        rt = _cudart()
        torch.cuda.synchronize()
        before = _memory_state(rt, reset_high=True)
    n, rp, rT = fn(F, max_sweeps, fixed, 1e-10, 1e-10)
    torch.cuda.synchronize()
    if noalloc:
        mem = (before, _memory_state(rt))
    return n, rp, rT, pt.cpu().numpy(), Tt.cpu().numpy(), mem


def test_noalloc_matches_allocating_entry_point_twice(lib_built):
    """Two calls in a row through the C ABI, each equal (bit for bit, the tolerance of these
    FP64 tests) to sts_pt_sweeps on the same inputs; the second call reuses the shared
    scratch left behind by the first."""
    rng = np.random.default_rng(11)
    runs = [(sc.channel_case("c", 60, 10, 2.43, 0.00283, 2.5e-4, 100), False, 40),
            (sc.rayleigh_benard_case("rb", 24, 12, Nt=100), True, 5)]
    calls = 0
    for case, fixed, nmax in runs:
        meta, f, p, T = sweep_inputs(case)
        assert meta["Nx"] * meta["Ny"] <= 32768
        p0 = p * (1 + 1e-4 * rng.standard_normal(p.shape))
        T0 = T * (1 + 1e-4 * rng.standard_normal(T.shape))
        want = _run(meta, f, p0, T0, nmax, fixed, noalloc=False)
        got = _run(meta, f, p0, T0, nmax, fixed, noalloc=True)
        assert got[:3] == want[:3]
        np.testing.assert_array_equal(got[3], want[3])
        np.testing.assert_array_equal(got[4], want[4])
        # nothing was allocated: the stream-ordered pool saw no allocation during the call and
        # holds what it held, and the device's free memory is unchanged (checked from the second
        # call on: the first call in a process may load the library's device code, which the
        # CUDA runtime places in device memory)
        (free0, reserved0, _), (free1, reserved1, used_high) = got[5]
        assert reserved1 == reserved0 and used_high == 0
        if calls:
            assert free1 == free0
        calls += 1


def test_noalloc_rejects_meshes_beyond_its_limit(lib_built):
    import sts
    F = sts.SweepFields()
    F.Nx, F.Ny = 300, 200  # 60000 cells > 32768
    for n in ["cls", "hx", "hy", "p", "T"] + sts.SWEEP_INPUTS:
        setattr(F, n, 8)  # never dereferenced: the size check comes first
    with pytest.raises(sts.StsError) as e:
        sts.pt_sweeps_noalloc(F, 4, True, 1e-8, 1e-8)
    assert e.value.code == sts.STS_ERR_ARG and "limit" in str(e.value)
