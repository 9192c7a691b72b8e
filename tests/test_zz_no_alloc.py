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


def _run(meta, f, p0, T0, max_sweeps, fixed, noalloc):
    import sts
    import torch
    F, pt, Tt, keep = device_fields(meta, f, p0, T0)
    fn = sts.pt_sweeps_noalloc if noalloc else sts.pt_sweeps
    n, rp, rT = fn(F, max_sweeps, fixed, 1e-10, 1e-10)
    torch.cuda.synchronize()
    return n, rp, rT, pt.cpu().numpy(), Tt.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_twice(lib_built):
    """Two calls in a row through the C ABI, each equal (bit for bit, the tolerance of these
    FP64 tests) to sts_pt_sweeps on the same inputs; the second call reuses the shared
    scratch left behind by the first."""
    rng = np.random.default_rng(11)
    runs = [(sc.channel_case("c", 60, 10, 2.43, 0.00283, 2.5e-4, 100), False, 40),
            (sc.rayleigh_benard_case("rb", 24, 12, Nt=100), True, 5)]
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


def test_noalloc_rejects_meshes_beyond_its_limit(lib_built):
    import sts
    F = sts.SweepFields()
    F.Nx, F.Ny = 300, 200  # 60000 cells > 32768
    for n in ["cls", "hx", "hy", "p", "T"] + sts.SWEEP_INPUTS:
        setattr(F, n, 8)  # never dereferenced: the size check comes first
    with pytest.raises(sts.StsError) as e:
        sts.pt_sweeps_noalloc(F, 4, True, 1e-8, 1e-8)
    assert e.value.code == sts.STS_ERR_ARG and "limit" in str(e.value)
