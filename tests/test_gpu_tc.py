"""The BF16 tensor-core GEMM (tcgen05 MMAs fed by TMA, FP32 accumulation in tensor memory) of the
learned warm start's network against an FP32 product of the same BF16 values (numpy)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bf16_bits(x):
    """Round-to-nearest-even BF16 bit patterns of float32 values, and the values they hold."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    return r, (r.astype(np.uint32) << 16).view(np.float32)


def tc_gemm(A, B, relu=False, bias=None):
    import sts
    lib = sts.load()
    M, K = A.shape
    N = B.shape[0]
    a, av = bf16_bits(A)
    b, bv = bf16_bits(B)
    D = np.zeros((M, N), np.float32)
    lib.sts_tc_gemm.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                C.c_int]
    bb = None if bias is None else np.ascontiguousarray(bias, np.float32)
    r = lib.sts_tc_gemm(a.ctypes.data, b.ctypes.data, M, N, K, int(relu), None if bb is None else bb.ctypes.data,
                        D.ctypes.data, 0)
    assert r == 0, r
    ref = av.astype(np.float64) @ bv.astype(np.float64).T
    if bias is not None:
        ref = ref + bias
    if relu:
        ref = np.maximum(ref, 0)
    return D, ref


@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (256, 128, 128), (384, 256, 576), (200, 32, 72), (130, 96, 200),
                                   (1024, 512, 64), (640, 288, 1152)])
def test_tc_gemm_matches_fp32_product(M, N, K, lib_built):
    rng = np.random.default_rng(M * 7 + N * 3 + K)
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((N, K)).astype(np.float32)
    D, ref = tc_gemm(A, B)
    scale = np.sqrt(K)
    np.testing.assert_allclose(D, ref, rtol=1e-4, atol=1e-4 * scale)


def test_tc_gemm_bias_relu_epilogue(lib_built):
    rng = np.random.default_rng(5)
    A = rng.standard_normal((256, 96)).astype(np.float32)
    B = rng.standard_normal((64, 96)).astype(np.float32)
    bias = rng.standard_normal(64).astype(np.float32)
    D, ref = tc_gemm(A, B, relu=True, bias=bias)
    np.testing.assert_allclose(D, ref, rtol=1e-4, atol=1e-3)
    assert (D >= 0).all()
