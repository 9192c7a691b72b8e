// BF16 tensor-core GEMM of the learned warm start's network (tcgen05 + TMA, sm_103a).
//
// D[M x N] = epilogue(A[M x K] * B[N x K]^T): A and B row-major BF16 with K contiguous (both
// operands K-major), FP32 accumulation in tensor memory.  One CTA of 128 threads per 128 x BN tile
// of D: warp 0 (one thread) streams 128 x 64 tiles of A and BN x 64 tiles of B into a 3- or 4-stage
// shared-memory ring with TMA (128-byte swizzle, zero fill past the edges); warp 1 (one thread)
// issues four 128 x BN x 16 tcgen05 MMAs per stage and releases the stage with tcgen05.commit;
// then all four warps read the accumulator rows of their tensor-memory lanes (warp w holds rows
// 32 w .. 32 w + 31) and apply the epilogue: scale, bias, ReLU, a ReLU-derivative gate, BF16 or
// FP32 store (FP32 may add to what is there).  The convolutions of the network are GEMMs over
// im2col rows (sts_unet.cu).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>

#include "sts_net.h"
#include "sts_tc.cuh"

namespace sts {
namespace {

constexpr int kBM = 128, kBK = 64;
constexpr uint32_t kWaitLimit = 1u << 22;  // polls of a pipeline barrier before the CTA gives up

// Pipeline depth: 4 stages for 256-wide tiles (one CTA per SM), 3 for narrower ones so that two or
// three CTAs fit on an SM and one's epilogue overlaps another's main loop.
template <int BN>
struct GemmSmem {
  static constexpr int kStages = BN >= 256 ? 4 : 3;
  static constexpr uint32_t kA = kBM * kBK * 2, kB = BN * kBK * 2;
  static constexpr uint32_t kBytes = kStages * (kA + kB) + 1024 + 256;
};

template <int BN>
__global__ void __launch_bounds__(128)
    k_gemm_tn(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, int M, int N, int K,
              GemmEpilogue e, unsigned* err) {
  using L = GemmSmem<BN>;
  constexpr int kStages = L::kStages;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  unsigned char* sa = smem;
  unsigned char* sb = smem + kStages * L::kA;
  uint64_t* full = (uint64_t*)(sb + kStages * L::kB);
  uint64_t* empty = full + kStages;
  uint64_t* done = empty + kStages;
  uint32_t* tslot = (uint32_t*)(done + 1);
  int* failed = (int*)(tslot + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * BN;
  const int nk = (K + kBK - 1) / kBK;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; s++) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(done, 1);
    *failed = 0;
    tc::fence_barrier_init();
  }
  if (warp == 1) tc::tmem_alloc(tslot, BN);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  if (warp == 0 && lane == 0) {  // TMA producer
    for (int kb = 0; kb < nk; kb++) {
      const int s = kb % kStages;
      const uint32_t ph = (uint32_t)(kb / kStages) & 1u;
      if (!tc::mbar_wait(&empty[s], ph ^ 1u, kWaitLimit)) {
        atomicExch(failed, 1);
        break;
      }
      tc::mbar_arrive_expect_tx(&full[s], L::kA + L::kB);
      tc::tma_load_2d(sa + s * L::kA, &ta, kb * kBK, m0, &full[s]);
      tc::tma_load_2d(sb + s * L::kB, &tb, kb * kBK, n0, &full[s]);
    }
  } else if (warp == 1 && lane == 0) {  // MMA issuer
    const uint32_t idesc = tc::idesc_bf16_f32(kBM, BN);
    for (int kb = 0; kb < nk; kb++) {
      const int s = kb % kStages;
      const uint32_t ph = (uint32_t)(kb / kStages) & 1u;
      if (!tc::mbar_wait(&full[s], ph, kWaitLimit)) {
        atomicExch(failed, 1);
        break;
      }
      tc::fence_after_sync();
      const uint32_t a0 = tc::smem_u32(sa + s * L::kA), b0 = tc::smem_u32(sb + s * L::kB);
#pragma unroll
      for (int k = 0; k < kBK / 16; k++)
        tc::mma_bf16(tmem, tc::sw128_desc(a0 + 32u * k), tc::sw128_desc(b0 + 32u * k), idesc, (kb | k) ? 1u : 0u);
      tc::mma_commit(&empty[s]);
    }
    tc::mma_commit(done);  // arrives once every MMA issued above has completed
  }
  __syncwarp();
  if (!tc::mbar_wait(done, 0u, kWaitLimit)) atomicExch(failed, 1);
  tc::fence_after_sync();
  __syncwarp();
  const bool ok = (*(volatile int*)failed) == 0;
  const int row = m0 + warp * 32 + lane;
#pragma unroll 1
  for (int c = 0; c < BN; c += 16) {
    float v[16];
    tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
    const int n = n0 + c;
    if (!ok || row >= M || n >= N) continue;
#pragma unroll
    for (int q = 0; q < 16; q++) {
      float x = e.alpha * v[q];
      if (e.bias && n + q < N) x += e.bias[n + q];
      if (e.relu) x = fmaxf(x, 0.f);
      if (e.gate && n + q < N && !(__bfloat162float(((const __nv_bfloat16*)e.gate)[(size_t)row * e.ldg + n + q]) > 0.f))
        x = 0.f;
      v[q] = x;
    }
    if (e.out_bf16) {
      __nv_bfloat16* o = (__nv_bfloat16*)e.out + (size_t)row * e.ldo + n;
      if (n + 16 <= N && (e.ldo % 8) == 0) {
        uint32_t w[8];
#pragma unroll
        for (int q = 0; q < 8; q++) {
          __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * q], v[2 * q + 1]);
          w[q] = *(uint32_t*)&h;
        }
        ((uint4*)o)[0] = make_uint4(w[0], w[1], w[2], w[3]);
        ((uint4*)o)[1] = make_uint4(w[4], w[5], w[6], w[7]);
      } else {
        for (int q = 0; q < 16 && n + q < N; q++) o[q] = __float2bfloat16_rn(v[q]);
      }
    } else {
      float* o = (float*)e.out + (size_t)row * e.ldo + n;
      for (int q = 0; q < 16 && n + q < N; q++) o[q] = e.accumulate ? o[q] + v[q] : v[q];
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 1) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, BN);
  }
  if (threadIdx.x == 0 && *(volatile int*)failed) atomicOr(err, 1u);
}

// The driver's tensor-map encoder, looked up through the runtime (the library does not link the
// driver library itself).
PFN_cuTensorMapEncodeTiled_v12000 encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  }
  return fn;
}

// Tensor map of a row-major BF16 matrix [rows][ld] read in boxes of 64 K-values x box_rows rows.
bool encode(CUtensorMap* m, const void* p, int K, int rows, int ld, int box_rows) {
  auto fn = encoder();
  if (!fn) return false;
  cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
  cuuint32_t es[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(p), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN>
cudaError_t launch(const void* A, int lda, const void* B, int ldb, int M, int N, int K, const GemmEpilogue& e,
                   unsigned* err, cudaStream_t s) {
  CUtensorMap ta, tb;
  if (!encode(&ta, A, K, M, lda, kBM) || !encode(&tb, B, K, N, ldb, BN)) return cudaErrorInvalidValue;
  static bool attr = false;
  if (!attr) {
    const cudaError_t r =
        cudaFuncSetAttribute(k_gemm_tn<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GemmSmem<BN>::kBytes);
    if (r != cudaSuccess) return r;
    attr = true;
  }
  dim3 grid((M + kBM - 1) / kBM, (N + BN - 1) / BN);
  k_gemm_tn<BN><<<grid, 128, GemmSmem<BN>::kBytes, s>>>(ta, tb, M, N, K, e, err);
  return cudaGetLastError();
}

}  // namespace

cudaError_t gemm_bf16_tn(const void* A, int lda, const void* B, int ldb, int M, int N, int K, const GemmEpilogue& e,
                         unsigned* err, cudaStream_t s) {
  if (M <= 0 || N <= 0 || K <= 0) return cudaSuccess;
  // TMA: 16-byte aligned bases and row pitches (K values: multiples of 8)
  if ((lda % 8) || (ldb % 8) || ((uintptr_t)A % 16) || ((uintptr_t)B % 16) || K > lda || K > ldb)
    return cudaErrorInvalidValue;
  if (N <= 32) return launch<32>(A, lda, B, ldb, M, N, K, e, err, s);
  if (N <= 64) return launch<64>(A, lda, B, ldb, M, N, K, e, err, s);
  if (N <= 128) return launch<128>(A, lda, B, ldb, M, N, K, e, err, s);
  return launch<256>(A, lda, B, ldb, M, N, K, e, err, s);
}

}  // namespace sts

// ---------------------------------------------------------------------------
// C ABI: self-check of the tensor-core GEMM on host data.
#include "../../include/sts_gb300.h"

extern "C" int sts_tc_gemm(const unsigned short* A, const unsigned short* B, int M, int N, int K, int relu,
                           const float* bias, float* D, int device) {
  if (!A || !B || !D || M <= 0 || N <= 0 || K <= 0 || (K % 8)) return STS_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return STS_ERR_CUDA;
  void *dA = nullptr, *dB = nullptr, *dD = nullptr, *dbias = nullptr;
  unsigned* derr = nullptr;
  unsigned herr = 0;
  cudaError_t r = cudaMalloc(&dA, (size_t)M * K * 2);
  if (r == cudaSuccess) r = cudaMalloc(&dB, (size_t)N * K * 2);
  if (r == cudaSuccess) r = cudaMalloc(&dD, (size_t)M * N * 4);
  if (r == cudaSuccess) r = cudaMalloc(&dbias, (size_t)N * 4);
  if (r == cudaSuccess) r = cudaMalloc(&derr, 4);
  if (r == cudaSuccess) r = cudaMemcpy(dA, A, (size_t)M * K * 2, cudaMemcpyHostToDevice);
  if (r == cudaSuccess) r = cudaMemcpy(dB, B, (size_t)N * K * 2, cudaMemcpyHostToDevice);
  if (r == cudaSuccess && bias) r = cudaMemcpy(dbias, bias, (size_t)N * 4, cudaMemcpyHostToDevice);
  if (r == cudaSuccess) r = cudaMemset(derr, 0, 4);
  if (r == cudaSuccess) {
    sts::GemmEpilogue e;
    e.out = dD;
    e.ldo = N;
    e.relu = relu;
    e.bias = bias ? (const float*)dbias : nullptr;
    r = sts::gemm_bf16_tn(dA, K, dB, K, M, N, K, e, derr, 0);
  }
  if (r == cudaSuccess) r = cudaMemcpy(D, dD, (size_t)M * N * 4, cudaMemcpyDeviceToHost);
  if (r == cudaSuccess) r = cudaMemcpy(&herr, derr, 4, cudaMemcpyDeviceToHost);
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dD);
  cudaFree(dbias);
  cudaFree(derr);
  if (r != cudaSuccess) return STS_ERR_CUDA;
  return herr ? STS_ERR_TIMEOUT : STS_OK;
}
