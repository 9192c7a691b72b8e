// The learned warm start's network: BF16 tensor-core GEMM (sts_net.cu) and the U-Net built on it
// (sts_unet.cu).
#pragma once
#include <cuda_runtime.h>

namespace sts {

// Epilogue of gemm_bf16_tn, applied per element of D = A * B^T (row m, column n):
//   x = alpha * acc + bias[n] (bias optional); x = max(x, 0) if relu; x = 0 where
//   gate[m * ldg + n] <= 0 (gate optional: the derivative of a ReLU whose output is gate);
//   stored to out[m * ldo + n] as BF16 (out_bf16) or FP32 (added to the value there if accumulate).
struct GemmEpilogue {
  void* out = nullptr;
  int ldo = 0;
  int out_bf16 = 0;
  int accumulate = 0;
  float alpha = 1.f;
  const float* bias = nullptr;
  int relu = 0;
  const void* gate = nullptr;  // __nv_bfloat16
  int ldg = 0;
};

// D[M x N] = epilogue(A[M x K] * B[N x K]^T) on `s`: A and B row-major BF16 (leading dimensions
// lda, ldb in elements, multiples of 8; bases 16-byte aligned), FP32 accumulation on the tensor
// cores (tcgen05).  *err (device) receives bit 0 if a pipeline wait gave up.
cudaError_t gemm_bf16_tn(const void* A, int lda, const void* B, int ldb, int M, int N, int K, const GemmEpilogue& e,
                         unsigned* err, cudaStream_t s);

}  // namespace sts
