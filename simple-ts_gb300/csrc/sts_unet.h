// U-Net of the learned warm start (sts_unet.cu): BF16 weights and activations, FP32 accumulation,
// forward, backward and Adam on the GPU; every convolution a tcgen05 GEMM.
#pragma once
#include <cuda_runtime.h>

#include <memory>
#include <vector>

namespace sts {

struct UNetImpl;

class UNet {
 public:
  // in_ch input and out_ch output channels per pixel (both at most 8 here: the input is padded to
  // 8 channels, the head to 8 outputs), base channels C0 (a multiple of 8), levels L >= 1; buffers
  // for batches of up to max_batch crops of H x W pixels (H and W multiples of 2^(L-1)).  Weights
  // are drawn from `seed` (uniform, He-scaled).  Errors are reported through ok().
  UNet(int in_ch, int out_ch, int base_ch, int levels, int max_batch, int H, int W, unsigned long long seed,
       cudaStream_t s);
  ~UNet();
  bool ok() const;
  const char* error() const;
  long long param_count() const;
  // FP32 master weights (layer order: every conv's Wt [9 C_in][C_out] then its bias, the head's
  // Wt [C0][8] and bias [8]); set_params also refreshes the BF16 copies.
  cudaError_t get_params(float* host) const;
  cudaError_t set_params(const float* host);
  // Forward on device input x [B][H][W][in_ch] (FP32); y [B][H][W][out_ch] (FP32, device).
  cudaError_t forward(const float* x, int B, float* y);
  // After forward: the loss against target [B][H][W][out_ch] with per-pixel weights (NULL: 1),
  // backward into the gradient buffer (*loss_dev receives the loss, device FP32).
  cudaError_t backward_mse(const float* target, const float* weight, int B, float* loss_dev);
  // After forward: only the loss (as backward_mse computes it), of the forward's output or, with
  // zero_prediction, of an output of zeros (the forward's output is then overwritten).
  cudaError_t loss(const float* target, const float* weight, int B, float* loss_dev, bool zero_prediction);
  // Backward from a given output gradient gy [B][H][W][out_ch] (device FP32).
  cudaError_t backward(const float* gy, int B);
  const float* grads() const;  // device, param_count() values in the layout of get_params
  // One Adam step with learning rate lr on the current gradients.
  cudaError_t adam(float lr);
  unsigned* error_flag() const;  // device word; bit 0: a GEMM pipeline wait gave up
  void set_stream(cudaStream_t s);  // the stream later calls queue their work on

 private:
  std::unique_ptr<UNetImpl> d;
};

}  // namespace sts
