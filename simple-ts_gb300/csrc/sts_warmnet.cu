// Network warm start (warm_start 5): the learned 3x3 stencil of warm_start 4, corrected on a window
// around the moving front by the U-Net (sts_unet.cu, BF16 tcgen05 GEMMs), which is trained on the GPU
// on step pairs the solver itself produces.
//
// No counterpart in the reference, which starts every step's sweeps from the previous step's p and
// T.  Plain Jacobi still iterates to the same residual tolerance; only the initial iterate changes.
//
// Per step, after the sweeps and the stencil's kernels (k_conv_next has stored the step's
// difference D_r = x_{n+1} - x_n and its maximum; k_conv_predict has flagged the active cells and
// put the stencil's start x_{n+1} + S in cnext there):
//   k_net_target: the window gathered at the previous step gets its target, the stencil's error on
//     its flagged cells in units of that window's scale, (D_r - S) / s, and the largest error;
//   k_net_head (one thread): the completed pair is counted; the coming window's slot of the replay
//     ring and its scales (inputs: max |D_r| per field; target: that largest error);
//   k_net_locate: the cell of the largest |D_r| of p (lowest index among equals);
//   k_net_gather: a window of H x W cells centred there (clamped to the mesh): the network input
//     (8 channels: D_r, D_r-1, D_r-2 of p and T over their field's max |D_r|, and the stencil's
//     predicted change S over the same), S and the flags, into the inference buffer and the slot;
//   k_net_commit (one thread): the window's origin;
//   the U-Net forward on the inference buffer (a child graph);
//   k_net_apply: where the network is enabled, cnext += s * output on the window's flagged cells,
//     field by field, if on the window completed this step the network's correction had left a
//     smaller largest error than the stencil's own (the gate: the sweep count follows the largest
//     error of the start, and consecutive windows of a front are alike; T's gate stays shut, see
//     kNetGateMarginT).  k_net_target measures both on that window from its target and the output
//     still held from its forward pass.
// Training (sts_warm_net_train) draws batches of completed slots from the ring between steps.
#include <cuda_runtime.h>

#include <cstdint>

#include "sts_common.cuh"
#include "sts_warmnet.h"

namespace sts {

__global__ void k_net_target(Geo g, NetState* ns, NetBuffers nb) {
  const int H = nb.H, W = nb.W;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (!ns->have_win) return;
  const unsigned r = g.ctl->warm_ready;
  float e[kNetOut] = {0.f, 0.f}, es[kNetOut] = {0.f, 0.f}, en[kNetOut] = {0.f, 0.f};
  if (k < H * W) {
    const int i = ns->i0 + k % W, j = ns->j0 + k / W, n = i + j * g.Nx;
    float* tgt = nb.replay + (size_t)ns->slot * nb.slot_floats + (size_t)H * W * kNetIn;
    float* wp = tgt + (size_t)H * W * kNetOut + k;
    const float* S = tgt + (size_t)H * W * (kNetOut + 1);
    const bool flagged = *wp > 0.f;
    bool outlier = false;
    for (int f = 0; f < kNetOut; f++) {
      const float err = flagged ? g.cD[f][r % kConvRing][n] - S[(size_t)k * kNetOut + f] : 0.f;
      const float t = err / ns->s[f];
      outlier = outlier || !(fabsf(t) <= kNetTargetClip);
      tgt[(size_t)k * kNetOut + f] = fminf(fmaxf(t, -kNetTargetClip), kNetTargetClip);
      e[f] = fabsf(err);
      if (flagged) {  // the gate's errors: the network's output for this window is still in infer_out
        const float o = fminf(fmaxf(nb.infer_out[(size_t)k * kNetOut + f], -kNetTargetClip), kNetTargetClip);
        es[f] = fabsf(t);
        en[f] = fabsf(t - o);
      }
    }
    if (outlier) *wp = 0.f;  // a pixel far outside the window's scale is left out of training
  }
  for (int f = 0; f < kNetOut; f++) {
    unsigned v = __float_as_uint(e[f]), a = __float_as_uint(es[f]), b = __float_as_uint(en[f]);
    for (int o = 16; o > 0; o >>= 1) {
      v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
      a = max(a, __shfl_xor_sync(0xffffffffu, a, o));
      b = max(b, __shfl_xor_sync(0xffffffffu, b, o));
    }
    if ((threadIdx.x & 31) == 0) {
      if (v) atomicMax(&ns->err_bits[f], v);
      if (a) atomicMax(&ns->gate_es[f], a);
      if (b) atomicMax(&ns->gate_en[f], b);
    }
  }
}

// One thread: the pending window's pair is complete; the coming window takes the next slot, its
// inputs are scaled by the step change's maximum and its target by the stencil's largest error on
// the completed window (never below kNetScaleFloor of the change, so that the windows before the
// stencil acts do not get a vanishing scale).
__global__ void k_net_head(Geo g, NetState* ns, int slots) {
  const unsigned r = g.ctl->warm_ready;
  if (ns->have_win) ns->count++;
  for (int f = 0; f < kNetOut; f++) {
    const float m = __uint_as_float(g.ctl->conv_max[r & 1][f]);
    ns->m[f] = m > 0.f ? m : 1.f;
    const float e = ns->have_win ? __uint_as_float(ns->err_bits[f]) : 0.f;
    ns->s[f] = fmaxf(e, kNetScaleFloor * ns->m[f]);
    ns->err_bits[f] = 0u;
    // the gate (non-negative floats order like their bit patterns; NaN never passes)
    const unsigned a = ns->gate_es[f], b = ns->gate_en[f];
    ns->gate[f] = (ns->have_win && a != 0u && a < 0x7f800000u && b < 0x7f800000u &&
                   __uint_as_float(b) < (f ? kNetGateMarginT : kNetGateMarginP) * __uint_as_float(a)) ? 1u : 0u;
    ns->gate_es[f] = 0u;
    ns->gate_en[f] = 0u;
  }
  ns->argmax = 0xffffffffu;
  ns->slot = (int)(ns->count % (unsigned)slots);
}

__global__ void k_net_locate(Geo g, NetState* ns) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i >= g.Nx || j >= g.Ny) return;
  const unsigned r = g.ctl->warm_ready;
  const int n = i + j * g.Nx;
  if (cls_o(g.cls[n]) && __float_as_uint(fabsf(g.cD[0][r % kConvRing][n])) == g.ctl->conv_max[r & 1][0])
    atomicMin(&ns->argmax, (unsigned)n);
}

// The window of H x W cells centred on the located cell (clamped to the mesh): the network input,
// the stencil's predicted change S and the flags (weight 1 where the stencil's start is used).
__global__ void k_net_gather(Geo g, NetState* ns, NetBuffers nb) {
  const int H = nb.H, W = nb.W;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned am = ns->argmax;
  const int ci = am == 0xffffffffu ? g.Nx / 2 : (int)(am % (unsigned)g.Nx);
  const int cj = am == 0xffffffffu ? g.Ny / 2 : (int)(am / (unsigned)g.Nx);
  const int i0 = min(max(ci - W / 2, 0), g.Nx - W), j0 = min(max(cj - H / 2, 0), g.Ny - H);
  if (k >= H * W) return;
  const unsigned r = g.ctl->warm_ready, cur = g.ctl->cur;
  const int i = i0 + k % W, j = j0 + k / W, n = i + j * g.Nx;
  const uint8_t b = g.cact[r & 1][n];
  float in[kNetIn], S[kNetOut], w = 0.f;
  for (int f = 0; f < kNetOut; f++) {
    const float inv = 1.f / ns->m[f];
    in[f] = g.cD[f][r % kConvRing][n] * inv;
    in[2 + f] = g.cD[f][(r + kConvRing - 1) % kConvRing][n] * inv;
    in[6 + f] = g.cD[f][(r + kConvRing - 2) % kConvRing][n] * inv;
    const bool used = (b >> (2 + f)) & 1u;
    S[f] = used ? (float)(g.cnext[f][n] - (f ? g.T[cur][n] : g.p[cur][n])) : 0.f;
    in[4 + f] = S[f] * inv;
    if (used) w = 1.f;
  }
  float* rec = nb.replay + (size_t)ns->slot * nb.slot_floats;
  float* tgt = rec + (size_t)H * W * kNetIn;
  for (int c = 0; c < kNetIn; c++) {
    nb.infer_in[(size_t)k * kNetIn + c] = in[c];
    rec[(size_t)k * kNetIn + c] = in[c];
  }
  tgt[(size_t)H * W * kNetOut + k] = w;
  float* Srec = tgt + (size_t)H * W * (kNetOut + 1);
  for (int f = 0; f < kNetOut; f++) Srec[(size_t)k * kNetOut + f] = S[f];
  nb.infer_w[k] = w;
}

// One thread, after the gather: the window's origin and the pending pair.
__global__ void k_net_commit(Geo g, NetState* ns, NetBuffers nb) {
  const unsigned am = ns->argmax;
  const int ci = am == 0xffffffffu ? g.Nx / 2 : (int)(am % (unsigned)g.Nx);
  const int cj = am == 0xffffffffu ? g.Ny / 2 : (int)(am / (unsigned)g.Nx);
  ns->i0 = min(max(ci - nb.W / 2, 0), g.Nx - nb.W);
  ns->j0 = min(max(cj - nb.H / 2, 0), g.Ny - nb.H);
  ns->have_win = 1;
}

__global__ void k_net_apply(Geo g, NetState* ns, NetBuffers nb) {
  const int H = nb.H, W = nb.W;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k == 0 && ns->enabled)
    for (int f = 0; f < kNetOut; f++) ns->steps_on[f] += ns->gate[f];
  if (k >= H * W || !ns->enabled || !(nb.infer_w[k] > 0.f)) return;
  const unsigned r = g.ctl->warm_ready;
  const int i = ns->i0 + k % W, j = ns->j0 + k / W, n = i + j * g.Nx;
  const uint8_t b = g.cact[r & 1][n];
  for (int f = 0; f < kNetOut; f++)
    if (((b >> (2 + f)) & 1u) && ns->gate[f]) {
      const float o = fminf(fmaxf(nb.infer_out[(size_t)k * kNetOut + f], -kNetTargetClip), kNetTargetClip);
      g.cnext[f][n] += (double)(ns->s[f] * o);
    }
}

// Training batch: the listed slots' inputs, targets and weights side by side.
__global__ void k_net_batch(NetBuffers nb, const int* slots, int B, float* x, float* t, float* w) {
  const size_t px = (size_t)nb.H * nb.W;
  const size_t n = (size_t)B * px;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
    const size_t b = k / px, p = k % px;
    const float* rec = nb.replay + (size_t)slots[b] * nb.slot_floats;
    const float* tgt = rec + px * kNetIn;
    for (int c = 0; c < kNetIn; c++) x[k * kNetIn + c] = rec[p * kNetIn + c];
    for (int c = 0; c < kNetOut; c++) t[k * kNetOut + c] = tgt[p * kNetOut + c];
    w[k] = tgt[px * kNetOut + p];
  }
}

}  // namespace sts
