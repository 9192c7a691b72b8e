// Network warm start (warm_start 5): device state and kernels (sts_warmnet.cu).
#pragma once
#include "sts_common.cuh"

namespace sts {

constexpr int kNetIn = 8, kNetOut = 2;
constexpr float kNetScaleFloor = 1e-4f;  // smallest target scale, relative to the step change's maximum
constexpr float kNetTargetClip = 8.f;    // targets (and outputs) beyond this many scales are clipped
// the gate opens for p (T) when the network left less than this fraction of the stencil's
// largest error on the window completed last; T's stays shut (on the 2048x256 and 1200x120
// channels its correction added sweeps wherever it opened)
constexpr float kNetGateMarginP = 1.0f, kNetGateMarginT = 0.0f;

// Device-side bookkeeping of the window and the replay ring.
struct NetState {
  int i0, j0;                 // origin of the window gathered last (its pair awaits its target)
  int slot;                   // its replay slot
  int have_win;               // a window was gathered
  unsigned count;             // completed pairs (targets written)
  unsigned argmax;            // located cell
  unsigned err_bits[kNetOut]; // largest stencil error on the completed window (float bits)
  float m[kNetOut];           // input scale of the window: max |D_r| per field
  float s[kNetOut];           // target and output scale of the window
  unsigned enabled;           // apply the network's correction
  // the gate: on the completed window, the largest stencil error |t| and the largest error left
  // after the network's correction |t - o| over its flagged cells (scaled, float bits); the
  // coming window takes field f's correction only if the latter was the smaller
  unsigned gate_es[kNetOut], gate_en[kNetOut];
  unsigned gate[kNetOut];
  unsigned steps_on[kNetOut];  // steps whose window took field f's correction
};

// Buffers: the replay ring of `slots` records of slot_floats floats each (per window pixel: 8
// inputs, then 2 targets, 1 weight, 2 stencil changes), the inference input and weights, and the
// network's output.
struct NetBuffers {
  int H, W;
  size_t slot_floats;
  float* replay;
  float* infer_in;
  float* infer_w;
  float* infer_out;
};

__global__ void k_net_target(Geo g, NetState* ns, NetBuffers nb);
__global__ void k_net_head(Geo g, NetState* ns, int slots);
__global__ void k_net_locate(Geo g, NetState* ns);
__global__ void k_net_gather(Geo g, NetState* ns, NetBuffers nb);
__global__ void k_net_commit(Geo g, NetState* ns, NetBuffers nb);
__global__ void k_net_apply(Geo g, NetState* ns, NetBuffers nb);
__global__ void k_net_batch(NetBuffers nb, const int* slots, int B, float* x, float* t, float* w);

}  // namespace sts
