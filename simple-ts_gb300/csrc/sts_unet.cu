// U-Net of the learned warm start: forward, backward and Adam on the GPU, BF16 weights and
// activations, FP32 accumulation, every convolution a tensor-core GEMM (gemm_bf16_tn, tcgen05).
//
// Layout: activations NHWC (pixel-major, channels contiguous) over a batch of B crops of H x W
// pixels; pixel p = (b H + y) W + x.  A 3x3 convolution (zero padding, cross-correlation) of an
// input X [P][C] is the GEMM Z = im2col(X) W^T + b with im2col(X)[p][t C + c] = X[p + off(t)][c],
// tap t = 3 (dy + 1) + (dx + 1), and W [N][9C] (its transpose Wt [9C][N] is the FP32 master
// copy).  Backward: dZ = dY (Y > 0); dWt = im2col(X)^T dZ (GEMM over pixels; both operands
// transposed to pixel-contiguous rows first); db = column sums of dZ; dX = col2im(dZ W) (the GEMM
// with Wt, then the nine shifted contributions summed per input pixel).
//
// Network (levels L, base channels C0, C_l = C0 2^l): encoder level l: conv C_in -> C_l, conv
// C_l -> C_l (ReLU after each), 2x2 average pooling between levels; decoder level l = L-2 .. 0:
// nearest-neighbour upsampling of the level below, concatenated with the encoder output of level l
// (C_l+1 + C_l channels), conv -> C_l, conv C_l -> C_l; head: 1x1 conv C0 -> out (no ReLU; its
// weights are padded to 8 outputs, the extra ones held at zero).  No counterpart in the reference.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "sts_net.h"
#include "sts_unet.h"

namespace sts {
namespace {

using bf16 = __nv_bfloat16;

__global__ void k_im2col(const bf16* __restrict__ X, bf16* __restrict__ P, int B, int H, int W, int C) {
  // one thread per (pixel, tap, 8 channels): 16-byte copies
  const int c8 = C / 8;
  const long long n = (long long)B * H * W * 9 * c8;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(k % c8);
    const int t = (int)((k / c8) % 9);
    const long long p = k / (c8 * 9);
    const int x = (int)(p % W), y = (int)((p / W) % H);
    const long long b = p / ((long long)W * H);
    const int yy = y + t / 3 - 1, xx = x + t % 3 - 1;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (yy >= 0 && yy < H && xx >= 0 && xx < W) v = *(const uint4*)(X + ((b * H + yy) * W + xx) * C + q * 8);
    *(uint4*)(P + p * 9 * C + t * C + q * 8) = v;
  }
}

// Transposed im2col: PT[t C + c][p] (rows of ld >= P pixels; taps = 9 for a 3x3 window, 1 for the
// plain transpose of X).  Writes are coalesced along p.
__global__ void k_im2col_t(const bf16* __restrict__ X, bf16* __restrict__ PT, int B, int H, int W, int C, int taps,
                           int ld) {
  const long long P = (long long)B * H * W;
  const long long n = (long long)taps * C * ld;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const long long p = k % ld;
    const int r = (int)(k / ld);
    const int c = r % C, t = r / C;
    bf16 v = __float2bfloat16(0.f);
    if (p < P) {
      const int x = (int)(p % W), y = (int)((p / W) % H);
      const long long b = p / ((long long)W * H);
      const int dy = taps == 9 ? t / 3 - 1 : 0, dx = taps == 9 ? t % 3 - 1 : 0;
      const int yy = y + dy, xx = x + dx;
      if (yy >= 0 && yy < H && xx >= 0 && xx < W) v = X[((b * H + yy) * W + xx) * C + c];
    }
    PT[(long long)r * ld + p] = v;
  }
}

// dZ = gY (Y > 0) (no gate when Y is null) as BF16, in both layouts: dZ [P][N] and dZT [N][ld].
__global__ void k_gate(const float* __restrict__ gY, const bf16* __restrict__ Y, bf16* __restrict__ dZ,
                       bf16* __restrict__ dZT, long long P, int N, int ldz, int ldT) {
  const long long n = P * N;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const long long p = k / N;
    const int c = (int)(k % N);
    float g = gY[p * N + c];
    if (Y && !(__bfloat162float(Y[p * N + c]) > 0.f)) g = 0.f;
    const bf16 h = __float2bfloat16_rn(g);
    dZ[p * ldz + c] = h;
    dZT[(long long)c * ldT + p] = h;
  }
  // the padding columns of dZ (ldz > N) and pixels of dZT (ldT > P) stay as cleared
}

// db[n] = sum_p dZ[p][n] (FP32): one CTA per output channel.
__global__ void k_bias_grad(const bf16* __restrict__ dZT, float* __restrict__ db, long long P, int ldT) {
  __shared__ float red[256];
  const int n = blockIdx.x;
  float s = 0.f;
  for (long long p = threadIdx.x; p < P; p += blockDim.x) s += __bfloat162float(dZT[(long long)n * ldT + p]);
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) db[n] = red[0];
}

// gX[q][c] += sum over taps t of dP[q - off(t)][t C + c] (source pixels inside the crop).
__global__ void k_col2im(const float* __restrict__ dP, float* __restrict__ gX, int B, int H, int W, int C) {
  const long long n = (long long)B * H * W * C;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(k % C);
    const long long q = k / C;
    const int x = (int)(q % W), y = (int)((q / W) % H);
    const long long b = q / ((long long)W * H);
    float s = 0.f;
    for (int t = 0; t < 9; t++) {
      const int yy = y - (t / 3 - 1), xx = x - (t % 3 - 1);
      if (yy >= 0 && yy < H && xx >= 0 && xx < W) s += dP[((b * H + yy) * W + xx) * 9 * C + t * C + c];
    }
    gX[k] += s;
  }
}

// 2x2 average pooling (H, W even): Y [B][H/2][W/2][C].
__global__ void k_pool(const bf16* __restrict__ X, bf16* __restrict__ Y, int B, int H, int W, int C) {
  const int h = H / 2, w = W / 2;
  const long long n = (long long)B * h * w * C;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(k % C);
    const long long q = k / C;
    const int x = (int)(q % w), y = (int)((q / w) % h);
    const long long b = q / ((long long)w * h);
    const long long base = ((b * H + 2 * y) * W + 2 * x) * C + c;
    const float s = __bfloat162float(X[base]) + __bfloat162float(X[base + C]) + __bfloat162float(X[base + (long long)W * C]) +
                    __bfloat162float(X[base + (long long)W * C + C]);
    Y[k] = __float2bfloat16_rn(0.25f * s);
  }
}

__global__ void k_pool_back(const float* __restrict__ gY, float* __restrict__ gX, int B, int H, int W, int C) {
  const long long n = (long long)B * H * W * C;
  const int h = H / 2, w = W / 2;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(k % C);
    const long long q = k / C;
    const int x = (int)(q % W), y = (int)((q / W) % H);
    const long long b = q / ((long long)W * H);
    gX[k] += 0.25f * gY[((b * h + y / 2) * w + x / 2) * C + c];
  }
}

// out [B][H][W][C1 + C2]: channels 0..C1-1 the nearest-neighbour upsampling of low [B][H/2][W/2][C1],
// then skip [B][H][W][C2].
__global__ void k_upcat(const bf16* __restrict__ low, const bf16* __restrict__ skip, bf16* __restrict__ out, int B,
                        int H, int W, int C1, int C2) {
  const int C = C1 + C2, h = H / 2, w = W / 2;
  const long long n = (long long)B * H * W * C;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(k % C);
    const long long q = k / C;
    if (c < C1) {
      const int x = (int)(q % W), y = (int)((q / W) % H);
      const long long b = q / ((long long)W * H);
      out[k] = low[((b * h + y / 2) * w + x / 2) * C1 + c];
    } else {
      out[k] = skip[q * C2 + (c - C1)];
    }
  }
}

__global__ void k_upcat_back(const float* __restrict__ gOut, float* __restrict__ gLow, float* __restrict__ gSkip, int B,
                             int H, int W, int C1, int C2) {
  const int C = C1 + C2, h = H / 2, w = W / 2;
  // gSkip: one thread per fine pixel and skip channel
  const long long n = (long long)B * H * W * C2;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(k % C2);
    const long long q = k / C2;
    gSkip[k] += gOut[q * C + C1 + c];
  }
  // gLow: one thread per coarse pixel and low channel, the sum of its four fine pixels
  const long long m = (long long)B * h * w * C1;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < m; k += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(k % C1);
    const long long q = k / C1;
    const int x = (int)(q % w), y = (int)((q / w) % h);
    const long long b = q / ((long long)w * h);
    const long long f = (b * H + 2 * y) * W + 2 * x;
    gLow[k] += gOut[f * C + c] + gOut[(f + 1) * C + c] + gOut[(f + W) * C + c] + gOut[(f + W + 1) * C + c];
  }
}

// Weighted squared error of the head's first `out` channels (of ldy) against the target
// [P][out], weight per pixel (NULL: 1): loss = sum w (y - t)^2 / sum w; gY = d loss / d y.
__global__ void k_mse(const float* __restrict__ y, int ldy, const float* __restrict__ t, const float* __restrict__ w,
                      float* __restrict__ gY, long long P, int out, float inv_wsum, float* __restrict__ loss) {
  float s = 0.f;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < P * ldy; k += (long long)gridDim.x * blockDim.x) {
    const long long p = k / ldy;
    const int c = (int)(k % ldy);
    float g = 0.f;
    if (c < out) {
      const float wp = w ? w[p] : 1.f;
      const float d = y[k] - t[p * out + c];
      s += wp * d * d;
      g = 2.f * wp * d * inv_wsum;
    }
    gY[k] = g;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, s * inv_wsum);
}

// Adam (Kingma & Ba), bias-corrected step sizes given by the host.
__global__ void k_adam(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v, const float* __restrict__ g,
                       long long n, float lr_t, float b1, float b2, float eps) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const float gk = g[k];
    const float mk = b1 * m[k] + (1.f - b1) * gk;
    const float vk = b2 * v[k] + (1.f - b2) * gk * gk;
    m[k] = mk;
    v[k] = vk;
    w[k] -= lr_t * mk / (sqrtf(vk) + eps);
  }
}

// The BF16 copies of one layer's weights from the FP32 master Wt [K][N]: W [N][K] (the forward GEMM's
// B operand) and Wt [K][N] (the backward-data GEMM's B operand).
__global__ void k_emit(const float* __restrict__ Wt32, bf16* __restrict__ W, bf16* __restrict__ Wt, int K, int N) {
  const long long n = (long long)K * N;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(k / N), c = (int)(k % N);
    const bf16 h = __float2bfloat16_rn(Wt32[k]);
    Wt[k] = h;
    W[(long long)c * K + r] = h;
  }
}

inline int grid_for(long long n) {
  long long g = (n + 255) / 256;
  return (int)(g < 1 ? 1 : (g > 8192 ? 8192 : g));
}

}  // namespace
}  // namespace sts

namespace sts {
namespace {

__global__ void k_pack_input(const float* __restrict__ x, int in_ch, bf16* __restrict__ y, long long P) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < P * 8; k += (long long)gridDim.x * blockDim.x) {
    const long long p = k / 8;
    const int c = (int)(k % 8);
    y[k] = __float2bfloat16_rn(c < in_ch ? x[p * in_ch + c] : 0.f);
  }
}

__global__ void k_unpad(const float* __restrict__ h, float* __restrict__ y, int out_ch, long long P) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < P * out_ch; k += (long long)gridDim.x * blockDim.x)
    y[k] = h[(k / out_ch) * 8 + k % out_ch];
}

__global__ void k_pad_grad(const float* __restrict__ gy, float* __restrict__ gh, int out_ch, long long P) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < P * 8; k += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(k % 8);
    gh[k] = c < out_ch ? gy[(k / 8) * out_ch + c] : 0.f;
  }
}

enum OpKind { OP_CONV, OP_POOL, OP_UPCAT, OP_HEAD };

struct Op {
  OpKind kind;
  int level;        // resolution level of the op's output
  int cin, cout;    // channels (UPCAT: cin = low channels, cout = skip channels)
  int taps;         // 9, or 1 for the head
  int a, b, out;    // activation indices (b: the skip of UPCAT)
  long long off;    // CONV/HEAD: offset of Wt in the parameters (bias follows)
  int layer;        // CONV/HEAD: index of the BF16 weight copies
};

}  // namespace

struct UNetImpl {
  int in_ch, out_ch, C0, L, maxB, H, W;
  cudaStream_t s;
  std::string err;
  std::vector<void*> allocs;
  long long nparams = 0;
  float *params = nullptr, *grads = nullptr, *m = nullptr, *v = nullptr;
  int adam_t = 0;
  // activations: index 0 is the packed input [P0][8]; the head's FP32 output separately
  std::vector<bf16*> act;
  std::vector<float*> gact;
  std::vector<int> act_level, act_ch;
  float *head_out = nullptr, *g_head = nullptr, *loss = nullptr;
  std::vector<Op> ops;
  std::vector<bf16*> Wb, Wtb;  // per layer: W [N][K] and Wt [K][N]
  std::vector<int> lk, ln;     // per layer: K, N
  bf16 *col = nullptr, *colT = nullptr, *dZ = nullptr, *dZT = nullptr;
  float* dP = nullptr;
  unsigned* errw = nullptr;

  long long P(int level, int B) const { return (long long)B * (H >> level) * (W >> level); }
  long long ldT(int level, int B) const { return (P(level, B) + 7) / 8 * 8; }

  template <class T>
  bool alloc(T** p, size_t n) {
    void* q = nullptr;
    if (cudaMalloc(&q, sizeof(T) * (n ? n : 1)) != cudaSuccess) {
      err = "cudaMalloc failed";
      return false;
    }
    cudaMemsetAsync(q, 0, sizeof(T) * (n ? n : 1), s);
    allocs.push_back(q);
    *p = (T*)q;
    return true;
  }
  int new_act(int level, int ch) {
    act_level.push_back(level);
    act_ch.push_back(ch);
    act.push_back(nullptr);
    gact.push_back(nullptr);
    return (int)act.size() - 1;
  }
  cudaError_t emit(int layer) {
    const Op* op = nullptr;
    for (const Op& o : ops)
      if ((o.kind == OP_CONV || o.kind == OP_HEAD) && o.layer == layer) op = &o;
    k_emit<<<grid_for((long long)lk[layer] * ln[layer]), 256, 0, s>>>(params + op->off, Wb[layer], Wtb[layer],
                                                                        lk[layer], ln[layer]);
    return cudaGetLastError();
  }
};

UNet::UNet(int in_ch, int out_ch, int base_ch, int levels, int max_batch, int H, int W, unsigned long long seed,
           cudaStream_t s)
    : d(new UNetImpl) {
  UNetImpl& u = *d;
  u.in_ch = in_ch;
  u.out_ch = out_ch;
  u.C0 = base_ch;
  u.L = levels;
  u.maxB = max_batch;
  u.H = H;
  u.W = W;
  u.s = s;
  const int div = 1 << (levels - 1);
  if (in_ch < 1 || in_ch > 8 || out_ch < 1 || out_ch > 8 || base_ch < 8 || base_ch % 8 || levels < 1 || levels > 6 ||
      max_batch < 1 || H % div || W % div || H < div || W < div) {
    u.err = "bad network shape";
    return;
  }
  // the op list and the activations
  long long off = 0;
  int layer = 0;
  auto ch = [&](int l) { return base_ch << l; };
  auto conv = [&](int a, int level, int cin, int cout) {
    const int o = u.new_act(level, cout);
    u.ops.push_back({OP_CONV, level, cin, cout, 9, a, -1, o, off, layer++});
    off += (long long)9 * cin * cout + cout;
    return o;
  };
  const int x = u.new_act(0, 8);
  std::vector<int> enc(levels);
  int cur = conv(conv(x, 0, 8, ch(0)), 0, ch(0), ch(0));
  enc[0] = cur;
  for (int l = 1; l < levels; l++) {
    const int p = u.new_act(l, ch(l - 1));
    u.ops.push_back({OP_POOL, l, ch(l - 1), ch(l - 1), 0, enc[l - 1], -1, p, 0, -1});
    cur = conv(conv(p, l, ch(l - 1), ch(l)), l, ch(l), ch(l));
    enc[l] = cur;
  }
  for (int l = levels - 2; l >= 0; l--) {
    const int c = u.new_act(l, ch(l + 1) + ch(l));
    u.ops.push_back({OP_UPCAT, l, ch(l + 1), ch(l), 0, cur, enc[l], c, 0, -1});
    cur = conv(conv(c, l, ch(l + 1) + ch(l), ch(l)), l, ch(l), ch(l));
  }
  u.ops.push_back({OP_HEAD, 0, ch(0), 8, 1, cur, -1, -1, off, layer++});
  off += (long long)ch(0) * 8 + 8;
  u.nparams = off;
  // buffers
  if (!u.alloc(&u.params, off) || !u.alloc(&u.grads, off) || !u.alloc(&u.m, off) || !u.alloc(&u.v, off) ||
      !u.alloc(&u.errw, 1) || !u.alloc(&u.loss, 1))
    return;
  for (size_t k = 0; k < u.act.size(); k++) {
    const size_t n = (size_t)u.P(u.act_level[k], max_batch) * u.act_ch[k];
    if (!u.alloc(&u.act[k], n) || !u.alloc(&u.gact[k], n)) return;
  }
  if (!u.alloc(&u.head_out, (size_t)u.P(0, max_batch) * 8) || !u.alloc(&u.g_head, (size_t)u.P(0, max_batch) * 8)) return;
  size_t ncol = 0, ncolT = 0, ndz = 0, ndzT = 0;
  for (const Op& o : u.ops) {
    if (o.kind != OP_CONV && o.kind != OP_HEAD) continue;
    const size_t P = (size_t)u.P(o.level, max_batch), lt = (size_t)u.ldT(o.level, max_batch);
    ncol = std::max(ncol, P * o.taps * o.cin);
    ncolT = std::max(ncolT, lt * o.taps * o.cin);
    ndz = std::max(ndz, P * o.cout);
    ndzT = std::max(ndzT, lt * o.cout);
    bf16 *w1, *w2;
    if (!u.alloc(&w1, (size_t)o.taps * o.cin * o.cout) || !u.alloc(&w2, (size_t)o.taps * o.cin * o.cout)) return;
    u.Wb.push_back(w1);
    u.Wtb.push_back(w2);
    u.lk.push_back(o.taps * o.cin);
    u.ln.push_back(o.cout);
  }
  if (!u.alloc(&u.col, ncol) || !u.alloc(&u.colT, ncolT) || !u.alloc(&u.dP, ncol) || !u.alloc(&u.dZ, ndz) ||
      !u.alloc(&u.dZT, ndzT))
    return;
  // weights: uniform in +-sqrt(6 / fan_in) (He), biases 0; the head's padding outputs 0
  std::vector<float> h(off, 0.f);
  unsigned long long st = seed * 6364136223846793005ULL + 1442695040888963407ULL;
  auto uni = [&]() {
    st = st * 6364136223846793005ULL + 1442695040888963407ULL;
    return (double)(st >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
  };
  for (const Op& o : u.ops) {
    if (o.kind != OP_CONV && o.kind != OP_HEAD) continue;
    const long long K = (long long)o.taps * o.cin;
    const double a = std::sqrt(6.0 / (double)K);
    for (long long r = 0; r < K; r++)
      for (int c = 0; c < o.cout; c++) {
        const bool live = o.kind == OP_CONV || c < out_ch;
        h[o.off + r * o.cout + c] = live ? (float)(a * uni()) : 0.f;
      }
  }
  if (set_params(h.data()) != cudaSuccess) u.err = "weight upload failed";
}

UNet::~UNet() {
  if (d)
    for (void* p : d->allocs) cudaFree(p);
}
bool UNet::ok() const { return d->err.empty(); }
const char* UNet::error() const { return d->err.c_str(); }
long long UNet::param_count() const { return d->nparams; }
const float* UNet::grads() const { return d->grads; }
unsigned* UNet::error_flag() const { return d->errw; }
void UNet::set_stream(cudaStream_t s) { d->s = s; }

cudaError_t UNet::get_params(float* host) const {
  cudaError_t r = cudaMemcpyAsync(host, d->params, sizeof(float) * d->nparams, cudaMemcpyDeviceToHost, d->s);
  if (r == cudaSuccess) r = cudaStreamSynchronize(d->s);
  return r;
}

cudaError_t UNet::set_params(const float* host) {
  UNetImpl& u = *d;
  cudaError_t r = cudaMemcpyAsync(u.params, host, sizeof(float) * u.nparams, cudaMemcpyHostToDevice, u.s);
  for (size_t k = 0; k < u.Wb.size() && r == cudaSuccess; k++) r = u.emit((int)k);
  if (r == cudaSuccess) r = cudaStreamSynchronize(u.s);
  return r;
}

cudaError_t UNet::forward(const float* x, int B, float* y) {
  UNetImpl& u = *d;
  if (!ok() || B < 1 || B > u.maxB) return cudaErrorInvalidValue;
  const long long P0 = u.P(0, B);
  k_pack_input<<<grid_for(P0 * 8), 256, 0, u.s>>>(x, u.in_ch, u.act[0], P0);
  for (const Op& o : u.ops) {
    const int Hl = u.H >> o.level, Wl = u.W >> o.level;
    const long long P = u.P(o.level, B);
    cudaError_t r = cudaSuccess;
    if (o.kind == OP_POOL) {
      k_pool<<<grid_for(P * o.cin), 256, 0, u.s>>>(u.act[o.a], u.act[o.out], B, Hl * 2, Wl * 2, o.cin);
    } else if (o.kind == OP_UPCAT) {
      k_upcat<<<grid_for(P * (o.cin + o.cout)), 256, 0, u.s>>>(u.act[o.a], u.act[o.b], u.act[o.out], B, Hl, Wl, o.cin,
                                                               o.cout);
    } else if (o.kind == OP_CONV) {
      k_im2col<<<grid_for(P * 9 * (o.cin / 8)), 256, 0, u.s>>>(u.act[o.a], u.col, B, Hl, Wl, o.cin);
      GemmEpilogue e;
      e.out = u.act[o.out];
      e.ldo = o.cout;
      e.out_bf16 = 1;
      e.bias = u.params + o.off + (long long)9 * o.cin * o.cout;
      e.relu = 1;
      r = gemm_bf16_tn(u.col, 9 * o.cin, u.Wb[o.layer], 9 * o.cin, (int)P, o.cout, 9 * o.cin, e, u.errw, u.s);
    } else {  // head: 1x1, FP32 out
      GemmEpilogue e;
      e.out = u.head_out;
      e.ldo = 8;
      e.bias = u.params + o.off + (long long)o.cin * 8;
      r = gemm_bf16_tn(u.act[o.a], o.cin, u.Wb[o.layer], o.cin, (int)P, 8, o.cin, e, u.errw, u.s);
    }
    if (r != cudaSuccess) return r;
  }
  if (y) k_unpad<<<grid_for(P0 * u.out_ch), 256, 0, u.s>>>(u.head_out, y, u.out_ch, P0);
  return cudaGetLastError();
}

cudaError_t UNet::backward_mse(const float* target, const float* weight, int B, float* loss_dev) {
  UNetImpl& u = *d;
  const long long P0 = u.P(0, B);
  cudaMemsetAsync(loss_dev, 0, sizeof(float), u.s);
  k_mse<<<grid_for(P0 * 8), 256, 0, u.s>>>(u.head_out, 8, target, weight, u.g_head, P0, u.out_ch,
                                           1.0f / (float)(P0 * u.out_ch), loss_dev);
  return backward(nullptr, B);
}

cudaError_t UNet::loss(const float* target, const float* weight, int B, float* loss_dev, bool zero_prediction) {
  UNetImpl& u = *d;
  const long long P0 = u.P(0, B);
  if (zero_prediction) cudaMemsetAsync(u.head_out, 0, sizeof(float) * P0 * 8, u.s);
  cudaMemsetAsync(loss_dev, 0, sizeof(float), u.s);
  k_mse<<<grid_for(P0 * 8), 256, 0, u.s>>>(u.head_out, 8, target, weight, u.g_head, P0, u.out_ch,
                                           1.0f / (float)(P0 * u.out_ch), loss_dev);
  return cudaGetLastError();
}

cudaError_t UNet::backward(const float* gy, int B) {
  UNetImpl& u = *d;
  if (!ok() || B < 1 || B > u.maxB) return cudaErrorInvalidValue;
  const long long P0 = u.P(0, B);
  if (gy) k_pad_grad<<<grid_for(P0 * 8), 256, 0, u.s>>>(gy, u.g_head, u.out_ch, P0);
  for (size_t k = 0; k < u.gact.size(); k++)
    cudaMemsetAsync(u.gact[k], 0, sizeof(float) * u.P(u.act_level[k], B) * u.act_ch[k], u.s);
  for (int q = (int)u.ops.size() - 1; q >= 0; q--) {
    const Op& o = u.ops[q];
    const int Hl = u.H >> o.level, Wl = u.W >> o.level;
    const long long P = u.P(o.level, B), lt = u.ldT(o.level, B);
    cudaError_t r = cudaSuccess;
    if (o.kind == OP_POOL) {
      k_pool_back<<<grid_for(P * 4 * o.cin), 256, 0, u.s>>>(u.gact[o.out], u.gact[o.a], B, Hl * 2, Wl * 2, o.cin);
    } else if (o.kind == OP_UPCAT) {
      k_upcat_back<<<grid_for(P * o.cout), 256, 0, u.s>>>(u.gact[o.out], u.gact[o.a], u.gact[o.b], B, Hl, Wl, o.cin,
                                                          o.cout);
    } else {
      const bool head = o.kind == OP_HEAD;
      const int K = o.taps * o.cin, N = o.cout;
      float* gW = u.grads + o.off;
      float* gb = gW + (long long)K * N;
      // dZ (and its transpose) from the output gradient, gated by the ReLU
      cudaMemsetAsync(u.dZT, 0, sizeof(bf16) * lt * N, u.s);
      k_gate<<<grid_for(P * N), 256, 0, u.s>>>(head ? u.g_head : u.gact[o.out], head ? nullptr : u.act[o.out], u.dZ,
                                               u.dZT, P, N, N, (int)lt);
      k_bias_grad<<<N, 256, 0, u.s>>>(u.dZT, gb, P, (int)lt);
      // dWt [K][N] = im2col(X)^T dZ: a GEMM over the pixels
      k_im2col_t<<<grid_for((long long)K * lt), 256, 0, u.s>>>(u.act[o.a], u.colT, B, Hl, Wl, o.cin, o.taps, (int)lt);
      GemmEpilogue ew;
      ew.out = gW;
      ew.ldo = N;
      r = gemm_bf16_tn(u.colT, (int)lt, u.dZT, (int)lt, K, N, (int)P, ew, u.errw, u.s);
      if (r != cudaSuccess) return r;
      // dX: dZ Wt^T, then the taps' contributions summed per input pixel; not needed for the input
      if (o.a != 0) {
        GemmEpilogue ex;
        if (head) {
          ex.out = u.gact[o.a];
          ex.ldo = o.cin;
          ex.accumulate = 1;
          r = gemm_bf16_tn(u.dZ, N, u.Wtb[o.layer], N, (int)P, o.cin, N, ex, u.errw, u.s);
        } else {
          ex.out = u.dP;
          ex.ldo = K;
          r = gemm_bf16_tn(u.dZ, N, u.Wtb[o.layer], N, (int)P, K, N, ex, u.errw, u.s);
          if (r == cudaSuccess)
            k_col2im<<<grid_for(P * o.cin), 256, 0, u.s>>>(u.dP, u.gact[o.a], B, Hl, Wl, o.cin);
        }
      }
    }
    if (r != cudaSuccess) return r;
  }
  return cudaGetLastError();
}

cudaError_t UNet::adam(float lr) {
  UNetImpl& u = *d;
  u.adam_t++;
  const float b1 = 0.9f, b2 = 0.999f;
  const float lr_t = lr * (float)(std::sqrt(1.0 - std::pow((double)b2, u.adam_t)) / (1.0 - std::pow((double)b1, u.adam_t)));
  k_adam<<<grid_for(u.nparams), 256, 0, u.s>>>(u.params, u.m, u.v, u.grads, u.nparams, lr_t, b1, b2, 1e-8f);
  for (size_t k = 0; k < u.Wb.size(); k++)
    if (cudaError_t r = u.emit((int)k)) return r;
  return cudaGetLastError();
}

}  // namespace sts

// ---------------------------------------------------------------------------
// C ABI: the network on host arrays (training and checking outside a solver).
#include "../../include/sts_gb300.h"

struct sts_net {
  int device = 0, H = 0, W = 0, in_ch = 0, out_ch = 0, maxB = 0;
  cudaStream_t s = nullptr;
  std::unique_ptr<sts::UNet> net;
  float *x = nullptr, *y = nullptr, *t = nullptr, *loss = nullptr;
  ~sts_net() {
    net.reset();
    cudaFree(x);
    cudaFree(y);
    cudaFree(t);
    cudaFree(loss);
    if (s) cudaStreamDestroy(s);
  }
};

namespace {
int net_status(sts_net* n, cudaError_t r) {
  if (r != cudaSuccess) return STS_ERR_CUDA;
  if (cudaStreamSynchronize(n->s) != cudaSuccess) return STS_ERR_CUDA;
  unsigned e = 0;
  if (cudaMemcpy(&e, n->net->error_flag(), sizeof(unsigned), cudaMemcpyDeviceToHost) != cudaSuccess) return STS_ERR_CUDA;
  return e ? STS_ERR_TIMEOUT : STS_OK;
}
}  // namespace

extern "C" {

int sts_net_create(int in_ch, int out_ch, int base_ch, int levels, int max_batch, int H, int W, unsigned long long seed,
                   int device, sts_net** out) {
  if (!out) return STS_ERR_ARG;
  *out = nullptr;
  if (cudaSetDevice(device) != cudaSuccess) return STS_ERR_CUDA;
  std::unique_ptr<sts_net> n(new sts_net);
  n->device = device;
  n->H = H;
  n->W = W;
  n->in_ch = in_ch;
  n->out_ch = out_ch;
  n->maxB = max_batch;
  if (cudaStreamCreateWithFlags(&n->s, cudaStreamNonBlocking) != cudaSuccess) return STS_ERR_CUDA;
  n->net.reset(new sts::UNet(in_ch, out_ch, base_ch, levels, max_batch, H, W, seed, n->s));
  if (!n->net->ok()) return STS_ERR_ARG;
  const size_t P = (size_t)max_batch * H * W;
  if (cudaMalloc(&n->x, sizeof(float) * P * in_ch) != cudaSuccess ||
      cudaMalloc(&n->y, sizeof(float) * P * out_ch) != cudaSuccess ||
      cudaMalloc(&n->t, sizeof(float) * P * out_ch) != cudaSuccess || cudaMalloc(&n->loss, sizeof(float)) != cudaSuccess)
    return STS_ERR_CUDA;
  *out = n.release();
  return STS_OK;
}

long long sts_net_param_count(sts_net* n) { return n ? n->net->param_count() : -1; }

int sts_net_get_params(sts_net* n, float* out) {
  if (!n || !out) return STS_ERR_ARG;
  cudaSetDevice(n->device);
  return n->net->get_params(out) == cudaSuccess ? STS_OK : STS_ERR_CUDA;
}

int sts_net_set_params(sts_net* n, const float* in) {
  if (!n || !in) return STS_ERR_ARG;
  cudaSetDevice(n->device);
  return n->net->set_params(in) == cudaSuccess ? STS_OK : STS_ERR_CUDA;
}

int sts_net_forward(sts_net* n, const float* x, int B, float* y) {
  if (!n || !x || !y || B < 1 || B > n->maxB) return STS_ERR_ARG;
  cudaSetDevice(n->device);
  const size_t P = (size_t)B * n->H * n->W;
  cudaError_t r = cudaMemcpyAsync(n->x, x, sizeof(float) * P * n->in_ch, cudaMemcpyHostToDevice, n->s);
  if (r == cudaSuccess) r = n->net->forward(n->x, B, n->y);
  if (r == cudaSuccess) r = cudaMemcpyAsync(y, n->y, sizeof(float) * P * n->out_ch, cudaMemcpyDeviceToHost, n->s);
  return net_status(n, r);
}

int sts_net_backward(sts_net* n, const float* gy, int B, float* grads) {
  if (!n || !gy || !grads || B < 1 || B > n->maxB) return STS_ERR_ARG;
  cudaSetDevice(n->device);
  const size_t P = (size_t)B * n->H * n->W;
  cudaError_t r = cudaMemcpyAsync(n->t, gy, sizeof(float) * P * n->out_ch, cudaMemcpyHostToDevice, n->s);
  if (r == cudaSuccess) r = n->net->backward(n->t, B);
  if (r == cudaSuccess)
    r = cudaMemcpyAsync(grads, n->net->grads(), sizeof(float) * n->net->param_count(), cudaMemcpyDeviceToHost, n->s);
  return net_status(n, r);
}

int sts_net_train_step(sts_net* n, const float* x, const float* target, int B, float lr, float* loss) {
  if (!n || !x || !target || B < 1 || B > n->maxB) return STS_ERR_ARG;
  cudaSetDevice(n->device);
  const size_t P = (size_t)B * n->H * n->W;
  cudaError_t r = cudaMemcpyAsync(n->x, x, sizeof(float) * P * n->in_ch, cudaMemcpyHostToDevice, n->s);
  if (r == cudaSuccess) r = cudaMemcpyAsync(n->t, target, sizeof(float) * P * n->out_ch, cudaMemcpyHostToDevice, n->s);
  if (r == cudaSuccess) r = n->net->forward(n->x, B, nullptr);
  if (r == cudaSuccess) r = n->net->backward_mse(n->t, nullptr, B, n->loss);
  if (r == cudaSuccess) r = n->net->adam(lr);
  float l = 0.f;
  if (r == cudaSuccess) r = cudaMemcpyAsync(&l, n->loss, sizeof(float), cudaMemcpyDeviceToHost, n->s);
  const int st = net_status(n, r);
  if (loss) *loss = l;
  return st;
}

void sts_net_destroy(sts_net* n) {
  if (n) {
    cudaSetDevice(n->device);
    delete n;
  }
}

}  // extern "C"
