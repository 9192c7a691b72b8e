// Convolutional warm start of the p-T sweeps (warm_start 4), learned on the run's own trajectory.
//
// No counterpart in the reference, which starts every step's sweeps from the previous step's
// p and T.  Here the sweeps start from a prediction of the step's change; plain Jacobi still
// iterates to the same residual tolerance, so only the number of sweeps changes.
//
// Model, per field (p and T separately): with D_t = x_t - x_{t-1} the step differences on the
// solved cells (stored in FP32), the change of the coming step at cell c is predicted as a linear
// combination of 36 features of c's 3x3 neighbourhood in the last four differences: the time
// basis D_t, D_t - D_{t-1}, and the second and third differences, each resolved in space into
// value, gradient and curvature along x and then along y (a 3-point polynomial basis, which keeps
// the least-squares problem well conditioned).  The stencil is applied where the solution moves:
// cells within 3 cells (diamond) of a cell with |D_t| > 0.1 max |D_t|.  Elsewhere the start is
// quadratic extrapolation in time (warm_start 2).  The 36 weights are refitted every step by
// least squares over the last kConvWin steps: each step contributes the pair (features of the
// previous step on its active cells, this step's difference), so the model tracks moving fronts
// (a shock that advances a fraction of a cell per step) that extrapolation in time cannot.
//
// Arithmetic: FP32 features; normal-equation terms summed in FP32 over the rows of a strip of 32x2
// cells (cell order), then with compensated FP32 sums (Neumaier) over the non-empty strips of each
// segment of kConvSeg strips and over the non-empty segments, both in index order; FP64 over the
// window in slot order; a ridge of 1e-11 of the mean diagonal; Gauss-Jordan elimination in FP32.  This file is compiled without fused multiply-adds and every sum has a
// fixed order, so the result does not depend on scheduling and the CPU oracle reproduces it bit
// for bit.  (GB300's FP64 pipe does about 2 adds per clock per SM: the sums over strips stay on
// the FP32 pipes and are spread over many CTAs.)
//
// Per step: k_step_begin stores the newest differences, writes the quadratic start and folds
// max |D| (conv_step_begin_cell, conv_block_max); then, in the step's first outer iteration and
// in a graph beside the assembly kernel (which reads neither p nor T of the iterate; the sweep loop
// waits for both), conv_gram (per-strip terms of the newest
// training pair), conv_reduce (segment sums and the pair's total), conv_solve (one CTA per
// field: window, ridge, elimination) and conv_apply (active flags of the newest difference,
// start).
#include <cuda_runtime.h>

#include "sts_common.cuh"
#include "sts_kernels.h"

#include "sts_device.cuh"

namespace sts {
namespace {

constexpr float kConvAlpha = 0.1f;   // a cell is a source when |D| > kConvAlpha * max |D|
constexpr int kConvReach = 3;        // a source activates the cells within this many steps
constexpr double kConvRidge = 1e-11; // ridge, relative to the mean diagonal of the Gram matrix

__device__ __forceinline__ bool solved_cell(const Geo& g, int n) { return cls_o(g.cls[n]) != 0; }

// The 36 features of a cell from its 3x3 neighbourhood in the last four differences:
// D(k, dj, di) returns D_{t-k} at the neighbour (dj, di) (k = 0..3, offsets -1..1).
template <class Load>
__device__ __forceinline__ void conv_features_from(Load D, float* out) {
  float S[4][3][3];
  for (int dj = -1; dj <= 1; dj++)
    for (int di = -1; di <= 1; di++) {
      const float d0 = D(0, dj, di), d1 = D(1, dj, di), d2 = D(2, dj, di), d3 = D(3, dj, di);
      const float t1 = d0 - d1, t1b = d1 - d2, t1c = d2 - d3;
      const float t2 = t1 - t1b, t2b = t1b - t1c;
      S[0][dj + 1][di + 1] = d0;
      S[1][dj + 1][di + 1] = t1;
      S[2][dj + 1][di + 1] = t2;
      S[3][dj + 1][di + 1] = t2 - t2b;
    }
  for (int k = 0; k < 4; k++) {
    float row[3][3];  // [y offset][value, x gradient, x curvature]
    for (int r = 0; r < 3; r++) {
      const float w = S[k][r][0], c = S[k][r][1], e = S[k][r][2];
      row[r][0] = c;
      row[r][1] = 0.5f * (e - w);
      row[r][2] = (e + w) - 2.0f * c;
    }
    for (int q = 0; q < 3; q++) {
      const float s = row[0][q], c = row[1][q], nn = row[2][q];
      out[k * 9 + q * 3 + 0] = c;
      out[k * 9 + q * 3 + 1] = 0.5f * (nn - s);
      out[k * 9 + q * 3 + 2] = (nn + s) - 2.0f * c;
    }
  }
}

// Term e of the normal equations: entry (a, b), a <= b, of the upper triangle in row order for
// e < 666, then the right-hand side of feature e - 666 (b == kConvFeat, the target).  Row a
// starts at term a n - a (a - 1) / 2 (n = kConvFeat); a comes from the quadratic formula and an
// integer correction.
__device__ __forceinline__ void conv_term(int e, int& a, int& b) {
  constexpr int n = kConvFeat, tri = n * (n + 1) / 2;
  if (e >= tri) {
    a = e - tri;
    b = n;
    return;
  }
  auto start = [](int r) { return r * n - r * (r - 1) / 2; };
  int r = (int)(((2 * n + 1) - sqrtf((float)((2 * n + 1) * (2 * n + 1) - 8 * e))) * 0.5f);
  r = max(0, min(r, n - 1));
  while (r + 1 < n && start(r + 1) <= e) r++;
  while (start(r) > e) r--;
  a = r;
  b = r + (e - start(r));
}

// Copies N values into shared memory with NT threads: every thread first loads its values into
// registers (all loads in flight together), then stores them.  load(k) returns value k.
template <int N, int NT, class Load>
__device__ __forceinline__ void stage(float* dst, int tid, Load load) {
  constexpr int kPer = (N + NT - 1) / NT;
  float v[kPer];
#pragma unroll
  for (int u = 0; u < kPer; u++) {
    const int k = tid + u * NT;
    v[u] = (k < N) ? load(k) : 0.f;
  }
#pragma unroll
  for (int u = 0; u < kPer; u++) {
    const int k = tid + u * NT;
    if (k < N) dst[k] = v[u];
  }
}

// Compensated summation (Neumaier): s + c carries the sum to about twice FP32 precision.
__device__ __forceinline__ void neumaier(float& s, float& c, float x) {
  const float t = s + x;
  if (fabsf(s) >= fabsf(x)) c = c + ((s - t) + x);
  else c = c + ((x - t) + s);
  s = t;
}

// One CTA per strip of 32x2 cells: the FP32 normal-equation terms of the newest training pair
// (features of the previous step on its active cells, target the newest difference).  A strip
// without active cells only records that.
__device__ __forceinline__ void conv_gram_body(const Geo& g) {
  const Ctl* ctl = g.ctl;
  const unsigned r = ctl->warm_ready;
  if (r < 5 || ctl->Iter != 0) return;  // a training pair needs five differences; first outer iteration only
  const unsigned h = r - 1;
  const int Nx = g.Nx, Ny = g.Ny;
  const int nsx = (Nx + kConvStripX - 1) / kConvStripX, nsy = (Ny + kConvStripY - 1) / kConvStripY;
  if ((int)blockIdx.x >= nsx || (int)blockIdx.y >= nsy) return;
  const int strip = blockIdx.x + blockIdx.y * nsx, nstrips = nsx * nsy;
  const int tid = threadIdx.x + kConvStripX * threadIdx.y;
  const int i = blockIdx.x * kConvStripX + threadIdx.x, j = blockIdx.y * kConvStripY + threadIdx.y;
  const bool in = i < Nx && j < Ny;
  const int n = i + j * Nx;
  const unsigned bits = in ? g.cact[(h - 1) & 1][n] : 0u;
  if (!__syncthreads_or(bits != 0u)) {
    if (tid < 2) g.cnrows[tid * nstrips + strip] = 0;
    return;
  }
  // the previous step's four differences over the strip and a margin of one (clamped to the mesh)
  const int i0 = blockIdx.x * kConvStripX, j0 = blockIdx.y * kConvStripY;
  constexpr int kFx = kConvStripX + 2, kFy = kConvStripY + 2;
  __shared__ float Df[2][4][kFy][kFx];
  stage<2 * 4 * kFy * kFx, kConvStripX * kConvStripY>(&Df[0][0][0][0], tid, [&](int k) {
    const int f = k / (4 * kFy * kFx), rem = k - f * (4 * kFy * kFx);
    const int t = rem / (kFy * kFx), rem2 = rem - t * (kFy * kFx), yy = rem2 / kFx, xx = rem2 - yy * kFx;
    const int jj = min(max(j0 - 1 + yy, 0), Ny - 1), ii = min(max(i0 - 1 + xx, 0), Nx - 1);
    return g.cD[f][(h - 1 - t) % kConvRing][ii + jj * Nx];
  });
  __shared__ float Tg[2][kConvStripY][kConvStripX];  // the target: the newest difference
  stage<2 * kConvStripY * kConvStripX, kConvStripX * kConvStripY>(&Tg[0][0][0], tid, [&](int k) {
    const int f = k / (kConvStripY * kConvStripX), rem = k - f * (kConvStripY * kConvStripX);
    const int yy = rem / kConvStripX, xx = rem - yy * kConvStripX;
    const int jj = min(j0 + yy, Ny - 1), ii = min(i0 + xx, Nx - 1);
    return g.cD[f][h % kConvRing][ii + jj * Nx];
  });
  __shared__ float F[kConvStripX * kConvStripY][kConvFeat + 1];
  __shared__ int wcount[kConvStripY];
  const int lane = threadIdx.x;
  __syncthreads();
  for (int f = 0; f < 2; f++) {
    const bool act = (bits >> f) & 1u;
    const unsigned bal = __ballot_sync(0xffffffffu, act);
    if (lane == 0) wcount[threadIdx.y] = __popc(bal);
    __syncthreads();
    int nrows = 0, pos = 0;
    for (int w = 0; w < kConvStripY; w++) {
      if (w < (int)threadIdx.y) pos += wcount[w];
      nrows += wcount[w];
    }
    pos += __popc(bal & ((1u << lane) - 1u));
    if (act) {
      const int x0 = threadIdx.x + 1, y0 = threadIdx.y + 1;
      conv_features_from([&](int k, int dj, int di) { return Df[f][k][y0 + dj][x0 + di]; }, F[pos]);
      F[pos][kConvFeat] = Tg[f][threadIdx.y][threadIdx.x];
    }
    __syncthreads();
    if (tid == 0) g.cnrows[f * nstrips + strip] = nrows;
    if (nrows > 0) {
      // each thread's terms e = tid + 64 k accumulate side by side (every term still sums its
      // rows in order)
      constexpr int kNT = kConvStripX * kConvStripY, kPerT = (kConvTerms + kNT - 1) / kNT;
      int ta[kPerT], tb[kPerT];
      float acc[kPerT];
      for (int k = 0; k < kPerT; k++) {
        const int e = tid + k * kNT;
        if (e < kConvTerms) conv_term(e, ta[k], tb[k]);
        else ta[k] = tb[k] = 0;
        acc[k] = 0.f;
      }
      for (int q = 0; q < nrows; q++)
#pragma unroll
        for (int k = 0; k < kPerT; k++) acc[k] = acc[k] + F[q][ta[k]] * F[q][tb[k]];
      float* out = g.cpart + ((size_t)strip * 2 + f) * kConvTerms;
      for (int k = 0; k < kPerT; k++) {
        const int e = tid + k * kNT;
        if (e < kConvTerms) out[e] = acc[k];
      }
    }
    __syncthreads();
  }
}

// CTA (segment, field x 3 blocks of 256 terms): the sums over the non-empty strips of a segment of
// kConvSeg strips, in strip order.  The last CTA of each (field, term block) to finish -- a ticket
// counter -- then sums the non-empty segments in order and writes the pair's FP64 window slot.
__device__ __forceinline__ void conv_reduce_body(const Geo& g) {
  Ctl* ctl = g.ctl;
  const unsigned r = ctl->warm_ready;
  if (r < 5 || ctl->Iter != 0) return;  // no training pair yet, or not the step's first outer iteration
  const unsigned pair = r - 5;
  const int nsx = (g.Nx + kConvStripX - 1) / kConvStripX, nsy = (g.Ny + kConvStripY - 1) / kConvStripY;
  const int nstrips = nsx * nsy, nseg = (nstrips + kConvSeg - 1) / kConvSeg;
  const int seg = blockIdx.x, yb = blockIdx.y, f = yb / 3, tid = threadIdx.x;
  if (seg >= nseg) return;
  const int e = (yb % 3) * 256 + tid, s0 = seg * kConvSeg, ns = min(kConvSeg, nstrips - s0);
  __shared__ int cnt[kConvSeg];
  __shared__ bool last;
  if (tid < ns) cnt[tid] = g.cnrows[f * nstrips + s0 + tid];
  __syncthreads();
  if (tid == 0) {
    int rows = 0;
    for (int q = 0; q < ns; q++) rows += cnt[q];
    g.cseg_rows[yb * nseg + seg] = rows;
  }
  if (e < kConvTerms) {
    float sum = 0.f, cmp = 0.f;
    for (int q0 = 0; q0 < ns; q0 += 16) {  // sixteen loads in flight, then the ordered sum
      float v[16];
#pragma unroll
      for (int u = 0; u < 16; u++) {
        const int q = q0 + u;
        v[u] = (q < ns && cnt[q] > 0) ? g.cpart[((size_t)(s0 + q) * 2 + f) * kConvTerms + e] : 0.f;
      }
#pragma unroll
      for (int u = 0; u < 16; u++)
        if (q0 + u < ns && cnt[q0 + u] > 0) neumaier(sum, cmp, v[u]);
    }
    g.cseg[((size_t)seg * 2 + f) * kConvTerms + e] = sum + cmp;
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) {
    const unsigned t = atomicAdd(&ctl->conv_ticket[yb], 1u);
    last = (t == (unsigned)nseg - 1u);
    if (last) ctl->conv_ticket[yb] = 0u;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  if (e >= kConvTerms) return;
  const int* rows = g.cseg_rows + yb * nseg;
  float sum = 0.f, cmp = 0.f;
  for (int q0 = 0; q0 < nseg; q0 += 16) {
    float v[16];
    int rw[16];
#pragma unroll
    for (int u = 0; u < 16; u++) {
      const int q = q0 + u;
      rw[u] = q < nseg ? rows[q] : 0;
      v[u] = q < nseg ? g.cseg[((size_t)q * 2 + f) * kConvTerms + e] : 0.f;
    }
#pragma unroll
    for (int u = 0; u < 16; u++)
      if (rw[u] > 0) neumaier(sum, cmp, v[u]);
  }
  g.cgram[((size_t)(pair % kConvWin) * 2 + f) * kConvTerms + e] = (double)(sum + cmp);
}

// One CTA of 256 threads per field: once the window is full, the FP64 window sum, the ridge, and
// the FP32 system solved by Gauss-Jordan elimination without pivoting (the matrix is symmetric
// positive definite): at pivot k, with u_j = M_kj / M_kk (a reciprocal, then products), row k
// becomes u and every other row i has M_ij - M_ik u_j, j > k, the right-hand side included; after
// the last pivot the right-hand side holds the weights.  Two buffers, one barrier per pivot.
__device__ __forceinline__ void conv_solve_body(const Geo& g) {
  Ctl* ctl = g.ctl;
  const unsigned r = ctl->warm_ready;
  const int f = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  if (ctl->Iter != 0) return;  // the step's first outer iteration only
  if (r < 5 || r - 5 + 1 < (unsigned)kConvWin) {  // the window is not full yet
    if (tid == 0) ctl->conv_ok[f] = 0u;
    return;
  }
  constexpr int n = kConvFeat, W = n + 1;
  __shared__ double G[kConvTerms];
  __shared__ float M[2][n][W + 1];
  __shared__ double lam;
  for (int e = tid; e < kConvTerms; e += nt) {
    double x[kConvWin];
#pragma unroll
    for (int q = 0; q < kConvWin; q++) x[q] = g.cgram[((size_t)q * 2 + f) * kConvTerms + e];
    double v = 0.0;
#pragma unroll
    for (int q = 0; q < kConvWin; q++) v = v + x[q];
    G[e] = v;
  }
  __syncthreads();
  if (tid == 0) {
    double tr = 0.0;
    for (int a = 0, e = 0; a < n; a++) {
      tr = tr + G[e];  // entry (a, a)
      e += n - a;      // first entry of the next row
    }
    lam = kConvRidge * tr / (double)n;
  }
  __syncthreads();
  for (int e = tid; e < kConvTerms; e += nt) {
    int a, b;
    conv_term(e, a, b);
    if (b == n) M[0][a][n] = (float)G[e];
    else if (a == b) M[0][a][a] = (float)(G[e] + lam);
    else M[0][a][b] = M[0][b][a] = (float)G[e];
  }
  __syncthreads();
  for (int k = 0; k < n; k++) {
    const float (*src)[W + 1] = M[k & 1];
    float (*dst)[W + 1] = M[(k + 1) & 1];
    const float piv = src[k][k];
    if (!(piv > 0.f && piv < 3.0e38f)) {  // the same decision in every thread
      if (tid == 0) ctl->conv_ok[f] = 0u;
      return;
    }
    const float rp = 1.0f / piv;
    const int ncol = n - k;  // columns k+1 .. n
    for (int idx = tid; idx < n * ncol; idx += nt) {
      const int i = idx / ncol, j = k + 1 + (idx - i * ncol);
      const float u = src[k][j] * rp;
      dst[i][j] = (i == k) ? u : src[i][j] - src[i][k] * u;
    }
    __syncthreads();
  }
  const float (*fin)[W + 1] = M[n & 1];
  if (tid < n) ctl->conv_w[f][tid] = fin[tid][n];
  if (tid == 0) {
    bool finite = true;
    for (int k = 0; k < n; k++) finite = finite && isfinite(fin[k][n]);
    ctl->conv_ok[f] = finite ? 1u : 0u;
  }
}

// Per 32x8 tile: the active flags of the newest difference (cells within kConvReach steps of a
// source, |D_h| > kConvAlpha max |D_h|; x wrapped on periodic meshes), then on the active cells
// the stencil's start x_h + sum_k w_k feature_k.
__device__ __forceinline__ void conv_apply_body(const Geo& g) {
  const Ctl* ctl = g.ctl;
  const unsigned r = ctl->warm_ready, cur = ctl->cur;
  if (r < 1 || ctl->Iter != 0) return;  // the step's first outer iteration only
  const unsigned h = r - 1;
  const int Nx = g.Nx, Ny = g.Ny;
  constexpr int TX = 32, TY = 8, R = kConvReach, HX = TX + 2 * R, HY = TY + 2 * R;
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  if (i0 >= Nx || j0 >= Ny) return;
  const int tid = threadIdx.x + threadIdx.y * TX;
  const int i = i0 + threadIdx.x, j = j0 + threadIdx.y;
  const bool in = i < Nx && j < Ny;
  const int n = i + j * Nx;
  const bool per = g.bits & F_PERIODIC;
  __shared__ float Dh[2][HY][HX];
  stage<2 * HY * HX, TX * TY>(&Dh[0][0][0], tid, [&](int k) {
    const int f = k / (HY * HX), rem = k - f * (HY * HX);
    const int yy = rem / HX, xx = rem - yy * HX, jj = j0 - R + yy;
    int ii = i0 - R + xx;
    if (per) ii = (ii + Nx) % Nx;
    return (jj >= 0 && jj < Ny && ii >= 0 && ii < Nx) ? g.cD[f][h % kConvRing][ii + jj * Nx] : 0.f;
  });
  __syncthreads();
  unsigned bits = 0;
  if (in && solved_cell(g, n)) {
    const float thr0 = kConvAlpha * __uint_as_float(ctl->conv_max[h & 1][0]);
    const float thr1 = kConvAlpha * __uint_as_float(ctl->conv_max[h & 1][1]);
    for (int dj = -R; dj <= R; dj++) {
      const int rx = R - (dj < 0 ? -dj : dj);
      for (int di = -rx; di <= rx; di++) {
        const int yy = threadIdx.y + R + dj, xx = threadIdx.x + R + di;
        if (fabsf(Dh[0][yy][xx]) > thr0) bits |= 1u;
        if (fabsf(Dh[1][yy][xx]) > thr1) bits |= 2u;
      }
    }
  }
  if (in) g.cact[h & 1][n] = (uint8_t)bits;
  const unsigned use = (ctl->conv_ok[0] ? 1u : 0u) | (ctl->conv_ok[1] ? 2u : 0u);
  if (!__syncthreads_or((bits & use) != 0u)) return;
  // the four newest differences over the tile and a margin of one (clamped to the mesh)
  __shared__ float Dt[2][4][TY + 2][TX + 2];
  stage<2 * 4 * (TY + 2) * (TX + 2), TX * TY>(&Dt[0][0][0][0], tid, [&](int k) {
    const int f = k / (4 * (TY + 2) * (TX + 2)), rem = k - f * (4 * (TY + 2) * (TX + 2));
    const int t = rem / ((TY + 2) * (TX + 2)), rem2 = rem - t * ((TY + 2) * (TX + 2));
    const int yy = rem2 / (TX + 2), xx = rem2 - yy * (TX + 2);
    const int jj = min(max(j0 - 1 + yy, 0), Ny - 1), ii = min(max(i0 - 1 + xx, 0), Nx - 1);
    return g.cD[f][(h - t) % kConvRing][ii + jj * Nx];
  });
  __syncthreads();
  for (int f = 0; f < 2; f++) {
    if (!((bits & use) >> f & 1u)) continue;
    float feat[kConvFeat];
    const int x0 = threadIdx.x + 1, y0 = threadIdx.y + 1;
    conv_features_from([&](int k, int dj, int di) { return Dt[f][k][y0 + dj][x0 + di]; }, feat);
    float corr = 0.f;
    for (int k = 0; k < kConvFeat; k++) corr = corr + ctl->conv_w[f][k] * feat[k];
    if (f == 0) g.p[cur][n] = g.p_m[0][n] + (double)corr;
    else g.T[cur][n] = g.T_m[0][n] + (double)corr;
  }
}

}  // namespace

__global__ void k_conv_gram(Geo g) { conv_gram_body(g); }
__global__ void k_conv_reduce(Geo g) { conv_reduce_body(g); }
__global__ void k_conv_solve(Geo g) { conv_solve_body(g); }
__global__ void k_conv_apply(Geo g) { conv_apply_body(g); }
__global__ void kb_conv_reduce(const Geo* gs) {
  __shared__ Geo sg;
  if (!stage_geo(sg, gs)) return;
  conv_reduce_body(sg);
}
__global__ void kb_conv_gram(const Geo* gs) {
  __shared__ Geo sg;
  if (!stage_geo(sg, gs)) return;
  conv_gram_body(sg);
}
__global__ void kb_conv_solve(const Geo* gs) {
  __shared__ Geo sg;
  if (!stage_geo(sg, gs)) return;
  conv_solve_body(sg);
}
__global__ void kb_conv_apply(const Geo* gs) {
  __shared__ Geo sg;
  if (!stage_geo(sg, gs)) return;
  conv_apply_body(sg);
}

}  // namespace sts
