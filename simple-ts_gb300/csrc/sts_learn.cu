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
// cells (cell order), then with compensated FP32 sums (Neumaier) over the strips with rows of each
// 32x8 tile (strip order), over the tiles with rows (tile order) and over the window (slot order);
// a ridge of 1e-11 of the mean diagonal (FP64 trace); Gauss-Jordan elimination in FP32.  This
// file is compiled without fused multiply-adds and every sum has a fixed order, so the result does
// not depend on scheduling and the CPU oracle reproduces it bit for bit.  (GB300's FP64 pipe does
// about 2 adds per clock per SM: the sums stay on the FP32 pipes.)
//
// Per step: k_step_begin stores the newest differences, writes the quadratic start, takes the
// stencil's start where one was prepared, and clears the coming maximum (conv_step_begin_cell,
// conv_block_max).  After the sweeps, beside the correction and boundary kernels (which write p
// and T only outside the solved cells; the step ends when both are done): conv_gram forms the
// terms of the training pair whose target is the coming difference, conv_solve fits the weights,
// conv_next stores the coming difference and its maximum, and conv_predict flags the active cells
// and prepares the next step's start there -- everything the next step's start needs, computed
// from the final iterate while the GPU is mostly idle.
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

// One CTA per tile of 32x8 cells, i.e. four strips of 32x2 cells, at the end of a step (after the
// sweeps): the normal-equation terms of the training pair whose target is the coming difference
// D_{h+1} = x_{n+1} - x_n -- the step's final iterate less the start-of-step value, rounded to
// FP32 exactly as the next step's start stores it -- and whose features are those of the newest
// stored difference D_h on its active cells; summed in FP32 over each strip's rows in cell order,
// then over the tile's strips with rows in strip order (compensated).  A tile without active
// cells only records that.  (The pair is the one the next step would form; forming it now lets
// the fit run beside the step's last kernels instead of on the next step's path.)
__device__ __forceinline__ void conv_gram_body(const Geo& g) {
  const Ctl* ctl = g.ctl;
  const unsigned r = ctl->warm_ready, cur = ctl->cur;
  // conv_next folds the coming difference's maximum once this kernel is done (with several
  // outer iterations, only the last one's counts)
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x < 2 && threadIdx.y == 0)
    const_cast<Ctl*>(ctl)->conv_max[r & 1][threadIdx.x] = 0u;
  if (r < 4) return;  // the features need four stored differences
  const unsigned h = r - 1;
  const int Nx = g.Nx, Ny = g.Ny;
  constexpr int TX = 32, TY = 8, NS = TY / kConvStripY, SR = kConvStripX * kConvStripY;
  const int ntx = (Nx + TX - 1) / TX, nty = (Ny + TY - 1) / TY, ntiles = ntx * nty;
  if ((int)blockIdx.x >= ntx || (int)blockIdx.y >= nty) return;
  const int tile = blockIdx.x + blockIdx.y * ntx;
  const int tid = threadIdx.x + TX * threadIdx.y, lane = threadIdx.x;
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  const int i = i0 + threadIdx.x, j = j0 + threadIdx.y;
  const bool in = i < Nx && j < Ny;
  const int n = i + j * Nx;
  const unsigned bits = in ? g.cact[h & 1][n] : 0u;
  if (!__syncthreads_or(bits != 0u)) {
    if (tid < 2) g.crows[tid * ntiles + tile] = 0;
    return;
  }
  __shared__ float Df[4][TY + 2][TX + 2];          // D_{h..h-3} of one field, margin one (clamped)
  __shared__ float F[NS][SR][kConvFeat + 1];       // per strip: active rows' features and target
  __shared__ int wcount[TY];
  float* P = &F[0][0][0];                          // the strips' terms, after F is used: [NS][kConvTerms]
  const int s = threadIdx.y / kConvStripY, t64 = threadIdx.x + TX * (threadIdx.y % kConvStripY);
  for (int f = 0; f < 2; f++) {
    stage<4 * (TY + 2) * (TX + 2), TX * TY>(&Df[0][0][0], tid, [&](int k) {
      const int t = k / ((TY + 2) * (TX + 2)), rem = k - t * ((TY + 2) * (TX + 2));
      const int yy = rem / (TX + 2), xx = rem - yy * (TX + 2);
      const int jj = min(max(j0 - 1 + yy, 0), Ny - 1), ii = min(max(i0 - 1 + xx, 0), Nx - 1);
      return g.cD[f][(h - t) % kConvRing][ii + jj * Nx];
    });
    const bool act = (bits >> f) & 1u;  // active cells are solved cells
    const float target = act ? (float)((f ? g.T[cur][n] : g.p[cur][n]) - (f ? g.T_m[0][n] : g.p_m[0][n])) : 0.f;
    const unsigned bal = __ballot_sync(0xffffffffu, act);
    if (lane == 0) wcount[threadIdx.y] = __popc(bal);
    __syncthreads();
    int nr[NS];
    for (int q = 0; q < NS; q++) nr[q] = wcount[kConvStripY * q] + wcount[kConvStripY * q + 1];
    const int pos = ((threadIdx.y % kConvStripY) ? wcount[threadIdx.y - 1] : 0) + __popc(bal & ((1u << lane) - 1u));
    if (act) {
      const int x0 = threadIdx.x + 1, y0 = threadIdx.y + 1;
      conv_features_from([&](int k, int dj, int di) { return Df[k][y0 + dj][x0 + di]; }, F[s][pos]);
      F[s][pos][kConvFeat] = target;
    }
    __syncthreads();
    // each strip's 64 threads: terms e = t64 + 64 k accumulate side by side, every term over the
    // strip's rows in order
    constexpr int kPerT = (kConvTerms + SR - 1) / SR;
    float acc[kPerT];
    for (int k = 0; k < kPerT; k++) acc[k] = 0.f;
    if (nr[s] > 0) {
      int ta[kPerT], tb[kPerT];
      for (int k = 0; k < kPerT; k++) {
        const int e = t64 + k * SR;
        if (e < kConvTerms) conv_term(e, ta[k], tb[k]);
        else ta[k] = tb[k] = 0;
      }
      for (int q = 0; q < nr[s]; q++)
#pragma unroll
        for (int k = 0; k < kPerT; k++) acc[k] = acc[k] + F[s][q][ta[k]] * F[s][q][tb[k]];
    }
    __syncthreads();  // F is read no more: its space takes the strips' terms
    for (int k = 0; k < kPerT; k++) {
      const int e = t64 + k * SR;
      if (e < kConvTerms) P[s * kConvTerms + e] = acc[k];
    }
    __syncthreads();
    for (int e = tid; e < kConvTerms; e += TX * TY) {
      float sum = 0.f, cmp = 0.f;
      for (int q = 0; q < NS; q++)
        if (nr[q] > 0) neumaier(sum, cmp, P[q * kConvTerms + e]);
      g.cpart[((size_t)tile * 2 + f) * kConvTerms + e] = sum + cmp;
    }
    if (tid == 0) g.crows[f * ntiles + tile] = nr[0] + nr[1] + nr[2] + nr[3];
    __syncthreads();
  }
}

// One CTA of kConvSolveThreads (1024) threads per field, after conv_gram: the pair's total over the
// tiles with rows (tile order, compensated FP32; one thread per term, sixteen tiles' values in
// flight) into the window ring; once the window is full, the weights for the next step: the window
// sum (slot order, compensated), the ridge (FP64 trace), and the FP32 system solved by Gauss-Jordan
// elimination without pivoting (the matrix is symmetric positive definite): at pivot k, with
// u_j = M_kj (1 / M_kk), row k becomes u and every other row i has M_ij - M_ik u_j, j > k, the
// right-hand side included; after the last pivot the right-hand side holds the weights.  Thread
// (c, g) owns column c and rows g, g + 27; two buffers, one barrier per pivot.  Which thread
// computes a value changes no bit: every sum keeps its order, every entry its formula.
constexpr int kSolveCols = kConvFeat + 1, kSolveRowGroups = 27, kSolveThreads = kConvSolveThreads;
static_assert(kSolveCols * kSolveRowGroups <= kSolveThreads, "launch size of k_conv_solve");
static_assert(kConvTerms <= kSolveThreads, "one term per thread");

__device__ __forceinline__ void conv_solve_body(const Geo& g) {
  Ctl* ctl = g.ctl;
  const unsigned r = ctl->warm_ready;
  const int f = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  if (r < 4) {
    if (tid == 0) ctl->conv_ok[f] = 0u;
    return;
  }
  const unsigned pair = r - 4;  // pairs formed so far, less one
  constexpr int TX = 32, TY = 8;
  const int ntiles = ((g.Nx + TX - 1) / TX) * ((g.Ny + TY - 1) / TY);
  constexpr int kChunk = 4096, kFlags = (kChunk + kSolveThreads - 1) / kSolveThreads, kAhead = 16;
  __shared__ int list[kChunk];
  __shared__ int wsum[32];
  __shared__ int count;
  float sum = 0.f, cmp = 0.f;
  const int e = tid;  // this thread's term (threads at or beyond kConvTerms only help with the lists)
  const int* rows = g.crows + f * ntiles;
  for (int t0 = 0; t0 < ntiles; t0 += kChunk) {
    // ordered list of the chunk's tiles with rows: block-wide exclusive scan of the flags
    int fl[kFlags], mine = 0;
#pragma unroll
    for (int q = 0; q < kFlags; q++) {
      const int t = t0 + tid * kFlags + q;
      fl[q] = (t < ntiles && tid * kFlags + q < kChunk) ? (rows[t] > 0) : 0;
    }
    for (int q = 0; q < kFlags; q++) mine += fl[q];
    const int lane = tid & 31, warp = tid >> 5, nw = (nt + 31) >> 5;
    int incl = mine;
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    int before = 0, total = 0;
    for (int w = 0; w < nw; w++) {
      if (w < warp) before += wsum[w];
      total += wsum[w];
    }
    int pos = before + incl - mine;
    for (int q = 0; q < kFlags; q++)
      if (fl[q]) list[pos++] = t0 + tid * kFlags + q;
    if (tid == 0) count = total;
    __syncthreads();
    const int cnt = count;
    if (e < kConvTerms)
      for (int q0 = 0; q0 < cnt; q0 += kAhead) {  // kAhead tiles' loads in flight, then the ordered sums
        float v[kAhead];
#pragma unroll
        for (int u = 0; u < kAhead; u++)
          v[u] = (q0 + u < cnt) ? g.cpart[((size_t)list[q0 + u] * 2 + f) * kConvTerms + e] : 0.f;
#pragma unroll
        for (int u = 0; u < kAhead; u++)
          if (q0 + u < cnt) neumaier(sum, cmp, v[u]);
      }
    __syncthreads();
  }
  if (e < kConvTerms) g.cgram[((size_t)(pair % kConvWin) * 2 + f) * kConvTerms + e] = sum + cmp;
  __syncthreads();
  if (pair + 1 < (unsigned)kConvWin) {
    if (tid == 0) ctl->conv_ok[f] = 0u;
    return;
  }
  constexpr int n = kConvFeat, W = n + 1;
  __shared__ float Gw[kConvTerms];
  __shared__ float M[2][n][W + 1];
  __shared__ double lam;
  if (e < kConvTerms) {
    float x[kConvWin];
#pragma unroll
    for (int q = 0; q < kConvWin; q++) x[q] = g.cgram[((size_t)q * 2 + f) * kConvTerms + e];
    float ws = 0.f, wc = 0.f;
#pragma unroll
    for (int q = 0; q < kConvWin; q++) neumaier(ws, wc, x[q]);
    Gw[e] = ws + wc;
  }
  __syncthreads();
  if (tid == 0) {
    double tr = 0.0;
    for (int a = 0, e = 0; a < n; a++) {
      tr = tr + (double)Gw[e];  // entry (a, a)
      e += n - a;               // first entry of the next row
    }
    lam = kConvRidge * tr / (double)n;
  }
  __syncthreads();
  for (int e = tid; e < kConvTerms; e += nt) {
    int a, b;
    conv_term(e, a, b);
    if (b == n) M[0][a][n] = Gw[e];
    else if (a == b) M[0][a][a] = (float)((double)Gw[e] + lam);
    else M[0][a][b] = M[0][b][a] = Gw[e];
  }
  __syncthreads();
  const int c = tid % kSolveCols, rg = tid / kSolveCols;
  for (int k = 0; k < n; k++) {
    const float (*src)[W + 1] = M[k & 1];
    float (*dst)[W + 1] = M[(k + 1) & 1];
    const float piv = src[k][k];
    if (!(piv > 0.f && piv < 3.0e38f)) {  // the same decision in every thread
      if (tid == 0) ctl->conv_ok[f] = 0u;
      return;
    }
    if (c > k && rg < kSolveRowGroups) {
      const float u = src[k][c] * (1.0f / piv);
      for (int i = rg; i < n; i += kSolveRowGroups) dst[i][c] = (i == k) ? u : src[i][c] - src[i][k] * u;
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

// End of a step, all cells, one CTA per 32x8 tile: the coming difference D_r = x_{n+1} - x_n
// (FP32; 0 off the solved cells) into its ring slot -- the value the next step's start stores
// there again -- its per-field maximum over the tile, and over the mesh (cleared by conv_gram), for
// the active flags.
__device__ __forceinline__ void conv_next_body(const Geo& g) {
  Cell c = cell(g);
  const Ctl* ctl = g.ctl;
  const unsigned r = ctl->warm_ready, cur = ctl->cur;
  unsigned m[2] = {0u, 0u};
  if (c.ok) {
    const int n = c.ij;
    float d[2] = {0.f, 0.f};
    if (solved_cell(g, n)) {
      d[0] = (float)(g.p[cur][n] - g.p_m[0][n]);
      d[1] = (float)(g.T[cur][n] - g.T_m[0][n]);
      m[0] = __float_as_uint(fabsf(d[0]));
      m[1] = __float_as_uint(fabsf(d[1]));
    }
    g.cD[0][r % kConvRing][n] = d[0];
    g.cD[1][r % kConvRing][n] = d[1];
  }
  __shared__ unsigned wm[2][32];
  const int tid = threadIdx.x + threadIdx.y * blockDim.x, lane = tid & 31, warp = tid >> 5;
  const int nw = (blockDim.x * blockDim.y + 31) >> 5;
  for (int f = 0; f < 2; f++) {
    const unsigned v = __reduce_max_sync(0xffffffffu, m[f]);
    if (lane == 0) wm[f][warp] = v;
  }
  __syncthreads();
  if (tid < 2) {
    unsigned v = 0;
    for (int w = 0; w < nw; w++) v = max(v, wm[tid][w]);
    const int ntx = (g.Nx + 31) / 32, nty = (g.Ny + 7) / 8;
    if ((int)blockIdx.x < ntx && (int)blockIdx.y < nty) g.ctmax[tid * ntx * nty + blockIdx.x + blockIdx.y * ntx] = v;
    if (v) atomicMax(&g.ctl->conv_max[r & 1][tid], v);
  }
}

// End of a step, per 32x8 tile: the active flags of the coming difference D_r (cells within
// kConvReach steps of a source, |D_r| > kConvAlpha max |D_r|; x wrapped on periodic meshes), and
// on the active cells, with the weights just fitted, the stencil's start for the next step,
// x_{n+1} + sum_k w_k feature_k, kept in cnext and flagged for k_step_begin (bits 2 and 3).
// A tile none of whose 3x3 neighbouring tiles holds a source (their maxima from conv_next; the
// reach is shorter than a tile) has no active cell and only clears its flags; the front covers a
// few percent of the tiles.  Tiles whose reach wraps around a periodic mesh take the per-cell test.
__device__ __forceinline__ void conv_predict_body(const Geo& g) {
  const Ctl* ctl = g.ctl;
  const unsigned r = ctl->warm_ready, cur = ctl->cur;
  const int Nx = g.Nx, Ny = g.Ny;
  constexpr int TX = 32, TY = 8, R = kConvReach, HX = TX + 2 * R, HY = TY + 2 * R;
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  if (i0 >= Nx || j0 >= Ny) return;
  const int tid = threadIdx.x + threadIdx.y * TX;
  const int i = i0 + threadIdx.x, j = j0 + threadIdx.y;
  const bool in = i < Nx && j < Ny;
  const int n = i + j * Nx;
  const bool per = g.bits & F_PERIODIC;
  const float thr0 = kConvAlpha * __uint_as_float(ctl->conv_max[r & 1][0]);
  const float thr1 = kConvAlpha * __uint_as_float(ctl->conv_max[r & 1][1]);
  {
    const int ntx = (Nx + TX - 1) / TX, nty = (Ny + TY - 1) / TY;
    bool near = per && (i0 - R < 0 || i0 + TX - 1 + R >= Nx);
    if (tid < 18) {
      const int f = tid / 9, q = tid - 9 * f, tx = (int)blockIdx.x + q % 3 - 1, ty = (int)blockIdx.y + q / 3 - 1;
      if (tx >= 0 && tx < ntx && ty >= 0 && ty < nty)
        near = near || __uint_as_float(g.ctmax[f * ntx * nty + tx + ty * ntx]) > (f ? thr1 : thr0);
    }
    if (!__syncthreads_or(near)) {
      if (in) g.cact[r & 1][n] = 0;
      return;
    }
  }
  __shared__ float Dh[2][HY][HX];
  stage<2 * HY * HX, TX * TY>(&Dh[0][0][0], tid, [&](int k) {
    const int f = k / (HY * HX), rem = k - f * (HY * HX);
    const int yy = rem / HX, xx = rem - yy * HX, jj = j0 - R + yy;
    int ii = i0 - R + xx;
    if (per) ii = (ii + Nx) % Nx;
    return (jj >= 0 && jj < Ny && ii >= 0 && ii < Nx) ? g.cD[f][r % kConvRing][ii + jj * Nx] : 0.f;
  });
  __syncthreads();
  unsigned bits = 0;
  if (in && solved_cell(g, n)) {
    for (int dj = -R; dj <= R; dj++) {
      const int rx = R - (dj < 0 ? -dj : dj);
      for (int di = -rx; di <= rx; di++) {
        const int yy = threadIdx.y + R + dj, xx = threadIdx.x + R + di;
        if (fabsf(Dh[0][yy][xx]) > thr0) bits |= 1u;
        if (fabsf(Dh[1][yy][xx]) > thr1) bits |= 2u;
      }
    }
  }
  const unsigned use = bits & ((ctl->conv_ok[0] ? 1u : 0u) | (ctl->conv_ok[1] ? 2u : 0u));
  if (in) g.cact[r & 1][n] = (uint8_t)(bits | (use << 2));
  if (!__syncthreads_or(use != 0u)) return;
  // the four newest differences over the tile and a margin of one (clamped to the mesh)
  __shared__ float Dt[2][4][TY + 2][TX + 2];
  stage<2 * 4 * (TY + 2) * (TX + 2), TX * TY>(&Dt[0][0][0][0], tid, [&](int k) {
    const int f = k / (4 * (TY + 2) * (TX + 2)), rem = k - f * (4 * (TY + 2) * (TX + 2));
    const int t = rem / ((TY + 2) * (TX + 2)), rem2 = rem - t * ((TY + 2) * (TX + 2));
    const int yy = rem2 / (TX + 2), xx = rem2 - yy * (TX + 2);
    const int jj = min(max(j0 - 1 + yy, 0), Ny - 1), ii = min(max(i0 - 1 + xx, 0), Nx - 1);
    return g.cD[f][(r - t) % kConvRing][ii + jj * Nx];
  });
  __syncthreads();
  for (int f = 0; f < 2; f++) {
    if (!((use >> f) & 1u)) continue;
    float feat[kConvFeat];
    const int x0 = threadIdx.x + 1, y0 = threadIdx.y + 1;
    conv_features_from([&](int k, int dj, int di) { return Dt[f][k][y0 + dj][x0 + di]; }, feat);
    float corr = 0.f;
    for (int k = 0; k < kConvFeat; k++) corr = corr + ctl->conv_w[f][k] * feat[k];
    g.cnext[f][n] = (f == 0 ? g.p[cur][n] : g.T[cur][n]) + (double)corr;
  }
}

}  // namespace

__global__ void k_conv_gram(Geo g) { conv_gram_body(g); }
__global__ void __launch_bounds__(kConvSolveThreads) k_conv_solve(Geo g) { conv_solve_body(g); }
__global__ void k_conv_next(Geo g) { conv_next_body(g); }
__global__ void k_conv_predict(Geo g) { conv_predict_body(g); }
__global__ void kb_conv_gram(const Geo* gs) {
  __shared__ Geo sg;
  if (!stage_geo(sg, gs)) return;
  conv_gram_body(sg);
}
__global__ void __launch_bounds__(kConvSolveThreads) kb_conv_solve(const Geo* gs) {
  __shared__ Geo sg;
  if (!stage_geo(sg, gs)) return;
  conv_solve_body(sg);
}
__global__ void kb_conv_next(const Geo* gs) {
  __shared__ Geo sg;
  if (!stage_geo(sg, gs)) return;
  conv_next_body(sg);
}
__global__ void kb_conv_predict(const Geo* gs) {
  __shared__ Geo sg;
  if (!stage_geo(sg, gs)) return;
  conv_predict_body(sg);
}

}  // namespace sts
