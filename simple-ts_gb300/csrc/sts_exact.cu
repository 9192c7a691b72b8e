// FP64 kernels of the SIMPLE-TS time step, bit-exact with the reference CPU solver.
//
// This translation unit is compiled with --fmad=false: every expression keeps the
// reference's operand order and rounding (no fused multiply-add), and division and
// sqrt are IEEE round-to-nearest, so each field matches the serial reference
// solver bit for bit.  One thread owns one cell (i, j); a per-cell class byte
// says which of the reference's two formula variants applies (interior list
// "nch" or boundary list "bc", SIMPLE_TS_MPI.cpp:8581-9063).
//
// Kernels per outer iteration: assemble -> sweep x S -> correct -> face_rho ->
// boundary -> flux_diff.  The sweep count S is decided on the device by the last
// block of each sweep (SIMPLE_TS_MPI.cpp:4099-4107), which also drives the CUDA
// graph's conditional WHILE node.
#include <cuda_runtime.h>
#include <math_constants.h>

#include "sts_common.cuh"
#include "sts_kernels.h"

#include "sts_device.cuh"

namespace sts {

// ---------------------------------------------------------------------------
// start of a time step: *_pr copies and per-step counters (SIMPLE_TS_MPI.cpp:3233-3260)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void k_step_begin_body(const Geo& g, int counters, unsigned long long h_outer, int in_graph) {
  Cell c = cell(g);
  Ctl* ctl = g.ctl;
  const unsigned cur = ctl->cur;
  // warm_start 4: the newest step differences and their maxima (the model's kernels follow)
  const unsigned conv_r = ctl->warm_ready;
  unsigned conv_m[2] = {0u, 0u};
  if (c.ok) {
    g.u_pr[c.ij] = g.u[c.ij];
    g.v_pr[c.ij] = g.v[c.ij];
    g.p_pr[c.ij] = g.p[cur][c.ij];
    g.T_pr[c.ij] = g.T[cur][c.ij];
    g.rho_pr[c.ij] = g.rho[c.ij];
    // warm start: the sweeps of this step start from p, T extrapolated in time on the solved
    // cells (the first step, without history, from the current values)
    if (counters && (g.warm_start == 1 || g.warm_start == 2) && cls_o(g.cls[c.ij])) {
      const int n = c.ij;
      const double x = g.p[cur][n], y = g.T[cur][n];
      const unsigned r = ctl->warm_ready;
      if (r == 0) {
        g.p_m[0][n] = x; g.p_m[1][n] = x;
        g.T_m[0][n] = y; g.T_m[1][n] = y;
      } else {
        if (g.warm_start == 2 && r >= 2) {
          g.p[cur][n] = 3.0 * (x - g.p_m[0][n]) + g.p_m[1][n];
          g.T[cur][n] = 3.0 * (y - g.T_m[0][n]) + g.T_m[1][n];
        } else {
          g.p[cur][n] = x + (x - g.p_m[0][n]);
          g.T[cur][n] = y + (y - g.T_m[0][n]);
        }
        g.p_m[1][n] = g.p_m[0][n]; g.p_m[0][n] = x;
        g.T_m[1][n] = g.T_m[0][n]; g.T_m[0][n] = y;
      }
    }
    if (counters && g.warm_start == 4) {
      if (cls_o(g.cls[c.ij])) {
        conv_step_begin_cell(g, c.ij, cur, conv_r, conv_m);
      } else if (conv_r >= 1) {
        g.cD[0][(conv_r - 1) % kConvRing][c.ij] = 0.f;
        g.cD[1][(conv_r - 1) % kConvRing][c.ij] = 0.f;
      }
    }
  }
  if (counters && g.warm_start == 4) conv_block_max(g, conv_r, conv_m);
  if (counters && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0) {
    if (in_graph) cudaGraphSetConditional((cudaGraphConditionalHandle)h_outer, 1);
    for (unsigned k = 0; k < ctl->Iter && k < 64; k++) {
      ctl->res_p[k] = 0; ctl->res_T[k] = 0; ctl->res_p0[k] = 0; ctl->res_T0[k] = 0; ctl->sweeps[k] = 0;
    }
    ctl->it += g.ht;
    ctl->it_counter++;
    ctl->Iter_pr2 = ctl->Iter_pr1;
    ctl->Iter_pr1 = ctl->Iter;
    ctl->Iter = 0;
    ctl->continue_iter = 1;
    ctl->step_sweeps = 0;
  }
}
__global__ void k_step_begin(Geo g, int counters, unsigned long long h_outer, int in_graph) {
  k_step_begin_body(g, counters, h_outer, in_graph);
}
// The same, with the state u, v, p, T first read from device-addressable host buffers (when
// given): every thread stores its cell's values before the step's copies read them back.
__global__ void k_step_begin_in(Geo g, unsigned long long h_outer, int in_graph, const double* u_in,
                                const double* v_in, const double* p_in, const double* T_in) {
  const Cell c = cell(g);
  if (u_in && c.ok) {
    const unsigned cur = g.ctl->cur;
    const double u = u_in[c.ij], v = v_in[c.ij], p = p_in[c.ij], T = T_in[c.ij];
    g.u[c.ij] = u;
    g.v[c.ij] = v;
    g.p[cur][c.ij] = p;
    g.T[cur][c.ij] = T;
  }
  k_step_begin_body(g, 1, h_outer, in_graph);
}

// Batched start of a step: a case takes part while its run goes on and steps are left; cases
// that stopped skip every kernel of the step (stage_geo reads the flag).
__global__ void kb_step_begin(const Geo* gs) {
  __shared__ Geo sg;
  stage_geo(sg, gs);
  Ctl* ctl = sg.ctl;
  const bool running = ctl->continue_step && ctl->steps_left > 0;
  __syncthreads();
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0) ctl->running = running ? 1u : 0u;
  if (running) k_step_begin_body(sg, 1, 0ull, 0);
}

// Steps the next batched launch may take, for every case.
__global__ void kb_set_steps(const Geo* gs, int ncases, unsigned n) {
  for (int c = threadIdx.x; c < ncases; c += blockDim.x) gs[c].ctl->steps_left = n;
}

// The batched step loop goes on while any case runs and has steps left: sets the graph's loop
// condition, or *flag outside a graph.
__global__ void kb_continue(const Geo* gs, int ncases, unsigned long long h_step, unsigned* flag) {
  int any = 0;
  for (int c = threadIdx.x; c < ncases; c += blockDim.x) {
    const Ctl* ctl = gs[c].ctl;
    any |= (ctl->continue_step && ctl->steps_left > 0) ? 1 : 0;
  }
  any = __syncthreads_or(any);
  if (threadIdx.x == 0) {
    if (flag) *flag = any ? 1u : 0u;
    else cudaGraphSetConditional((cudaGraphConditionalHandle)h_step, any ? 1 : 0);
  }
}

// ---------------------------------------------------------------------------
// Learned warm start (mode 3).  The sweeps of a step start from x_n + w0 D_n + w1 D_{n-1} +
// w2 D_{n-2} (D_t = x_t - x_{t-1} on the solved cells), a linear predictor fitted by least
// squares on the solver's own trajectory: over the last kWarmWin steps s, D_s is regressed on
// d(s-1) = (D_{s-1}, D_{s-1} - D_{s-2}, D_{s-1} - 2 D_{s-2} + D_{s-3}) -- the span of the three
// previous differences in a basis that stays well conditioned on smooth trajectories.  Each
// step adds its target's Gram and right-hand-side terms (products of the FP64 differences
// rounded to FP32, summed per CTA in FP32 and across CTAs in FP64 in a fixed order) and drops
// the oldest; the 3x3 system is solved by Cramer's rule.  Until kWarmWin + 3 differences exist,
// or when the system is nearly singular, the weights are those of quadratic extrapolation
// (linear on the second step).  p and T have their own weights.
// warm_diff: the new difference and its normal-equation terms; warm_fit: one CTA per case
// sums them and solves; warm_apply: the initial iterate.
// ---------------------------------------------------------------------------
constexpr int kWarmTerms = 9;  // per field: Gram entries 00 01 02 11 12 22, then right-hand sides 0 1 2

__device__ __forceinline__ void warm_diff_body(const Geo& g) {
  Cell c = cell(g);
  const Ctl* ctl = g.ctl;
  const unsigned r = ctl->warm_ready, cur = ctl->cur;
  float t[2 * kWarmTerms];
  for (int k = 0; k < 2 * kWarmTerms; k++) t[k] = 0.f;
  if (c.ok && cls_o(g.cls[c.ij])) {
    const int n = c.ij;
    const double x = g.p[cur][n], y = g.T[cur][n];
    if (r >= 1) {
      const unsigned h = r - 1;
      const double dn[2] = {x - g.p_m[0][n], y - g.T_m[0][n]};
      g.Dp[h % kWarmRing][n] = dn[0];
      g.DT[h % kWarmRing][n] = dn[1];
      if (h >= 3) {
        for (int f = 0; f < 2; f++) {
          double* const* R = f ? g.DT : g.Dp;
          const double d1 = R[(h - 1) % kWarmRing][n], d2 = R[(h - 2) % kWarmRing][n], d3 = R[(h - 3) % kWarmRing][n];
          const float a0 = (float)d1, a1 = (float)(d1 - d2), a2 = (float)(d1 - 2.0 * d2 + d3), yy = (float)dn[f];
          float* o = t + f * kWarmTerms;
          o[0] = a0 * a0; o[1] = a0 * a1; o[2] = a0 * a2; o[3] = a1 * a1; o[4] = a1 * a2; o[5] = a2 * a2;
          o[6] = a0 * yy; o[7] = a1 * yy; o[8] = a2 * yy;
        }
      }
    }
    g.p_m[0][n] = x;
    g.T_m[0][n] = y;
  }
  // CTA sums, written as partials indexed by the case's own 32x8 tiling, so one case alone and
  // the same case in a batch (whose grid is that of the largest case) add them in the same order
  __shared__ float part[8][2 * kWarmTerms];
  const int tid = threadIdx.x + threadIdx.y * blockDim.x, lane = tid & 31, warp = tid >> 5;
  for (int k = 0; k < 2 * kWarmTerms; k++) {
    float v = t[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) part[warp][k] = v;
  }
  __syncthreads();
  const int tx = (g.Nx + 31) / 32, ty = (g.Ny + 7) / 8;
  if (tid < 2 * kWarmTerms && (int)blockIdx.x < tx && (int)blockIdx.y < ty) {
    float v = 0.f;
    for (int w = 0; w < (int)((blockDim.x * blockDim.y) >> 5); w++) v += part[w][tid];
    g.warm_part[(blockIdx.x + blockIdx.y * tx) * (2 * kWarmTerms) + tid] = v;
  }
}

__device__ __forceinline__ double det3(const double m[3][3]) {
  return m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
         m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
}

// One CTA of 32 x 2*kWarmTerms threads per case: warp k sums term k over the case's CTAs.
__device__ __forceinline__ void warm_fit_body(const Geo& g) {
  Ctl* ctl = g.ctl;
  const unsigned r = ctl->warm_ready;
  const int nblocks = ((g.Nx + 31) / 32) * ((g.Ny + 7) / 8);
  const int tid = threadIdx.x + threadIdx.y * blockDim.x, lane = tid & 31, k = tid >> 5;
  __shared__ double sum[2 * kWarmTerms];
  if (r >= 4 && k < 2 * kWarmTerms) {
    double v = 0.0;
    for (int b = lane; b < nblocks; b += 32) v += (double)g.warm_part[b * (2 * kWarmTerms) + k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) sum[k] = v;
  }
  __syncthreads();
  if (tid != 0) return;
  if (r == 0) {
    ctl->warm_ready = 1;
    return;
  }
  const unsigned h = r - 1, have = h + 1;
  if (h >= 3)
    for (int q = 0; q < 2 * kWarmTerms; q++) ctl->warm_acc[h % kWarmWin][q / kWarmTerms][q % kWarmTerms] = sum[q];
  for (int f = 0; f < 2; f++) {
    double w[3] = {2.0, -1.0, 0.0};
    if (have < 2) {
      w[0] = 1.0;
      w[1] = 0.0;
    }
    if (have >= 3u + kWarmWin) {
      double a[kWarmTerms] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      for (int s2 = 0; s2 < kWarmWin; s2++)
        for (int q = 0; q < kWarmTerms; q++) a[q] += ctl->warm_acc[s2][f][q];
      const double G[3][3] = {{a[0], a[1], a[2]}, {a[1], a[3], a[4]}, {a[2], a[4], a[5]}};
      const double rhs[3] = {a[6], a[7], a[8]};
      const double det = det3(G), scale = G[0][0] * G[1][1] * G[2][2];
      if (scale > 0 && fabs(det) > 1e-6 * scale) {
        double cc[3];
        for (int i = 0; i < 3; i++) {
          double Gi[3][3];
          for (int x = 0; x < 3; x++)
            for (int y = 0; y < 3; y++) Gi[x][y] = (y == i) ? rhs[x] : G[x][y];
          cc[i] = det3(Gi) / det;
        }
        w[0] = cc[0] + cc[1] + cc[2];
        w[1] = -cc[1] - 2.0 * cc[2];
        w[2] = cc[2];
      }
    }
    for (int q = 0; q < 3; q++) ctl->warm_w[f][q] = w[q];
  }
  ctl->warm_ready = r + 1;
}

__device__ __forceinline__ void warm_apply_body(const Geo& g) {
  Cell c = cell(g);
  const Ctl* ctl = g.ctl;
  const unsigned r = ctl->warm_ready;  // already counts this step
  if (r < 2 || !c.ok || !cls_o(g.cls[c.ij])) return;
  const unsigned h = r - 2, have = h + 1, cur = ctl->cur;
  const int n = c.ij;
  double ep = ctl->warm_w[0][0] * g.Dp[h % kWarmRing][n];
  double eT = ctl->warm_w[1][0] * g.DT[h % kWarmRing][n];
  if (have >= 2) {
    ep += ctl->warm_w[0][1] * g.Dp[(h - 1) % kWarmRing][n];
    eT += ctl->warm_w[1][1] * g.DT[(h - 1) % kWarmRing][n];
  }
  if (have >= 3) {
    ep += ctl->warm_w[0][2] * g.Dp[(h - 2) % kWarmRing][n];
    eT += ctl->warm_w[1][2] * g.DT[(h - 2) % kWarmRing][n];
  }
  g.p[cur][n] += ep;
  g.T[cur][n] += eT;
}

__global__ void k_warm_diff(Geo g) { warm_diff_body(g); }
__global__ void k_warm_fit(Geo g) { warm_fit_body(g); }
__global__ void k_warm_apply(Geo g) { warm_apply_body(g); }
__global__ void kb_warm_diff(const Geo* gs) {
  __shared__ Geo sg;
  if (!stage_geo(sg, gs)) return;
  warm_diff_body(sg);
}
__global__ void kb_warm_fit(const Geo* gs) {
  __shared__ Geo sg;
  if (!stage_geo(sg, gs)) return;
  warm_fit_body(sg);
}
__global__ void kb_warm_apply(const Geo* gs) {
  __shared__ Geo sg;
  if (!stage_geo(sg, gs)) return;
  warm_apply_body(sg);
}

// ---------------------------------------------------------------------------
// momentum coefficients (u: SIMPLE_TS_MPI.cpp:3269-3344 bc, :3478-3545 nch;
// v: :3373-3450 bc, :3561-3630 nch) and the energy source ScT1 (:3655-3756)
// ---------------------------------------------------------------------------
// The interior form's corner term of ScT1 at cell (i, j) (s0 below): it belongs to the mesh
// vertex at the cell's lower-left corner, and s1, s2, s3 of a cell are s0 of its east, north and
// north-east neighbours whenever those neighbours are the plain i+1 / j+1 cells (same operands,
// same operations, so the same bits).
__device__ __forceinline__ double corner_s0(const Geo& g, const Nb& d) {
  const int i = d.i, j = d.j, jm = j - (0 < j ? 1 : 0);
  return div_cr(g.u[d.ij] - g.u[d.ij_1], g.hy[jm] + g.hy[j], g.ryy_m[j]) +
         div_cr(g.v[d.ij] - g.v[d.i_1j], g.hx[d.i_1] + g.hx[i], g.rxx_m[i]);
}

// Two more shared terms of the interior forms.  The u part of cell (i, j) takes
// sT·(v_N - v)·2/3 at (i, j) and at (i-1, j): staged at (i, j) is the west one, and the east
// neighbour's staged term is the cell's own whenever that neighbour is the plain i+1 cell.  The
// v part takes sT·(u_E - u)·2/3 at (i, j) and at (i, j-1): staged at (i, j) is the south one,
// and the north neighbour's staged term is the cell's own whenever that neighbour exists.
__device__ __forceinline__ double west_term_v(const Geo& g, const Nb& d) {
  return div_cr(g.sqrt_T[d.i_1j] * (g.v[d.i_1j1] - g.v[d.i_1j]) * 2.0, 3.0, g.r3);
}
__device__ __forceinline__ double south_term_u(const Geo& g, const Nb& d) {
  return div_cr(g.sqrt_T[d.ij_1] * (g.u[d.i1j_1] - g.u[d.ij_1]) * 2.0, 3.0, g.r3);
}

constexpr int kAsmCorners = 400;  // corners of the largest block shape the tuner uses (128x2 + 1)

__device__ __forceinline__ void assemble_body(const Geo& g, unsigned long long h_sweep, int in_graph) {
  // shared terms of the block's cells and of one more column and row, computed once each by
  // the block's threads in turn
  __shared__ double corner[kAsmCorners], west_v[kAsmCorners], south_u[kAsmCorners];
  const int W1 = blockDim.x + 1, ncorner = W1 * (blockDim.y + 1);
  const bool shared_corners = ncorner <= kAsmCorners;
  if (shared_corners) {
    const int tid = threadIdx.x + threadIdx.y * blockDim.x, nthr = blockDim.x * blockDim.y;
    const int i0 = blockIdx.x * blockDim.x, j0 = blockIdx.y * blockDim.y;
    for (int q = tid; q < ncorner; q += nthr) {
      const int py = q / W1, px = q - py * W1, ci = i0 + px, cj = j0 + py;
      double s = 0.0, w = 0.0, z = 0.0;
      if (ci < g.Nx && cj < g.Ny) {
        const Nb e = neighbours(ci, cj, g.Nx, g.Ny, g.bits & F_PERIODIC);
        s = corner_s0(g, e);
        w = west_term_v(g, e);
        z = south_term_u(g, e);
      }
      corner[q] = s;
      west_v[q] = w;
      south_u[q] = z;
    }
    __syncthreads();
  }
  Cell c = cell(g);
  Ctl* ctl = g.ctl;
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0) {
    ctl->Iter_p_c = 0;
    ctl->pt_done = 0;
    ctl->res_bits_p = 0;
    ctl->res_bits_T = 0;
    ctl->res_bits_u = 0;
    ctl->res_bits_v = 0;
    if (in_graph) cudaGraphSetConditional((cudaGraphConditionalHandle)h_sweep, 1);
  }
  if (!c.ok) return;
  const uint8_t cl = g.cls[c.ij];
  if (!(cl & 0x3F)) return;
  const int i = c.i, j = c.j, Nx = g.Nx;
  const Nb d = neighbours(i, j, g.Nx, g.Ny, g.bits & F_PERIODIC);
  // east: d.i1 is i + 1 (no clamp or wrap); north: the cell above exists
  const int q = threadIdx.x + threadIdx.y * W1;
  const bool east = shared_corners && d.i1 == i + 1, north = shared_corners && j + 1 < g.Ny;
  const double cT = ctl->cT, cPch = ctl->cPch, ht = g.ht;
  const double* __restrict__ hx = g.hx;
  const double* __restrict__ hy = g.hy;
  const double* __restrict__ u = g.u;
  const double* __restrict__ v = g.v;
  const double* __restrict__ Fx = g.Fx;
  const double* __restrict__ Fy = g.Fy;
  const double* __restrict__ sT = g.sqrt_T;
  const double* __restrict__ rho = g.rho;
  const double* __restrict__ rho_pr = g.rho_pr;
  auto B = [&](int k) -> double { return cls_fluid(g.cls[k]) ? 1.0 : 0.0; };
  auto BB = [&](int k) -> bool { return cls_fluid(g.cls[k]); };

  const int cu = cls_u(cl);
  if (cu) {
    const double F_xu1 = 0.5 * (Fx[d.i_1j] + Fx[d.ij]);
    const double F_xu2 = 0.5 * (Fx[d.ij] + Fx[d.i1j]);
    double Scu;
    if (cu == CLS_BC) {
      Scu = cT * (div_cr(B(d.i1j) * u[d.i1j] * sT[d.ij] * hy[j], hx[i] * 3.0, g.r3x[i]) +
                  div_cr(B(d.i_2j) * u[d.i_1j] * sT[d.i_1j] * hy[j], hx[d.i_1] * 3.0, g.r3x[d.i_1]) +
                  g.Gamma_yf[d.ij1] * (v[d.ij1] * B(d.ij1) - v[d.i_1j1] * B(d.i_1j1)) -
                  g.Gamma_yf[d.ij] * (v[d.ij] * B(d.ij_1) - v[d.i_1j] * B(d.i_1j_1)) -
                  div_cr(sT[d.ij] * (v[d.ij1] * B(d.ij1) - v[d.ij] * B(d.ij_1)) * 2.0, 3.0, g.r3) +
                  div_cr(sT[d.i_1j] * (v[d.i_1j1] * B(d.i_1j1) - v[d.i_1j] * B(d.i_1j_1)) * 2.0, 3.0, g.r3));
    } else {
      const double wE = east ? west_v[q + 1] : div_cr(sT[d.ij] * (v[d.ij1] - v[d.ij]) * 2.0, 3.0, g.r3);
      const double wW = shared_corners ? west_v[q] : west_term_v(g, d);
      Scu = cT * (div_cr(u[d.i1j] * sT[d.ij] * hy[j], hx[i] * 3.0, g.r3x[i]) +
                  div_cr(u[d.i_1j] * sT[d.i_1j] * hy[j], hx[d.i_1] * 3.0, g.r3x[d.i_1]) +
                  g.Gamma_yf[d.ij1] * (v[d.ij1] - v[d.i_1j1]) - g.Gamma_yf[d.ij] * (v[d.ij] - v[d.i_1j]) - wE + wW);
    }
    const double Spu = div_cr(-(g.D_ux[d.ij] + g.D_ux[d.i1j]), 3.0, g.r3);
    const double au1 = dmax0(0, F_xu1) + g.D_ux[d.ij];
    const double au2 = dmax0(0, -F_xu2) + g.D_ux[d.i1j];
    const double au3 = 0.5 * (dmax0(0, Fy[d.i_1j]) + dmax0(0, Fy[d.ij])) + g.D_uy[d.ij];
    const double au4 = 0.5 * (dmax0(0, -Fy[d.i_1j1]) + dmax0(0, -Fy[d.ij1])) + g.D_uy[d.ij1];
    const double bu3 = div_cr((rho_pr[d.i_1j] * hx[d.i_1] + rho_pr[d.ij] * hx[i]) * g.u_pr[d.ij] * hy[j] * 0.5, ht, g.rht) + Scu;
    const double au0 = au1 + au2 + au3 + au4 + 0.5 * (-Fy[d.i_1j] - Fy[d.ij] + Fy[d.i_1j1] + Fy[d.ij1]) + F_xu2 - F_xu1 -
                       Spu + div_cr((rho[d.i_1j] * hx[d.i_1] + rho[d.ij] * hx[i]) * hy[j] * 0.5, ht, g.rht);
    double up;
    if (cu == CLS_BC)
      up = div_z(au1 * B(d.i1j) * u[d.i_1j] + au2 * B(d.i_2j) * u[d.i1j] + au3 * u[d.ij_1] + au4 * u[d.ij1] + bu3, au0);
    else
      up = div_z(au1 * u[d.i_1j] + au2 * u[d.i1j] + au3 * u[d.ij_1] + au4 * u[d.ij1] + bu3, au0);
    const double dpc = cPch * hy[j] / au0;
    const double hr = hy[j] * g.rho_u[d.ij];
    g.u_pseudo[d.ij] = up;
    g.d12[d.ij] = dpc;
    g.apx[d.ij] = dpc * hr;
    g.bpx[d.ij] = (cu == CLS_BC) ? B(d.i_1j) * B(d.ij) * hr * up : hr * up;
  }

  const int cv = cls_v(cl);
  if (cv) {
    const int jm = j - ((j - 1) >= 0 ? 1 : 0);
    const int far = d.ij_1 - ((j - 2) >= 0 ? Nx : 0);
    const double F_yv3 = 0.5 * (Fy[d.ij_1] + Fy[d.ij]);
    const double F_yv4 = 0.5 * (Fy[d.ij] + Fy[d.ij1]);
    double Scv;
    if (cv == CLS_BC) {
      Scv = cT * (div_cr(B(d.ij1) * v[d.ij1] * sT[d.ij] * hx[i], hy[j] * 3.0, g.r3y[j]) +
                  div_cr(B(far) * v[d.ij_1] * sT[d.ij_1] * hx[i], hy[jm] * 3.0, g.r3y[jm]) +
                  g.Gamma_xf[d.i1j] * (u[d.i1j] * B(d.i1j) - u[d.i1j_1] * B(d.i1j_1)) -
                  g.Gamma_xf[d.ij] * (u[d.ij] * B(d.i_1j) - u[d.ij_1] * B(d.i_1j_1)) -
                  div_cr(sT[d.ij] * (u[d.i1j] * B(d.i1j) - u[d.ij] * B(d.i_1j)) * 2.0, 3.0, g.r3) +
                  div_cr(sT[d.ij_1] * (u[d.i1j_1] * B(d.i1j_1) - u[d.ij_1] * B(d.i_1j_1)) * 2.0, 3.0, g.r3)) -
            g.c_Fr_v * (rho[d.ij_1] * hx[i] * 0.5 * hy[jm] + rho[d.ij] * hx[i] * 0.5 * hy[j]);
    } else {
      const double zN = north ? south_u[q + W1] : div_cr(sT[d.ij] * (u[d.i1j] - u[d.ij]) * 2.0, 3.0, g.r3);
      const double zS = shared_corners ? south_u[q] : south_term_u(g, d);
      Scv = cT * (div_cr(v[d.ij1] * sT[d.ij] * hx[i], hy[j] * 3.0, g.r3y[j]) +
                  div_cr(v[d.ij_1] * sT[d.ij_1] * hx[i], hy[j - 1] * 3.0, g.r3y[j - 1]) +
                  g.Gamma_xf[d.i1j] * (u[d.i1j] - u[d.i1j_1]) - g.Gamma_xf[d.ij] * (u[d.ij] - u[d.ij_1]) - zN + zS) -
            g.c_Fr_v * (rho[d.ij_1] * hx[i] * 0.5 * hy[j - 1] + rho[d.ij] * hx[i] * 0.5 * hy[j]);
    }
    const double Spv = div_cr(-(g.D_vy[d.ij] + g.D_vy[d.ij1]), 3.0, g.r3);
    const double av1 = 0.5 * (dmax0(0, Fx[d.ij]) + dmax0(0, Fx[d.ij_1])) + g.D_vx[d.ij];
    const double av2 = 0.5 * (dmax0(0, -Fx[d.i1j]) + dmax0(0, -Fx[d.i1j_1])) + g.D_vx[d.i1j];
    const double av3 = dmax0(0, F_yv3) + g.D_vy[d.ij];
    const double av4 = dmax0(0, -F_yv4) + g.D_vy[d.ij1];
    const double bv3 = div_cr((rho_pr[d.ij_1] * hy[j - 1] + rho_pr[d.ij] * hy[j]) * g.v_pr[d.ij] * hx[i] * 0.5, ht, g.rht) + Scv;
    const double av0 = av1 + av2 + av3 + av4 + 0.5 * (Fx[d.i1j] - Fx[d.ij] + Fx[d.i1j_1] - Fx[d.ij_1]) + F_yv4 - F_yv3 -
                       Spv + div_cr((rho[d.ij_1] * hy[j - 1] + rho[d.ij] * hy[j]) * hx[i] * 0.5, ht, g.rht);
    double vp;
    if (cv == CLS_BC)
      vp = div_z(av1 * v[d.i_1j] + av2 * v[d.i1j] + av3 * B(far) * v[d.ij_1] + av4 * B(d.ij1) * v[d.ij1] + bv3, av0);
    else
      vp = div_z(av1 * v[d.i_1j] + av2 * v[d.i1j] + av3 * v[d.ij_1] + av4 * v[d.ij1] + bv3, av0);
    const double dpc = cPch * hx[i] / av0;
    const double hr = hx[i] * g.rho_v[d.ij];
    g.v_pseudo[d.ij] = vp;
    g.d34[d.ij] = dpc;
    g.apy[d.ij] = dpc * hr;
    g.bpy[d.ij] = (cv == CLS_BC) ? B(d.ij - Nx) * B(d.ij) * hr * vp : hr * vp;
  }

  const int co = cls_o(cl);
  if (co) {
    const int jm = j - (0 < j ? 1 : 0), jp = j + (j < (Nx - 1) ? 1 : 0);  // j is compared with Nx here (:3677)
    double dudx, dvdy, s0, s1, s2, s3;
    if (co == CLS_BC) {
      dudx = div_cr(B(d.i1j) * u[d.i1j] - B(d.i_1j) * u[d.ij], hx[i], g.rhx[i]);
      dvdy = div_cr(B(d.ij1) * v[d.ij1] - B(d.ij_1) * v[d.ij], hy[j], g.rhy[j]);
      s0 = div_z(u[d.ij] - u[d.ij_1], (double)(BB(d.i_1j_1) && BB(d.ij_1)) * hy[jm] + hy[j]) +
           div_z(v[d.ij] - v[d.i_1j], (double)(BB(d.i_1j_1) && BB(d.i_1j)) * hx[d.i_1] + hx[i]);
      s1 = div_z(u[d.i1j] - u[d.i1j_1], (double)(BB(d.ij_1) && BB(d.i1j_1)) * hy[jm] + hy[j]) +
           div_z(v[d.i1j] - v[d.ij], hx[i] + (double)(BB(d.i1j_1) && BB(d.i1j)) * hx[d.i1]);
      s2 = div_z(u[d.ij1] - u[d.ij], hy[j] + (double)(BB(d.i_1j1) && BB(d.ij1)) * hy[jp]) +
           div_z(v[d.ij1] - v[d.i_1j1], (double)(BB(d.i_1j) && BB(d.i_1j1)) * hx[d.i_1] + hx[i]);
      s3 = div_z(u[d.i1j1] - u[d.i1j], hy[j] + (double)(BB(d.ij1) && BB(d.i1j1)) * hy[jp]) +
           div_z(v[d.i1j1] - v[d.ij1], hx[i] + (double)(BB(d.i1j) && BB(d.i1j1)) * hx[d.i1]);
    } else {
      // the interior cells' sums hy[jm] + hy[j], hy[j] + hy[jp] and their x counterparts have
      // correctly rounded reciprocal tables (jp as here, clamped to the mesh for the table)
      const double rym = g.ryy_m[j], ryp = g.ryy_p[j], rxm = g.rxx_m[i], rxp = g.rxx_p[i];
      dudx = div_cr(u[d.i1j] - u[d.ij], hx[i], g.rhx[i]);
      dvdy = div_cr(v[d.ij1] - v[d.ij], hy[j], g.rhy[j]);
      // north corners also need jp = j + 1
      const bool north_c = north && j < Nx - 1;
      s0 = shared_corners ? corner[q]
                          : div_cr(u[d.ij] - u[d.ij_1], hy[jm] + hy[j], rym) +
                                div_cr(v[d.ij] - v[d.i_1j], hx[d.i_1] + hx[i], rxm);
      s1 = east ? corner[q + 1]
                : div_cr(u[d.i1j] - u[d.i1j_1], hy[jm] + hy[j], rym) + div_cr(v[d.i1j] - v[d.ij], hx[i] + hx[d.i1], rxp);
      s2 = north_c ? corner[q + W1]
                 : div_cr(u[d.ij1] - u[d.ij], hy[j] + hy[jp], ryp) + div_cr(v[d.ij1] - v[d.i_1j1], hx[d.i_1] + hx[i], rxm);
      s3 = (east && north_c)
               ? corner[q + W1 + 1]
               : div_cr(u[d.i1j1] - u[d.i1j], hy[j] + hy[jp], ryp) + div_cr(v[d.i1j1] - v[d.ij1], hx[i] + hx[d.i1], rxp);
    }
    g.ScT1[d.ij] = ht * sT[d.ij] * g.cT2 * hx[i] * hy[j] *
                       (2.0 * (dudx * dudx + dvdy * dvdy) + s0 * s0 + s1 * s1 + s2 * s2 + s3 * s3 -
                        div_cr((dudx + dvdy) * (dudx + dvdy) * 2.0, 3.0, g.r3)) +
                   g.p_pr[d.ij] * hx[i] * hy[j];
  }
}
__global__ void k_assemble(Geo g, unsigned long long h_sweep, int in_graph) { assemble_body(g, h_sweep, in_graph); }
__global__ void kb_assemble(const Geo* gs, unsigned long long h_sweep, int in_graph) {
  __shared__ Geo sg;
  if (!stage_geo(sg, gs)) return;
  assemble_body(sg, h_sweep, in_graph);
}

// ---------------------------------------------------------------------------
// one coupled p-T Jacobi sweep with the EOS substitution (SIMPLE_TS_MPI.cpp:3786-4131).
// Reads buffer `cur`, writes buffer `cur^1` for every cell (unsolved cells copy through,
// which keeps both buffers identical there exactly as the reference's memcpy + swap do).
// ---------------------------------------------------------------------------
// The first sweep of an outer iteration evaluates the reference expressions in full and
// stores their loop-invariant parts (identical operations, so identical bits); later sweeps
// reuse them and keep the reference's order for every term that involves the iterate.
// Invariants: a_k = aT_k, or aT_k * T_wall for a wall neighbour (the bc form multiplies the
// wall temperature by aT_k and adds exact zeros), divu, the T denominator, the p_pr/T_pr
// term and ht * (sum of the p coefficients).
// RCP (the persistent loop): the first sweep also stores RN(1/den_T) in inv[8] and later sweeps
// divide by den_T through it (div_cr, the same bits as the IEEE quotient) and read hx hy from the
// per-cell table instead of multiplying.
template <bool FIRST, bool RCP = false>
__device__ __forceinline__ void sweep_cell(const Geo& g, const Cell& c, const double* __restrict__ P,
                                           const double* __restrict__ TT, double* __restrict__ pn,
                                           double* __restrict__ Tn, double& rp, double& rT) {
  const uint8_t cl = g.cls[c.ij];
  const int co = cls_o(cl);
  if (!co) {
    pn[c.ij] = P[c.ij];
    Tn[c.ij] = TT[c.ij];
    return;
  }
  const int i = c.i, j = c.j;
  const Nb d = neighbours(i, j, g.Nx, g.Ny, g.bits & F_PERIODIC);
  const double* __restrict__ Fx = g.Fx;
  const double* __restrict__ Fy = g.Fy;
  const double* __restrict__ hx = g.hx;
  const double* __restrict__ hy = g.hy;
  const double* __restrict__ apx = g.apx;
  const double* __restrict__ apy = g.apy;
  const double ht = g.ht;
  const int ij = d.ij;
  double Tnew, pnew;
  if (FIRST) {
    const double aT1 = dmax0(0, Fx[d.ij]) + g.DTx[d.ij];
    const double aT2 = dmax0(0, -Fx[d.i1j]) + g.DTx[d.i1j];
    const double aT3 = dmax0(0, Fy[d.ij]) + g.DTy[d.ij];
    const double aT4 = dmax0(0, -Fy[d.ij1]) + g.DTy[d.ij1];
    const double divu = (g.u[d.i1j] - g.u[d.ij]) * hy[j] + (g.v[d.ij1] - g.v[d.ij]) * hx[i];
    const double denT =
        ht * (aT1 + aT2 + aT3 + aT4 + Fx[d.i1j] - Fx[d.ij] + Fy[d.ij1] - Fy[d.ij]) + hx[i] * hy[j] * g.rho[d.ij];
    double w1 = aT1, w2 = aT2, w3 = aT3, w4 = aT4;
    if (co == CLS_BC) {
      auto B = [&](int k) -> double { return cls_fluid(g.cls[k]) ? 1.0 : 0.0; };
      auto NB = [&](int k) -> double { return cls_fluid(g.cls[k]) ? 0.0 : 1.0; };
      Tnew = (ht * (aT1 * (B(d.i_1j) * TT[d.i_1j] + NB(d.i_1j) * g.Tw_u[d.ij]) +
                    aT2 * (B(d.i1j) * TT[d.i1j] + NB(d.i1j) * g.Tw_u[d.i1j]) +
                    aT3 * (B(d.ij_1) * TT[d.ij_1] + NB(d.ij_1) * g.Tw_v[d.ij]) +
                    aT4 * (B(d.ij1) * TT[d.ij1] + NB(d.ij1) * g.Tw_v[d.ij1]) + (1.0 - g.gamma1) * P[d.ij] * divu) +
              g.ScT1[d.ij]) /
             denT;
      if (!cls_fluid(g.cls[d.i_1j])) w1 = aT1 * g.Tw_u[d.ij];
      if (!cls_fluid(g.cls[d.i1j])) w2 = aT2 * g.Tw_u[d.i1j];
      if (!cls_fluid(g.cls[d.ij_1])) w3 = aT3 * g.Tw_v[d.ij];
      if (!cls_fluid(g.cls[d.ij1])) w4 = aT4 * g.Tw_v[d.ij1];
    } else {
      Tnew = (ht * (aT1 * TT[d.i_1j] + aT2 * TT[d.i1j] + aT3 * TT[d.ij_1] + aT4 * TT[d.ij1] +
                    (1.0 - g.gamma1) * P[d.ij] * divu) +
              g.ScT1[d.ij]) /
             denT;
    }
    const double pc = g.p_pr[d.ij] * hx[i] * hy[j] / (g.T_pr[d.ij]);
    const double sa = ht * (apx[d.ij] + apx[d.i1j] + apy[d.ij] + apy[d.ij1]);
    g.inv[0][ij] = w1;
    g.inv[1][ij] = w2;
    g.inv[2][ij] = w3;
    g.inv[3][ij] = w4;
    g.inv[4][ij] = divu;
    g.inv[5][ij] = denT;
    g.inv[6][ij] = pc;
    g.inv[7][ij] = sa;
    if (RCP) g.inv[8][ij] = 1.0 / denT;
    double num = apx[d.ij] * P[d.i_1j] + apx[d.i1j] * P[d.i1j] + apy[d.ij] * P[d.ij_1] + apy[d.ij1] * P[d.ij1] +
                 g.bpx[d.ij] - g.bpx[d.i1j] + g.bpy[d.ij] - g.bpy[d.ij1];
    if (co == CLS_BC) {
      const double gxb = ((g.bits & F_GIVEN_U_XB) && i == g.Nx_o0) ? 1.0 : 0.0;
      const double gxe = ((g.bits & F_GIVEN_U_XE) && i == g.Nx_o1 - 1) ? 1.0 : 0.0;
      num = num + gxb * Fx[d.ij] - gxe * Fx[d.i1j];
    }
    pnew = (ht * num + pc) / (sa + hx[i] * hy[j] / (Tnew));
  } else {
    const double w1 = g.inv[0][ij], w2 = g.inv[1][ij], w3 = g.inv[2][ij], w4 = g.inv[3][ij];
    double t1, t2, t3, t4;
    if (co == CLS_BC) {
      t1 = cls_fluid(g.cls[d.i_1j]) ? w1 * TT[d.i_1j] : w1;
      t2 = cls_fluid(g.cls[d.i1j]) ? w2 * TT[d.i1j] : w2;
      t3 = cls_fluid(g.cls[d.ij_1]) ? w3 * TT[d.ij_1] : w3;
      t4 = cls_fluid(g.cls[d.ij1]) ? w4 * TT[d.ij1] : w4;
    } else {
      t1 = w1 * TT[d.i_1j];
      t2 = w2 * TT[d.i1j];
      t3 = w3 * TT[d.ij_1];
      t4 = w4 * TT[d.ij1];
    }
    const double X = ht * (t1 + t2 + t3 + t4 + (1.0 - g.gamma1) * P[d.ij] * g.inv[4][ij]) + g.ScT1[d.ij];
    Tnew = RCP ? div_cr(X, g.inv[5][ij], g.inv[8][ij]) : X / g.inv[5][ij];
    double num = apx[d.ij] * P[d.i_1j] + apx[d.i1j] * P[d.i1j] + apy[d.ij] * P[d.ij_1] + apy[d.ij1] * P[d.ij1] +
                 g.bpx[d.ij] - g.bpx[d.i1j] + g.bpy[d.ij] - g.bpy[d.ij1];
    if (co == CLS_BC) {
      const double gxb = ((g.bits & F_GIVEN_U_XB) && i == g.Nx_o0) ? 1.0 : 0.0;
      const double gxe = ((g.bits & F_GIVEN_U_XE) && i == g.Nx_o1 - 1) ? 1.0 : 0.0;
      num = num + gxb * Fx[d.ij] - gxe * Fx[d.i1j];
    }
    const double H = RCP ? g.hxy[ij] : hx[i] * hy[j];  // the persistent loop reads the stored product
    pnew = (ht * num + g.inv[6][ij]) / (g.inv[7][ij] + H / (Tnew));
  }
  Tn[ij] = Tnew;
  pn[ij] = pnew;
  rT = fabs(Tnew - TT[ij]);
  rp = fabs(pnew - P[ij]);
}

template <bool FIRST>
__device__ __forceinline__ void sweep_body(const Geo& g, unsigned long long h_sweep, int in_graph) {
  Ctl* ctl = g.ctl;
  if (ctl->pt_done) {  // the loop already stopped: the launch is a no-op
    if (in_graph && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0)
      cudaGraphSetConditional((cudaGraphConditionalHandle)h_sweep, 0);
    return;
  }
  Cell c = cell(g);
  const unsigned cur = ctl->cur;
  double rp = 0, rT = 0;
  if (c.ok) sweep_cell<FIRST>(g, c, g.p[cur], g.T[cur], g.p[cur ^ 1], g.T[cur ^ 1], rp, rT);
  block_max2(rp, rT, &ctl->res_bits_p, &ctl->res_bits_T, &ctl->status);
  if (last_block(&ctl->block_count)) {
    // the reference's loop control, evaluated once per sweep (SIMPLE_TS_MPI.cpp:4087-4107)
    const unsigned I = ctl->Iter < 64 ? ctl->Iter : 63;
    const double res_p = as_d(atomicExch(&ctl->res_bits_p, 0ull));
    const double res_T = as_d(atomicExch(&ctl->res_bits_T, 0ull));
    ctl->res_p[I] = res_p;
    ctl->res_T[I] = res_T;
    if (ctl->Iter_p_c == 0) {
      ctl->res_p0[I] = res_p;
      ctl->res_T0[I] = res_T;
    }
    const unsigned n = ++ctl->Iter_p_c;
    bool cont;
    if (g.bits & F_FIXED_SWEEPS)
      cont = n < (unsigned)g.N_I_p_c;
    else
      cont = (n < 2) || ((n < (unsigned)g.N_I_p_c) && ((g.MaxError_p_c < res_p) || (g.MaxError_T < res_T)));
    ctl->cur = cur ^ 1;
    if (!cont) {
      ctl->pt_done = 1;
      ctl->sweeps[I] = n;
      ctl->step_sweeps += n;
    }
    if (in_graph) cudaGraphSetConditional((cudaGraphConditionalHandle)h_sweep, cont ? 1 : 0);
  }
}

__global__ void k_sweep_first(Geo g, unsigned long long h_sweep, int in_graph) { sweep_body<true>(g, h_sweep, in_graph); }

__global__ void k_sweep(Geo g, unsigned long long h_sweep, int in_graph) { sweep_body<false>(g, h_sweep, in_graph); }

// The whole sweep loop of one outer iteration, for one case or a batch, in one cooperative
// launch: the same cell arithmetic as k_sweep_first / k_sweep (so the same bits), one sweep per
// round of pt_loop_rounds.
struct ExactOps {
  static constexpr bool kCellList = true;  // a single case's sweeps split the solved cells evenly
  static __device__ __forceinline__ void pass(const Geo& g, const Cell& c, const LoopCase& s, double& rp, double& rT) {
    const double* P = g.p[s.cur];
    const double* TT = g.T[s.cur];
    double* pn = g.p[s.cur ^ 1];
    double* Tn = g.T[s.cur ^ 1];
    double a = 0, b = 0;
    if (s.phase == PS_FIRST) sweep_cell<true, true>(g, c, P, TT, pn, Tn, a, b);
    else sweep_cell<false, true>(g, c, P, TT, pn, Tn, a, b);
    rp = a;
    rT = b;
  }
  static __device__ __forceinline__ void pass32(const Geo&, const Cell&, const LoopCase&, float&, float&) {}
  static __device__ __forceinline__ void advance(const Geo& g, bool lead, LoopCase& s, double res_p, double res_T) {
    advance_fp64(g, lead, s, res_p, res_T);
  }
};

__global__ void __launch_bounds__(256, 4) k_pt_loop(Geo g, int ntiles, LoopCtl* lc) {
  pt_loop_rounds<ExactOps, true>(g, nullptr, nullptr, nullptr, 1, ntiles, lc);
}
__global__ void __launch_bounds__(256, 4) kb_pt_loop(const Geo* gs, const int* tile_case, const int* tile_first,
                                                     int ncases, int ntiles, LoopCtl* lc) {
  pt_loop_rounds<ExactOps, false>(gs[0], gs, tile_case, tile_first, ncases, ntiles, lc);
}

// ---------------------------------------------------------------------------
// velocity correction with L-inf residuals (SIMPLE_TS_MPI.cpp:4171-4305) and
// sqrt(T), rho = p/T (:4323-4330)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void correct_body(const Geo& g) {
  Cell c = cell(g);
  Ctl* ctl = g.ctl;
  const unsigned cur = ctl->cur;
  const double* __restrict__ p = g.p[cur];
  const double* __restrict__ T = g.T[cur];
  double ru = 0, rv = 0;
  if (c.ok) {
    const uint8_t cl = g.cls[c.ij];
    const int n = c.ij;
    if (cls_u(cl)) {
      const int w = (cls_u(cl) == CLS_BC && (g.bits & F_PERIODIC) && c.i == 0) ? n + g.Nx - 1 : n - 1;
      const double t = g.u[n];
      const double un = g.u_pseudo[n] - (p[n] - p[w]) * g.d12[n];
      g.u[n] = un;
      ru = fabs(un - t);
    }
    if (cls_v(cl)) {
      const double t = g.v[n];
      const double vn = g.v_pseudo[n] - (p[n] - p[n - g.Nx]) * g.d34[n];
      g.v[n] = vn;
      rv = fabs(vn - t);
    }
    g.sqrt_T[n] = sqrt(T[n]);
    g.rho[n] = cls_fluid(cl) ? p[n] / T[n] : 0.0;
  }
  block_max2(ru, rv, &ctl->res_bits_u, &ctl->res_bits_v, &ctl->status);
}
__global__ void k_correct(Geo g) {
  wait_for_predecessor();
  correct_body(g);
}
__global__ void kb_correct(const Geo* gs) {
  __shared__ Geo sg;
  if (!stage_geo(sg, gs)) return;
  correct_body(sg);
}

// Solve_rho_in_middle_points (SIMPLE_TS_MPI.cpp:10382-10437)
__device__ __forceinline__ void face_rho_body(const Geo& g) {
  Cell c = cell(g);
  if (!c.ok) return;
  const Nb d = neighbours(c.i, c.j, g.Nx, g.Ny, g.bits & F_PERIODIC);
  const double* __restrict__ rho = g.rho;
  const bool bw = cls_fluid(g.cls[d.i_1j]), bp = cls_fluid(g.cls[d.ij]), bs = cls_fluid(g.cls[d.ij_1]);
  double ru, rv;
  if (bw && bp) ru = upwind_rho(rho[d.i_1j], rho[d.ij], g.u[d.ij]);
  else if (bw != bp) ru = bw ? rho[d.i_1j] : rho[d.ij];
  else ru = 0.0;
  if (bs && bp) rv = upwind_rho(rho[d.ij_1], rho[d.ij], g.v[d.ij]);
  else if (bs != bp) rv = bs ? rho[d.ij_1] : rho[d.ij];
  else rv = 0.0;
  g.rho_u[d.ij] = ru;
  g.rho_v[d.ij] = rv;
}
__global__ void k_face_rho(Geo g) {
  wait_for_predecessor();
  face_rho_body(g);
}
__global__ void kb_face_rho(const Geo* gs) {
  __shared__ Geo sg;
  if (!stage_geo(sg, gs)) return;
  face_rho_body(sg);
}

// SolveFluxes (SIMPLE_TS_MPI.cpp:10440-10454) and SolveDiffisionTerms (:10457-10618)

// The linear interpolations of sqrt(T) behind Gamma_yf and Gamma_xf (LiY, LiX below) belong to
// cell faces: a cell's west interpolation in y is its west neighbour's own one, and its south
// interpolation in x is its south neighbour's own one, whenever those neighbours are the plain
// i-1 / j-1 cells.  A 32x8 block computes each once (with one more column on the west and one
// more row on the south) in shared memory; the operands and operations are those of the per-cell
// form, so the values are the same bits.
__device__ __forceinline__ double li_y_at(const Geo& g, int i, int j) {
  const Nb d = neighbours(i, j, g.Nx, g.Ny, g.bits & F_PERIODIC);
  const int jm = j - (0 < j ? 1 : 0);
  return div_cr(g.sqrt_T[d.ij_1] * g.hy[j] + g.sqrt_T[d.ij] * g.hy[jm], g.hy[jm] + g.hy[j], g.ryy_m[j]);
}
__device__ __forceinline__ double li_x_at(const Geo& g, int i, int j) {
  const Nb d = neighbours(i, j, g.Nx, g.Ny, g.bits & F_PERIODIC);
  return div_cr(g.sqrt_T[d.i_1j] * g.hx[i] + g.sqrt_T[d.ij] * g.hx[d.i_1], g.hx[d.i_1] + g.hx[i], g.rxx_m[i]);
}
constexpr int kFluxLy = 33 * 8, kFluxLx = 32 * 9;

// The reference's masked sum m_wall * sqrt(tw) + m_cell * h when the masks switch the wall term
// off (m_wall = 0, m_cell = 1): h itself whenever tw is a finite non-negative number (then
// 0 * sqrt(tw) is a zero) and h is not a zero (a zero added to h leaves it); any other operands
// take the sum as written.  It saves the square root where both cells of a face are fluid.
__device__ __forceinline__ double wall_term_off(double tw, double h) {
  return (tw >= 0.0 && tw < CUDART_INF && h != 0.0) ? h : 0.0 * sqrt(tw) + 1.0 * h;
}

// The diffusion coefficients' quotients of mesh widths at cell (i, j): divisions by mesh sums
// through their correctly rounded reciprocals (same bits as IEEE); a divisor (m1 h1 + m2 h2) with
// fluid masks m is h1, h2 or the rounded sum.  They depend on the mesh and the cell classes
// only, so k_flux_quotients evaluates them once per run into g.fq and the per-step kernel reads
// them (the same operands and operations, so the same bits); entries whose term is a plain zero
// hold 0.
__device__ __forceinline__ void flux_quotients(const Geo& g, int i, int j, double q[6]) {
  const Nb d = neighbours(i, j, g.Nx, g.Ny, g.bits & F_PERIODIC);
  const double* __restrict__ hx = g.hx;
  const double* __restrict__ hy = g.hy;
  const bool b_ws = cls_fluid(g.cls[d.i_1j_1]), b_s = cls_fluid(g.cls[d.ij_1]), b_w = cls_fluid(g.cls[d.i_1j]),
             b_p = cls_fluid(g.cls[d.ij]);
  const int jm = j - (0 < j ? 1 : 0);
  const double ry = g.ryy_m[j], rx = g.rxx_m[i];
  auto rsum = [](bool a, bool b, double r_both, double r_a, double r_b) { return a ? (b ? r_both : r_a) : r_b; };
  const bool all4 = b_ws && b_s && b_w && b_p;
  q[0] = div_cr(hy[j], hx[d.i_1], g.rhx[d.i_1]);
  if (all4)
    q[1] = div_cr(hx[i] + hx[d.i_1], hy[j] + hy[jm], ry);
  else if ((b_p && b_w) || (b_s && b_ws))
    q[1] = div_cr(hx[i] + hx[d.i_1], (double)(b_p * b_w) * hy[j] + (double)(b_s * b_ws) * hy[jm],
                  rsum(b_p && b_w, b_s && b_ws, ry, g.rhy[j], g.rhy[jm]));
  else
    q[1] = 0.0;
  if (all4)
    q[2] = div_cr(hy[j] + hy[jm], hx[i] + hx[d.i_1], rx);
  else if ((b_p && b_s) || (b_w && b_ws))
    q[2] = div_cr(hy[j] + hy[jm], (double)(b_p * b_s) * hx[i] + (double)(b_w * b_ws) * hx[d.i_1],
                  rsum(b_p && b_s, b_w && b_ws, rx, g.rhx[i], g.rhx[d.i_1]));
  else
    q[2] = 0.0;
  q[3] = div_cr(hx[i], hy[jm], g.rhy[jm]);
  // 1 / (0.5 s) = 2 (1 / s) exactly
  if (b_p && b_w)
    q[4] = div_cr(hy[j], 0.5 * (hx[i] + hx[d.i_1]), 2.0 * rx);
  else if (b_p || b_w)
    q[4] = div_cr(hy[j], 0.5 * ((double)b_p * hx[i] + (double)b_w * hx[d.i_1]),
                  2.0 * rsum(b_p, b_w, rx, g.rhx[i], g.rhx[d.i_1]));
  else
    q[4] = 0.0;
  if (b_p && b_s)
    q[5] = div_cr(hx[i], 0.5 * (hy[j] + hy[jm]), 2.0 * ry);
  else if (b_p || b_s)
    q[5] = div_cr(hx[i], 0.5 * ((double)b_p * hy[j] + (double)b_s * hy[jm]),
                  2.0 * rsum(b_p, b_s, ry, g.rhy[j], g.rhy[jm]));
  else
    q[5] = 0.0;
}
__global__ void k_flux_quotients(Geo g) {
  const Cell c = cell(g);
  if (!c.ok) return;
  double q[6];
  flux_quotients(g, c.i, c.j, q);
  for (int k = 0; k < 6; k++) const_cast<double*>(g.fq[k])[c.ij] = q[k];
  const_cast<double*>(g.hxy)[c.ij] = g.hx[c.i] * g.hy[c.j];
}

// ly, lx: the block's staged interpolations (null when the block is not 32x8)
__device__ __forceinline__ void flux_diff_cell(const Geo& g, const Cell& c, const double* ly, const double* lx) {
  const int i = c.i, j = c.j;
  const Nb d = neighbours(i, j, g.Nx, g.Ny, g.bits & F_PERIODIC);
  const double* __restrict__ hx = g.hx;
  const double* __restrict__ hy = g.hy;
  const double* __restrict__ sT = g.sqrt_T;
  const double* __restrict__ Tw_u = g.Tw_u;
  const double* __restrict__ Tw_v = g.Tw_v;
  const double cT = g.ctl->cT, cT1 = g.cT1;
  g.Fx[d.ij] = hy[j] * g.rho_u[d.ij] * g.u[d.ij];
  g.Fy[d.ij] = hx[i] * g.rho_v[d.ij] * g.v[d.ij];
  const bool b_ws = cls_fluid(g.cls[d.i_1j_1]), b_s = cls_fluid(g.cls[d.ij_1]), b_w = cls_fluid(g.cls[d.i_1j]),
             b_p = cls_fluid(g.cls[d.ij]);
  const int jm = j - (0 < j ? 1 : 0);
  const double ry = g.ryy_m[j], rx = g.rxx_m[i];
  auto LiY = [&](double f1, double f2) { return div_cr(f1 * hy[j] + f2 * hy[jm], hy[jm] + hy[j], ry); };
  auto LiX = [&](double f1, double f2) { return div_cr(f1 * hx[i] + f2 * hx[d.i_1], hx[d.i_1] + hx[i], rx); };
  const int x = threadIdx.x, y = threadIdx.y;
  const bool west = ly && d.i_1 == i - 1, south = lx && j > 0;
  auto ly_west = [&]() { return west ? ly[x + 33 * y] : LiY(sT[d.i_1j_1], sT[d.i_1j]); };
  auto ly_own = [&]() { return ly ? ly[x + 1 + 33 * y] : LiY(sT[d.ij_1], sT[d.ij]); };
  auto lx_south = [&]() { return south ? lx[x + 32 * y] : LiX(sT[d.i_1j_1], sT[d.ij_1]); };
  auto lx_own = [&]() { return lx ? lx[x + 32 * (y + 1)] : LiX(sT[d.i_1j], sT[d.ij]); };
  double Gy = g.Gamma_yf[d.ij], Gx = g.Gamma_xf[d.ij];
  if (b_ws && b_s && b_w && b_p) {
    Gy = 0.5 * (ly_west() + ly_own());
  } else if (b_ws || b_s || b_w || b_p) {
    Gy = 0.5 * ((double)(b_ws && b_w) * ly_west() +
                (double)(b_ws != b_w) * sqrt(Tw_v[d.i_1j]) +
                (double)(b_s && b_p) * ly_own() + (double)(b_s != b_p) * sqrt(Tw_v[d.ij]) +
                (double)((!(b_ws && b_w)) || (!(b_s && b_p))) * LiY(sqrt(Tw_u[d.ij_1]), sqrt(Tw_u[d.ij])));
  }
  g.Gamma_yf[d.ij] = Gy;
  g.D_ux[d.ij] = cT * sT[d.i_1j] * g.fq[0][d.ij];
  // where every mask is 1 the masked sums are the plain sums (1 * x = x exactly)
  if ((b_p && b_w) || (b_s && b_ws))
    g.D_uy[d.ij] = cT * Gy * g.fq[1][d.ij];
  else
    g.D_uy[d.ij] = 0;
  if (b_ws && b_s && b_w && b_p) {
    Gx = 0.5 * (lx_south() + lx_own());
  } else if (b_ws || b_s || b_w || b_p) {
    Gx = 0.5 * ((double)(b_ws && b_s) * lx_south() +
                (double)(b_ws != b_s) * sqrt(Tw_u[d.ij_1]) +
                (double)(b_w && b_p) * lx_own() + (double)(b_w != b_p) * sqrt(Tw_u[d.ij]) +
                (double)((!(b_ws && b_s)) || (!(b_w && b_p))) * LiX(sqrt(Tw_v[d.i_1j]), sqrt(Tw_v[d.ij])));
  }
  g.Gamma_xf[d.ij] = Gx;
  if ((b_p && b_s) || (b_w && b_ws))
    g.D_vx[d.ij] = cT * Gx * g.fq[2][d.ij];
  else
    g.D_vx[d.ij] = 0;
  g.D_vy[d.ij] = cT * sT[d.ij_1] * g.fq[3][d.ij];
  if (b_p && b_w)
    g.DTx[d.ij] = cT1 * g.fq[4][d.ij] * wall_term_off(Tw_u[d.ij], Hi(sT[d.i_1j], sT[d.ij], hx[d.i_1], hx[i]));
  else if (b_p || b_w)
    g.DTx[d.ij] = cT1 * g.fq[4][d.ij] *
                  ((double)((!b_p) || (!b_w)) * sqrt(Tw_u[d.ij]) +
                   (double)(b_p * b_w) * Hi(sT[d.i_1j], sT[d.ij], hx[d.i_1], hx[i]));
  else
    g.DTx[d.ij] = 0;
  if (b_p && b_s)
    g.DTy[d.ij] = cT1 * g.fq[5][d.ij] * wall_term_off(Tw_v[d.ij], Hi(sT[d.ij_1], sT[d.ij], hy[jm], hy[j]));
  else if (b_p || b_s)
    g.DTy[d.ij] = cT1 * g.fq[5][d.ij] *
                  ((double)((!b_p) || (!b_s)) * sqrt(Tw_v[d.ij]) +
                   (double)(b_p * b_s) * Hi(sT[d.ij_1], sT[d.ij], hy[jm], hy[j]));
  else
    g.DTy[d.ij] = 0;
}

// The zero-gradient temperature and pressure copies (phases `tail`) touch only ghost cells of p
// and T, which the fluxes and diffusion terms do not read, so the first CTA does them too.
__device__ __forceinline__ void flux_diff_body(const Geo& g, unsigned tail) {
  __shared__ double ly[kFluxLy], lx[kFluxLx];
  const bool staged = blockDim.x == 32 && blockDim.y == 8;
  if (staged) {
    const int tid = threadIdx.x + 32 * threadIdx.y, i0 = blockIdx.x * 32, j0 = blockIdx.y * 8;
    for (int q = tid; q < kFluxLy; q += 256) {  // faces of columns i0-1 .. i0+31
      const int py = q / 33, ci = i0 - 1 + (q - 33 * py), cj = j0 + py;
      ly[q] = (ci >= 0 && ci < g.Nx && cj < g.Ny) ? li_y_at(g, ci, cj) : 0.0;
    }
    for (int q = tid; q < kFluxLx; q += 256) {  // faces of rows j0-1 .. j0+7
      const int ci = i0 + (q & 31), cj = j0 - 1 + (q >> 5);
      lx[q] = (ci < g.Nx && cj >= 0 && cj < g.Ny) ? li_x_at(g, ci, cj) : 0.0;
    }
    __syncthreads();
  }
  Cell c = cell(g);
  if (c.ok) flux_diff_cell(g, c, staged ? ly : nullptr, staged ? lx : nullptr);
  if (tail && blockIdx.x == 0 && blockIdx.y == 0) {
    const int tid = threadIdx.x + threadIdx.y * blockDim.x, nt = blockDim.x * blockDim.y;
    const unsigned cur = g.ctl->cur;
    if (tail & PH_TEMP) phase_temp(g, g.T[cur], tid, nt);
    __syncthreads();
    if (tail & PH_PRES) phase_pres(g, g.p[cur], tid, nt);
  }
}
__global__ void k_flux_diff(Geo g, unsigned tail) {
  wait_for_predecessor();
  flux_diff_body(g, tail);
}
__global__ void kb_flux_diff(const Geo* gs, unsigned tail) {
  __shared__ Geo sg;
  if (!stage_geo(sg, gs)) return;
  flux_diff_body(sg, tail);
}

// ApplyBodiesConditionsToVariables on the device (SIMPLE_TS_MPI.cpp:6470-6584): a face takes the
// velocity of the body it belongs to, or of the body on its low side; body cells take p, T and rho = 0.
__global__ void k_apply_bodies(Geo g) {
  Cell c = cell(g);
  if (!c.ok) return;
  const unsigned cur = g.ctl->cur;
  const int i = c.i, j = c.j, n = c.ij;
  const uint32_t id = g.vol_id[n];
  const uint32_t idw = (i > 0) ? g.vol_id[n - 1] : 0u;
  const uint32_t ids = (j > 0) ? g.vol_id[n - g.Nx] : 0u;
  if (id >= 1) g.u[n] = g.bodies[id - 1].u;
  else if (idw >= 1) g.u[n] = g.bodies[idw - 1].u;
  if (id >= 1) g.v[n] = g.bodies[id - 1].v;
  else if (ids >= 1) g.v[n] = g.bodies[ids - 1].v;
  if (id >= 1) {
    g.p[cur][n] = g.bodies[id - 1].p;
    g.T[cur][n] = g.bodies[id - 1].T;
    g.rho[n] = cls_fluid(g.cls[n]) ? g.p[cur][n] / g.T[cur][n] : 0.0;
  }
}

// sqrt(T) and rho over all cells (SIMPLE_TS_MPI.cpp:2995-3001, :3020-3032)
__global__ void k_sqrt_rho(Geo g, int do_rho) {
  Cell c = cell(g);
  if (!c.ok) return;
  const unsigned cur = g.ctl->cur;
  const double T = g.T[cur][c.ij];
  g.sqrt_T[c.ij] = sqrt(T);
  if (do_rho) g.rho[c.ij] = cls_fluid(g.cls[c.ij]) ? g.p[cur][c.ij] / T : 0.0;
}

// ---------------------------------------------------------------------------
// Boundary work, in the reference's order.  The wall lists are O(perimeter) but carry FP64
// divisions, so they run one entry per thread over a grid (k_bnd_fused); the short column and
// row copies run in one CTA (the last of k_bnd_fused, k_boundary before the time loop) or in the
// first CTA of k_flux_diff.
// ---------------------------------------------------------------------------
// loop control after the velocity correction: SIMPLE_TS_MPI.cpp:4347-4361 (coefficients), :4406-4450
__device__ void do_control(const Geo& g, unsigned long long h_outer, int in_graph) {
  Ctl* ctl = g.ctl;
  const int TypeND = g.TypeND;
  if (TypeND == 1 || TypeND == 2) {
    ctl->cT = (1.0 / g.Re) * (ctl->u_given_xb_in_it * ctl->p_BC_xb / g.T_BC_xb);
    ctl->cPch = (TypeND == 1) ? 0.5 : ctl->u_given_xb_in_it * ctl->u_given_xb_in_it / (g.gamma1 * g.Ma * g.Ma);
  }
  const double ru = as_d(ctl->res_bits_u), rv = as_d(ctl->res_bits_v);
  ctl->res_u = ru;
  ctl->res_v = rv;
  const unsigned It = ++ctl->Iter;
  if (It == 1) {
    ctl->res_u0 = ru;
    ctl->res_v0 = rv;
  }
  const unsigned I = (It - 1) < 64 ? It - 1 : 63;
  const double rpI = ctl->res_p[I], rTI = ctl->res_T[I];
  const bool ci = (It < (unsigned)g.N_I) &&
                  (g.MaxError_Velocities < ru || g.MaxError_Velocities < rv || g.MaxError_p_c < rpI || g.MaxError_T < rTI);
  const double stop = g.MaxError_to_stop_program;
  const bool cs = ((double)ctl->it_counter < g.Nt) &&
                  ((!(It <= 1 && ctl->Iter_p_c <= 2)) || stop < ru || stop < rv || stop < ctl->res_p0[I] ||
                   stop < ctl->res_T0[I]);
  ctl->continue_iter = ci;
  ctl->continue_step = cs;
  if (in_graph) cudaGraphSetConditional((cudaGraphConditionalHandle)h_outer, ci ? 1 : 0);
}

// BoundaryConditions_Velocities_SlipBC_u (SIMPLE_TS_MPI.cpp:7098-7213), entry k; an entry performs
// only the writes that survive in the reference's sequential order (host-side analysis).
__device__ void do_slip_u(const Geo& g, int k) {
  const int Nx = g.Nx, Ny = g.Ny;
  const bool per = g.bits & F_PERIODIC;
  double* __restrict__ u = g.u;
  auto fl = [&](int q) { return cls_fluid(g.cls[q]); };
  const uint64_t bits = g.bits;
  const bool kl = bits & F_KN_LOCAL;

  const int node = g.slip_u[k];
  const uint8_t fin = g.slip_u_fin[k];
  const int j = node / Nx, i = node - j * Nx;
  const Nb d = neighbours(i, j, Nx, Ny, per);
  // the static operands of both sides (below / above) loaded together, before the choice, so
  // that the entry's loads do not wait on one another; u keeps its place in the reference's order
  const int vid = g.vol_id[d.ij], vid_s = g.vol_id[d.ij_1];
  const int jm = j - (0 < j ? 1 : 0), jp = j + (j < (Ny - 1) ? 1 : 0);
  const double hym = g.hy[jm], hyp = g.hy[jp];
  const double ru_s0 = g.rho_u[d.ij_1], ru_s1 = g.rho_u[d.i1j_1], ru_n0 = g.rho_u[d.ij1], ru_n1 = g.rho_u[d.i1j1];
  const bool f_s0 = fl(d.i_1j_1), f_s1 = fl(d.i1j_1), f_n0 = fl(d.i_1j1), f_n1 = fl(d.i1j1);
  const Body& Bd = g.bodies[vid - 1];
  const double FK = Bd.F_slip * g.Kn;
  if (vid_s == 0) {
    const double a_ij = kl ? FK / (ru_s0 * 0.5 * hym) : FK / (0.5 * hym);
    const double a_i1j = kl ? FK / (ru_s1 * 0.5 * hym) : FK / (0.5 * hym);
    if ((fin & 1) && f_s0) u[d.ij] = div_z(u[d.ij_1] * a_ij + Bd.u, 1.0 + a_ij);
    if ((fin & 2) && f_s1) u[d.i1j] = div_z(u[d.i1j_1] * a_i1j + Bd.u, 1.0 + a_i1j);
  } else {
    const double a_ij = kl ? FK / (ru_n0 * 0.5 * hyp) : FK / (0.5 * hyp);
    const double a_i1j = kl ? FK / (ru_n1 * 0.5 * hyp) : FK / (0.5 * hyp);
    if ((fin & 1) && f_n0) u[d.ij] = div_z(u[d.ij1] * a_ij + Bd.u, 1.0 + a_ij);
    if ((fin & 2) && f_n1) u[d.i1j] = div_z(u[d.i1j1] * a_i1j + Bd.u, 1.0 + a_i1j);
  }
}

// BoundaryConditions_Velocities_SlipBC_v (SIMPLE_TS_MPI.cpp:7216-7331), entry k
__device__ void do_slip_v(const Geo& g, int k) {
  const int Nx = g.Nx, Ny = g.Ny;
  const bool per = g.bits & F_PERIODIC;
  double* __restrict__ v = g.v;
  auto fl = [&](int q) { return cls_fluid(g.cls[q]); };
  const uint64_t bits = g.bits;
  const bool kl = bits & F_KN_LOCAL;

  const int node = g.slip_v[k];
  const uint8_t fin = g.slip_v_fin[k];
  const int j = node / Nx, i = node - j * Nx;
  const Nb d = neighbours(i, j, Nx, Ny, per);
  // as in do_slip_u: both sides' static operands (left / right) loaded together
  const int vid = g.vol_id[d.ij], vid_w = g.vol_id[d.i_1j];
  const double hxw = g.hx[d.i_1], hxe = g.hx[d.i1];
  const double rv_w0 = g.rho_v[d.i_1j], rv_w1 = g.rho_v[d.i_1j1], rv_e0 = g.rho_v[d.i1j], rv_e1 = g.rho_v[d.i1j1];
  const bool f_w0 = fl(d.i_1j_1), f_w1 = fl(d.i_1j1), f_e0 = fl(d.i1j_1), f_e1 = fl(d.i1j1);
  const Body& Bd = g.bodies[vid - 1];
  const double FK = Bd.F_slip * g.Kn;
  if (vid_w == 0) {
    const double a_ij = kl ? FK / (rv_w0 * 0.5 * hxw) : FK / (0.5 * hxw);
    const double a_ij1 = kl ? FK / (rv_w1 * 0.5 * hxw) : FK / (0.5 * hxw);
    if ((fin & 1) && f_w0) v[d.ij] = div_z(v[d.i_1j] * a_ij + Bd.v, 1.0 + a_ij);
    if ((fin & 2) && f_w1) v[d.ij1] = div_z(v[d.i_1j1] * a_ij1 + Bd.v, 1.0 + a_ij1);
  } else {
    const double a_ij = kl ? FK / (rv_e0 * 0.5 * hxe) : FK / (0.5 * hxe);
    const double a_ij1 = kl ? FK / (rv_e1 * 0.5 * hxe) : FK / (0.5 * hxe);
    if ((fin & 1) && f_e0) v[d.ij] = div_z(v[d.i1j] * a_ij + Bd.v, 1.0 + a_ij);
    if ((fin & 2) && f_e1) v[d.ij1] = div_z(v[d.i1j1] * a_ij1 + Bd.v, 1.0 + a_ij1);
  }
}

// BoundaryConditions_Temperature_TemperatureJumpBC (SIMPLE_TS_MPI.cpp:7744-8045), entry k
__device__ void do_tjump(const Geo& g, const double* __restrict__ T, int k) {
  const int Nx = g.Nx, Ny = g.Ny;
  const bool per = g.bits & F_PERIODIC;
  auto fl = [&](int q) { return cls_fluid(g.cls[q]); };
  const uint64_t bits = g.bits;
  const bool kl = bits & F_KN_LOCAL;

  const int node = g.tjump[k];
  const uint8_t fin = g.tjump_fin[k];
  const int j = node / Nx, i = node - j * Nx;
  const Nb d = neighbours(i, j, Nx, Ny, per);
  const int nb[4] = {d.i_1j, d.i1j, d.ij_1, d.ij1};
  const int dst[4] = {d.ij, d.i1j, d.ij, d.ij1};
  // every operand of the four sides loaded together (T and rho are not written here), so that the
  // sides do not wait on one another's loads
  bool fluid[4];
  int vid[4];
  for (int q = 0; q < 4; q++) {
    fluid[q] = fl(nb[q]);
    vid[q] = g.vol_id[nb[q]];
  }
  const double Tc = T[d.ij], rc = g.rho[d.ij], hxi = g.hx[i], hyj = g.hy[j];
  for (int q = 0; q < 4; q++) {
    if (fluid[q] || !(fin & (1 << q))) continue;
    const Body& Bd = g.bodies[vid[q] - 1];
    double* out = (q < 2) ? g.Tw_u : g.Tw_v;
    double val;
    if (Bd.jump) {
      const double FK = kl ? (Bd.F_jump * g.Kn) / rc : Bd.F_jump * g.Kn;
      const double a = FK / (0.5 * ((q < 2) ? hxi : hyj));
      val = (a * Tc + Bd.T) / (1.0 + a);
    } else if (Bd.dTdn0 != 0) {
      val = Tc;
    } else {
      val = Bd.T;
    }
    out[dst[q]] = val;
  }
}

// ..._TemperatureJumpBC_WriteToMassiveToWriteDataToFile (SIMPLE_TS_MPI.cpp:8048-8099), entry k
__device__ void do_tjump_write(const Geo& g, double* __restrict__ T, int k) {
  const int Nx = g.Nx, Ny = g.Ny;
  const bool per = g.bits & F_PERIODIC;
  auto fl = [&](int q) { return cls_fluid(g.cls[q]); };

  const int node = g.tjump[k];
  const uint8_t fin = g.tjump_wr_fin[k];
  const int j = node / Nx, i = node - j * Nx;
  const Nb d = neighbours(i, j, Nx, Ny, per);
  if ((fin & 1) && !fl(d.i_1j)) T[d.i_1j] = g.Tw_u[d.ij];
  if ((fin & 2) && !fl(d.i1j)) T[d.i1j] = g.Tw_u[d.i1j];
  if ((fin & 4) && !fl(d.ij_1)) T[d.ij_1] = g.Tw_v[d.ij];
  if ((fin & 8) && !fl(d.ij1)) T[d.ij1] = g.Tw_v[d.ij1];
}

// Single-CTA boundary work; `phases` selects the parts (PH_* in sts_kernels.h).
__device__ __forceinline__ void boundary_body(const Geo& g, unsigned phases, unsigned long long h_outer, int in_graph) {
  Ctl* ctl = g.ctl;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int Nx = g.Nx, Ny = g.Ny;
  const bool per = g.bits & F_PERIODIC;
  double* __restrict__ u = g.u;
  double* __restrict__ v = g.v;
  const unsigned cur = ctl->cur;
  double* __restrict__ p = g.p[cur];
  double* __restrict__ T = g.T[cur];
  auto fl = [&](int k) { return cls_fluid(g.cls[k]); };
  const uint64_t bits = g.bits;

  if ((phases & PH_CONTROL) && tid == 0) do_control(g, h_outer, in_graph);
  __syncthreads();

  if (phases & PH_SLIP_U)
    for (int k = tid; k < g.n_slip_u; k += nt) do_slip_u(g, k);
  __syncthreads();

  if (phases & PH_SLIP_V)
    for (int k = tid; k < g.n_slip_v; k += nt) do_slip_v(g, k);
  __syncthreads();

  // BoundaryConditions_Velocities (SIMPLE_TS_MPI.cpp:6790-7096), each loop a phase
  if ((phases & PH_VEL) && !per) {
    if (bits & F_DVDX0_XB) {
      for (int k = tid; k < Ny * g.Nx_v0; k += nt) {
        const int j = k / g.Nx_v0, i = k - j * g.Nx_v0, n = g.Nx_v0 + j * Nx;
        if (fl(n)) v[i + j * Nx] = v[n];
      }
      __syncthreads();
    }
    if (bits & F_DVDX0_XE) {
      const int w = Nx - g.Nx_v1;
      for (int k = tid; k < Ny * w; k += nt) {
        const int j = k / w, i = g.Nx_v1 + (k - j * w), n = g.Nx_v1 - 1 + j * Nx;
        if (fl(n)) v[i + j * Nx] = v[n];
      }
      __syncthreads();
    }
    if (bits & F_DVDY0_YB) {
      for (int k = tid; k < Nx * g.Ny_v0; k += nt) {
        const int jj = k / Nx, i = k - jj * Nx, n = i + g.Ny_v0 * Nx;
        if (fl(n)) v[i + jj * Nx] = v[n];
      }
      __syncthreads();
    }
    if (bits & F_DVDY0_YE) {
      const int w = Ny - g.Ny_v1;
      for (int k = tid; k < Nx * w; k += nt) {
        const int jj = k / Nx, i = k - jj * Nx, n = i + (g.Ny_v1 - 1) * Nx;
        if (fl(n)) v[i + (g.Ny_v1 + jj) * Nx] = v[n];
      }
      __syncthreads();
    }
    if (bits & F_DUDX0_XB) {
      for (int k = tid; k < Ny * g.Nx_u0; k += nt) {
        const int j = k / g.Nx_u0, i = k - j * g.Nx_u0, n = g.Nx_u0 + j * Nx;
        if (fl(n)) u[i + j * Nx] = u[n];
      }
      __syncthreads();
    }
    if (bits & F_DURHODX0_XB) {
      for (int j = tid; j < Ny; j += nt) {
        const int n = g.Nx_u0 - 1 + j * Nx;
        if (fl(n)) u[n] = div_z(g.rho_u[n + 1] * u[n + 1], g.rho_u[n]);
      }
      __syncthreads();
    }
    if (bits & F_DRHODT0_XB) {
      const int i = g.Nx_u0 - 1;
      for (int j = tid; j < Ny; j += nt) {
        const int n = i + j * Nx;
        // the reference reads one row past the array for a fluid cell in the top row; skipped here
        if (fl(n) && n + Nx < g.Na)
          u[n] = ((g.rho[n] - g.rho_pr[n]) * g.hx[i] * g.hy[j] / g.ht +
                  (g.rho_v[n + Nx] * v[n + Nx] - g.rho_v[n] * v[n]) * g.hx[i] + g.rho_u[n + 1] * u[n + 1] * g.hy[j]) /
                 (g.rho_u[n] * g.hy[j]);
      }
      __syncthreads();
    }
    if (bits & F_DUDX0_XE) {
      const int w = Nx - g.Nx_u1;
      for (int k = tid; k < Ny * w; k += nt) {
        const int j = k / w, i = g.Nx_u1 + (k - j * w), n = g.Nx_u1 - 1 + j * Nx;
        if (fl(n)) u[i + j * Nx] = u[n];
      }
      __syncthreads();
    }
    if (bits & F_DURHODX0_XE) {
      for (int j = tid; j < Ny; j += nt) {
        const int n = g.Nx_u1 - 1 + j * Nx;
        if (fl(n)) u[n + 1] = div_z(g.rho_u[n] * u[n], g.rho_u[n + 1]);
      }
      __syncthreads();
    }
    if (bits & F_DRHODT0_XE) {
      const int i = g.Nx_u1 - 1;
      for (int j = tid; j < Ny; j += nt) {
        const int n = i + j * Nx;
        if (fl(n) && n + Nx < g.Na)
          u[n + 1] = (-(g.rho[n] - g.rho_pr[n]) * g.hx[i] * g.hy[j] / g.ht -
                      (g.rho_v[n + Nx] * v[n + Nx] - g.rho_v[n] * v[n]) * g.hx[i] + g.rho_u[n] * u[n] * g.hy[j]) /
                     (g.rho_u[n + 1] * g.hy[j]);
      }
      __syncthreads();
    }
    if (bits & F_U_MINMOUT_XE) {  // the reference keeps the last row's rho_u for Min and Mout
      const double Min = g.rho_u[g.Nx_u0 + (Ny - 1) * Nx], Mout = g.rho_u[g.Nx_u1 + (Ny - 1) * Nx];
      __syncthreads();
      for (int j = tid; j < Ny; j += nt) {
        const int n = g.Nx_u1 - 1 + j * Nx;
        u[n + 1] = u[n] * Min / Mout;
      }
      __syncthreads();
    }
    if (bits & F_DUDY0_YB) {
      for (int k = tid; k < Nx * g.Ny_u0; k += nt) {
        const int jj = k / Nx, i = k - jj * Nx, n = i + g.Ny_u0 * Nx;
        if (fl(n)) u[i + jj * Nx] = u[n];
      }
      __syncthreads();
    }
    if (bits & F_DUDY0_YE) {
      const int w = Ny - g.Ny_u1;
      for (int k = tid; k < Nx * w; k += nt) {
        const int jj = k / Nx, i = k - jj * Nx, n = i + (g.Ny_u1 - 1) * Nx;
        if (fl(n)) u[i + (g.Ny_u1 + jj) * Nx] = u[n];
      }
      __syncthreads();
    }
  }
  __syncthreads();

  // BoundaryConditions_Pressure_begin_iteration_for_it (SIMPLE_TS_MPI.cpp:7430-7647)
  if ((phases & PH_PBEGIN) && !per) {
    __shared__ int ratio_side;  // 0: nothing, 1: inlet columns, 2: outlet columns
    // the inflow column is staged in shared memory by all threads; thread 0 then folds it
    // in the reference's order (the mean is an ordered sum)
    // (the column maximum and mean feed correction methods 1 and 2 and the pressure-control log)
    __shared__ double col_u[kMaxColumn], col_h[kMaxColumn];
    const bool need_col = (g.p_corr_method == 1 || g.p_corr_method == 2) || (bits & F_PRESSURE_BC);
    const bool staged = need_col && Ny <= kMaxColumn;
    if (staged) {
      for (int j = tid; j < Ny; j += nt) {
        const int n = g.Nx_u0 + j * Nx;
        col_u[j] = u[n];
        col_h[j] = fl(n) ? g.hy[j] : -1.0;  // negative height marks a body cell
      }
    }
    __syncthreads();
    if (tid == 0) {
      ratio_side = 0;
      if (need_col) {
        const int i = g.Nx_u0;
        double umax = u[0], mean = 0, hin = 0;
        for (int j = 0; j < Ny; j++) {
          const bool f = staged ? col_h[j] >= 0 : fl(i + j * Nx);
          if (!f) continue;
          const double uj = staged ? col_u[j] : u[i + j * Nx];
          const double hj = staged ? col_h[j] : g.hy[j];
          umax = (umax > uj) ? umax : uj;
          mean += uj * hj;
          hin += hj;
        }
        ctl->u_in_max = umax;
        ctl->u_in_mean = mean / hin;
      }
      const double umax = ctl->u_in_max, mean = ctl->u_in_mean;
      if (bits & F_GIVEN_REKN) ctl->u_given_xb = g.Re * g.Kn * sqrt(15.0 * 3.14159265358979323846 / 128.0);
      const double ug = ctl->u_given_xb;
      if (g.p_corr_method == 0) {
        ctl->u_given_xb_in_it = ug;
        if (bits & F_GIVEN_U_XB) {
          const int ii = g.Nx_o0;
          const int jj = (int)(((double)g.Ny_o1 - 1.0) - (double)g.Ny_o0);
          ctl->p_BC_xb = p[ii + jj * Nx];
        }
      } else if (g.p_corr_method == 1) {
        ctl->u_given_xb_in_it = umax;
      } else if (g.p_corr_method == 2) {
        ctl->u_given_xb_in_it = mean;
      }
      if ((bits & F_PRESSURE_BC) && (bits & F_RATIO_CORRECT)) {
        double pc = ctl->p_correction;
        if (bits & F_P_CORR_AUTO) {
          const double r = sqrt(ctl->res_u * ctl->res_u + ctl->res_v * ctl->res_v);
          double t;
          if (ctl->Iter_pr1 <= ctl->Iter_pr2 && ctl->Iter_pr1 < (unsigned)(g.N_I - 1)) t = pc * (1.0 + r);
          else t = pc * (1.0 - r);
          if (t < g.p_correction_min) t = g.p_correction_min;
          else if (g.p_correction_max < t) t = g.p_correction_max;
          pc = t;
          ctl->p_correction = pc;
        }
        const double ui = ctl->u_given_xb_in_it;
        const bool cxb = bits & F_CORRECT_P_XB;
        if (ui < (ug * (1.0 - g.u_given_xb_error))) {
          if (cxb) ctl->p_BC_xb = ctl->p_BC_xb * (1.0 + pc * (ug - ui) * (ug - ui));
          else {
            const double t = ctl->p_BC_xe * (1.0 - pc * (ug - ui) * (ug - ui));
            ctl->p_BC_xe = (t < 0.0) ? 0.0 : t;
          }
        } else if ((ug * (1.0 + g.u_given_xb_error)) < ui) {
          if (cxb) {
            const double t = ctl->p_BC_xb * (1.0 - pc * (ug - ui) * (ug - ui));
            ctl->p_BC_xb = (t > ctl->p_BC_xe) ? t : ctl->p_BC_xe;
          } else {
            const double t = ctl->p_BC_xb * (1.0 + pc * (ug - ui) * (ug - ui));
            ctl->p_BC_xe = (t > ctl->p_BC_xb) ? ctl->p_BC_xb : t;
          }
        }
        ratio_side = cxb ? 1 : 2;
      }
    }
    __syncthreads();
    if (ratio_side == 1) {
      const double pb = ctl->p_BC_xb, rb = ctl->p_BC_xb / g.T_BC_xb;
      for (int k = tid; k < Ny * g.Nx_o0; k += nt) {
        const int j = k / g.Nx_o0, i = k - j * g.Nx_o0, n = i + j * Nx;
        if (fl(n)) { p[n] = pb; g.rho[n] = rb; }
      }
    } else if (ratio_side == 2) {
      const double pe = ctl->p_BC_xe, re = ctl->p_BC_xe / g.T_BC_xe;
      const int w = Nx - g.Nx_o1;
      for (int k = tid; k < Ny * w; k += nt) {
        const int j = k / w, i = g.Nx_o1 + (k - j * w), n = i + j * Nx;
        if (fl(n)) { p[n] = pe; g.rho[n] = re; }
      }
    }
  }
  __syncthreads();

  // inlet/outlet pressure and temperature before the time loop (SIMPLE_TS_MPI.cpp:2942-2979)
  if ((phases & PH_PINIT) && (bits & F_PRESSURE_BC)) {
    for (int k = tid; k < Ny * Nx; k += nt) {
      const int j = k / Nx, i = k - j * Nx;
      if (!fl(k)) continue;
      if (i < g.Nx_o0) { p[k] = ctl->p_BC_xb; T[k] = g.T_BC_xb; }
      else if (i >= g.Nx_o1) { p[k] = ctl->p_BC_xe; T[k] = g.T_BC_xe; }
    }
  }
  __syncthreads();

  if (phases & (PH_TJUMP | PH_TJUMP_WRITE))
    for (int k = tid; k < g.n_tjump; k += nt) do_tjump(g, T, k);
  __syncthreads();

  if (phases & PH_TJUMP_WRITE)
    for (int k = tid; k < g.n_tjump; k += nt) do_tjump_write(g, T, k);
  __syncthreads();

  if (phases & PH_TEMP) phase_temp(g, T, tid, nt);
  __syncthreads();

  if (phases & PH_PRES) phase_pres(g, p, tid, nt);
}
__global__ void __launch_bounds__(1024) k_boundary(Geo g, unsigned phases, unsigned long long h_outer, int in_graph) { boundary_body(g, phases, h_outer, in_graph); }

// The boundary work of one outer iteration in one launch.  Over the whole grid, one entry per
// thread: the loop control (first thread), the slip-wall entries of u and of v (independent:
// they write u and v respectively, each entry only the writes that survive in the reference's
// sequential order) and, when they need nothing of the velocity and pressure phases
// (jump_beside), the temperature-jump entries.  The last CTA to finish then runs the column and
// row phases (PH_VEL | PH_PBEGIN), which read the slip walls' u and v and the control's
// residuals, and after them the jump entries when those read the inlet density that PH_PBEGIN
// writes: the reference's order (control, slip u, slip v, velocities, pressure begin) with the
// jump values wherever they see the same inputs.
__device__ __forceinline__ bool last_cta(unsigned* counter) {
  __shared__ bool last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();  // this CTA's writes before its ticket
    const unsigned t = atomicAdd(counter, 1u);
    last = (t == gridDim.x * gridDim.y - 1);
    if (last) {
      *counter = 0;
      __threadfence();  // every other CTA's writes before the reads that follow
    }
  }
  __syncthreads();
  return last;
}

// tail: the zero-gradient temperature and pressure copies (PH_TEMP, PH_PRES) after the jump walls,
// in the last CTA, where the flux kernel does not do them.
__device__ __forceinline__ void bnd_fused_body(const Geo& g, unsigned long long h_outer, int in_graph, int jump_beside,
                                               unsigned tail) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
  if (t == 0) do_control(g, h_outer, in_graph);
  const int nu = g.n_slip_u, nuv = nu + g.n_slip_v, n = nuv + (jump_beside ? g.n_tjump : 0);
  const double* T = g.T[g.ctl->cur];
  for (int k = t; k < n; k += nt) {
    if (k < nu) do_slip_u(g, k);
    else if (k < nuv) do_slip_v(g, k - nu);
    else do_tjump(g, T, k - nuv);
  }
  if (!last_cta(&g.ctl->bnd_count)) return;
  boundary_body(g, PH_VEL | PH_PBEGIN, 0ull, 0);
  if (!jump_beside) {
    __syncthreads();
    for (int k = threadIdx.x; k < g.n_tjump; k += blockDim.x) do_tjump(g, T, k);
  }
  if (tail) {
    const unsigned cur = g.ctl->cur;
    __syncthreads();
    if (tail & PH_TEMP) phase_temp(g, g.T[cur], threadIdx.x, blockDim.x);
    __syncthreads();
    if (tail & PH_PRES) phase_pres(g, g.p[cur], threadIdx.x, blockDim.x);
  }
}
__global__ void k_bnd_fused(Geo g, unsigned long long h_outer, int in_graph, int jump_beside, unsigned tail) {
  wait_for_predecessor();
  bnd_fused_body(g, h_outer, in_graph, jump_beside, tail);
}
__global__ void kb_bnd_fused(const Geo* gs, unsigned long long h_outer, int in_graph, int jump_beside) {
  __shared__ Geo sg;
  if (!stage_geo(sg, gs)) return;
  bnd_fused_body(sg, h_outer, in_graph, jump_beside, 0u);
}

// End of a time step: time-dependent inflow (SIMPLE_TS_MPI.cpp:8102-8144), per-step
// record and the multi-step loop condition.
__device__ __forceinline__ void step_end_body(const Geo& g, unsigned long long h_step, int in_graph) {
  Ctl* ctl = g.ctl;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int Nx = g.Nx, Ny = g.Ny;
  if ((g.bits & F_U_BY_TIME) && !(g.bits & F_PERIODIC)) {
    const double it = ctl->it;
    double ug;
    if (it <= g.t_BC_b) ug = g.u_BC_xb_t_BC_b;
    else if (g.t_BC_b < it && it <= g.t_BC_e)
      ug = ((g.u_BC_xb_t_BC_e - g.u_BC_xb_t_BC_b) / (g.t_BC_e - g.t_BC_b)) * (it - g.t_BC_b) + g.u_BC_xb_t_BC_b;
    else ug = g.u_BC_xb_t_BC_e;
    for (int k = tid; k < Ny * g.Nx_u0; k += nt) {
      const int j = k / g.Nx_u0, i = k - j * g.Nx_u0, n = i + j * Nx;
      if (cls_fluid(g.cls[n])) g.u[n] = ug;
    }
    __syncthreads();
    if (tid == 0) {
      ctl->u_gas_nd = ug;
      ctl->u_given_xb = ug;
    }
  }
  if (tid == 0) {
    if (g.warm_start == 1 || g.warm_start == 2 || g.warm_start == 4) ctl->warm_ready++;
    ctl->hist_sweeps[ctl->hist_n % 4096u] = ctl->step_sweeps;
    ctl->hist_n++;
    if (ctl->steps_left > 0) ctl->steps_left--;
    if (in_graph)
      cudaGraphSetConditional((cudaGraphConditionalHandle)h_step, (ctl->steps_left > 0 && ctl->continue_step) ? 1 : 0);
  }
}
__global__ void k_step_end(Geo g, unsigned long long h_step, int in_graph) { step_end_body(g, h_step, in_graph); }
__global__ void kb_step_end(const Geo* gs, unsigned long long h_step, int in_graph) {
  __shared__ Geo sg;
  if (!stage_geo(sg, gs)) return;
  step_end_body(sg, h_step, in_graph);
}

}  // namespace sts

namespace sts {

// Self-check of div_cr against the IEEE quotient on n pseudo-random operand pairs (a splitmix64
// stream from `seed`): random signs and significands, dividend exponents over 2^-920..2^920 (so
// some pairs take the IEEE fallback), divisor exponents over 2^-110..2^110, one divisor in eight
// with an all-ones significand, every fourth dividend formed as a rounded product q*b so that
// the quotient is exact or within an ulp of a representable number, and one dividend in sixteen
// a zero of either sign.  Each pair also checks div_z (the IEEE division with zero dividends
// answered directly) against the IEEE quotient, one divisor in eight then replaced by a zero
// of either sign, an infinity or NaN.  Counts the results that differ in any bit (the sign of
// a zero included).
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long& s) {
  unsigned long long z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ double make_double(unsigned long long bits, int exp_lo, int exp_hi, bool all_ones) {
  const unsigned long long mant = all_ones ? 0xFFFFFFFFFFFFFull : (bits & 0xFFFFFFFFFFFFFull);
  const int span = exp_hi - exp_lo + 1;
  const int e = exp_lo + (int)((bits >> 52) % (unsigned long long)span);
  const unsigned long long sign = (bits >> 63) << 63;
  return __longlong_as_double((long long)(sign | ((unsigned long long)(e + 1023) << 52) | mant));
}

// Global conservation sums of the current state (no counterpart in the reference; its
// SolveContinuityEquation, SIMPLE_TS_MPI.cpp:10621-10714, gives the local continuity residual).
// Per fluid cell (i, j), area A = hx_i hy_j, cell-centre velocities u_c = (u_ij + u_i+1,j) / 2,
// v_c = (v_ij + v_i,j+1) / 2 (the neighbour index clamped at the last column or row):
//   mass rho A, momentum rho A u_c and rho A v_c, internal energy rho A T / (gamma - 1),
//   kinetic energy rho A (u_c^2 + v_c^2)
// (energies per unit depth in units of rho0 R T0 L^2: velocities are in units of sqrt(2 R T0)).
// FP64 in a fixed order: each thread sums kConsChunk cells of a row in x order, then
// k_cons_final sums each row's chunks in order and the rows in y order.
__global__ void k_cons_partial(Geo g, unsigned cur, double* part, int nch) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (k >= nch || j >= g.Ny) return;
  const int Nx = g.Nx, Ny = g.Ny;
  const double* T = g.T[cur];
  double s[kConsQ] = {0.0, 0.0, 0.0, 0.0, 0.0};
  const int i1 = min(Nx, (k + 1) * kConsChunk);
  for (int i = k * kConsChunk; i < i1; i++) {
    const int n = i + j * Nx;
    if (!cls_fluid(g.cls[n])) continue;
    const int ne = (i + 1 < Nx) ? n + 1 : n, nn = (j + 1 < Ny) ? n + Nx : n;
    const double A = g.hx[i] * g.hy[j];
    const double uc = 0.5 * (g.u[n] + g.u[ne]), vc = 0.5 * (g.v[n] + g.v[nn]);
    const double m = g.rho[n] * A;
    s[0] = s[0] + m;
    s[1] = s[1] + m * uc;
    s[2] = s[2] + m * vc;
    s[3] = s[3] + (m * T[n]) / (g.gamma1 - 1.0);
    s[4] = s[4] + m * (uc * uc + vc * vc);
  }
  for (int q = 0; q < kConsQ; q++) part[((size_t)j * nch + k) * kConsQ + q] = s[q];
}

__global__ void k_cons_final(int Ny, int nch, const double* part, double* rows, double* out) {
  for (int j = threadIdx.x; j < Ny; j += blockDim.x)
    for (int q = 0; q < kConsQ; q++) {
      double s = 0.0;
      for (int k = 0; k < nch; k++) s = s + part[((size_t)j * nch + k) * kConsQ + q];
      rows[(size_t)j * kConsQ + q] = s;
    }
  __syncthreads();
  if (threadIdx.x < kConsQ) {
    double s = 0.0;
    for (int j = 0; j < Ny; j++) s = s + rows[(size_t)j * kConsQ + threadIdx.x];
    out[threadIdx.x] = s;
  }
}

// Self-check of the grid barrier's bounded wait: CTA `skip` (none when skip < 0) returns without
// arriving; every other CTA meets `rounds` barriers, each wait limited to spin_limit polls, and
// leaves at the first one that gives up (ST_BARRIER_TIMEOUT in lc->status).  Every CTA ends.
__global__ void k_barrier_probe(LoopCtl* lc, int skip, unsigned spin_limit, int rounds) {
  if ((int)blockIdx.x == skip) return;
  for (int r = 0; r < rounds; r++)
    if (!grid_barrier(lc, spin_limit)) return;
}

__global__ void k_check_division(unsigned long long n, unsigned long long seed, unsigned long long* bad) {
  unsigned long long local = 0;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < n; k += stride) {
    unsigned long long st = seed ^ (k * 0xD1B54A32D192ED03ull);
    const unsigned long long r1 = splitmix64(st), r2 = splitmix64(st), r3 = splitmix64(st);
    const double b = make_double(r2, -110, 110, (r3 & 7) == 0);
    double a = make_double(r1, -920, 920, false);
    if (((r3 >> 3) & 3) == 0) a = __dmul_rn(make_double(r1, -700, 700, false), b);
    if (((r3 >> 5) & 15) == 0) a = ((r3 >> 9) & 1) ? -0.0 : 0.0;  // signed zero dividends
    const double y = __ddiv_rn(1.0, b);
    const double q1 = div_cr(a, b, y), q2 = __ddiv_rn(a, b);
    if (__double_as_longlong(q1) != __double_as_longlong(q2)) local++;
    // div_z, also with zero, infinite and NaN divisors
    double bz = b;
    const unsigned sp = (unsigned)(r3 >> 12) & 31u;
    if (sp == 1) bz = ((r3 >> 17) & 1) ? -0.0 : 0.0;
    if (sp == 2) bz = ((r3 >> 17) & 1) ? -CUDART_INF : CUDART_INF;
    if (sp == 3) bz = CUDART_NAN;
    if (__double_as_longlong(div_z(a, bz)) != __double_as_longlong(__ddiv_rn(a, bz))) local++;
  }
  for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
  if ((threadIdx.x & 31) == 0 && local) atomicAdd(bad, local);
}

// The state exchange with host buffers the device can address (pinned or registered memory):
// one grid-stride pass moves all four fields, so the four transfers share the host link at
// once instead of queueing on the copy engines one after another.
__device__ __forceinline__ void move4_body(const double* __restrict__ a0, const double* __restrict__ a1,
                                           const double* __restrict__ a2, const double* __restrict__ a3, double* b0,
                                           double* b1, double* b2, double* b3, int n) {
  // every pointer 16-byte aligned: pairs of doubles, two pairs of each array in flight per thread
  // (the host link needs many bytes in flight); otherwise one double at a time
  const bool vec = ((reinterpret_cast<uintptr_t>(a0) | reinterpret_cast<uintptr_t>(a1) |
                     reinterpret_cast<uintptr_t>(a2) | reinterpret_cast<uintptr_t>(a3) |
                     reinterpret_cast<uintptr_t>(b0) | reinterpret_cast<uintptr_t>(b1) |
                     reinterpret_cast<uintptr_t>(b2) | reinterpret_cast<uintptr_t>(b3)) & 15u) == 0;
  const int t = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
  int done = 0;
  if (vec) {
    const int n2 = n / 2;
    const double2 *c0 = reinterpret_cast<const double2*>(a0), *c1 = reinterpret_cast<const double2*>(a1),
                  *c2 = reinterpret_cast<const double2*>(a2), *c3 = reinterpret_cast<const double2*>(a3);
    double2 *d0 = reinterpret_cast<double2*>(b0), *d1 = reinterpret_cast<double2*>(b1),
            *d2 = reinterpret_cast<double2*>(b2), *d3 = reinterpret_cast<double2*>(b3);
    for (int k = t; k < n2; k += 2 * nt) {
      const int k2 = k + nt;
      const bool two = k2 < n2;
      const double2 x0 = c0[k], x1 = c1[k], x2 = c2[k], x3 = c3[k];
      double2 y0 = x0, y1 = x1, y2 = x2, y3 = x3;
      if (two) {
        y0 = c0[k2];
        y1 = c1[k2];
        y2 = c2[k2];
        y3 = c3[k2];
      }
      d0[k] = x0;
      d1[k] = x1;
      d2[k] = x2;
      d3[k] = x3;
      if (two) {
        d0[k2] = y0;
        d1[k2] = y1;
        d2[k2] = y2;
        d3[k2] = y3;
      }
    }
    done = 2 * n2;
  }
  for (int k = done + t; k < n; k += nt) {
    b0[k] = a0[k];
    b1[k] = a1[k];
    b2[k] = a2[k];
    b3[k] = a3[k];
  }
}
__global__ void k_move4(const double* __restrict__ a0, const double* __restrict__ a1, const double* __restrict__ a2,
                        const double* __restrict__ a3, double* b0, double* b1, double* b2, double* b3, int n) {
  move4_body(a0, a1, a2, a3, b0, b1, b2, b3, n);
}
// The state u, v, p, T out to host buffers at the end of steps queued before it: the buffer with
// the latest p-T iterate is the one the device recorded (the host has not read it yet).
__global__ void k_move4_state_out(Geo g, double* b0, double* b1, double* b2, double* b3) {
  const unsigned cur = *(volatile const unsigned*)&g.ctl->cur;
  move4_body(g.u, g.v, g.p[cur], g.T[cur], b0, b1, b2, b3, g.Na);
}

// FP64 throughput of the device: every thread advances 8 independent chains `iters` times with
// one operation each (op 0: add, 1: multiply, 2: fused multiply-add), so the FP64 unit, not
// latency, sets the time.  The chains stay near 1 (factors and addends are tiny perturbations);
// each thread stores its sum so that nothing is optimised away.
__global__ void k_fp64_rate(int op, int iters, double c_mul, double c_add, double* out) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; k++) x[k] = 1.0 + (double)(threadIdx.x * 8 + k) * 1e-9;
  if (op == 0) {
    for (int it = 0; it < iters; it++)
#pragma unroll
      for (int k = 0; k < 8; k++) x[k] = __dadd_rn(x[k], c_add);
  } else if (op == 1) {
    for (int it = 0; it < iters; it++)
#pragma unroll
      for (int k = 0; k < 8; k++) x[k] = __dmul_rn(x[k], c_mul);
  } else {
    for (int it = 0; it < iters; it++)
#pragma unroll
      for (int k = 0; k < 8; k++) x[k] = __fma_rn(x[k], c_mul, c_add);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace sts

namespace sts {

// ---------------------------------------------------------------------------
// Diagnostics of the time loop.
// Drag-coefficient sums of WriteDragCoefficient (SIMPLE_TS_MPI.cpp:8147-8275): thread k adds up
// list k -- the cells of one flagged body that have a fluid neighbour, in the reference's loop
// order (i outer, j inner over the p/T solve range) -- sequentially, so the sums are the
// reference's bit for bit; out[12 k ..] = friction, pressure and area sums of the bottom,
// front, top and behind faces.  Thread nlist adds the inflow and outflow mass fluxes of the
// short-format summary (:8471-8491) into out[12 nlist], out[12 nlist + 1].
// ---------------------------------------------------------------------------
__global__ void k_drag(Geo g, const int* cells, const int* first, int nlist, double* out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int Nx = g.Nx, Ny = g.Ny;
  const double* u = g.u;
  const double* v = g.v;
  const double* p = g.p[g.ctl->cur];
  const double* hx = g.hx;
  const double* hy = g.hy;
  auto fl = [&](int q) { return cls_fluid(g.cls[q]); };
  if (k < nlist) {
    double fb = 0, pb = 0, sb = 0, ff = 0, pf = 0, sf = 0, ft = 0, pt = 0, st = 0, fh = 0, ph = 0, sh = 0;
    for (int q = first[k]; q < first[k + 1]; q++) {
      const int node = cells[q], j = node / Nx, i = node - j * Nx;
      const Nb d = neighbours(i, j, Nx, Ny, false);  // ij_function_i_and_j_to_the_boundaries
      if (fl(d.ij_1)) {
        const double h = hy[j - (j < (Ny - 1) ? 1 : 0)];
        fb += hx[i] * sqrt(g.Tw_v[d.ij]) * ((u[d.ij_1] - u[d.ij]) / h + (u[d.i1j_1] - u[d.i1j]) / h);
        pb += p[d.ij_1] * hx[i];
        sb += hx[i];
      }
      if (fl(d.i_1j)) {
        ff += hy[j] * sqrt(g.Tw_u[d.ij]) * ((v[d.i_1j] - v[d.ij]) / hx[d.i_1] + (v[d.i_1j1] - v[d.ij1]) / hx[d.i_1]);
        pf += p[d.i_1j] * hy[j];
        sf += hy[j];
      }
      if (fl(d.ij1)) {
        const double h = hy[j + (0 < j ? 1 : 0)];
        ft += hx[i] * sqrt(g.Tw_v[d.ij1]) * ((u[d.ij1] - u[d.ij]) / h + (u[d.i1j1] - u[d.i1j]) / h);
        pt += p[d.ij1] * hx[i];
        st += hx[i];
      }
      if (fl(d.i1j)) {
        fh += hy[j] * sqrt(g.Tw_u[d.i1j]) * ((v[d.i1j] - v[d.ij]) / hx[d.i1] + (v[d.i1j1] - v[d.ij1]) / hx[d.i1]);
        ph += p[d.i1j] * hy[j];
        sh += hy[j];
      }
    }
    double* o = out + 12 * k;
    o[0] = fb; o[1] = pb; o[2] = sb; o[3] = ff; o[4] = pf; o[5] = sf;
    o[6] = ft; o[7] = pt; o[8] = st; o[9] = fh; o[10] = ph; o[11] = sh;
  } else if (k == nlist) {
    double qb = 0, qe = 0;
    for (int j = 0; j < Ny; j++) {
      const int n = 0 + j * Nx;
      if (fl(n)) qb += g.rho[n] * u[n] * hy[j];
    }
    for (int j = 0; j < Ny; j++) {
      const int n = g.Nx_u1 + j * Nx;
      if (fl(n)) qe += g.rho[n] * u[n] * hy[j];
    }
    out[12 * nlist] = qb;
    out[12 * nlist + 1] = qe;
  }
}

// SolveFluxes (SIMPLE_TS_MPI.cpp:10440-10454) alone, as SolveContinuityEquation calls it.
__global__ void k_fluxes(Geo g) {
  Cell c = cell(g);
  if (!c.ok) return;
  g.Fx[c.ij] = g.hy[c.j] * g.rho_u[c.ij] * g.u[c.ij];
  g.Fy[c.ij] = g.hx[c.i] * g.rho_v[c.ij] * g.v[c.ij];
}

// The steady and unsteady continuity residuals of SolveContinuityEquation
// (SIMPLE_TS_MPI.cpp:10624-10641); cells of the last row and column stay zero.
__global__ void k_continuity(Geo g, double* st, double* ce) {
  Cell c = cell(g);
  if (!c.ok) return;
  if (c.i >= g.Nx - 1 || c.j >= g.Ny - 1) {
    st[c.ij] = 0.0;
    ce[c.ij] = 0.0;
    return;
  }
  const Nb d = neighbours(c.i, c.j, g.Nx, g.Ny, g.bits & F_PERIODIC);
  const double s = g.Fx[d.i1j] - g.Fx[d.ij] + g.Fy[d.ij1] - g.Fy[d.ij];
  st[d.ij] = s;
  ce[d.ij] = (g.rho[d.ij] - g.rho_pr[d.ij]) * g.hx[c.i] * g.hy[c.j] / g.ht + s;
}

}  // namespace sts
