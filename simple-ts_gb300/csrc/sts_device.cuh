// Device helpers shared by the kernel translation units (each .cu gets its own copy).
#pragma once
#include <cuda_runtime.h>

#include "sts_common.cuh"

namespace sts {
namespace {

__device__ __forceinline__ double dmax0(double a, double b) { return a > b ? a : b; }
__device__ __forceinline__ double upwind_rho(double r0, double r1, double v1) {
  return (v1 == 0) ? (0.5 * (r0 + r1)) : ((v1 > 0) ? r0 : r1);
}
__device__ __forceinline__ double Li(double f1, double f2, double h1, double h2) {
  return (f1 * h2 + f2 * h1) / (h1 + h2);
}
__device__ __forceinline__ double Hi(double f1, double f2, double h1, double h2) {
  return (h1 + h2) * f1 * f2 / (h1 * f2 + h2 * f1);
}
__device__ __forceinline__ double as_d(unsigned long long b) { return __longlong_as_double((long long)b); }
__device__ __forceinline__ unsigned long long as_b(double d) { return (unsigned long long)__double_as_longlong(d); }

// Correctly rounded a / b from y = RN(1/b), the division by a correctly rounded reciprocal of
// P. Markstein (IBM J. Res. Develop. 34(1), 1990; Muller et al., Handbook of Floating-Point
// Arithmetic, 2nd ed., sec. 4.9): q0 = RN(a y) is within two units in the last place of a/b;
// one correction with the fused remainder makes it faithful, and for a faithful q the remainder
// r = a - b q is exact and RN(q + r y) = RN(a / b).  Valid when nothing overflows or underflows:
// operands outside 2^-900 <= |a| <= 2^900 or 2^-100 <= |b| <= 2^100 (zeros, subnormals,
// infinities and NaN included) take the IEEE division instead.  Explicit _rn intrinsics, so the
// result does not depend on the file's contraction flags.
__device__ __forceinline__ double div_cr(double a, double b, double y) {
  const unsigned ea = ((unsigned)__double2hiint(a) >> 20) & 0x7ffu;
  const unsigned eb = ((unsigned)__double2hiint(b) >> 20) & 0x7ffu;
  if (ea - 123u > 1800u || eb - 923u > 200u) return __ddiv_rn(a, b);
  double q = __dmul_rn(a, y);
  double r = __fma_rn(-b, q, a);
  q = __fma_rn(r, y, q);
  r = __fma_rn(-b, q, a);
  return __fma_rn(r, y, q);
}

constexpr int kMaxColumn = 1024;  // rows staged in shared memory by the inflow-column reductions

// Running maximum that ignores NaN exactly like "if (m < fabs(r)) m = fabs(r)".
__device__ __forceinline__ double mx(double m, double x) { return (m < x) ? x : m; }

// Block-wide max of two non-negative values, folded into global maxima by bit pattern
// (for non-negative IEEE doubles the bit patterns order like the values).
__device__ void block_max2(double a, double b, unsigned long long* ga, unsigned long long* gb, unsigned int* status) {
  __shared__ double sa[32], sb[32];
  const int lane = (threadIdx.x + threadIdx.y * blockDim.x) & 31;
  const int warp = (threadIdx.x + threadIdx.y * blockDim.x) >> 5;
  const int nw = (blockDim.x * blockDim.y + 31) >> 5;
  if (!(a <= 1.7976931348623157e308) && a == a) atomicOr(status, 1u);  // +inf
  if (a != a || b != b) atomicOr(status, 1u);                           // NaN
  for (int o = 16; o > 0; o >>= 1) {
    a = mx(a, __shfl_xor_sync(0xffffffffu, a, o));
    b = mx(b, __shfl_xor_sync(0xffffffffu, b, o));
  }
  if (lane == 0) { sa[warp] = a; sb[warp] = b; }
  __syncthreads();
  if (warp == 0) {
    a = lane < nw ? sa[lane] : 0.0;
    b = lane < nw ? sb[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      a = mx(a, __shfl_xor_sync(0xffffffffu, a, o));
      b = mx(b, __shfl_xor_sync(0xffffffffu, b, o));
    }
    if (lane == 0) {
      if (a > 0) atomicMax(ga, as_b(a));
      if (b > 0) atomicMax(gb, as_b(b));
    }
  }
}

// True for exactly one thread in the grid: the last thread (0,0) of the last block to finish.
__device__ bool last_block(unsigned int* counter) {
  __shared__ bool last;
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    __threadfence();
    const unsigned int nb = gridDim.x * gridDim.y;
    const unsigned int t = atomicAdd(counter, 1u);
    last = (t == nb - 1);
    if (last) *counter = 0;
  }
  __syncthreads();
  return last && threadIdx.x == 0 && threadIdx.y == 0;
}

struct Cell {
  int i, j, ij;
  bool ok;
};
__device__ __forceinline__ Cell cell(const Geo& g) {
  Cell c;
  c.i = blockIdx.x * blockDim.x + threadIdx.x;
  c.j = blockIdx.y * blockDim.y + threadIdx.y;
  c.ok = c.i < g.Nx && c.j < g.Ny;
  c.ij = c.i + c.j * g.Nx;
  return c;
}

// ---------------------------------------------------------------------------
// Persistent sweep loops: one launch runs every p-T sweep of an outer iteration.  The grid is
// no larger than the number of CTAs that fit on the GPU at once (cooperative launch), each CTA
// takes 32x8-cell tiles in a grid-stride loop, and the CTAs meet at a grid barrier after every
// sweep, where each reads the sweep's residual maxima and applies the stop rule itself.
// ---------------------------------------------------------------------------
constexpr unsigned kSpinLimit = 1u << 24;  // barrier polls before giving up (about a second)

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Grid-wide barrier on the counter/generation pair of the control block.  A CTA that waits
// longer than kSpinLimit polls sets ST_BARRIER_TIMEOUT and returns false, so a launch whose
// CTAs are not all resident ends with an error status instead of hanging.
__device__ bool grid_barrier(Ctl* ctl) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    const unsigned g0 = ld_acquire(&ctl->bar_gen);
    __threadfence();
    int good = 1;
    if (atomicAdd(&ctl->bar_count, 1u) == gridDim.x * gridDim.y - 1) {
      atomicExch(&ctl->bar_count, 0u);
      __threadfence();
      atomicAdd(&ctl->bar_gen, 1u);
    } else {
      unsigned spins = 0;
      while (ld_acquire(&ctl->bar_gen) == g0) {
        if (++spins > kSpinLimit) {
          atomicOr(&ctl->status, ST_BARRIER_TIMEOUT);
          good = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    ok = good;
  }
  __syncthreads();
  return ok;
}

__device__ __forceinline__ double ld_res(const unsigned long long* p) {
  return as_d(*(const volatile unsigned long long*)p);
}

// Cell of thread (x, y) in tile t of a 32x8 tiling (tx tiles per row).
__device__ __forceinline__ Cell tile_cell(const Geo& g, int t, int tx) {
  Cell c;
  const int ty = t / tx;
  c.i = (t - ty * tx) * 32 + threadIdx.x;
  c.j = ty * 8 + threadIdx.y;
  c.ok = c.i < g.Nx && c.j < g.Ny;
  c.ij = c.i + c.j * g.Nx;
  return c;
}

// Folds a sweep's per-CTA residual maxima into slot n % 3, clears the slot sweep n+1 will use
// (its last readers passed the barrier of sweep n-1 before this CTA could reach sweep n), meets
// the other CTAs at the barrier and returns the sweep's global maxima.  False on a barrier timeout.
__device__ __forceinline__ bool sweep_residual(Ctl* ctl, unsigned n, double rp, double rT, double& res_p,
                                               double& res_T) {
  const unsigned slot = n % 3, next = (n + 1) % 3;
  block_max2(rp, rT, &ctl->rb_p[slot], &ctl->rb_T[slot], &ctl->status);
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0) {
    ctl->rb_p[next] = 0ull;
    ctl->rb_T[next] = 0ull;
  }
  if (!grid_barrier(ctl)) return false;
  res_p = ld_res(&ctl->rb_p[slot]);
  res_T = ld_res(&ctl->rb_T[slot]);
  return true;
}

// The reference's stop rule of the sweep loop (SIMPLE_TS_MPI.cpp:4087-4107), n sweeps taken.
__device__ __forceinline__ bool sweep_continues(const Geo& g, unsigned n, double res_p, double res_T) {
  if (g.bits & F_FIXED_SWEEPS) return n < (unsigned)g.N_I_p_c;
  return (n < 2) || ((n < (unsigned)g.N_I_p_c) && ((g.MaxError_p_c < res_p) || (g.MaxError_T < res_T)));
}

// Bookkeeping of a finished loop by the last CTA to leave: current buffer, sweep counts, and
// the residual slots cleared for the next launch.
__device__ __forceinline__ void pt_loop_finish(Ctl* ctl, unsigned cur, unsigned n, unsigned I) {
  if (last_block(&ctl->block_count)) {
    ctl->cur = cur;
    ctl->Iter_p_c = n;
    ctl->pt_done = 1;
    ctl->sweeps[I] = n;
    ctl->step_sweeps += n;
    for (int k = 0; k < 3; k++) {
      ctl->rb_p[k] = 0ull;
      ctl->rb_T[k] = 0ull;
    }
  }
}

// Records the residuals of sweep n (1-based) of outer iteration I (one thread of CTA 0).
__device__ __forceinline__ void record_residual(Ctl* ctl, unsigned n, unsigned I, double res_p, double res_T) {
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0) {
    ctl->res_p[I] = res_p;
    ctl->res_T[I] = res_T;
    if (n == 1) {
      ctl->res_p0[I] = res_p;
      ctl->res_T0[I] = res_T;
    }
  }
}

// Zero-gradient copies into the ghost cells outside the p/T solve range, side by side in the
// reference's order (x begin, x end, y begin, y end); a ghost cell takes the value of the
// nearest solved cell of its row or column when that cell is fluid.  Called by every thread
// of one CTA.  Pure copies, so every build of it gives the same bits.
__device__ __forceinline__ void zero_gradient_ghosts(const Geo& g, double* __restrict__ f, uint64_t xb, uint64_t xe,
                                                     uint64_t yb, uint64_t ye, int tid, int nt) {
  const int Nx = g.Nx, Ny = g.Ny;
  const uint64_t bits = g.bits;
  if (bits & F_PERIODIC) return;
  auto fl = [&](int q) { return cls_fluid(g.cls[q]); };
  if (bits & xb) {
    for (int k = tid; k < Ny * g.Nx_o0; k += nt) {
      const int j = k / g.Nx_o0, i = k - j * g.Nx_o0, n = g.Nx_o0 + j * Nx;
      if (fl(n)) f[i + j * Nx] = f[n];
    }
    __syncthreads();
  }
  if (bits & xe) {
    const int w = Nx - g.Nx_o1;
    for (int k = tid; k < Ny * w; k += nt) {
      const int j = k / w, i = g.Nx_o1 + (k - j * w), n = g.Nx_o1 - 1 + j * Nx;
      if (fl(n)) f[i + j * Nx] = f[n];
    }
    __syncthreads();
  }
  if (bits & yb) {
    for (int k = tid; k < Nx * g.Ny_o0; k += nt) {
      const int jj = k / Nx, i = k - jj * Nx, n = i + g.Ny_o0 * Nx;
      if (fl(n)) f[i + jj * Nx] = f[n];
    }
    __syncthreads();
  }
  if (bits & ye) {
    const int w = Ny - g.Ny_o1;
    for (int k = tid; k < Nx * w; k += nt) {
      const int jj = k / Nx, i = k - jj * Nx, n = i + (g.Ny_o1 - 1) * Nx;
      if (fl(n)) f[i + (g.Ny_o1 + jj) * Nx] = f[n];
    }
    __syncthreads();
  }
}

// BoundaryConditions_Temperature (SIMPLE_TS_MPI.cpp:7650-7741)
__device__ __forceinline__ void phase_temp(const Geo& g, double* __restrict__ T, int tid, int nt) {
  zero_gradient_ghosts(g, T, F_DTDX0_XB, F_DTDX0_XE, F_DTDY0_YB, F_DTDY0_YE, tid, nt);
}

// BoundaryConditions_Pressure (SIMPLE_TS_MPI.cpp:7335-7428)
__device__ __forceinline__ void phase_pres(const Geo& g, double* __restrict__ p, int tid, int nt) {
  zero_gradient_ghosts(g, p, F_DPDX0_XB, F_DPDX0_XE, F_DPDY0_YB, F_DPDY0_YE, tid, nt);
}

}  // namespace

}  // namespace sts
