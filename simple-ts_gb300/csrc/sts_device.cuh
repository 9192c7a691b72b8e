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
