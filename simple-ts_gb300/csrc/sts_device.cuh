// Device helpers shared by the kernel translation units (each .cu gets its own copy).
#pragma once
#include <cuda_runtime.h>

#include "sts_common.cuh"

namespace sts {
namespace {

__device__ __forceinline__ double dmax0(double a, double b) { return a > b ? a : b; }
// Face density upwind of velocity v1 (the mean when v1 is zero).  The two tests of v1 are made
// on its bit pattern (the integer pipes; GB300's FP64 unit is the scarce one): zero of either
// sign -> the mean; positive and not NaN (+inf included) -> r0; anything else -> r1, as the
// comparisons v1 == 0 and v1 > 0 decide.
__device__ __forceinline__ double upwind_rho(double r0, double r1, double v1) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v1), mag = b & 0x7fffffffffffffffull;
  if (mag == 0ull) return 0.5 * (r0 + r1);
  return ((b >> 63) == 0ull && mag <= 0x7ff0000000000000ull) ? r0 : r1;
}
__device__ __forceinline__ double Li(double f1, double f2, double h1, double h2) {
  return (f1 * h2 + f2 * h1) / (h1 + h2);
}
__device__ __forceinline__ double Hi(double f1, double f2, double h1, double h2) {
  return (h1 + h2) * f1 * f2 / (h1 * f2 + h2 * f1);
}
__device__ __forceinline__ double as_d(unsigned long long b) { return __longlong_as_double((long long)b); }
__device__ __forceinline__ unsigned long long as_b(double d) { return (unsigned long long)__double_as_longlong(d); }

// Kernels that the step graph launches before their predecessor has completed (a programmatic
// dependency: launched once every CTA of the predecessor has finished) wait here, before their
// first access to memory, until the predecessor has completed and its writes are visible.
// Launched any other way the wait returns at once.
__device__ __forceinline__ void wait_for_predecessor() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// The IEEE quotient, out of line: the rare operands div_cr cannot take branch here instead of
// being evaluated (predicated) beside every fast division.
__device__ __noinline__ double div_ieee(double a, double b) { return __ddiv_rn(a, b); }

// The IEEE quotient a / b, with zero dividends answered directly: for every b that is neither
// zero nor NaN, 0 / b is the zero whose sign is sign(a) xor sign(b), which a * copysign(1, b)
// gives exactly; every other pair takes the division.  Zero dividends are common in the fields
// (v vanishes over much of a channel) and slow for the IEEE division.
__device__ __forceinline__ double div_z(double a, double b) {
  if (a == 0.0 && (b > 0.0 || b < 0.0)) return __dmul_rn(a, copysign(1.0, b));
  return __ddiv_rn(a, b);
}

// Correctly rounded a / b from y = RN(1/b), the division by a correctly rounded reciprocal of
// P. Markstein (IBM J. Res. Develop. 34(1), 1990; Muller et al., Handbook of Floating-Point
// Arithmetic, 2nd ed., sec. 4.9): q0 = RN(a y) is within two units in the last place of a/b;
// one correction with the fused remainder makes it faithful, and for a faithful q the remainder
// r = a - b q is exact and RN(q + r y) = RN(a / b).  Valid when nothing overflows or underflows:
// operands outside 2^-900 <= |a| <= 2^900 or 2^-100 <= |b| <= 2^100 (subnormals, infinities
// and NaN included) take the IEEE division instead.  A zero dividend is exact: a y is the zero
// whose sign is sign(a) xor sign(b) (y carries b's sign), the IEEE quotient 0 / b; zeros are
// common in the fields (v vanishes over much of a channel), so they stay on the fast path.
// Explicit _rn intrinsics, so the result does not depend on the file's contraction flags.
__device__ __forceinline__ double div_cr(double a, double b, double y) {
  const unsigned ha = (unsigned)__double2hiint(a);
  const unsigned ea = (ha >> 20) & 0x7ffu;
  const unsigned eb = ((unsigned)__double2hiint(b) >> 20) & 0x7ffu;
  const bool za = ((ha & 0x7fffffffu) | (unsigned)__double2loint(a)) == 0u;
  if ((ea - 123u > 1800u && !za) || eb - 923u > 200u) return div_ieee(a, b);
  double q = __dmul_rn(a, y);
  if (za) return q;
  double r = __fma_rn(-b, q, a);
  q = __fma_rn(r, y, q);
  r = __fma_rn(-b, q, a);
  return __fma_rn(r, y, q);
}

// Convolutional warm start (warm_start 4), at the start of a step on a solved cell n holding
// x = p_n, y = T_n: the newest step differences D (FP32, ring slot r-1), the quadratic start of
// warm_start 2, replaced by the stencil's start where the end of the previous step prepared one;
// m receives |D| as float bit patterns for the per-field maximum.
__device__ __forceinline__ void conv_step_begin_cell(const Geo& g, int n, unsigned cur, unsigned r, unsigned m[2]) {
  const double x = g.p[cur][n], y = g.T[cur][n];
  if (r == 0) {
    g.p_m[0][n] = x; g.p_m[1][n] = x;
    g.T_m[0][n] = y; g.T_m[1][n] = y;
    return;
  }
  const double dx = x - g.p_m[0][n], dy = y - g.T_m[0][n];
  const float fx = (float)dx, fy = (float)dy;
  g.cD[0][(r - 1) % kConvRing][n] = fx;
  g.cD[1][(r - 1) % kConvRing][n] = fy;
  m[0] = __float_as_uint(fabsf(fx));
  m[1] = __float_as_uint(fabsf(fy));
  if (r >= 2) {
    g.p[cur][n] = 3.0 * dx + g.p_m[1][n];
    g.T[cur][n] = 3.0 * dy + g.T_m[1][n];
  } else {
    g.p[cur][n] = x + dx;
    g.T[cur][n] = y + dy;
  }
  g.p_m[1][n] = g.p_m[0][n]; g.p_m[0][n] = x;
  g.T_m[1][n] = g.T_m[0][n]; g.T_m[0][n] = y;
  // the stencil's start, prepared at the end of the previous step on the cells it flagged
  const uint8_t b = g.cact[(r - 1) & 1][n];
  if (b & 4u) g.p[cur][n] = g.cnext[0][n];
  if (b & 8u) g.T[cur][n] = g.cnext[1][n];
}

// Per-field maximum of |D| over the block, folded into the step's slot (non-negative floats
// order like their bit patterns; NaN lands above every number); the other parity's slot, the next
// step's, is cleared by the first block.  Every thread of the block calls this.
__device__ __forceinline__ void conv_block_max(const Geo& g, unsigned r, const unsigned m[2]) {
  if (r == 0) return;
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
    if (v) atomicMax(&g.ctl->conv_max[(r - 1) & 1][tid], v);
    if (blockIdx.x == 0 && blockIdx.y == 0) g.ctl->conv_max[r & 1][tid] = 0u;
  }
}

constexpr int kMaxColumn = 1024;  // rows staged in shared memory by the inflow-column reductions

// Running maximum that ignores NaN exactly like "if (m < fabs(r)) m = fabs(r)".
__device__ __forceinline__ double mx(double m, double x) { return (m < x) ? x : m; }

// Block-wide max of two non-negative values, folded into global maxima by bit pattern: for
// non-negative IEEE numbers the bit patterns order like the values, so the reduction runs on
// the integer pipes (the FP64 pipe is the scarce one).  NaN is left out of the maximum, as the
// reference's "if (m < fabs(r)) m = fabs(r)" leaves it out, and flagged in *status together
// with +inf.
__device__ __forceinline__ unsigned long long umax64(unsigned long long a, unsigned long long b) { return a > b ? a : b; }

__device__ void block_max2_bits(unsigned long long a, unsigned long long b, unsigned long long* ga,
                                unsigned long long* gb) {
  __shared__ unsigned long long sa[32], sb[32];
  const int lane = (threadIdx.x + threadIdx.y * blockDim.x) & 31;
  const int warp = (threadIdx.x + threadIdx.y * blockDim.x) >> 5;
  const int nw = (blockDim.x * blockDim.y + 31) >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    a = umax64(a, __shfl_xor_sync(0xffffffffu, a, o));
    b = umax64(b, __shfl_xor_sync(0xffffffffu, b, o));
  }
  if (lane == 0) { sa[warp] = a; sb[warp] = b; }
  __syncthreads();
  if (warp == 0) {
    a = lane < nw ? sa[lane] : 0ull;
    b = lane < nw ? sb[lane] : 0ull;
    for (int o = 16; o > 0; o >>= 1) {
      a = umax64(a, __shfl_xor_sync(0xffffffffu, a, o));
      b = umax64(b, __shfl_xor_sync(0xffffffffu, b, o));
    }
    if (lane == 0) {
      if (a) atomicMax(ga, a);
      if (b) atomicMax(gb, b);
    }
  }
}

// Bit pattern of a residual for the maximum: NaN and +inf set the status bit, NaN counts as 0.
__device__ __forceinline__ unsigned long long res_bits(double x, unsigned int* status) {
  const unsigned long long m = as_b(x) & 0x7fffffffffffffffull;
  if (m >= 0x7ff0000000000000ull) {
    atomicOr(status, 1u);
    if (m > 0x7ff0000000000000ull) return 0ull;
  }
  return m;
}

__device__ __forceinline__ void block_max2(double a, double b, unsigned long long* ga, unsigned long long* gb,
                                           unsigned int* status) {
  block_max2_bits(res_bits(a, status), res_bits(b, status), ga, gb);
}

// Bit pattern of an FP32 residual for the maximum, with block_max2_f's rule: NaN and +inf set the
// status bit, NaN counts as 0.
__device__ __forceinline__ unsigned res_bits_f(float x, unsigned int* status) {
  unsigned m = __float_as_uint(x) & 0x7fffffffu;
  if (m >= 0x7f800000u) {
    atomicOr(status, 1u);
    if (m > 0x7f800000u) m = 0u;
  }
  return m;
}

// The same for FP32 residuals: reduced as 32-bit patterns, folded in as doubles (exact widening).
__device__ void block_max2_f(float a, float b, unsigned long long* ga, unsigned long long* gb, unsigned int* status) {
  __shared__ unsigned sa[32], sb[32];
  unsigned ua = __float_as_uint(a) & 0x7fffffffu, ub = __float_as_uint(b) & 0x7fffffffu;
  if (ua >= 0x7f800000u || ub >= 0x7f800000u) {
    atomicOr(status, 1u);
    if (ua > 0x7f800000u) ua = 0u;
    if (ub > 0x7f800000u) ub = 0u;
  }
  const int lane = (threadIdx.x + threadIdx.y * blockDim.x) & 31;
  const int warp = (threadIdx.x + threadIdx.y * blockDim.x) >> 5;
  const int nw = (blockDim.x * blockDim.y + 31) >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    ua = max(ua, __shfl_xor_sync(0xffffffffu, ua, o));
    ub = max(ub, __shfl_xor_sync(0xffffffffu, ub, o));
  }
  if (lane == 0) { sa[warp] = ua; sb[warp] = ub; }
  __syncthreads();
  if (warp == 0) {
    ua = lane < nw ? sa[lane] : 0u;
    ub = lane < nw ? sb[lane] : 0u;
    for (int o = 16; o > 0; o >>= 1) {
      ua = max(ua, __shfl_xor_sync(0xffffffffu, ua, o));
      ub = max(ub, __shfl_xor_sync(0xffffffffu, ub, o));
    }
    if (lane == 0) {
      if (ua) atomicMax(ga, as_b((double)__uint_as_float(ua)));
      if (ub) atomicMax(gb, as_b((double)__uint_as_float(ub)));
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

__device__ __forceinline__ unsigned atom_add_acq_rel(unsigned* p, unsigned v) {
  unsigned old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}
__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed(unsigned* p, unsigned v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Grid-wide barrier on the counter/generation pair of a LoopCtl.  The CTA's writes are ordered
// before thread 0's arrival by the CTA barrier; the arrival is an acquire-release add, so the
// last arriver has acquired every earlier arrival; it resets the counter and publishes the next
// generation with a release store, which the others acquire before their CTA barrier releases
// their threads (acquire/release pairs instead of full fences: about 0.5 us less per barrier
// with 608 CTAs).  A CTA that waits longer than spin_limit polls sets ST_BARRIER_TIMEOUT and
// returns false, so a launch whose CTAs are not all resident ends with an error status instead
// of hanging.
__device__ bool grid_barrier(LoopCtl* lc, unsigned spin_limit = kSpinLimit) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    const unsigned g0 = ld_acquire(&lc->bar_gen);
    int good = 1;
    if (atom_add_acq_rel(&lc->bar_count, 1u) == gridDim.x * gridDim.y - 1) {
      st_relaxed(&lc->bar_count, 0u);
      st_release(&lc->bar_gen, g0 + 1u);
    } else {
      unsigned spins = 0;
      while (ld_acquire(&lc->bar_gen) == g0) {
        if (++spins > spin_limit) {
          atomicOr(&lc->status, ST_BARRIER_TIMEOUT);
          good = 0;
          break;
        }
        __nanosleep(64);
      }
    }
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

// The reference's stop rule of the sweep loop (SIMPLE_TS_MPI.cpp:4087-4107), n sweeps taken.
__device__ __forceinline__ bool sweep_continues(const Geo& g, unsigned n, double res_p, double res_T) {
  if (g.bits & F_FIXED_SWEEPS) return n < (unsigned)g.N_I_p_c;
  return (n < 2) || ((n < (unsigned)g.N_I_p_c) && ((g.MaxError_p_c < res_p) || (g.MaxError_T < res_T)));
}

// Records the residuals of sweep n (1-based) of outer iteration I.
__device__ __forceinline__ void record_residual(Ctl* ctl, unsigned n, unsigned I, double res_p, double res_T) {
  ctl->res_p[I] = res_p;
  ctl->res_T[I] = res_T;
  if (n == 1) {
    ctl->res_p0[I] = res_p;
    ctl->res_T0[I] = res_T;
  }
}

// ---------------------------------------------------------------------------
// The persistent sweep loop of one or many cases.  Every case runs a small state machine
// (LoopCase) whose passes -- a sweep, or for the FP32-correction loop also the re-forming of
// an FP64 iterate -- all take one round.  In a round every CTA takes its share of the tiles of
// all cases still running, folds the pass's residual maxima into the case's slot round % 3,
// and meets the others at the grid barrier; then every CTA advances every case's state from
// the same numbers, so all CTAs agree without further communication.  The loop ends when
// every case has met its stop rule; the last CTA to leave writes the cases' loop results.
// Ops supplies pass() (one cell of the current pass) and advance() (the state transition).
// ---------------------------------------------------------------------------
enum : unsigned char { PS_FIRST = 0, PS_SWEEP = 1, PS_SWEEP32 = 2, PS_MATERIALIZE = 3, PS_CONFIRM = 4, PS_DONE = 255 };

struct LoopCase {
  unsigned n;     // sweeps counted so far (the reference's Iter_p_c)
  unsigned cur;   // FP64 buffer with the latest iterate
  unsigned base;  // FP64 buffer with the base of the FP32 corrections
  unsigned I;     // outer iteration (row of the residual records)
  unsigned char phase, ec, active, eprev;  // ec: correction buffer with the latest FP32 iterate,
                                          // eprev: the one with the iterate before it
};

// SINGLE: one case whose Geo g0 is a kernel parameter (gs, tile_case, tile_first unused).
// TB (single cases of the FP32-correction loop): a round of FP32 sweeps takes two sweeps per tile
// load (Ops::pass32_pair, tiles staged by TMA through `maps`, shared memory at tb_smem); the round's
// second residual pair goes to the rb2 slots, and the state advances sweep by sweep from them, so
// the loop stops at the same sweep with the same iterate as with one sweep per round.
template <class Ops, bool SINGLE, bool TB = false>
__device__ __forceinline__ void pt_loop_rounds(const Geo& g0, const Geo* __restrict__ gs,
                                               const int* __restrict__ tile_case, const int* __restrict__ tile_first,
                                               int ncases, int ntiles, LoopCtl* lc, const EMaps* maps = nullptr,
                                               void* tb_smem = nullptr) {
  unsigned tphase = 0;  // parity of the TMA barrier's next completion (TB)
  auto G = [&](int c) -> const Geo& { return SINGLE ? g0 : gs[c]; };
  __shared__ LoopCase sc[kMaxBatchCases];
  __shared__ bool last;
  const int tid = threadIdx.x + threadIdx.y * blockDim.x, nthr = blockDim.x * blockDim.y;
  const bool lead = blockIdx.x == 0 && blockIdx.y == 0;
  for (int c = tid; c < ncases; c += nthr) {
    const Ctl* ctl = G(c).ctl;
    LoopCase s;
    s.n = 0;
    s.cur = ctl->cur;
    s.base = s.cur;
    s.I = ctl->Iter < 64 ? ctl->Iter : 63;
    s.ec = 0;
    s.active = ctl->running ? 1 : 0;
    s.phase = s.active ? PS_FIRST : PS_DONE;
    s.eprev = 0;
    sc[c] = s;
  }
  __syncthreads();
  // Ops::kCellList, one case: each CTA takes an equal slice of the solved cells instead of
  // 32x8 tiles (tiles leave most SMs with four full tiles while the mean is lower: walls, bodies
  // and the last tile row); the unsolved cells are passed in the first pass only (copied, and
  // their correction terms zeroed), after which both iterate buffers hold the same values there
  // and every later pass would only copy them onto themselves.
  const bool by_list = Ops::kCellList && SINGLE && g0.pt_cells != nullptr;
  for (unsigned round = 0;; round++) {
    const unsigned slot = round % 3;
    if (by_list) {
      const LoopCase s = sc[0];
      const int per = (g0.n_pt_cells + (int)gridDim.x - 1) / (int)gridDim.x;
      const int k0 = (int)blockIdx.x * per, k1 = min(g0.n_pt_cells, k0 + per);
      auto list_cell = [&](unsigned e) {
        Cell cl;
        cl.i = (int)(e & 0xffffu);
        cl.j = (int)(e >> 16);
        cl.ok = true;
        cl.ij = cl.i + cl.j * g0.Nx;
        return cl;
      };
      unsigned* st = &g0.ctl->status;
      if (s.phase == PS_SWEEP32) {  // FP32 residuals: the thread's maximum, then the block's
        unsigned fp = 0, fT = 0;
        for (int k = k0 + tid; k < k1; k += nthr) {
          float a = 0.f, b = 0.f;
          Ops::pass32(g0, list_cell(g0.pt_cells[k]), s, a, b);
          fp = max(fp, res_bits_f(a, st));
          fT = max(fT, res_bits_f(b, st));
        }
        block_max2_f(__uint_as_float(fp), __uint_as_float(fT), &g0.ctl->rb_p[slot], &g0.ctl->rb_T[slot], st);
      } else if (s.phase != PS_DONE) {
        unsigned long long bp = 0, bT = 0;
        for (int k = k0 + tid; k < k1; k += nthr) {
          double a = 0, b = 0;
          Ops::pass(g0, list_cell(g0.pt_cells[k]), s, a, b);
          bp = umax64(bp, res_bits(a, st));
          bT = umax64(bT, res_bits(b, st));
        }
        if (s.phase == PS_FIRST) {
          const int perc = (g0.n_pt_copy + (int)gridDim.x - 1) / (int)gridDim.x;
          const int c0 = (int)blockIdx.x * perc, c1 = min(g0.n_pt_copy, c0 + perc);
          for (int k = c0 + tid; k < c1; k += nthr) {
            double a = 0, b = 0;
            Ops::pass(g0, list_cell(g0.pt_copy[k]), s, a, b);  // an unsolved cell: copied, no residual
          }
        }
        if (s.phase != PS_MATERIALIZE) block_max2_bits(bp, bT, &g0.ctl->rb_p[slot], &g0.ctl->rb_T[slot]);
      }
    }
    bool pair_round = false;
    if constexpr (TB) {
      if (sc[0].phase == PS_SWEEP32) {  // two FP32 sweeps per tile load
        pair_round = true;
        for (int t = (int)blockIdx.x; t < ntiles; t += gridDim.x)
          if (!Ops::pass32_pair(g0, t, sc[0], maps, tb_smem, tphase, slot)) break;
      }
    }
    for (int t = (by_list || pair_round) ? ntiles : (int)blockIdx.x; t < ntiles; t += gridDim.x) {
      const int c = SINGLE ? 0 : tile_case[t];
      const LoopCase s = sc[c];
      if (s.phase == PS_DONE) continue;  // uniform over the CTA
      const Geo& g = G(c);
      const Cell cl = tile_cell(g, SINGLE ? t : t - tile_first[c], (g.Nx + 31) / 32);
      if (s.phase == PS_SWEEP32) {  // FP32 residuals, reduced as floats
        float rp = 0.f, rT = 0.f;
        if (cl.ok) Ops::pass32(g, cl, s, rp, rT);
        block_max2_f(rp, rT, &g.ctl->rb_p[slot], &g.ctl->rb_T[slot], &g.ctl->status);
      } else {
        double rp = 0, rT = 0;
        if (cl.ok) Ops::pass(g, cl, s, rp, rT);
        if (s.phase != PS_MATERIALIZE) block_max2(rp, rT, &g.ctl->rb_p[slot], &g.ctl->rb_T[slot], &g.ctl->status);
      }
    }
    // clear the slot of the next round (its last readers passed the previous barrier)
    if (lead)
      for (int c = tid; c < ncases; c += nthr) {
        G(c).ctl->rb_p[(round + 1) % 3] = 0ull;
        G(c).ctl->rb_T[(round + 1) % 3] = 0ull;
        if (TB) {
          G(c).ctl->rb2_p[(round + 1) % 3] = 0ull;
          G(c).ctl->rb2_T[(round + 1) % 3] = 0ull;
        }
      }
    if (!grid_barrier(lc)) break;
    int any = 0;
    for (int c = tid; c < ncases; c += nthr) {
      LoopCase s = sc[c];
      if (s.phase == PS_DONE) continue;
      double res_p = 0, res_T = 0;
      if (s.phase != PS_MATERIALIZE) {
        res_p = ld_res(&G(c).ctl->rb_p[slot]);
        res_T = ld_res(&G(c).ctl->rb_T[slot]);
      }
      Ops::advance(G(c), lead, s, res_p, res_T);
      if (TB && pair_round && s.phase == PS_SWEEP32)  // the round's second sweep
        Ops::advance(G(c), lead, s, ld_res(&G(c).ctl->rb2_p[slot]), ld_res(&G(c).ctl->rb2_T[slot]));
      sc[c] = s;
      any |= (s.phase != PS_DONE);
    }
    if (!__syncthreads_or(any)) break;
  }
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    last = atomicAdd(&lc->block_count, 1u) == gridDim.x * gridDim.y - 1;
    if (last) lc->block_count = 0;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  const unsigned lstatus = *(volatile unsigned*)&lc->status;
  for (int c = tid; c < ncases; c += nthr) {
    const LoopCase s = sc[c];
    if (!s.active) continue;
    Ctl* ctl = G(c).ctl;
    if (lstatus) atomicOr(&ctl->status, lstatus);  // a barrier timeout ends the run of every case
    ctl->cur = s.cur;
    ctl->Iter_p_c = s.n;
    ctl->pt_done = 1;
    ctl->sweeps[s.I] = s.n;
    ctl->step_sweeps += s.n;
    for (int k = 0; k < 3; k++) {
      ctl->rb_p[k] = 0ull;
      ctl->rb_T[k] = 0ull;
      ctl->rb2_p[k] = 0ull;
      ctl->rb2_T[k] = 0ull;
    }
  }
}

// The FP64 loops' state transition (exact and mode-1 sweeps): count the sweep, flip the
// buffers, apply the stop rule.
__device__ __forceinline__ void advance_fp64(const Geo& g, bool lead, LoopCase& s, double res_p, double res_T) {
  s.n++;
  s.cur ^= 1;
  if (lead) record_residual(g.ctl, s.n, s.I, res_p, res_T);
  s.phase = sweep_continues(g, s.n, res_p, res_T) ? PS_SWEEP : PS_DONE;
}

// A batched kernel's CTA (x, y, z) works on case z: the case's Geo is staged in shared memory.
// Returns whether the case takes part in the current step.
__device__ __forceinline__ bool stage_geo(Geo& sg, const Geo* __restrict__ gs, unsigned which) {
  const int tid = threadIdx.x + threadIdx.y * blockDim.x, nthr = blockDim.x * blockDim.y;
  const unsigned* src = reinterpret_cast<const unsigned*>(&gs[which]);
  unsigned* dst = reinterpret_cast<unsigned*>(&sg);
  for (int k = tid; k < (int)(sizeof(Geo) / 4); k += nthr) dst[k] = src[k];
  __syncthreads();
  return *(volatile unsigned*)&sg.ctl->running != 0;
}
__device__ __forceinline__ bool stage_geo(Geo& sg, const Geo* __restrict__ gs) { return stage_geo(sg, gs, blockIdx.z); }

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
