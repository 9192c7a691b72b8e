// Shared host/device definitions for the GB300 SIMPLE-TS time step.
//
// Data layout in HBM: every field is a dense double[Nx*Ny] array with
// ij = i + j*Nx (x fastest), the same indexing as the reference
// (SIMPLE_TS_MPI.cpp:140-153, :2384-2464), so dumps are byte-compatible.
// Static per-cell information is packed in one byte per cell (CellClass),
// replacing the reference's rule vectors (SIMPLE_TS_MPI.cpp:8581-9063).
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define STS_HD __host__ __device__ __forceinline__
#else
#define STS_HD inline
#endif

#include <cuda.h>  // CUtensorMap

namespace sts {

// Per-cell class byte.
//   bits 0-1: u-face class, bits 2-3: v-face class, bits 4-5: p/T cell class
//             (0 = not solved, 1 = interior list "nch", 2 = boundary list "bc")
//   bit 6   : fluid (vol_inf_fb == 0)
enum : uint8_t { CLS_NONE = 0, CLS_NCH = 1, CLS_BC = 2 };
STS_HD int cls_u(uint8_t c) { return c & 3; }
STS_HD int cls_v(uint8_t c) { return (c >> 2) & 3; }
STS_HD int cls_o(uint8_t c) { return (c >> 4) & 3; }
STS_HD bool cls_fluid(uint8_t c) { return (c >> 6) & 1; }

// Body properties used by the wall conditions (Polyhedrons_Objects.h, Circles_Objects.h).
struct Body {
  double u, v, p, T;
  double F_slip, F_jump, dTdn0;
  int slip, jump;
};

// Bits of Flags.bits: boundary-condition switches read from EnteredData.txt.
enum FlagBit : uint64_t {
  F_PERIODIC = 1ull << 0,
  F_PRESSURE_BC = 1ull << 1,
  F_GIVEN_U_XB = 1ull << 2,
  F_GIVEN_U_XE = 1ull << 3,
  F_DVDX0_XB = 1ull << 4,
  F_DVDX0_XE = 1ull << 5,
  F_DVDY0_YB = 1ull << 6,
  F_DVDY0_YE = 1ull << 7,
  F_DUDX0_XB = 1ull << 8,
  F_DURHODX0_XB = 1ull << 9,
  F_DRHODT0_XB = 1ull << 10,
  F_DUDX0_XE = 1ull << 11,
  F_DURHODX0_XE = 1ull << 12,
  F_DRHODT0_XE = 1ull << 13,
  F_U_MINMOUT_XE = 1ull << 14,
  F_DUDY0_YB = 1ull << 15,
  F_DUDY0_YE = 1ull << 16,
  F_DPDX0_XB = 1ull << 17,
  F_DPDX0_XE = 1ull << 18,
  F_DPDY0_YB = 1ull << 19,
  F_DPDY0_YE = 1ull << 20,
  F_DTDX0_XB = 1ull << 21,
  F_DTDX0_XE = 1ull << 22,
  F_DTDY0_YB = 1ull << 23,
  F_DTDY0_YE = 1ull << 24,
  F_KN_LOCAL = 1ull << 25,
  F_GIVEN_REKN = 1ull << 26,
  F_RATIO_CORRECT = 1ull << 27,
  F_P_CORR_AUTO = 1ull << 28,
  F_CORRECT_P_XB = 1ull << 29,
  F_U_BY_TIME = 1ull << 30,
  F_FIXED_SWEEPS = 1ull << 31,
};

// Mutable scalars of the run, resident in device memory so that the whole
// step (including the data-dependent sweep count) runs without host round trips.
struct Ctl {
  // nondimensional coefficients refreshed every outer iteration (SIMPLE_TS_MPI.cpp:4347-4361)
  double cT, cPch;
  // inflow / pressure-control state (SIMPLE_TS_MPI.cpp:7430-7647)
  double p_BC_xb, p_BC_xe, u_given_xb, u_given_xb_in_it, u_in_max, u_in_mean, p_correction, u_gas_nd;
  double it;  // physical time
  // residuals
  double res_u, res_v, res_u0, res_v0;
  unsigned long long res_bits_p, res_bits_T;  // running max of the current sweep (bit patterns)
  unsigned long long res_bits_u, res_bits_v;
  double res_p[64], res_T[64], res_p0[64], res_T0[64];  // per outer iteration (N_I <= 64)
  unsigned int sweeps[64];
  // loop control
  unsigned int cur;        // which of the two p/T buffers holds the current iterate
  unsigned int Iter, Iter_pr1, Iter_pr2, Iter_p_c;
  unsigned int it_counter;
  unsigned int pt_done;    // the sweep loop of this outer iteration has stopped
  unsigned int continue_iter, continue_step;
  unsigned int steps_left; // multi-step graph launches count down here
  unsigned int block_count;  // last-block detection
  unsigned int bnd_count;    // last-CTA detection of the fused boundary kernel
  unsigned int status;     // ST_* bits
  unsigned int step_sweeps;  // sum of sweeps in the current step
  // per-step record (ring of the last 4096 steps)
  unsigned int hist_n;
  unsigned int hist_sweeps[4096];
  // mixed-precision sweep loop statistics
  unsigned int sweeps32;      // FP32 sweeps taken in this run
  unsigned int rebases;       // FP64 re-basings of the FP32 corrections in this run
  // persistent sweep loop: per-sweep residual maxima (three slots used in rotation; all zero
  // between launches)
  unsigned long long rb_p[3], rb_T[3];
  // the second sweep of a temporally blocked FP32 round (two sweeps per round), same rotation
  unsigned long long rb2_p[3], rb2_T[3];
  unsigned int running;       // the case takes part in the current step (batches; 1 otherwise)
  unsigned int warm_ready;    // steps of history the warm start has
  // mode 3: per step, the normal-equation terms of its newest target (6 Gram entries and 3
  // right-hand sides, for p and for T) over the last kWarmWin steps, and the fitted weights
  double warm_acc[6][2][9];
  double warm_w[2][3];
  // mode 4: max |D| of the newest step difference per field (float bit patterns, by step
  // parity), the fitted stencil weights and whether this step's fit succeeded, per field
  unsigned int conv_max[2][2];
  float conv_w[2][36];
  unsigned int conv_ok[2];
};

// Learned warm start: differences kept, and steps of the least-squares window.
constexpr int kWarmRing = 4, kWarmWin = 6;

// Convolutional warm start (mode 4): features per cell (4 time-difference orders x 9 spatial
// basis values of the 3x3 neighbourhood), normal-equation terms per field (upper triangle of the
// 36x36 Gram matrix, then the 36 right-hand sides), steps in the least-squares window, ring of
// stored step differences, and the strips of 32x2 cells whose FP32 partial sums are kept apart.
constexpr int kConvFeat = 36, kConvTerms = kConvFeat * (kConvFeat + 1) / 2 + kConvFeat, kConvWin = 6,
              kConvRing = 5, kConvStripX = 32, kConvStripY = 2;

// Most cases one batch may hold (the sweep loop keeps their state in shared memory).
constexpr int kMaxBatchCases = 256;

// Grid barrier and exit ticket of one persistent sweep-loop launch (one per context or batch).
struct LoopCtl {
  unsigned int bar_count, bar_gen, status, block_count;
};

// TMA tensor maps of the three FP32 correction buffers of e_T and e_p (the temporally blocked
// FP32 sweeps load their tiles with them); a kernel parameter.
struct EMaps {  // aligned as CUtensorMap (128 bytes)
  CUtensorMap eT[3], ep[3];
};

// Bits of Ctl::status.
enum : unsigned { ST_NONFINITE = 1u, ST_BARRIER_TIMEOUT = 2u };

// Everything a kernel needs: constant parameters and device pointers.
struct Geo {
  int Nx, Ny, Na;
  uint64_t bits;  // FlagBit
  // solve ranges (define_area_for_solving, SIMPLE_TS_MPI.cpp:6009-6191)
  int Nx_u0, Nx_u1, Ny_u0, Ny_u1, Nx_v0, Nx_v1, Ny_v0, Ny_v1, Nx_o0, Nx_o1, Ny_o0, Ny_o1;
  // constants
  double ht, gamma1, Kn, cT1, cT2, c_Fr_v, Re, Ma, T_BC_xb, T_BC_xe, u_given_xb_error, p_correction_min,
      p_correction_max, MaxError_Velocities, MaxError_p_c, MaxError_T, MaxError_to_stop_program, Nt;
  double t_BC_b, t_BC_e, u_BC_xb_t_BC_b, u_BC_xb_t_BC_e;
  int TypeND, N_I, N_I_p_c, p_corr_method;
  // static geometry
  const double *hx, *hy;
  const uint8_t* cls;
  const uint32_t* vol_id;
  const Body* bodies;  // bodies[id-1]
  // wall lists; the flag arrays say which of an entry's writes survive in the
  // reference's sequential order (bit0: first write, bit1: second, ...)
  const int *slip_u, *slip_v, *tjump;
  const uint8_t *slip_u_fin, *slip_v_fin, *tjump_fin, *tjump_wr_fin;
  int n_slip_u, n_slip_v, n_tjump;
  // the cells the p-T sweeps solve (p/T class set) and the other cells, row-major, each packed
  // as i | j << 16: a single case's FP64 sweep loops split the solved cells evenly over their
  // CTAs, and copy the others through in the first sweep of a loop only
  const unsigned *pt_cells, *pt_copy;
  int n_pt_cells, n_pt_copy;
  // fields
  double *u, *v, *u_pr, *v_pr, *p[2], *T[2], *p_pr, *T_pr, *rho, *rho_pr, *sqrt_T, *rho_u, *rho_v;
  double *Fx, *Fy, *D_ux, *D_uy, *D_vx, *D_vy, *DTx, *DTy, *Gamma_xf, *Gamma_yf;
  double *u_pseudo, *v_pseudo, *d12, *d34, *apx, *apy, *bpx, *bpy, *ScT1, *Tw_u, *Tw_v;
  double* inv[9];  // loop-invariant parts of the sweep, written by the first sweep of an outer iteration
  Ctl* ctl;
  // correctly rounded reciprocals of the mesh quantities the kernels divide by: 1/hx, 1/hy,
  // 1/(hx[i-1]+hx[i]), 1/(hx[i]+hx[i+1]), the same in y, 1/(3 hx), 1/(3 hy), 1/ht and 1/3
  const double *rhx, *rhy, *rxx_m, *rxx_p, *ryy_m, *ryy_p, *r3x, *r3y;
  double rht, r3;
  // the quotients of mesh widths that the diffusion coefficients take per cell (static: widths
  // and fluid masks), computed once by k_flux_quotients with the divisions of the per-step
  // form: [0] D_ux, [1] D_uy, [2] D_vx, [3] D_vy, [4] DTx, [5] DTy
  const double* fq[6];
  // hx[i] hy[j] per cell (static; the product the sweeps would form, the same bits), also filled
  // by k_flux_quotients
  const double* hxy;
  // --- precision modes 1 and 2 ---
  // FP32 correction sweeps: coefficients c[0..4] of the T correction, a[0..3] of the p
  // numerator, the base-sweep values T1, H/T1, p1, Den and the defects dT, dp; e_p/e_T are the
  // corrections in three buffers used in rotation, rows of Nxe floats (Nx rounded up to a multiple
  // of 4, so that a row starts on a 16-byte boundary for TMA)
  float *c32[5], *a32[4], *T1, *hT, *q1, *den1, *dT, *dp;
  float *ep[3], *eT[3];
  int Nxe;
  int precision;  // 0 bit-exact FP64, 1 FP64 with reciprocal/FMA arithmetic, 2 = 1 + FP32 correction sweeps
  // warm start of the sweeps: 0 none (the reference), 1 linear and 2 quadratic extrapolation in
  // time of p and T on the solved cells, 3 the fitted linear predictor, 4 the fitted 3x3 stencil
  // predictor on the cells where the solution moves; p_m[k], T_m[k] hold the values of k+1
  // steps back
  int warm_start;
  double *p_m[2], *T_m[2];
  // mode 3: ring of the last kWarmRing step differences of p and T, per-CTA partial sums
  double *Dp[4], *DT[4];
  float* warm_part;
  // mode 4: ring of step differences per field (FP32), active-cell flags by step parity (bit 0 p,
  // bit 1 T; bits 2 and 3: the stencil's start in cnext for p, T), per-tile (32x8) sums of the newest training pair's terms [tile][field][term] and row
  // counts [field][tile], sums of the last kConvWin pairs [slot][field][term]
  float* cD[2][kConvRing];
  uint8_t* cact[2];
  double* cnext[2];  // the stencil's start for the next step, on the cells flagged for it
  float* cpart;
  int* crows;
  float* cgram;
  unsigned* ctmax;  // [field][tile]: largest |D| of the coming difference per 32x8 tile (FP32 bits)
};

// Neighbour indices of one cell: ij_function / ij_function_PeriodicBC (SIMPLE_TS_MPI.cpp:140-232).
struct Nb {
  int i, j, ij, i_1, i_2, i1, i_1j, i1j, ij_1, ij1, i_1j_1, i_1j1, i1j_1, i1j1, i_2j;
};

STS_HD Nb neighbours(int i, int j, int Nx, int Ny, bool periodic) {
  Nb d;
  d.i = i;
  d.j = j;
  d.ij = i + j * Nx;
  const int dn = (j > 0) ? 1 : 0, up = (j < Ny - 1) ? 1 : 0;
  if (periodic) {
    d.i_1 = (i == 0) ? Nx - 1 : i - 1;
    d.i_2 = (i == 1) ? Nx - 1 : ((i == 0) ? Nx - 2 : i - 2);
    d.i1 = (i == Nx - 1) ? 0 : i + 1;
  } else {
    d.i_1 = i - (i > 0 ? 1 : 0);
    d.i_2 = i - (i > 0 ? 1 : 0) - (i > 1 ? 1 : 0);
    d.i1 = i + (i < Nx - 1 ? 1 : 0);
  }
  d.i_1j = d.i_1 + j * Nx;
  d.i1j = d.i1 + j * Nx;
  d.ij_1 = i + (j - dn) * Nx;
  d.ij1 = i + (j + up) * Nx;
  d.i_1j_1 = d.i_1 + (j - dn) * Nx;
  d.i_1j1 = d.i_1 + (j + up) * Nx;
  d.i1j_1 = d.i1 + (j - dn) * Nx;
  d.i1j1 = d.i1 + (j + up) * Nx;
  d.i_2j = d.i_2 + j * Nx;
  return d;
}

}  // namespace sts
