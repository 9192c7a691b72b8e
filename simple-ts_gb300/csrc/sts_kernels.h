// Kernel declarations of the GB300 SIMPLE-TS step (FP64, bit-exact variant in sts_exact.cu).
#pragma once
#include <cuda_runtime.h>

#include "sts_common.cuh"

namespace sts {

// Phases of k_boundary, run in this order when selected.
enum : unsigned {
  PH_CONTROL = 1u << 0,      // loop control after the velocity correction (SIMPLE_TS_MPI.cpp:4406-4450)
  PH_SLIP_U = 1u << 1,       // SIMPLE_TS_MPI.cpp:7098-7213
  PH_SLIP_V = 1u << 2,       // SIMPLE_TS_MPI.cpp:7216-7331
  PH_VEL = 1u << 3,          // SIMPLE_TS_MPI.cpp:6790-7096
  PH_PBEGIN = 1u << 4,       // SIMPLE_TS_MPI.cpp:7430-7647
  PH_TJUMP = 1u << 5,        // SIMPLE_TS_MPI.cpp:7744-8045
  PH_TJUMP_WRITE = 1u << 6,  // SIMPLE_TS_MPI.cpp:8048-8099 (output-time overwrite of wall temperatures)
  PH_TEMP = 1u << 7,         // SIMPLE_TS_MPI.cpp:7650-7741
  PH_PRES = 1u << 8,         // SIMPLE_TS_MPI.cpp:7335-7428
  PH_PINIT = 1u << 9,        // SIMPLE_TS_MPI.cpp:2942-2979 (set-up only)
  PH_ALL_STEP = PH_CONTROL | PH_SLIP_U | PH_SLIP_V | PH_VEL | PH_PBEGIN | PH_TJUMP | PH_TEMP | PH_PRES,
};

// Per-case kernels.  Each k_X takes the case's Geo by value; its batched form kb_X takes the
// device array of the batch's Geos and runs case blockIdx.z (cases outside the step return).
__global__ void k_step_begin(Geo g, int counters, unsigned long long h_outer, int in_graph);
__global__ void k_step_begin_in(Geo g, unsigned long long h_outer, int in_graph, const double* u_in,
                                const double* v_in, const double* p_in, const double* T_in);
__global__ void k_apply_bodies(Geo g);
__global__ void k_assemble(Geo g, unsigned long long h_sweep, int in_graph);
__global__ void k_sweep_first(Geo g, unsigned long long h_sweep, int in_graph);
__global__ void k_sweep(Geo g, unsigned long long h_sweep, int in_graph);
__global__ void k_correct(Geo g);
__global__ void k_face_rho(Geo g);
__global__ void k_flux_diff(Geo g, unsigned tail);
__global__ void k_flux_quotients(Geo g);
__global__ void k_bnd_fused(Geo g, unsigned long long h_outer, int in_graph, int jump_beside, unsigned tail);
__global__ void k_sqrt_rho(Geo g, int do_rho);
__global__ void k_boundary(Geo g, unsigned phases, unsigned long long h_outer, int in_graph);
__global__ void k_step_end(Geo g, unsigned long long h_step, int in_graph);
__global__ void k_warm_diff(Geo g);
__global__ void k_warm_fit(Geo g);
__global__ void k_warm_apply(Geo g);
__global__ void kb_warm_diff(const Geo* gs);
__global__ void kb_warm_fit(const Geo* gs);
__global__ void kb_warm_apply(const Geo* gs);
// convolutional warm start (warm_start 4), sts_learn.cu (k_step_begin stores the differences and
// takes the prepared start): at the end of a step k_conv_gram -> {k_conv_solve, k_conv_next} ->
// k_conv_predict; k_conv_gram, k_conv_next and k_conv_predict on the 32x8 cell tiles,
// k_conv_solve with one CTA of kConvSolveThreads per field
constexpr int kConvSolveThreads = 1024;
__global__ void k_conv_gram(Geo g);
__global__ void k_conv_solve(Geo g);
__global__ void k_conv_next(Geo g);
__global__ void k_conv_predict(Geo g);
__global__ void kb_conv_gram(const Geo* gs);
__global__ void kb_conv_solve(const Geo* gs);
__global__ void kb_conv_next(const Geo* gs);
__global__ void kb_conv_predict(const Geo* gs);
__global__ void kb_step_begin(const Geo* gs);
__global__ void kb_set_steps(const Geo* gs, int ncases, unsigned n);
__global__ void kb_continue(const Geo* gs, int ncases, unsigned long long h_step, unsigned* flag);
__global__ void kb_assemble(const Geo* gs, unsigned long long h_sweep, int in_graph);
__global__ void kb_correct(const Geo* gs);
__global__ void kb_face_rho(const Geo* gs);
__global__ void kb_flux_diff(const Geo* gs, unsigned tail);
__global__ void kb_bnd_fused(const Geo* gs, unsigned long long h_outer, int in_graph, int jump_beside);
__global__ void kb_step_end(const Geo* gs, unsigned long long h_step, int in_graph);
// The whole sweep loop of an outer iteration in one cooperative launch (grid <= resident CTAs):
// k_ for one case (ntiles 32x8 tiles), kb_ for ncases cases, where tile_case[t] is the case of
// global tile t and tile_first[c] the first tile of case c.
__global__ void k_pt_loop(Geo g, int ntiles, LoopCtl* lc);
__global__ void kb_pt_loop(const Geo* gs, const int* tile_case, const int* tile_first, int ncases, int ntiles,
                           LoopCtl* lc);
// diagnostics of the time loop: drag-coefficient and mass-flux sums, the fluxes alone, the
// continuity residuals
__global__ void k_drag(Geo g, const int* cells, const int* first, int nlist, double* out);
__global__ void k_fluxes(Geo g);
__global__ void k_continuity(Geo g, double* st, double* ce);
// self-check of the correctly rounded division by a reciprocal against IEEE division
__global__ void k_check_division(unsigned long long n, unsigned long long seed, unsigned long long* bad);
__global__ void k_barrier_probe(LoopCtl* lc, int skip, unsigned spin_limit, int rounds);
constexpr int kConsQ = 5, kConsChunk = 64;
__global__ void k_cons_partial(Geo g, unsigned cur, double* part, int nch);
__global__ void k_cons_final(int Ny, int nch, const double* part, double* rows, double* out);
__global__ void k_fp64_rate(int op, int iters, double c_mul, double c_add, double* out);
__global__ void k_move4(const double* a0, const double* a1, const double* a2, const double* a3, double* b0,
                        double* b1, double* b2, double* b3, int n);
__global__ void k_move4_state_out(Geo g, double* b0, double* b1, double* b2, double* b3);
// precision modes 1 and 2
__global__ void k_assemble_fast(Geo g, unsigned long long h_sweep, int in_graph);
__global__ void k_flux_diff_fast(Geo g, unsigned tail);
__global__ void kb_assemble_fast(const Geo* gs, unsigned long long h_sweep, int in_graph);
__global__ void kb_flux_diff_fast(const Geo* gs, unsigned tail);
__global__ void k_pt_loop_fast(Geo g, int ntiles, LoopCtl* lc);
__global__ void k_pt_loop_mixed(Geo g, int ntiles, LoopCtl* lc);
__global__ void kb_pt_loop_fast(const Geo* gs, const int* tile_case, const int* tile_first, int ncases, int ntiles,
                                LoopCtl* lc);
__global__ void kb_pt_loop_mixed(const Geo* gs, const int* tile_case, const int* tile_first, int ncases, int ntiles,
                                 LoopCtl* lc);
// precision mode 3: double-float arithmetic in the FP64-bound kernels
__global__ void k_check_df(unsigned long long n, unsigned long long seed, unsigned long long* err);
__global__ void k_assemble_df(Geo g, unsigned long long h_sweep, int in_graph);
__global__ void kb_assemble_df(const Geo* gs, unsigned long long h_sweep, int in_graph);
__global__ void k_flux_diff_df(Geo g, unsigned tail);
__global__ void kb_flux_diff_df(const Geo* gs, unsigned tail);
__global__ void k_correct_df(Geo g);
__global__ void kb_correct_df(const Geo* gs);
__global__ void k_pt_loop_mixed_df(Geo g, int ntiles, LoopCtl* lc);
// the FP32-correction loops with two FP32 sweeps per tile load (temporal blocking, TMA-staged tiles)
__global__ void k_pt_loop_mixed_tb(Geo g, int ntiles, LoopCtl* lc, const __grid_constant__ EMaps maps);
__global__ void k_pt_loop_mixed_df_tb(Geo g, int ntiles, LoopCtl* lc, const __grid_constant__ EMaps maps);
__global__ void kb_pt_loop_mixed_df(const Geo* gs, const int* tile_case, const int* tile_first, int ncases, int ntiles,
                                    LoopCtl* lc);

}  // namespace sts
