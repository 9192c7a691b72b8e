// Mixed-precision variants of the SIMPLE-TS step kernels (precision modes 1 and 2).
//
// The assembly and the flux/diffusion kernels keep FP64 and the reference's formulas, but
// divide by static mesh sums through precomputed reciprocals, let the compiler fuse
// multiply-adds, and take one division per pseudo-velocity instead of two.  These are FP64
// results within a few ulps of the reference, not bit-exact ones; the bit-exact kernels are
// in sts_exact.cu.  k_sweep32 is the FP32 correction sweep described in sts_exact.cu
// (k_sweep_first_mixed).
#include <cuda_runtime.h>

#include "sts_common.cuh"
#include "sts_device.cuh"
#include "sts_kernels.h"

namespace sts {

// u/v momentum coefficients and ScT1 (SIMPLE_TS_MPI.cpp:3269-3756) with reciprocal multiplies.
__device__ __forceinline__ void assemble_fast_body(const Geo& g, unsigned long long h_sweep, int in_graph) {
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
  const double cT = ctl->cT, cPch = ctl->cPch, ht = g.ht, rht = g.rht;
  const double third = 1.0 / 3.0, two_third = 2.0 / 3.0;
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
  const bool bc_u = cls_u(cl) == CLS_BC, bc_v = cls_v(cl) == CLS_BC, bc_o = cls_o(cl) == CLS_BC;

  if (cls_u(cl)) {
    const double F_xu1 = 0.5 * (Fx[d.i_1j] + Fx[d.ij]);
    const double F_xu2 = 0.5 * (Fx[d.ij] + Fx[d.i1j]);
    const double r3a = third * g.rhx[i], r3b = third * g.rhx[d.i_1];
    const double m1 = bc_u ? B(d.i1j) : 1.0, m2 = bc_u ? B(d.i_2j) : 1.0;
    const double mN = bc_u ? B(d.ij1) : 1.0, mNW = bc_u ? B(d.i_1j1) : 1.0;
    const double mS = bc_u ? B(d.ij_1) : 1.0, mSW = bc_u ? B(d.i_1j_1) : 1.0;
    const double Scu = cT * (m1 * u[d.i1j] * sT[d.ij] * hy[j] * r3a + m2 * u[d.i_1j] * sT[d.i_1j] * hy[j] * r3b +
                             g.Gamma_yf[d.ij1] * (v[d.ij1] * mN - v[d.i_1j1] * mNW) -
                             g.Gamma_yf[d.ij] * (v[d.ij] * mS - v[d.i_1j] * mSW) -
                             sT[d.ij] * (v[d.ij1] * mN - v[d.ij] * mS) * two_third +
                             sT[d.i_1j] * (v[d.i_1j1] * mNW - v[d.i_1j] * mSW) * two_third);
    const double Spu = -(g.D_ux[d.ij] + g.D_ux[d.i1j]) * third;
    const double au1 = fmax(0.0, F_xu1) + g.D_ux[d.ij];
    const double au2 = fmax(0.0, -F_xu2) + g.D_ux[d.i1j];
    const double au3 = 0.5 * (fmax(0.0, Fy[d.i_1j]) + fmax(0.0, Fy[d.ij])) + g.D_uy[d.ij];
    const double au4 = 0.5 * (fmax(0.0, -Fy[d.i_1j1]) + fmax(0.0, -Fy[d.ij1])) + g.D_uy[d.ij1];
    const double bu3 = (rho_pr[d.i_1j] * hx[d.i_1] + rho_pr[d.ij] * hx[i]) * g.u_pr[d.ij] * hy[j] * 0.5 * rht + Scu;
    const double au0 = au1 + au2 + au3 + au4 + 0.5 * (-Fy[d.i_1j] - Fy[d.ij] + Fy[d.i_1j1] + Fy[d.ij1]) + F_xu2 -
                       F_xu1 - Spu + (rho[d.i_1j] * hx[d.i_1] + rho[d.ij] * hx[i]) * hy[j] * 0.5 * rht;
    const double rau0 = 1.0 / au0;
    const double up = (au1 * m1 * u[d.i_1j] + au2 * m2 * u[d.i1j] + au3 * u[d.ij_1] + au4 * u[d.ij1] + bu3) * rau0;
    const double dpc = cPch * hy[j] * rau0;
    const double hr = hy[j] * g.rho_u[d.ij];
    g.u_pseudo[d.ij] = up;
    g.d12[d.ij] = dpc;
    g.apx[d.ij] = dpc * hr;
    g.bpx[d.ij] = bc_u ? B(d.i_1j) * B(d.ij) * hr * up : hr * up;
  }

  if (cls_v(cl)) {
    const int jm = j - ((j - 1) >= 0 ? 1 : 0);
    const int far = d.ij_1 - ((j - 2) >= 0 ? Nx : 0);
    const double F_yv3 = 0.5 * (Fy[d.ij_1] + Fy[d.ij]);
    const double F_yv4 = 0.5 * (Fy[d.ij] + Fy[d.ij1]);
    const double r3a = third * g.rhy[j], r3b = third * g.rhy[jm];
    const double mN = bc_v ? B(d.ij1) : 1.0, mF = bc_v ? B(far) : 1.0;
    const double mE = bc_v ? B(d.i1j) : 1.0, mSE = bc_v ? B(d.i1j_1) : 1.0;
    const double mW = bc_v ? B(d.i_1j) : 1.0, mSW = bc_v ? B(d.i_1j_1) : 1.0;
    const double Scv = cT * (mN * v[d.ij1] * sT[d.ij] * hx[i] * r3a + mF * v[d.ij_1] * sT[d.ij_1] * hx[i] * r3b +
                             g.Gamma_xf[d.i1j] * (u[d.i1j] * mE - u[d.i1j_1] * mSE) -
                             g.Gamma_xf[d.ij] * (u[d.ij] * mW - u[d.ij_1] * mSW) -
                             sT[d.ij] * (u[d.i1j] * mE - u[d.ij] * mW) * two_third +
                             sT[d.ij_1] * (u[d.i1j_1] * mSE - u[d.ij_1] * mSW) * two_third) -
                       g.c_Fr_v * (rho[d.ij_1] * hx[i] * 0.5 * hy[jm] + rho[d.ij] * hx[i] * 0.5 * hy[j]);
    const double Spv = -(g.D_vy[d.ij] + g.D_vy[d.ij1]) * third;
    const double av1 = 0.5 * (fmax(0.0, Fx[d.ij]) + fmax(0.0, Fx[d.ij_1])) + g.D_vx[d.ij];
    const double av2 = 0.5 * (fmax(0.0, -Fx[d.i1j]) + fmax(0.0, -Fx[d.i1j_1])) + g.D_vx[d.i1j];
    const double av3 = fmax(0.0, F_yv3) + g.D_vy[d.ij];
    const double av4 = fmax(0.0, -F_yv4) + g.D_vy[d.ij1];
    const double bv3 = (rho_pr[d.ij_1] * hy[j - 1] + rho_pr[d.ij] * hy[j]) * g.v_pr[d.ij] * hx[i] * 0.5 * rht + Scv;
    const double av0 = av1 + av2 + av3 + av4 + 0.5 * (Fx[d.i1j] - Fx[d.ij] + Fx[d.i1j_1] - Fx[d.ij_1]) + F_yv4 -
                       F_yv3 - Spv + (rho[d.ij_1] * hy[j - 1] + rho[d.ij] * hy[j]) * hx[i] * 0.5 * rht;
    const double rav0 = 1.0 / av0;
    const double vp = (av1 * v[d.i_1j] + av2 * v[d.i1j] + av3 * mF * v[d.ij_1] + av4 * mN * v[d.ij1] + bv3) * rav0;
    const double dpc = cPch * hx[i] * rav0;
    const double hr = hx[i] * g.rho_v[d.ij];
    g.v_pseudo[d.ij] = vp;
    g.d34[d.ij] = dpc;
    g.apy[d.ij] = dpc * hr;
    g.bpy[d.ij] = bc_v ? B(d.ij - Nx) * B(d.ij) * hr * vp : hr * vp;
  }

  if (cls_o(cl)) {
    double dudx, dvdy, s0, s1, s2, s3;
    if (bc_o) {
      dudx = (B(d.i1j) * u[d.i1j] - B(d.i_1j) * u[d.ij]) * g.rhx[i];
      dvdy = (B(d.ij1) * v[d.ij1] - B(d.ij_1) * v[d.ij]) * g.rhy[j];
      // (mask * h_low + h) picks h alone or the two-cell sum
      const double ys = (BB(d.i_1j_1) && BB(d.ij_1)) ? g.ryy_m[j] : g.rhy[j];
      const double xs = (BB(d.i_1j_1) && BB(d.i_1j)) ? g.rxx_m[i] : g.rhx[i];
      const double ys1 = (BB(d.ij_1) && BB(d.i1j_1)) ? g.ryy_m[j] : g.rhy[j];
      const double xs1 = (BB(d.i1j_1) && BB(d.i1j)) ? g.rxx_p[i] : g.rhx[i];
      const double yn2 = (BB(d.i_1j1) && BB(d.ij1)) ? g.ryy_p[j] : g.rhy[j];
      const double xs2 = (BB(d.i_1j) && BB(d.i_1j1)) ? g.rxx_m[i] : g.rhx[i];
      const double yn3 = (BB(d.ij1) && BB(d.i1j1)) ? g.ryy_p[j] : g.rhy[j];
      const double xs3 = (BB(d.i1j) && BB(d.i1j1)) ? g.rxx_p[i] : g.rhx[i];
      s0 = (u[d.ij] - u[d.ij_1]) * ys + (v[d.ij] - v[d.i_1j]) * xs;
      s1 = (u[d.i1j] - u[d.i1j_1]) * ys1 + (v[d.i1j] - v[d.ij]) * xs1;
      s2 = (u[d.ij1] - u[d.ij]) * yn2 + (v[d.ij1] - v[d.i_1j1]) * xs2;
      s3 = (u[d.i1j1] - u[d.i1j]) * yn3 + (v[d.i1j1] - v[d.ij1]) * xs3;
    } else {
      dudx = (u[d.i1j] - u[d.ij]) * g.rhx[i];
      dvdy = (v[d.ij1] - v[d.ij]) * g.rhy[j];
      s0 = (u[d.ij] - u[d.ij_1]) * g.ryy_m[j] + (v[d.ij] - v[d.i_1j]) * g.rxx_m[i];
      s1 = (u[d.i1j] - u[d.i1j_1]) * g.ryy_m[j] + (v[d.i1j] - v[d.ij]) * g.rxx_p[i];
      s2 = (u[d.ij1] - u[d.ij]) * g.ryy_p[j] + (v[d.ij1] - v[d.i_1j1]) * g.rxx_m[i];
      s3 = (u[d.i1j1] - u[d.i1j]) * g.ryy_p[j] + (v[d.i1j1] - v[d.ij1]) * g.rxx_p[i];
    }
    const double dd = dudx + dvdy;
    g.ScT1[d.ij] = ht * sT[d.ij] * g.cT2 * hx[i] * hy[j] *
                       (2.0 * (dudx * dudx + dvdy * dvdy) + s0 * s0 + s1 * s1 + s2 * s2 + s3 * s3 - dd * dd * two_third) +
                   g.p_pr[d.ij] * hx[i] * hy[j];
  }
}
__global__ void k_assemble_fast(Geo g, unsigned long long h_sweep, int in_graph) { assemble_fast_body(g, h_sweep, in_graph); }
__global__ void kb_assemble_fast(const Geo* gs, unsigned long long h_sweep, int in_graph) {
  __shared__ Geo sg;
  if (!stage_geo(sg, gs)) return;
  assemble_fast_body(sg, h_sweep, in_graph);
}

// Fluxes and diffusion coefficients (SIMPLE_TS_MPI.cpp:10440-10618) with reciprocal multiplies.
__device__ __forceinline__ void flux_diff_fast_body(const Geo& g, unsigned tail) {
  Cell c = cell(g);
  if (c.ok) {
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
    auto LiY = [&](double f1, double f2) { return (f1 * hy[j] + f2 * hy[jm]) * ry; };
    auto LiX = [&](double f1, double f2) { return (f1 * hx[i] + f2 * hx[d.i_1]) * rx; };
    double Gy = g.Gamma_yf[d.ij], Gx = g.Gamma_xf[d.ij];
    if (b_ws && b_s && b_w && b_p) {
      Gy = 0.5 * (LiY(sT[d.i_1j_1], sT[d.i_1j]) + LiY(sT[d.ij_1], sT[d.ij]));
      Gx = 0.5 * (LiX(sT[d.i_1j_1], sT[d.ij_1]) + LiX(sT[d.i_1j], sT[d.ij]));
    } else if (b_ws || b_s || b_w || b_p) {
      Gy = 0.5 * ((b_ws && b_w) ? LiY(sT[d.i_1j_1], sT[d.i_1j]) : 0.0) + 0.5 * ((b_ws != b_w) ? sqrt(Tw_v[d.i_1j]) : 0.0) +
           0.5 * ((b_s && b_p) ? LiY(sT[d.ij_1], sT[d.ij]) : 0.0) + 0.5 * ((b_s != b_p) ? sqrt(Tw_v[d.ij]) : 0.0) +
           0.5 * (((!(b_ws && b_w)) || (!(b_s && b_p))) ? LiY(sqrt(Tw_u[d.ij_1]), sqrt(Tw_u[d.ij])) : 0.0);
      Gx = 0.5 * ((b_ws && b_s) ? LiX(sT[d.i_1j_1], sT[d.ij_1]) : 0.0) + 0.5 * ((b_ws != b_s) ? sqrt(Tw_u[d.ij_1]) : 0.0) +
           0.5 * ((b_w && b_p) ? LiX(sT[d.i_1j], sT[d.ij]) : 0.0) + 0.5 * ((b_w != b_p) ? sqrt(Tw_u[d.ij]) : 0.0) +
           0.5 * (((!(b_ws && b_s)) || (!(b_w && b_p))) ? LiX(sqrt(Tw_v[d.i_1j]), sqrt(Tw_v[d.ij])) : 0.0);
    }
    g.Gamma_yf[d.ij] = Gy;
    g.Gamma_xf[d.ij] = Gx;
    g.D_ux[d.ij] = cT * sT[d.i_1j] * hy[j] * g.rhx[d.i_1];
    g.D_vy[d.ij] = cT * sT[d.ij_1] * hx[i] * g.rhy[jm];
    const bool pw = b_p && b_w, sws = b_s && b_ws, ps = b_p && b_s, wws = b_w && b_ws;
    g.D_uy[d.ij] = (pw || sws) ? cT * Gy * (hx[i] + hx[d.i_1]) * ((pw && sws) ? ry : (pw ? g.rhy[j] : g.rhy[jm])) : 0.0;
    g.D_vx[d.ij] = (ps || wws) ? cT * Gx * (hy[j] + hy[jm]) * ((ps && wws) ? rx : (ps ? g.rhx[i] : g.rhx[d.i_1])) : 0.0;
    if (b_p || b_w) {
      const double rs = pw ? rx : (b_p ? g.rhx[i] : g.rhx[d.i_1]);
      const double face = pw ? (hx[d.i_1] + hx[i]) * sT[d.i_1j] * sT[d.ij] / (hx[d.i_1] * sT[d.ij] + hx[i] * sT[d.i_1j])
                             : sqrt(Tw_u[d.ij]);
      g.DTx[d.ij] = cT1 * hy[j] * 2.0 * rs * face;
    } else {
      g.DTx[d.ij] = 0.0;
    }
    if (b_p || b_s) {
      const double rs = ps ? ry : (b_p ? g.rhy[j] : g.rhy[jm]);
      const double face = ps ? (hy[jm] + hy[j]) * sT[d.ij_1] * sT[d.ij] / (hy[jm] * sT[d.ij] + hy[j] * sT[d.ij_1])
                             : sqrt(Tw_v[d.ij]);
      g.DTy[d.ij] = cT1 * hx[i] * 2.0 * rs * face;
    } else {
      g.DTy[d.ij] = 0.0;
    }
  }
  if (tail && blockIdx.x == 0 && blockIdx.y == 0) {
    const int tid = threadIdx.x + threadIdx.y * blockDim.x, nt = blockDim.x * blockDim.y;
    const unsigned cur = g.ctl->cur;
    if (tail & PH_TEMP) phase_temp(g, g.T[cur], tid, nt);
    __syncthreads();
    if (tail & PH_PRES) phase_pres(g, g.p[cur], tid, nt);
  }
}
__global__ void k_flux_diff_fast(Geo g, unsigned tail) { flux_diff_fast_body(g, tail); }
__global__ void kb_flux_diff_fast(const Geo* gs, unsigned tail) {
  __shared__ Geo sg;
  if (!stage_geo(sg, gs)) return;
  flux_diff_fast_body(sg, tail);
}

// ---------------------------------------------------------------------------
// p-T sweeps with reciprocal multiplies (precision modes 1 and 2): the reference's update
// (SIMPLE_TS_MPI.cpp:3786-4131) with 1/den_T stored once per outer iteration and the pressure
// denominator sa + H/T_new folded into one division, p_new = N T_new / (sa T_new + H).
// The first sweep stores the loop invariants of a cell in inv[0..7]: the four neighbour weights
// (a wall neighbour's weight already multiplied by the wall temperature), divu, 1/den_T, the
// p_pr/T_pr term and ht * (sum of the p coefficients).  Returns false for unsolved cells, which
// copy through.
// ---------------------------------------------------------------------------
template <bool FIRST>
__device__ __forceinline__ bool sweep_cell_fast(const Geo& g, const Cell& c, const double* __restrict__ P,
                                                const double* __restrict__ TT, double* __restrict__ pn,
                                                double* __restrict__ Tn, double& Tnew, double& pnew, double& sa) {
  const int ij = c.ij;
  const uint8_t cl = g.cls[ij];
  const int co = cls_o(cl);
  if (!co) {
    pnew = P[ij];
    Tnew = TT[ij];
    pn[ij] = pnew;
    Tn[ij] = Tnew;
    return false;
  }
  const int i = c.i, j = c.j;
  const Nb d = neighbours(i, j, g.Nx, g.Ny, g.bits & F_PERIODIC);
  const double* __restrict__ apx = g.apx;
  const double* __restrict__ apy = g.apy;
  const double ht = g.ht, H = g.hx[i] * g.hy[j];
  auto fl = [&](int k) { return cls_fluid(g.cls[k]); };
  double w1, w2, w3, w4, divu, rden, pc;
  if (FIRST) {
    const double* __restrict__ Fx = g.Fx;
    const double* __restrict__ Fy = g.Fy;
    const double aT1 = fmax(0.0, Fx[d.ij]) + g.DTx[d.ij];
    const double aT2 = fmax(0.0, -Fx[d.i1j]) + g.DTx[d.i1j];
    const double aT3 = fmax(0.0, Fy[d.ij]) + g.DTy[d.ij];
    const double aT4 = fmax(0.0, -Fy[d.ij1]) + g.DTy[d.ij1];
    divu = (g.u[d.i1j] - g.u[d.ij]) * g.hy[j] + (g.v[d.ij1] - g.v[d.ij]) * g.hx[i];
    rden = 1.0 / (ht * (aT1 + aT2 + aT3 + aT4 + Fx[d.i1j] - Fx[d.ij] + Fy[d.ij1] - Fy[d.ij]) + H * g.rho[ij]);
    w1 = aT1; w2 = aT2; w3 = aT3; w4 = aT4;
    if (co == CLS_BC) {
      if (!fl(d.i_1j)) w1 = aT1 * g.Tw_u[ij];
      if (!fl(d.i1j)) w2 = aT2 * g.Tw_u[d.i1j];
      if (!fl(d.ij_1)) w3 = aT3 * g.Tw_v[ij];
      if (!fl(d.ij1)) w4 = aT4 * g.Tw_v[d.ij1];
    }
    pc = g.p_pr[ij] * H / g.T_pr[ij];
    sa = ht * (apx[ij] + apx[d.i1j] + apy[ij] + apy[d.ij1]);
    g.inv[0][ij] = w1; g.inv[1][ij] = w2; g.inv[2][ij] = w3; g.inv[3][ij] = w4;
    g.inv[4][ij] = divu; g.inv[5][ij] = rden; g.inv[6][ij] = pc; g.inv[7][ij] = sa;
  } else {
    w1 = g.inv[0][ij]; w2 = g.inv[1][ij]; w3 = g.inv[2][ij]; w4 = g.inv[3][ij];
    divu = g.inv[4][ij]; rden = g.inv[5][ij]; pc = g.inv[6][ij]; sa = g.inv[7][ij];
  }
  double t1, t2, t3, t4;
  if (co == CLS_BC) {
    t1 = fl(d.i_1j) ? w1 * TT[d.i_1j] : w1;
    t2 = fl(d.i1j) ? w2 * TT[d.i1j] : w2;
    t3 = fl(d.ij_1) ? w3 * TT[d.ij_1] : w3;
    t4 = fl(d.ij1) ? w4 * TT[d.ij1] : w4;
  } else {
    t1 = w1 * TT[d.i_1j];
    t2 = w2 * TT[d.i1j];
    t3 = w3 * TT[d.ij_1];
    t4 = w4 * TT[d.ij1];
  }
  Tnew = (ht * (t1 + t2 + t3 + t4 + (1.0 - g.gamma1) * P[ij] * divu) + g.ScT1[ij]) * rden;
  double num = apx[ij] * P[d.i_1j] + apx[d.i1j] * P[d.i1j] + apy[ij] * P[d.ij_1] + apy[d.ij1] * P[d.ij1] +
               g.bpx[ij] - g.bpx[d.i1j] + g.bpy[ij] - g.bpy[d.ij1];
  if (co == CLS_BC) {
    if ((g.bits & F_GIVEN_U_XB) && i == g.Nx_o0) num += g.Fx[ij];
    if ((g.bits & F_GIVEN_U_XE) && i == g.Nx_o1 - 1) num -= g.Fx[d.i1j];
  }
  pnew = (ht * num + pc) * Tnew / (sa * Tnew + H);
  Tn[ij] = Tnew;
  pn[ij] = pnew;
  return true;
}

// The sweep loop of mode 1 (see k_pt_loop).
struct FastOps {
  static __device__ __forceinline__ void pass(const Geo& g, const Cell& c, const LoopCase& s, double& rp, double& rT) {
    const double* P = g.p[s.cur];
    const double* TT = g.T[s.cur];
    double Tnew, pnew, sa;
    const bool solved = (s.phase == PS_FIRST)
                            ? sweep_cell_fast<true>(g, c, P, TT, g.p[s.cur ^ 1], g.T[s.cur ^ 1], Tnew, pnew, sa)
                            : sweep_cell_fast<false>(g, c, P, TT, g.p[s.cur ^ 1], g.T[s.cur ^ 1], Tnew, pnew, sa);
    if (!solved) return;
    rp = fabs(pnew - P[c.ij]);
    rT = fabs(Tnew - TT[c.ij]);
  }
  static __device__ __forceinline__ void pass32(const Geo&, const Cell&, const LoopCase&, float&, float&) {}
  static __device__ __forceinline__ void advance(const Geo& g, bool lead, LoopCase& s, double res_p, double res_T) {
    advance_fp64(g, lead, s, res_p, res_T);
  }
};

__global__ void __launch_bounds__(256, 4) k_pt_loop_fast(Geo g, int ntiles, LoopCtl* lc) {
  pt_loop_rounds<FastOps, true>(g, nullptr, nullptr, nullptr, 1, ntiles, lc);
}
__global__ void __launch_bounds__(256, 4) kb_pt_loop_fast(const Geo* gs, const int* tile_case, const int* tile_first,
                                                          int ncases, int ntiles, LoopCtl* lc) {
  pt_loop_rounds<FastOps, false>(gs[0], gs, tile_case, tile_first, ncases, ntiles, lc);
}

// ---------------------------------------------------------------------------
// Mixed-precision sweep loop (precision mode 2, tolerance-terminated loops).  Within one outer
// iteration the Jacobi map G is affine in the neighbour temperatures and pressures except for
// the 1/T_new term of the pressure denominator.  Writing the iterate as x = b + e (b: FP64 base,
// e: FP32 correction), an FP64 sweep from b gives x1 = G(b) and the defect d = x1 - b, and every
// later sweep is e' = d + (G(b + e) - G(b)), evaluated in FP32 from the correction alone:
//   dT   = sum_k c_k e_T,k + c_5 e_p,P                (c_k = ht w_k / den_T, c_5 = ht (1-gamma) divu / den_T)
//   e_T' = d_T + dT
//   q    = (H/T1) dT / (T1 + dT)                      (H = hx hy, T1 = T of x1)
//   e_p' = d_p + (sum_k a_k e_p,k + p1 q) / (Den1 - q)  (a_k = ht apx/apy, p1 = p of x1, Den1 = sa + H/T1)
// which is the exact difference of two FP64 updates, so FP32 only rounds correction-sized numbers.
// When the FP32 sweeps meet the reference's stop rule at sweep n, the iterate of sweep n-1 is
// formed in FP64 (b + e) and sweep n is recomputed in FP64; its residual decides.  If it misses
// the tolerance, the FP64 pair (x_{n-1}, x_n) becomes the new base and defect and the FP32 sweeps
// go on from there with corrections of residual size.  A cell whose FP32 update is below the
// resolution of its correction (kFloor32 |e|) counts as converged for the FP32 stop test only.
// ---------------------------------------------------------------------------
constexpr float kFloor32 = 8.0f / 16777216.0f;  // 8 units in the last place of an FP32 number

// Base values of the FP32 corrections taken from an FP64 sweep x -> x1 of a solved cell.
__device__ __forceinline__ void set_base(const Geo& g, const Cell& c, double T0, double p0, double T1, double p1,
                                         double sa) {
  const int ij = c.ij;
  const double hT = g.hx[c.i] * g.hy[c.j] / T1;
  g.T1[ij] = (float)T1;
  g.hT[ij] = (float)hT;
  g.q1[ij] = (float)p1;
  g.den1[ij] = (float)(sa + hT);
  const float dT = (float)(T1 - T0), dp = (float)(p1 - p0);
  g.dT[ij] = dT;
  g.dp[ij] = dp;
  g.eT[0][ij] = dT;
  g.ep[0][ij] = dp;
}

// One FP32 correction sweep of a solved cell: e (buffer src) -> e' (buffer src ^ 1).
__device__ __forceinline__ void sweep32_cell(const Geo& g, const Cell& c, unsigned src, float& rp, float& rT) {
  const int ij = c.ij;
  const Nb d = neighbours(c.i, c.j, g.Nx, g.Ny, g.bits & F_PERIODIC);
  const float* __restrict__ ep = g.ep[src];
  const float* __restrict__ eT = g.eT[src];
  const float dT = g.c32[0][ij] * eT[d.i_1j] + g.c32[1][ij] * eT[d.i1j] + g.c32[2][ij] * eT[d.ij_1] +
                   g.c32[3][ij] * eT[d.ij1] + g.c32[4][ij] * ep[ij];
  const float eTnew = g.dT[ij] + dT;
  const float q = g.hT[ij] * dT / (g.T1[ij] + dT);
  const float num = g.a32[0][ij] * ep[d.i_1j] + g.a32[1][ij] * ep[d.i1j] + g.a32[2][ij] * ep[d.ij_1] +
                    g.a32[3][ij] * ep[d.ij1];
  const float epnew = g.dp[ij] + (num + g.q1[ij] * q) / (g.den1[ij] - q);
  g.eT[src ^ 1][ij] = eTnew;
  g.ep[src ^ 1][ij] = epnew;
  const float aT = fabsf(eTnew - eT[ij]), ap = fabsf(epnew - ep[ij]);
  rT = aT <= kFloor32 * fabsf(eTnew) ? 0.0f : aT;
  rp = ap <= kFloor32 * fabsf(epnew) ? 0.0f : ap;
}

struct MixedOps {
  static __device__ __forceinline__ void pass(const Geo& g, const Cell& c, const LoopCase& s, double& rp, double& rT) {
    const int ij = c.ij;
    const unsigned base = s.base;
    switch (s.phase) {
      case PS_FIRST: {  // FP64 sweep from b into base ^ 1, with the FP32 coefficients of this outer iteration
        const double* P = g.p[base];
        const double* TT = g.T[base];
        double Tnew, pnew, sa;
        if (!sweep_cell_fast<true>(g, c, P, TT, g.p[base ^ 1], g.T[base ^ 1], Tnew, pnew, sa)) {
          g.dT[ij] = 0.0f; g.dp[ij] = 0.0f;
          g.eT[0][ij] = 0.0f; g.ep[0][ij] = 0.0f; g.eT[1][ij] = 0.0f; g.ep[1][ij] = 0.0f;
          return;
        }
        rp = fabs(pnew - P[ij]);
        rT = fabs(Tnew - TT[ij]);
        const Nb d = neighbours(c.i, c.j, g.Nx, g.Ny, g.bits & F_PERIODIC);
        const double ht = g.ht, r = ht * g.inv[5][ij];
        const int nb[4] = {d.i_1j, d.i1j, d.ij_1, d.ij1};
        for (int k = 0; k < 4; k++)  // a wall neighbour's term is a constant and sits in the defect
          g.c32[k][ij] = (cls_o(g.cls[ij]) == CLS_NCH || cls_fluid(g.cls[nb[k]])) ? (float)(r * g.inv[k][ij]) : 0.0f;
        g.c32[4][ij] = (float)(r * (1.0 - g.gamma1) * g.inv[4][ij]);
        g.a32[0][ij] = (float)(ht * g.apx[ij]);
        g.a32[1][ij] = (float)(ht * g.apx[d.i1j]);
        g.a32[2][ij] = (float)(ht * g.apy[ij]);
        g.a32[3][ij] = (float)(ht * g.apy[d.ij1]);
        set_base(g, c, TT[ij], P[ij], Tnew, pnew, sa);
        return;
      }
      case PS_MATERIALIZE:  // the iterate of the sweep before the last FP32 one, in FP64
        g.p[base ^ 1][ij] = g.p[base][ij] + (double)g.ep[s.ec ^ 1][ij];
        g.T[base ^ 1][ij] = g.T[base][ij] + (double)g.eT[s.ec ^ 1][ij];
        return;
      case PS_CONFIRM: {  // that sweep again in FP64 into the base buffer; exports for a re-basing
        const double* P = g.p[base ^ 1];
        const double* TT = g.T[base ^ 1];
        double Tnew, pnew, sa;
        if (!sweep_cell_fast<false>(g, c, P, TT, g.p[base], g.T[base], Tnew, pnew, sa)) return;
        rp = fabs(pnew - P[ij]);
        rT = fabs(Tnew - TT[ij]);
        set_base(g, c, TT[ij], P[ij], Tnew, pnew, sa);
        return;
      }
      default:
        return;
    }
  }
  static __device__ __forceinline__ void pass32(const Geo& g, const Cell& c, const LoopCase& s, float& rp, float& rT) {
    if (cls_o(g.cls[c.ij])) sweep32_cell(g, c, s.ec, rp, rT);
  }
  static __device__ __forceinline__ void advance(const Geo& g, bool lead, LoopCase& s, double res_p, double res_T) {
    Ctl* ctl = g.ctl;
    switch (s.phase) {
      case PS_FIRST:
        s.n = 1;
        if (lead) record_residual(ctl, s.n, s.I, res_p, res_T);
        s.cur = s.base ^ 1;
        s.ec = 0;
        s.phase = (s.n >= (unsigned)g.N_I_p_c) ? PS_DONE : PS_SWEEP32;  // a single sweep: x1 is the result
        break;
      case PS_SWEEP32:
        s.n++;
        s.ec ^= 1;
        if (lead) ctl->sweeps32++;
        s.phase = ((s.n < (unsigned)g.N_I_p_c) && ((g.MaxError_p_c < res_p) || (g.MaxError_T < res_T)))
                      ? PS_SWEEP32 : PS_MATERIALIZE;
        break;
      case PS_MATERIALIZE:
        s.n--;
        s.phase = PS_CONFIRM;
        break;
      case PS_CONFIRM:
        s.n++;
        if (lead) record_residual(ctl, s.n, s.I, res_p, res_T);
        s.cur = s.base;
        if (!sweep_continues(g, s.n, res_p, res_T)) {
          s.phase = PS_DONE;
        } else {  // re-base: x_{n-1} (buffer base ^ 1) and the defect x_n - x_{n-1} written by the pass
          s.base ^= 1;
          s.cur = s.base ^ 1;
          s.ec = 0;
          if (lead) ctl->rebases++;
          s.phase = PS_SWEEP32;
        }
        break;
      default:
        break;
    }
  }
};

__global__ void __launch_bounds__(256, 4) k_pt_loop_mixed(Geo g, int ntiles, LoopCtl* lc) {
  pt_loop_rounds<MixedOps, true>(g, nullptr, nullptr, nullptr, 1, ntiles, lc);
}
__global__ void __launch_bounds__(256, 4) kb_pt_loop_mixed(const Geo* gs, const int* tile_case, const int* tile_first,
                                                          int ncases, int ntiles, LoopCtl* lc) {
  pt_loop_rounds<MixedOps, false>(gs[0], gs, tile_case, tile_first, ncases, ntiles, lc);
}

}  // namespace sts
