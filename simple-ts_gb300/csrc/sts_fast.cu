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
__global__ void k_assemble_fast(Geo g, unsigned long long h_sweep, int in_graph) {
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

// Fluxes and diffusion coefficients (SIMPLE_TS_MPI.cpp:10440-10618) with reciprocal multiplies.
__global__ void k_flux_diff_fast(Geo g, unsigned tail) {
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

// FP32 correction sweep (see k_sweep_first_mixed): e' = d + (G(b + e) - G(b)).
__global__ void k_sweep32(Geo g, unsigned long long h_sweep, int in_graph) {
  Ctl* ctl = g.ctl;
  if (ctl->pt_done || ctl->stop32) {
    if (in_graph && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0)
      cudaGraphSetConditional((cudaGraphConditionalHandle)h_sweep, 0);
    return;
  }
  Cell c = cell(g);
  const unsigned src = ctl->ecur;
  const float* __restrict__ ep = g.ep[src];
  const float* __restrict__ eT = g.eT[src];
  float* __restrict__ epn = g.ep[src ^ 1];
  float* __restrict__ eTn = g.eT[src ^ 1];
  float rp = 0.f, rT = 0.f;
  if (c.ok && cls_o(g.cls[c.ij])) {
    const int ij = c.ij;
    const Nb d = neighbours(c.i, c.j, g.Nx, g.Ny, g.bits & F_PERIODIC);
    const float dT = g.c32[0][ij] * eT[d.i_1j] + g.c32[1][ij] * eT[d.i1j] + g.c32[2][ij] * eT[d.ij_1] +
                     g.c32[3][ij] * eT[d.ij1] + g.c32[4][ij] * ep[ij];
    const float eTnew = g.dT[ij] + dT;
    const float T1 = g.T1[ij];
    const float H = (float)(g.hx[c.i] * g.hy[c.j]);
    const float gg = H * dT / (T1 * (T1 + dT));
    const float num = g.a32[0][ij] * ep[d.i_1j] + g.a32[1][ij] * ep[d.i1j] + g.a32[2][ij] * ep[d.ij_1] +
                      g.a32[3][ij] * ep[d.ij1];
    const float epnew = g.dp[ij] + (num + g.q1[ij] * gg) / (g.den1[ij] - gg);
    eTn[ij] = eTnew;
    epn[ij] = epnew;
    rT = fabsf(eTnew - eT[ij]);
    rp = fabsf(epnew - ep[ij]);
  }
  block_max2((double)rp, (double)rT, &ctl->res_bits_p, &ctl->res_bits_T, &ctl->status);
  if (last_block(&ctl->block_count)) {
    const unsigned I = ctl->Iter < 64 ? ctl->Iter : 63;
    const double res_p = as_d(atomicExch(&ctl->res_bits_p, 0ull));
    const double res_T = as_d(atomicExch(&ctl->res_bits_T, 0ull));
    ctl->res_p[I] = res_p;
    ctl->res_T[I] = res_T;
    const unsigned n = ++ctl->Iter_p_c;
    ctl->sweeps32++;
    const bool cont = (n < 2) || ((n < (unsigned)g.N_I_p_c) && ((g.MaxError_p_c < res_p) || (g.MaxError_T < res_T)));
    ctl->ecur = src ^ 1;
    if (!cont) ctl->stop32 = 1;
    if (in_graph) cudaGraphSetConditional((cudaGraphConditionalHandle)h_sweep, cont ? 1 : 0);
  }
}

}  // namespace sts
