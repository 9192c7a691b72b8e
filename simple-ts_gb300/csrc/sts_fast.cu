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
#include "sts_df.cuh"
#include "sts_kernels.h"
#include "sts_tc.cuh"

namespace sts {

// u/v momentum coefficients and ScT1 (SIMPLE_TS_MPI.cpp:3269-3756) with reciprocal multiplies,
// in FP64 (R = double) or double-float (R = df).
// parts: bit 0 the u faces, bit 1 the v faces, bit 2 ScT1 (the double-float kernel runs the three
// as separate CTAs, for three times the warps on a latency-bound kernel).
template <class R>
__device__ __forceinline__ void assemble_t(const Geo& g, unsigned long long h_sweep, int in_graph, unsigned parts = 7u) {
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
  const R cT = num<R>(ctl->cT), cPch = num<R>(ctl->cPch), ht = num<R>(g.ht), rht = num<R>(g.rht);
  const R third = num<R>(1.0 / 3.0), two_third = num<R>(2.0 / 3.0), one = num<R>(1.0), half = num<R>(0.5);
  const Arr<R> hx{g.hx}, hy{g.hy}, u{g.u}, v{g.v}, Fx{g.Fx}, Fy{g.Fy}, sT{g.sqrt_T}, rho{g.rho}, rho_pr{g.rho_pr};
  auto A = [](const double* p) { return Arr<R>{p}; };
  auto B = [&](int k) -> R { return cls_fluid(g.cls[k]) ? one : num<R>(0.0); };
  auto BB = [&](int k) -> bool { return cls_fluid(g.cls[k]); };
  const bool bc_u = cls_u(cl) == CLS_BC, bc_v = cls_v(cl) == CLS_BC, bc_o = cls_o(cl) == CLS_BC;

  if ((parts & 1u) && cls_u(cl)) {
    const R F_xu1 = half * (Fx[d.i_1j] + Fx[d.ij]);
    const R F_xu2 = half * (Fx[d.ij] + Fx[d.i1j]);
    const R r3a = third * A(g.rhx)[i], r3b = third * A(g.rhx)[d.i_1];
    const R m1 = bc_u ? B(d.i1j) : one, m2 = bc_u ? B(d.i_2j) : one;
    const R mN = bc_u ? B(d.ij1) : one, mNW = bc_u ? B(d.i_1j1) : one;
    const R mS = bc_u ? B(d.ij_1) : one, mSW = bc_u ? B(d.i_1j_1) : one;
    const R Scu = cT * (m1 * u[d.i1j] * sT[d.ij] * hy[j] * r3a + m2 * u[d.i_1j] * sT[d.i_1j] * hy[j] * r3b +
                             A(g.Gamma_yf)[d.ij1] * (v[d.ij1] * mN - v[d.i_1j1] * mNW) -
                             A(g.Gamma_yf)[d.ij] * (v[d.ij] * mS - v[d.i_1j] * mSW) -
                             sT[d.ij] * (v[d.ij1] * mN - v[d.ij] * mS) * two_third +
                             sT[d.i_1j] * (v[d.i_1j1] * mNW - v[d.i_1j] * mSW) * two_third);
    const R Spu = -(A(g.D_ux)[d.ij] + A(g.D_ux)[d.i1j]) * third;
    const R au1 = fmax0(F_xu1) + A(g.D_ux)[d.ij];
    const R au2 = fmax0(-F_xu2) + A(g.D_ux)[d.i1j];
    const R au3 = half * (fmax0(Fy[d.i_1j]) + fmax0(Fy[d.ij])) + A(g.D_uy)[d.ij];
    const R au4 = half * (fmax0(-Fy[d.i_1j1]) + fmax0(-Fy[d.ij1])) + A(g.D_uy)[d.ij1];
    const R bu3 = (rho_pr[d.i_1j] * hx[d.i_1] + rho_pr[d.ij] * hx[i]) * A(g.u_pr)[d.ij] * hy[j] * half * rht + Scu;
    const R au0 = au1 + au2 + au3 + au4 + half * (-Fy[d.i_1j] - Fy[d.ij] + Fy[d.i_1j1] + Fy[d.ij1]) + F_xu2 -
                       F_xu1 - Spu + (rho[d.i_1j] * hx[d.i_1] + rho[d.ij] * hx[i]) * hy[j] * half * rht;
    const R rau0 = one / au0;
    const R up = (au1 * m1 * u[d.i_1j] + au2 * m2 * u[d.i1j] + au3 * u[d.ij_1] + au4 * u[d.ij1] + bu3) * rau0;
    const R dpc = cPch * hy[j] * rau0;
    const R hr = hy[j] * A(g.rho_u)[d.ij];
    g.u_pseudo[d.ij] = to_double(up);
    g.d12[d.ij] = to_double(dpc);
    g.apx[d.ij] = to_double(dpc * hr);
    g.bpx[d.ij] = to_double(bc_u ? B(d.i_1j) * B(d.ij) * hr * up : hr * up);
  }

  if ((parts & 2u) && cls_v(cl)) {
    const int jm = j - ((j - 1) >= 0 ? 1 : 0);
    const int far = d.ij_1 - ((j - 2) >= 0 ? Nx : 0);
    const R F_yv3 = half * (Fy[d.ij_1] + Fy[d.ij]);
    const R F_yv4 = half * (Fy[d.ij] + Fy[d.ij1]);
    const R r3a = third * A(g.rhy)[j], r3b = third * A(g.rhy)[jm];
    const R mN = bc_v ? B(d.ij1) : one, mF = bc_v ? B(far) : one;
    const R mE = bc_v ? B(d.i1j) : one, mSE = bc_v ? B(d.i1j_1) : one;
    const R mW = bc_v ? B(d.i_1j) : one, mSW = bc_v ? B(d.i_1j_1) : one;
    const R Scv = cT * (mN * v[d.ij1] * sT[d.ij] * hx[i] * r3a + mF * v[d.ij_1] * sT[d.ij_1] * hx[i] * r3b +
                             A(g.Gamma_xf)[d.i1j] * (u[d.i1j] * mE - u[d.i1j_1] * mSE) -
                             A(g.Gamma_xf)[d.ij] * (u[d.ij] * mW - u[d.ij_1] * mSW) -
                             sT[d.ij] * (u[d.i1j] * mE - u[d.ij] * mW) * two_third +
                             sT[d.ij_1] * (u[d.i1j_1] * mSE - u[d.ij_1] * mSW) * two_third) -
                       num<R>(g.c_Fr_v) * (rho[d.ij_1] * hx[i] * half * hy[jm] + rho[d.ij] * hx[i] * half * hy[j]);
    const R Spv = -(A(g.D_vy)[d.ij] + A(g.D_vy)[d.ij1]) * third;
    const R av1 = half * (fmax0(Fx[d.ij]) + fmax0(Fx[d.ij_1])) + A(g.D_vx)[d.ij];
    const R av2 = half * (fmax0(-Fx[d.i1j]) + fmax0(-Fx[d.i1j_1])) + A(g.D_vx)[d.i1j];
    const R av3 = fmax0(F_yv3) + A(g.D_vy)[d.ij];
    const R av4 = fmax0(-F_yv4) + A(g.D_vy)[d.ij1];
    const R bv3 = (rho_pr[d.ij_1] * hy[j - 1] + rho_pr[d.ij] * hy[j]) * A(g.v_pr)[d.ij] * hx[i] * half * rht + Scv;
    const R av0 = av1 + av2 + av3 + av4 + half * (Fx[d.i1j] - Fx[d.ij] + Fx[d.i1j_1] - Fx[d.ij_1]) + F_yv4 -
                       F_yv3 - Spv + (rho[d.ij_1] * hy[j - 1] + rho[d.ij] * hy[j]) * hx[i] * half * rht;
    const R rav0 = one / av0;
    const R vp = (av1 * v[d.i_1j] + av2 * v[d.i1j] + av3 * mF * v[d.ij_1] + av4 * mN * v[d.ij1] + bv3) * rav0;
    const R dpc = cPch * hx[i] * rav0;
    const R hr = hx[i] * A(g.rho_v)[d.ij];
    g.v_pseudo[d.ij] = to_double(vp);
    g.d34[d.ij] = to_double(dpc);
    g.apy[d.ij] = to_double(dpc * hr);
    g.bpy[d.ij] = to_double(bc_v ? B(d.ij - Nx) * B(d.ij) * hr * vp : hr * vp);
  }

  if ((parts & 4u) && cls_o(cl)) {
    R dudx, dvdy, s0, s1, s2, s3;
    if (bc_o) {
      dudx = (B(d.i1j) * u[d.i1j] - B(d.i_1j) * u[d.ij]) * A(g.rhx)[i];
      dvdy = (B(d.ij1) * v[d.ij1] - B(d.ij_1) * v[d.ij]) * A(g.rhy)[j];
      // (mask * h_low + h) picks h alone or the two-cell sum
      const R ys = (BB(d.i_1j_1) && BB(d.ij_1)) ? A(g.ryy_m)[j] : A(g.rhy)[j];
      const R xs = (BB(d.i_1j_1) && BB(d.i_1j)) ? A(g.rxx_m)[i] : A(g.rhx)[i];
      const R ys1 = (BB(d.ij_1) && BB(d.i1j_1)) ? A(g.ryy_m)[j] : A(g.rhy)[j];
      const R xs1 = (BB(d.i1j_1) && BB(d.i1j)) ? A(g.rxx_p)[i] : A(g.rhx)[i];
      const R yn2 = (BB(d.i_1j1) && BB(d.ij1)) ? A(g.ryy_p)[j] : A(g.rhy)[j];
      const R xs2 = (BB(d.i_1j) && BB(d.i_1j1)) ? A(g.rxx_m)[i] : A(g.rhx)[i];
      const R yn3 = (BB(d.ij1) && BB(d.i1j1)) ? A(g.ryy_p)[j] : A(g.rhy)[j];
      const R xs3 = (BB(d.i1j) && BB(d.i1j1)) ? A(g.rxx_p)[i] : A(g.rhx)[i];
      s0 = (u[d.ij] - u[d.ij_1]) * ys + (v[d.ij] - v[d.i_1j]) * xs;
      s1 = (u[d.i1j] - u[d.i1j_1]) * ys1 + (v[d.i1j] - v[d.ij]) * xs1;
      s2 = (u[d.ij1] - u[d.ij]) * yn2 + (v[d.ij1] - v[d.i_1j1]) * xs2;
      s3 = (u[d.i1j1] - u[d.i1j]) * yn3 + (v[d.i1j1] - v[d.ij1]) * xs3;
    } else {
      dudx = (u[d.i1j] - u[d.ij]) * A(g.rhx)[i];
      dvdy = (v[d.ij1] - v[d.ij]) * A(g.rhy)[j];
      s0 = (u[d.ij] - u[d.ij_1]) * A(g.ryy_m)[j] + (v[d.ij] - v[d.i_1j]) * A(g.rxx_m)[i];
      s1 = (u[d.i1j] - u[d.i1j_1]) * A(g.ryy_m)[j] + (v[d.i1j] - v[d.ij]) * A(g.rxx_p)[i];
      s2 = (u[d.ij1] - u[d.ij]) * A(g.ryy_p)[j] + (v[d.ij1] - v[d.i_1j1]) * A(g.rxx_m)[i];
      s3 = (u[d.i1j1] - u[d.i1j]) * A(g.ryy_p)[j] + (v[d.i1j1] - v[d.ij1]) * A(g.rxx_p)[i];
    }
    const R dd = dudx + dvdy;
    g.ScT1[d.ij] = to_double(ht * sT[d.ij] * num<R>(g.cT2) * hx[i] * hy[j] *
                       (num<R>(2.0) * (dudx * dudx + dvdy * dvdy) + s0 * s0 + s1 * s1 + s2 * s2 + s3 * s3 - dd * dd * two_third) +
                   A(g.p_pr)[d.ij] * hx[i] * hy[j]);
  }
}
__device__ __forceinline__ void assemble_fast_body(const Geo& g, unsigned long long h_sweep, int in_graph) {
  assemble_t<double>(g, h_sweep, in_graph);
}
__global__ void k_assemble_fast(Geo g, unsigned long long h_sweep, int in_graph) { assemble_fast_body(g, h_sweep, in_graph); }
__global__ void kb_assemble_fast(const Geo* gs, unsigned long long h_sweep, int in_graph) {
  __shared__ Geo sg;
  if (!stage_geo(sg, gs)) return;
  assemble_fast_body(sg, h_sweep, in_graph);
}

// Fluxes and diffusion coefficients (SIMPLE_TS_MPI.cpp:10440-10618) with reciprocal multiplies,
// in FP64 (R = double) or double-float (R = df).  Gamma keeps its stored value where no branch
// computes it (no FP64 -> double-float -> FP64 round trip).
template <class R>
__device__ __forceinline__ void flux_diff_t(const Geo& g, unsigned tail) {
  Cell c = cell(g);
  if (c.ok) {
    const int i = c.i, j = c.j;
    const Nb d = neighbours(i, j, g.Nx, g.Ny, g.bits & F_PERIODIC);
    const Arr<R> hx{g.hx}, hy{g.hy}, sT{g.sqrt_T}, Tw_u{g.Tw_u}, Tw_v{g.Tw_v}, rhx{g.rhx}, rhy{g.rhy};
    const R cT = num<R>(g.ctl->cT), cT1 = num<R>(g.cT1), half = num<R>(0.5), zero = num<R>(0.0);
    g.Fx[d.ij] = to_double(hy[j] * Arr<R>{g.rho_u}[d.ij] * Arr<R>{g.u}[d.ij]);
    g.Fy[d.ij] = to_double(hx[i] * Arr<R>{g.rho_v}[d.ij] * Arr<R>{g.v}[d.ij]);
    const bool b_ws = cls_fluid(g.cls[d.i_1j_1]), b_s = cls_fluid(g.cls[d.ij_1]), b_w = cls_fluid(g.cls[d.i_1j]),
               b_p = cls_fluid(g.cls[d.ij]);
    const int jm = j - (0 < j ? 1 : 0);
    const R ry = Arr<R>{g.ryy_m}[j], rx = Arr<R>{g.rxx_m}[i];
    auto LiY = [&](R f1, R f2) { return (f1 * hy[j] + f2 * hy[jm]) * ry; };
    auto LiX = [&](R f1, R f2) { return (f1 * hx[i] + f2 * hx[d.i_1]) * rx; };
    R Gy, Gx;
    if (b_ws && b_s && b_w && b_p) {
      Gy = half * (LiY(sT[d.i_1j_1], sT[d.i_1j]) + LiY(sT[d.ij_1], sT[d.ij]));
      Gx = half * (LiX(sT[d.i_1j_1], sT[d.ij_1]) + LiX(sT[d.i_1j], sT[d.ij]));
      g.Gamma_yf[d.ij] = to_double(Gy);
      g.Gamma_xf[d.ij] = to_double(Gx);
    } else if (b_ws || b_s || b_w || b_p) {
      Gy = half * ((b_ws && b_w) ? LiY(sT[d.i_1j_1], sT[d.i_1j]) : zero) +
           half * ((b_ws != b_w) ? dsqrt(Tw_v[d.i_1j]) : zero) + half * ((b_s && b_p) ? LiY(sT[d.ij_1], sT[d.ij]) : zero) +
           half * ((b_s != b_p) ? dsqrt(Tw_v[d.ij]) : zero) +
           half * (((!(b_ws && b_w)) || (!(b_s && b_p))) ? LiY(dsqrt(Tw_u[d.ij_1]), dsqrt(Tw_u[d.ij])) : zero);
      Gx = half * ((b_ws && b_s) ? LiX(sT[d.i_1j_1], sT[d.ij_1]) : zero) +
           half * ((b_ws != b_s) ? dsqrt(Tw_u[d.ij_1]) : zero) + half * ((b_w && b_p) ? LiX(sT[d.i_1j], sT[d.ij]) : zero) +
           half * ((b_w != b_p) ? dsqrt(Tw_u[d.ij]) : zero) +
           half * (((!(b_ws && b_s)) || (!(b_w && b_p))) ? LiX(dsqrt(Tw_v[d.i_1j]), dsqrt(Tw_v[d.ij])) : zero);
      g.Gamma_yf[d.ij] = to_double(Gy);
      g.Gamma_xf[d.ij] = to_double(Gx);
    } else {
      Gy = Arr<R>{g.Gamma_yf}[d.ij];
      Gx = Arr<R>{g.Gamma_xf}[d.ij];
    }
    g.D_ux[d.ij] = to_double(cT * sT[d.i_1j] * hy[j] * rhx[d.i_1]);
    g.D_vy[d.ij] = to_double(cT * sT[d.ij_1] * hx[i] * rhy[jm]);
    const bool pw = b_p && b_w, sws = b_s && b_ws, ps = b_p && b_s, wws = b_w && b_ws;
    g.D_uy[d.ij] =
        (pw || sws) ? to_double(cT * Gy * (hx[i] + hx[d.i_1]) * ((pw && sws) ? ry : (pw ? rhy[j] : rhy[jm]))) : 0.0;
    g.D_vx[d.ij] =
        (ps || wws) ? to_double(cT * Gx * (hy[j] + hy[jm]) * ((ps && wws) ? rx : (ps ? rhx[i] : rhx[d.i_1]))) : 0.0;
    if (b_p || b_w) {
      const R rs = pw ? rx : (b_p ? rhx[i] : rhx[d.i_1]);
      const R face = pw ? (hx[d.i_1] + hx[i]) * sT[d.i_1j] * sT[d.ij] / (hx[d.i_1] * sT[d.ij] + hx[i] * sT[d.i_1j])
                        : dsqrt(Tw_u[d.ij]);
      g.DTx[d.ij] = to_double(cT1 * hy[j] * num<R>(2.0) * rs * face);
    } else {
      g.DTx[d.ij] = 0.0;
    }
    if (b_p || b_s) {
      const R rs = ps ? ry : (b_p ? rhy[j] : rhy[jm]);
      const R face = ps ? (hy[jm] + hy[j]) * sT[d.ij_1] * sT[d.ij] / (hy[jm] * sT[d.ij] + hy[j] * sT[d.ij_1])
                        : dsqrt(Tw_v[d.ij]);
      g.DTy[d.ij] = to_double(cT1 * hx[i] * num<R>(2.0) * rs * face);
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
__device__ __forceinline__ void flux_diff_fast_body(const Geo& g, unsigned tail) { flux_diff_t<double>(g, tail); }
__global__ void k_flux_diff_fast(Geo g, unsigned tail) {
  wait_for_predecessor();
  flux_diff_fast_body(g, tail);
}
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
template <bool FIRST, class R>
__device__ __forceinline__ bool sweep_cell_t(const Geo& g, const Cell& c, const double* __restrict__ P,
                                             const double* __restrict__ TT, double* __restrict__ pn,
                                             double* __restrict__ Tn, R& Tnew, R& pnew, R& sa) {
  const int ij = c.ij;
  const uint8_t cl = g.cls[ij];
  const int co = cls_o(cl);
  if (!co) {
    pn[ij] = P[ij];
    Tn[ij] = TT[ij];
    pnew = num<R>(P[ij]);
    Tnew = num<R>(TT[ij]);
    return false;
  }
  const int i = c.i, j = c.j;
  const Nb d = neighbours(i, j, g.Nx, g.Ny, g.bits & F_PERIODIC);
  const Arr<R> apx{g.apx}, apy{g.apy}, Pv{P}, Tv{TT};
  const R ht = num<R>(g.ht), H = num<R>(g.hx[i]) * num<R>(g.hy[j]);
  auto fl = [&](int k) { return cls_fluid(g.cls[k]); };
  R w1, w2, w3, w4, divu, rden, pc;
  if (FIRST) {
    const Arr<R> Fx{g.Fx}, Fy{g.Fy}, DTx{g.DTx}, DTy{g.DTy}, u{g.u}, v{g.v};
    const R aT1 = fmax0(Fx[d.ij]) + DTx[d.ij];
    const R aT2 = fmax0(-Fx[d.i1j]) + DTx[d.i1j];
    const R aT3 = fmax0(Fy[d.ij]) + DTy[d.ij];
    const R aT4 = fmax0(-Fy[d.ij1]) + DTy[d.ij1];
    divu = (u[d.i1j] - u[d.ij]) * num<R>(g.hy[j]) + (v[d.ij1] - v[d.ij]) * num<R>(g.hx[i]);
    rden = num<R>(1.0) / (ht * (aT1 + aT2 + aT3 + aT4 + Fx[d.i1j] - Fx[d.ij] + Fy[d.ij1] - Fy[d.ij]) +
                          H * num<R>(g.rho[ij]));
    w1 = aT1; w2 = aT2; w3 = aT3; w4 = aT4;
    if (co == CLS_BC) {
      if (!fl(d.i_1j)) w1 = aT1 * num<R>(g.Tw_u[ij]);
      if (!fl(d.i1j)) w2 = aT2 * num<R>(g.Tw_u[d.i1j]);
      if (!fl(d.ij_1)) w3 = aT3 * num<R>(g.Tw_v[ij]);
      if (!fl(d.ij1)) w4 = aT4 * num<R>(g.Tw_v[d.ij1]);
    }
    pc = num<R>(g.p_pr[ij]) * H / num<R>(g.T_pr[ij]);
    sa = ht * (apx[ij] + apx[d.i1j] + apy[ij] + apy[d.ij1]);
    g.inv[0][ij] = to_double(w1); g.inv[1][ij] = to_double(w2); g.inv[2][ij] = to_double(w3);
    g.inv[3][ij] = to_double(w4); g.inv[4][ij] = to_double(divu); g.inv[5][ij] = to_double(rden);
    g.inv[6][ij] = to_double(pc); g.inv[7][ij] = to_double(sa);
  } else {
    w1 = num<R>(g.inv[0][ij]); w2 = num<R>(g.inv[1][ij]); w3 = num<R>(g.inv[2][ij]); w4 = num<R>(g.inv[3][ij]);
    divu = num<R>(g.inv[4][ij]); rden = num<R>(g.inv[5][ij]); pc = num<R>(g.inv[6][ij]); sa = num<R>(g.inv[7][ij]);
  }
  R t1, t2, t3, t4;
  if (co == CLS_BC) {
    t1 = fl(d.i_1j) ? w1 * Tv[d.i_1j] : w1;
    t2 = fl(d.i1j) ? w2 * Tv[d.i1j] : w2;
    t3 = fl(d.ij_1) ? w3 * Tv[d.ij_1] : w3;
    t4 = fl(d.ij1) ? w4 * Tv[d.ij1] : w4;
  } else {
    t1 = w1 * Tv[d.i_1j];
    t2 = w2 * Tv[d.i1j];
    t3 = w3 * Tv[d.ij_1];
    t4 = w4 * Tv[d.ij1];
  }
  Tnew = (ht * (t1 + t2 + t3 + t4 + num<R>(1.0 - g.gamma1) * Pv[ij] * divu) + num<R>(g.ScT1[ij])) * rden;
  R nm = apx[ij] * Pv[d.i_1j] + apx[d.i1j] * Pv[d.i1j] + apy[ij] * Pv[d.ij_1] + apy[d.ij1] * Pv[d.ij1] +
         num<R>(g.bpx[ij]) - num<R>(g.bpx[d.i1j]) + num<R>(g.bpy[ij]) - num<R>(g.bpy[d.ij1]);
  if (co == CLS_BC) {
    if ((g.bits & F_GIVEN_U_XB) && i == g.Nx_o0) nm = nm + num<R>(g.Fx[ij]);
    if ((g.bits & F_GIVEN_U_XE) && i == g.Nx_o1 - 1) nm = nm - num<R>(g.Fx[d.i1j]);
  }
  pnew = (ht * nm + pc) * Tnew / (sa * Tnew + H);
  Tn[ij] = to_double(Tnew);
  pn[ij] = to_double(pnew);
  return true;
}
template <bool FIRST>
__device__ __forceinline__ bool sweep_cell_fast(const Geo& g, const Cell& c, const double* __restrict__ P,
                                                const double* __restrict__ TT, double* __restrict__ pn,
                                                double* __restrict__ Tn, double& Tnew, double& pnew, double& sa) {
  return sweep_cell_t<FIRST, double>(g, c, P, TT, pn, Tn, Tnew, pnew, sa);
}

// The sweep loop of mode 1 (see k_pt_loop).
struct FastOps {
  static constexpr bool kCellList = true;
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

// Index of cell (i, j) in the FP32 correction buffers (rows of g.Nxe floats).
__device__ __forceinline__ int eix(const Geo& g, int i, int j) { return i + j * g.Nxe; }

// Base values of the FP32 corrections taken from an FP64 sweep x -> x1 of a solved cell
// (x, x1 in FP64 or double-float).
template <class R>
__device__ __forceinline__ void set_base(const Geo& g, const Cell& c, R T0, R p0, R T1, R p1, R sa) {
  const int ij = c.ij, e = eix(g, c.i, c.j);
  // the FP32 sweeps' coefficients are formed in FP32 (they only steer the corrections; the
  // FP64 passes decide the converged iterate), which keeps an FP64 division off this pass
  const float T1f = to_float(T1);
  const float hT = ((float)g.hx[c.i] * (float)g.hy[c.j]) / T1f;
  g.T1[ij] = T1f;
  g.hT[ij] = hT;
  g.q1[ij] = to_float(p1);
  g.den1[ij] = to_float(sa) + hT;
  const float dT = to_float(T1 - T0), dp = to_float(p1 - p0);
  g.dT[ij] = dT;
  g.dp[ij] = dp;
  g.eT[0][e] = dT;
  g.ep[0][e] = dp;
}

// One FP32 correction update of solved cell ij from its corrections (centre P and neighbours W, E,
// S, N of e_T and e_p); both the one-sweep pass and the two-sweep tile pass use it, so their
// arithmetic is the same expression.
__device__ __forceinline__ void sweep32_math(const Geo& g, int ij, float TW, float TE, float TS, float TN, float pP,
                                             float pW, float pE, float pS, float pN, float TP, float& eTnew,
                                             float& epnew, float& rp, float& rT) {
  const float dT = g.c32[0][ij] * TW + g.c32[1][ij] * TE + g.c32[2][ij] * TS + g.c32[3][ij] * TN + g.c32[4][ij] * pP;
  eTnew = g.dT[ij] + dT;
  const float q = g.hT[ij] * dT / (g.T1[ij] + dT);
  const float num = g.a32[0][ij] * pW + g.a32[1][ij] * pE + g.a32[2][ij] * pS + g.a32[3][ij] * pN;
  epnew = g.dp[ij] + (num + g.q1[ij] * q) / (g.den1[ij] - q);
  const float aT = fabsf(eTnew - TP), ap = fabsf(epnew - pP);
  rT = aT <= kFloor32 * fabsf(eTnew) ? 0.0f : aT;
  rp = ap <= kFloor32 * fabsf(epnew) ? 0.0f : ap;
}

// One FP32 correction sweep of a solved cell: e (buffer src) -> e' (buffer dst).
__device__ __forceinline__ void sweep32_cell(const Geo& g, const Cell& c, unsigned src, unsigned dst, float& rp,
                                             float& rT) {
  const Nb d = neighbours(c.i, c.j, g.Nx, g.Ny, g.bits & F_PERIODIC);
  const int jm = c.j > 0 ? c.j - 1 : c.j, jp = c.j < g.Ny - 1 ? c.j + 1 : c.j;
  const int P = eix(g, c.i, c.j), W = eix(g, d.i_1, c.j), E = eix(g, d.i1, c.j), S = eix(g, c.i, jm),
            N = eix(g, c.i, jp);
  const float* __restrict__ ep = g.ep[src];
  const float* __restrict__ eT = g.eT[src];
  float eTnew, epnew;
  sweep32_math(g, c.ij, eT[W], eT[E], eT[S], eT[N], ep[P], ep[W], ep[E], ep[S], ep[N], eT[P], eTnew, epnew, rp, rT);
  g.eT[dst][P] = eTnew;
  g.ep[dst][P] = epnew;
}

__device__ __forceinline__ unsigned next_buf(unsigned b) { return b == 2u ? 0u : b + 1u; }

// Shared memory of the two-sweep tile pass: the corrections of the tile and a margin of two cells
// (one TMA box of 40 x 12 floats per field, x starting 4 cells left of the tile so that the start
// is a multiple of 16 bytes), the first sweep's values of the tile and a margin of one cell, and the
// TMA completion barrier.
struct Tile2Smem {
  alignas(128) float E0[2][12][40];
  float E1[2][10][34];
  alignas(8) uint64_t bar;
};

// Two FP32 correction sweeps of the 32x8 tile t in one round (temporal blocking).  The first sweep
// updates the tile and a margin of one cell in shared memory, the second the tile, each cell with
// sweep32_math and the neighbours of neighbours() (x wraps on periodic meshes, indices clamp at the
// mesh edges), so every value is the one the one-sweep passes would compute; the tile's values of
// both sweeps go to the next two buffers and both sweeps' residual maxima to the round's two slot
// pairs.  Returns false if the TMA load did not complete in time (status flagged).
__device__ bool sweep32_pair_tile(const Geo& g, int t, const LoopCase& s, const EMaps* maps, Tile2Smem& sm,
                                  unsigned& tphase, unsigned slot) {
  const int tx = (g.Nx + 31) / 32, tyi = t / tx;
  const int i0 = (t - tyi * tx) * 32, j0 = tyi * 8;
  const int tid = threadIdx.x + 32 * threadIdx.y;
  const unsigned src = s.ec, d1 = next_buf(src), d2 = next_buf(d1);
  const bool per = g.bits & F_PERIODIC;
  const int Nx = g.Nx, Ny = g.Ny;
  __syncthreads();  // the previous tile's readers of the shared arrays are done
  if (tid == 0) {
    tc::mbar_arrive_expect_tx(&sm.bar, 2u * 12u * 40u * 4u);
    tc::tma_load_2d(&sm.E0[0][0][0], &maps->eT[src], i0 - 4, j0 - 2, &sm.bar);
    tc::tma_load_2d(&sm.E0[1][0][0], &maps->ep[src], i0 - 4, j0 - 2, &sm.bar);
  }
  const bool got = tc::mbar_wait(&sm.bar, tphase, 1u << 22);
  tphase ^= 1u;
  if (!__syncthreads_and(got)) {
    if (tid == 0) atomicOr(&g.ctl->status, ST_BARRIER_TIMEOUT);
    return false;
  }
  if (per) {  // the margin columns outside [0, Nx) hold the wrapped cells
    for (int k = tid; k < 12 * 40; k += 256) {
      const int yy = k / 40, xx = k - yy * 40, i = i0 - 4 + xx, j = j0 - 2 + yy;
      if ((i < 0 || i >= Nx) && j >= 0 && j < Ny) {
        const int wi = ((i % Nx) + Nx) % Nx;
        sm.E0[0][yy][xx] = g.eT[src][eix(g, wi, j)];
        sm.E0[1][yy][xx] = g.ep[src][eix(g, wi, j)];
      }
    }
    __syncthreads();
  }
  unsigned* st = &g.ctl->status;
  unsigned r1p = 0u, r1T = 0u;  // residual maxima as bit patterns (NaN counts as 0 and is flagged)
  float r2p = 0.f, r2T = 0.f;
  // first sweep: the tile and a margin of one cell (cells outside the mesh and unsolved cells keep
  // their values)
  for (int k = tid; k < 10 * 34; k += 256) {
    const int yy = k / 34, xx = k - yy * 34, i = i0 - 1 + xx, j = j0 - 1 + yy;
    const int cx = xx + 3, cy = yy + 1;  // the cell in E0
    float vT = sm.E0[0][cy][cx], vp = sm.E0[1][cy][cx];
    if (j >= 0 && j < Ny && (per || (i >= 0 && i < Nx))) {
      const int gi = ((i % Nx) + Nx) % Nx, ij = gi + j * Nx;
      if (cls_o(g.cls[ij])) {
        const int xw = (per || gi > 0) ? cx - 1 : cx, xe = (per || gi < Nx - 1) ? cx + 1 : cx;
        const int ys = j > 0 ? cy - 1 : cy, yn = j < Ny - 1 ? cy + 1 : cy;
        const float(*T)[40] = sm.E0[0];
        const float(*p)[40] = sm.E0[1];
        float eTn, epn, rp, rT;
        sweep32_math(g, ij, T[cy][xw], T[cy][xe], T[ys][cx], T[yn][cx], p[cy][cx], p[cy][xw], p[cy][xe], p[ys][cx],
                     p[yn][cx], T[cy][cx], eTn, epn, rp, rT);
        vT = eTn;
        vp = epn;
        if (i >= i0 && i < i0 + 32 && i < Nx && j >= j0 && j < j0 + 8) {  // a cell of the tile: value, residual
          g.eT[d1][eix(g, gi, j)] = eTn;
          g.ep[d1][eix(g, gi, j)] = epn;
          r1p = max(r1p, res_bits_f(rp, st));
          r1T = max(r1T, res_bits_f(rT, st));
        }
      }
    }
    sm.E1[0][yy][xx] = vT;
    sm.E1[1][yy][xx] = vp;
  }
  __syncthreads();
  // second sweep: the tile's cells, one per thread
  {
    const int i = i0 + threadIdx.x, j = j0 + threadIdx.y;
    if (i < Nx && j < Ny) {
      const int ij = i + j * Nx;
      if (cls_o(g.cls[ij])) {
        const int cx = threadIdx.x + 1, cy = threadIdx.y + 1;  // the cell in E1
        const int xw = (per || i > 0) ? cx - 1 : cx, xe = (per || i < Nx - 1) ? cx + 1 : cx;
        const int ys = j > 0 ? cy - 1 : cy, yn = j < Ny - 1 ? cy + 1 : cy;
        const float(*T)[34] = sm.E1[0];
        const float(*p)[34] = sm.E1[1];
        float eTn, epn;
        sweep32_math(g, ij, T[cy][xw], T[cy][xe], T[ys][cx], T[yn][cx], p[cy][cx], p[cy][xw], p[cy][xe], p[ys][cx],
                     p[yn][cx], T[cy][cx], eTn, epn, r2p, r2T);
        g.eT[d2][eix(g, i, j)] = eTn;
        g.ep[d2][eix(g, i, j)] = epn;
      }
    }
  }
  block_max2_f(__uint_as_float(r1p), __uint_as_float(r1T), &g.ctl->rb_p[slot], &g.ctl->rb_T[slot], st);
  block_max2_f(r2p, r2T, &g.ctl->rb2_p[slot], &g.ctl->rb2_T[slot], st);
  return true;
}

// R: the arithmetic of the FP64 sweeps (FP64, or double-float in precision mode 3).
template <class R>
struct MixedOpsT {
  static constexpr bool kCellList = false;  // measured slower with the cell list
  static __device__ __forceinline__ void pass(const Geo& g, const Cell& c, const LoopCase& s, double& rp, double& rT) {
    const int ij = c.ij;
    const unsigned base = s.base;
    switch (s.phase) {
      case PS_FIRST: {  // FP64 sweep from b into base ^ 1, with the FP32 coefficients of this outer iteration
        const double* P = g.p[base];
        const double* TT = g.T[base];
        R Tnew, pnew, sa;
        if (!sweep_cell_t<true, R>(g, c, P, TT, g.p[base ^ 1], g.T[base ^ 1], Tnew, pnew, sa)) {
          g.dT[ij] = 0.0f; g.dp[ij] = 0.0f;
          const int e = eix(g, c.i, c.j);
          for (int b = 0; b < 3; b++) {
            g.eT[b][e] = 0.0f;
            g.ep[b][e] = 0.0f;
          }
          return;
        }
        const R P0 = num<R>(P[ij]), T0 = num<R>(TT[ij]);
        rp = to_double(dabs(pnew - P0));
        rT = to_double(dabs(Tnew - T0));
        const Nb d = neighbours(c.i, c.j, g.Nx, g.Ny, g.bits & F_PERIODIC);
        // the FP32 sweeps' coefficients, products formed in FP32
        const float ht = (float)g.ht, r = ht * (float)g.inv[5][ij];
        const int nb[4] = {d.i_1j, d.i1j, d.ij_1, d.ij1};
        for (int k = 0; k < 4; k++)  // a wall neighbour's term is a constant and sits in the defect
          g.c32[k][ij] = (cls_o(g.cls[ij]) == CLS_NCH || cls_fluid(g.cls[nb[k]])) ? r * (float)g.inv[k][ij] : 0.0f;
        g.c32[4][ij] = r * (float)(1.0 - g.gamma1) * (float)g.inv[4][ij];
        g.a32[0][ij] = ht * (float)g.apx[ij];
        g.a32[1][ij] = ht * (float)g.apx[d.i1j];
        g.a32[2][ij] = ht * (float)g.apy[ij];
        g.a32[3][ij] = ht * (float)g.apy[d.ij1];
        set_base<R>(g, c, T0, P0, Tnew, pnew, sa);
        return;
      }
      case PS_MATERIALIZE:  // the iterate of the sweep before the last FP32 one, in FP64
        g.p[base ^ 1][ij] = g.p[base][ij] + widen(g.ep[s.eprev][eix(g, c.i, c.j)]);
        g.T[base ^ 1][ij] = g.T[base][ij] + widen(g.eT[s.eprev][eix(g, c.i, c.j)]);
        return;
      case PS_CONFIRM: {  // that sweep again in FP64 into the base buffer; exports for a re-basing
        const double* P = g.p[base ^ 1];
        const double* TT = g.T[base ^ 1];
        R Tnew, pnew, sa;
        if (!sweep_cell_t<false, R>(g, c, P, TT, g.p[base], g.T[base], Tnew, pnew, sa)) return;
        const R P0 = num<R>(P[ij]), T0 = num<R>(TT[ij]);
        rp = to_double(dabs(pnew - P0));
        rT = to_double(dabs(Tnew - T0));
        set_base<R>(g, c, T0, P0, Tnew, pnew, sa);
        return;
      }
      default:
        return;
    }
  }
  static __device__ __forceinline__ void pass32(const Geo& g, const Cell& c, const LoopCase& s, float& rp, float& rT) {
    if (cls_o(g.cls[c.ij])) sweep32_cell(g, c, s.ec, next_buf(s.ec), rp, rT);
  }
  static __device__ __forceinline__ bool pass32_pair(const Geo& g, int t, const LoopCase& s, const EMaps* maps,
                                                     void* smem, unsigned& tphase, unsigned slot) {
    return sweep32_pair_tile(g, t, s, maps, *(Tile2Smem*)smem, tphase, slot);
  }
  static __device__ __forceinline__ void advance(const Geo& g, bool lead, LoopCase& s, double res_p, double res_T) {
    Ctl* ctl = g.ctl;
    switch (s.phase) {
      case PS_FIRST:
        s.n = 1;
        if (lead) record_residual(ctl, s.n, s.I, res_p, res_T);
        s.cur = s.base ^ 1;
        s.ec = 0;
        s.eprev = 0;
        s.phase = (s.n >= (unsigned)g.N_I_p_c) ? PS_DONE : PS_SWEEP32;  // a single sweep: x1 is the result
        break;
      case PS_SWEEP32:
        s.n++;
        s.eprev = s.ec;
        s.ec = next_buf(s.ec);
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
  pt_loop_rounds<MixedOpsT<double>, true>(g, nullptr, nullptr, nullptr, 1, ntiles, lc);
}

// The same loop with two FP32 sweeps per tile load (temporal blocking, tiles staged by TMA).
__device__ __forceinline__ void init_tile2(Tile2Smem& sm) {
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    tc::mbar_init(&sm.bar, 1);
    tc::fence_barrier_init();
  }
  __syncthreads();
}
__global__ void __launch_bounds__(256, 4) k_pt_loop_mixed_tb(Geo g, int ntiles, LoopCtl* lc,
                                                             const __grid_constant__ EMaps maps) {
  __shared__ Tile2Smem sm;
  init_tile2(sm);
  pt_loop_rounds<MixedOpsT<double>, true, true>(g, nullptr, nullptr, nullptr, 1, ntiles, lc, &maps, &sm);
}
__global__ void __launch_bounds__(256, 4) kb_pt_loop_mixed(const Geo* gs, const int* tile_case, const int* tile_first,
                                                          int ncases, int ntiles, LoopCtl* lc) {
  pt_loop_rounds<MixedOpsT<double>, false>(gs[0], gs, tile_case, tile_first, ncases, ntiles, lc);
}

// Self-check of the double-float arithmetic against FP64 on n pseudo-random operand pairs of
// random sign and magnitude 2^-40 .. 2^40: the largest relative error of the FP64 -> double-float
// conversion and of add, multiply, divide and square root, as bit patterns in err[0..4] (folded
// with atomicMax; non-negative doubles order like their bits).  Additions are checked against
// |a| + |b| (the error bound of a double-word sum is relative to the operands, not the result).
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double rand_val(unsigned long long r) {
  const int e = (int)((r >> 52) % 81ull) - 40;
  const unsigned long long bits = ((r >> 63) << 63) | ((unsigned long long)(e + 1023) << 52) | (r & 0xFFFFFFFFFFFFFull);
  return __longlong_as_double((long long)bits);
}
__global__ void k_check_df(unsigned long long n, unsigned long long seed, unsigned long long* err) {
  double m[5] = {0, 0, 0, 0, 0};
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < n; k += stride) {
    const double a = rand_val(mix64(seed + 2 * k)), b = rand_val(mix64(seed + 2 * k + 1));
    const df A = to_df(a), B = to_df(b);
    m[0] = fmax(m[0], fabs(to_double(A) - a) / fabs(a));
    m[1] = fmax(m[1], fabs(to_double(A + B) - (a + b)) / (fabs(a) + fabs(b)));
    m[2] = fmax(m[2], fabs(to_double(A * B) - a * b) / fabs(a * b));
    m[3] = fmax(m[3], fabs(to_double(A / B) - a / b) / fabs(a / b));
    const double sa = ::sqrt(fabs(a));
    m[4] = fmax(m[4], fabs(to_double(dsqrt(dabs(A))) - sa) / sa);
  }
  for (int q = 0; q < 5; q++) atomicMax(&err[q], (unsigned long long)__double_as_longlong(m[q]));
}

// ---------------------------------------------------------------------------
// Precision mode 3: precision mode 2 with the FP64 arithmetic of the assembly, the fluxes and
// diffusion terms and the FP64 sweeps done in double-float (sts_df.cuh) on GB300's FP32 pipes;
// fields stay FP64 in memory, the FP32 correction sweeps are those of mode 2.
// ---------------------------------------------------------------------------
// grid z: 3 parts (k_) or 3 parts per case (kb_, z = 3 case + part)
__device__ __forceinline__ void assemble_df_part(const Geo& g, unsigned long long h_sweep, int in_graph, unsigned part) {
  switch (part) {  // each part compiled on its own (constant mask)
    case 0: assemble_t<df>(g, h_sweep, in_graph, 1u); break;
    case 1: assemble_t<df>(g, h_sweep, in_graph, 2u); break;
    default: assemble_t<df>(g, h_sweep, in_graph, 4u); break;
  }
}
__global__ void __launch_bounds__(256, 3) k_assemble_df(Geo g, unsigned long long h_sweep, int in_graph) {
  assemble_df_part(g, h_sweep, in_graph, blockIdx.z);
}
__global__ void __launch_bounds__(256, 3) kb_assemble_df(const Geo* gs, unsigned long long h_sweep, int in_graph) {
  __shared__ Geo sg;
  if (!stage_geo(sg, gs, blockIdx.z / 3)) return;
  assemble_df_part(sg, h_sweep, in_graph, blockIdx.z % 3);
}
// The velocity correction, sqrt(T) and the cell density of k_correct (SIMPLE_TS_MPI.cpp:4171-4330)
// for precision mode 3: the same formulas with their FP64 arithmetic in double-float -- the
// division p / T and the square root are what bind k_correct to GB300's FP64 unit -- and the
// fields FP64 in memory.  The residuals |u_new - u| are taken between the stored FP64 values.
__device__ __forceinline__ void correct_df_body(const Geo& g) {
  Cell c = cell(g);
  Ctl* ctl = g.ctl;
  const unsigned cur = ctl->cur;
  const double* __restrict__ p = g.p[cur];
  const double* __restrict__ T = g.T[cur];
  double ru = 0, rv = 0;
  if (c.ok) {
    const uint8_t cl = g.cls[c.ij];
    const int n = c.ij;
    const df pn = to_df(p[n]);
    if (cls_u(cl)) {
      const int w = (cls_u(cl) == CLS_BC && (g.bits & F_PERIODIC) && c.i == 0) ? n + g.Nx - 1 : n - 1;
      const double t = g.u[n];
      const double un = to_double(to_df(g.u_pseudo[n]) - (pn - to_df(p[w])) * to_df(g.d12[n]));
      g.u[n] = un;
      ru = fabs(un - t);
    }
    if (cls_v(cl)) {
      const double t = g.v[n];
      const double vn = to_double(to_df(g.v_pseudo[n]) - (pn - to_df(p[n - g.Nx])) * to_df(g.d34[n]));
      g.v[n] = vn;
      rv = fabs(vn - t);
    }
    const df Tn = to_df(T[n]);
    g.sqrt_T[n] = to_double(dsqrt(Tn));
    g.rho[n] = cls_fluid(cl) ? to_double(pn / Tn) : 0.0;
  }
  block_max2(ru, rv, &ctl->res_bits_u, &ctl->res_bits_v, &ctl->status);
}
__global__ void k_correct_df(Geo g) {
  wait_for_predecessor();
  correct_df_body(g);
}
__global__ void kb_correct_df(const Geo* gs) {
  __shared__ Geo sg;
  if (!stage_geo(sg, gs)) return;
  correct_df_body(sg);
}
__global__ void __launch_bounds__(256, 4) k_flux_diff_df(Geo g, unsigned tail) {
  wait_for_predecessor();
  flux_diff_t<df>(g, tail);
}
__global__ void __launch_bounds__(256, 4) kb_flux_diff_df(const Geo* gs, unsigned tail) {
  __shared__ Geo sg;
  if (!stage_geo(sg, gs)) return;
  flux_diff_t<df>(sg, tail);
}
__global__ void __launch_bounds__(256, 4) k_pt_loop_mixed_df(Geo g, int ntiles, LoopCtl* lc) {
  pt_loop_rounds<MixedOpsT<df>, true>(g, nullptr, nullptr, nullptr, 1, ntiles, lc);
}
__global__ void __launch_bounds__(256, 4) k_pt_loop_mixed_df_tb(Geo g, int ntiles, LoopCtl* lc,
                                                                const __grid_constant__ EMaps maps) {
  __shared__ Tile2Smem sm;
  init_tile2(sm);
  pt_loop_rounds<MixedOpsT<df>, true, true>(g, nullptr, nullptr, nullptr, 1, ntiles, lc, &maps, &sm);
}
__global__ void __launch_bounds__(256, 4) kb_pt_loop_mixed_df(const Geo* gs, const int* tile_case,
                                                             const int* tile_first, int ncases, int ntiles,
                                                             LoopCtl* lc) {
  pt_loop_rounds<MixedOpsT<df>, false>(gs[0], gs, tile_case, tile_first, ncases, ntiles, lc);
}

}  // namespace sts
