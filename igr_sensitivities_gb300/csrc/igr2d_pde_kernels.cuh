// 2D continuous adjoint (optimise-then-discretise, conservative Pi form,
// IGR_adjoints_2d/adjoint_pde.jl:41-611) on the forward kernels' tiling.
//
// Backward in time the adjoint a = (a_mux, a_muy, a_rho, a_E) advances by
//   d_tau a = +div F_dag(q, a) - S_loc(q) a + S_Sigma(q, Pi),
// with the primal q and Sigma frozen at the stored snapshot for all three
// stages of a step. Everything that depends on the snapshot alone is computed
// once per step (k2_pde_prep): the ten local-source coefficients (the
// pointwise q-derivatives of div F, :138-217), the nodal velocity gradients,
// grad(Sigma)/rho and R_tr of the nonlocal source (:381-466), 1/rho and the
// LLF wave speeds. Each stage then runs
//   k2_pde_b   (alpha > 0)  b = alpha w_i w_j Jx Jy (div a_mu + grad a_E . u)  (:337-364, :490-493)
//   Pi solve   (alpha > 0)  the forward's SIP operator and solver kernels, warm start = previous Pi
//   k2_pde_rk               adjoint DG operator + sources + SSP-RK3 combination
// so a stage reads the adjoint once and writes it once, like the forward.
#pragma once
#include "igr2d_kernels.cuh"

namespace igrgpu {

// Local-source coefficients per node: S_loc = C a with
//   S_mux = a_mux C0 + a_muy C1 + a_E C2,  S_muy = a_mux C3 + a_muy C4 + a_E C5,
//   S_rho = a_mux C6 + a_muy C7 + a_E C8,  S_E = a_E C9.
constexpr int PDE_SRC = 10;
// Nonlocal-source primal fields per node: d_x u_x, d_x u_y, d_y u_x, d_y u_y
// (of the nodal velocity), d_x Sigma / rho, d_y Sigma / rho, R_tr.
constexpr int PDE_NL = 7;

struct PdePrepArgs2D {
  const Tile2D* tiles; const Inst2D* inst; BasisDev B;
  const double *q[4], *S;
  double* invr;            // 1 / rho
  double* src[PDE_SRC];
  double* nl[PDE_NL];      // nullptr entries: not needed (alpha = 0)
  double *ws_x, *ws_y;     // |u_x| + c, |u_y| + c
};

template <int NP>
__global__ void __launch_bounds__(Tiling2D<NP>::NT) k2_pde_prep(PdePrepArgs2D a) {
  using TL = Tiling2D<NP>;
  constexpr int TE = TL::TE, NN = TL::NN;
  // x-derivatives (physical) of mux, muy, rho, E, Sigma, u_x, u_y; 1/rho
  __shared__ double s_dx[7][TE][NN];
  __shared__ double s_ir[TE][NN];
  const Tile2D tl = a.tiles[blockIdx.x];
  const Inst2D I = a.inst[tl.inst];
  const ElemView vr = elem_view<NP>(tl, I, 0), vc = elem_view<NP>(tl, I, 1);
  const BasisDev& B = a.B;
  const double invJx = I.ijx, invJy = I.ijy;
  if (vr.valid) {
    const int t = vr.t, e = vr.e;
    double f[7][NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const long long n = vr.base + t * NP + i;
      const double r = a.q[2][n], ir = 1.0 / r;  // one FP64 divide per node, shared by both phases
      s_ir[e][t * NP + i] = ir;
      f[0][i] = a.q[0][n]; f[1][i] = a.q[1][n]; f[2][i] = r; f[3][i] = a.q[3][n]; f[4][i] = a.S[n];
      f[5][i] = f[0][i] * ir; f[6][i] = f[1][i] * ir;
    }
#pragma unroll
    for (int v = 0; v < 7; ++v)
#pragma unroll
      for (int i = 0; i < NP; ++i) s_dx[v][e][t * NP + i] = dot_row<NP>(B, i, f[v]) * invJx;
  }
  __syncthreads();
  if (!vc.valid) return;
  const int t = vc.t, e = vc.e;
  double f[7][NP];
#pragma unroll
  for (int l = 0; l < NP; ++l) {
    const long long n = vc.base + l * NP + t;
    const double ir = s_ir[e][l * NP + t];
    f[0][l] = a.q[0][n]; f[1][l] = a.q[1][n]; f[2][l] = a.q[2][n]; f[3][l] = a.q[3][n]; f[4][l] = a.S[n];
    f[5][l] = f[0][l] * ir; f[6][l] = f[1][l] * ir;
  }
  const double g = I.gamma, gm = g - 1.0;
#pragma unroll
  for (int l = 0; l < NP; ++l) {
    const long long n = vc.base + l * NP + t;
    const int nd = l * NP + t;
    const double mxx = s_dx[0][e][nd], myx = s_dx[1][e][nd], rx = s_dx[2][e][nd], Ex = s_dx[3][e][nd], Sx = s_dx[4][e][nd];
    const double mxy = dot_row<NP>(B, l, f[0]) * invJy, myy = dot_row<NP>(B, l, f[1]) * invJy;
    const double ry = dot_row<NP>(B, l, f[2]) * invJy, Ey = dot_row<NP>(B, l, f[3]) * invJy;
    const double Sy = dot_row<NP>(B, l, f[4]) * invJy;
    const double mx = f[0][l], my = f[1][l], en = f[3][l], Sg = f[4][l];
    const double ir = s_ir[e][nd], ir2 = ir * ir, ir3 = ir2 * ir;
    const double ux = f[5][l], uy = f[6][l];
    // quotient-rule velocity gradients of the local source (adjoint_pde.jl:163-164)
    const double uxx = (mxx - ux * rx) * ir, uyy = (myy - uy * ry) * ir;
    const double m2 = fma(mx, mx, my * my);
    const double P = gm * (en - m2 * (0.5 * ir));
    const double Hb = en + P + Sg;
    const double Pr = gm * fma(ux, ux, uy * uy) * 0.5;
    const double mdx = fma(mx, mxx, my * myx), mdy = fma(mx, mxy, my * myy);
    const double Pbx = fma(gm, Ex - mdx * ir + m2 * rx * (0.5 * ir2), Sx);
    const double Pby = fma(gm, Ey - mdy * ir + m2 * ry * (0.5 * ir2), Sy);
    const double dPx_dmx = gm * (mx * rx * ir2 - mxx * ir);
    const double dPx_dmy = gm * (my * rx * ir2 - myx * ir);
    const double dPx_dr = gm * (mdx * ir2 - m2 * rx * ir3);
    const double dPy_dmx = gm * (mx * ry * ir2 - mxy * ir);
    const double dPy_dmy = gm * (my * ry * ir2 - myy * ir);
    const double dPy_dr = gm * (mdy * ir2 - m2 * ry * ir3);
    const double HEx = Ex + Pbx, HEy = Ey + Pby;
    const double c0 = mxx * ir + uxx - mx * rx * ir2 + dPx_dmx + uyy;                                   // dmx/dmx
    const double c3 = dPx_dmy + mxy * ir - mx * ry * ir2;                                              // dmx/dmy
    const double c6 = -mxx * ux * ir + mx * (ux * rx * ir2 - uxx * ir) + dPx_dr - mxy * uy * ir +
                      mx * (uy * ry * ir2 - uyy * ir);                                                 // dmx/drho
    const double c1 = myx * ir - my * rx * ir2 + dPy_dmx;                                              // dmy/dmx
    const double c4 = uxx + myy * ir + uyy - my * ry * ir2 + dPy_dmy;                                  // dmy/dmy
    const double c7 = -myx * ux * ir + my * (ux * rx * ir2 - uxx * ir) - myy * uy * ir +
                      my * (uy * ry * ir2 - uyy * ir) + dPy_dr;                                        // dmy/drho
    const double c2 = dPx_dmx * ux + HEx * ir - gm * ux * uxx - Hb * rx * ir2 + dPy_dmx * uy - gm * ux * uyy;  // dE/dmx
    const double c5 = dPx_dmy * ux - gm * uy * uxx + dPy_dmy * uy + HEy * ir - gm * uy * uyy - Hb * ry * ir2;  // dE/dmy
    const double c8 = dPx_dr * ux - HEx * ux * ir + Pr * uxx + Hb * (ux * rx * ir2 - uxx * ir) + dPy_dr * uy -
                      HEy * uy * ir + Pr * uyy + Hb * (uy * ry * ir2 - uyy * ir);                      // dE/drho
    const double c9 = g * (uxx + uyy);                                                                 // dE/dE
    a.src[0][n] = c0; a.src[1][n] = c1; a.src[2][n] = c2; a.src[3][n] = c3; a.src[4][n] = c4;
    a.src[5][n] = c5; a.src[6][n] = c6; a.src[7][n] = c7; a.src[8][n] = c8; a.src[9][n] = c9;
    a.invr[n] = ir;
    const double cs = sqrt(g * P * ir);
    a.ws_x[n] = fabs(ux) + cs;
    a.ws_y[n] = fabs(uy) + cs;
    if (a.nl[0]) {
      // nodal-velocity gradients (adjoint_pde.jl:391-404)
      const double nxx = s_dx[5][e][nd], nyx = s_dx[6][e][nd];
      const double nxy = dot_row<NP>(B, l, f[5]) * invJy, nyy = dot_row<NP>(B, l, f[6]) * invJy;
      const double dv = nxx + nyy;
      double R = fma(dv, dv, nxx * nxx);
      R = fma(2.0 * nxy, nyx, R);
      R = fma(nyy, nyy, R);
      a.nl[0][n] = nxx; a.nl[1][n] = nyx; a.nl[2][n] = nxy; a.nl[3][n] = nyy;
      a.nl[4][n] = Sx * ir; a.nl[5][n] = Sy * ir; a.nl[6][n] = R;
    }
  }
}

// b = alpha w_i w_j Jx Jy (d_x a_mux + d_y a_muy + u_x d_x a_E + u_y d_y a_E)
struct PdeBArgs2D {
  const Tile2D* tiles; const Inst2D* inst; BasisDev B;
  const double *a[4], *mx, *my, *invr;
  double* b;
};

template <int NP>
__global__ void __launch_bounds__(Tiling2D<NP>::NT) k2_pde_b(PdeBArgs2D a) {
  using TL = Tiling2D<NP>;
  constexpr int TE = TL::TE, NN = TL::NN;
  __shared__ double s_d[2][TE][NN];  // d_x a_mux, d_x a_E
  const Tile2D tl = a.tiles[blockIdx.x];
  const Inst2D I = a.inst[tl.inst];
  const ElemView vr = elem_view<NP>(tl, I, 0), vc = elem_view<NP>(tl, I, 1);
  const BasisDev& B = a.B;
  if (vr.valid) {
    const int t = vr.t, e = vr.e;
    double am[NP], aE[NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) { const long long n = vr.base + t * NP + i; am[i] = a.a[0][n]; aE[i] = a.a[3][n]; }
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      s_d[0][e][t * NP + i] = dot_row<NP>(B, i, am) * I.ijx;
      s_d[1][e][t * NP + i] = dot_row<NP>(B, i, aE) * I.ijx;
    }
  }
  __syncthreads();
  if (!vc.valid) return;
  const int t = vc.t, e = vc.e;
  double am[NP], aE[NP];
#pragma unroll
  for (int l = 0; l < NP; ++l) { const long long n = vc.base + l * NP + t; am[l] = a.a[1][n]; aE[l] = a.a[3][n]; }
  const double cw = I.alpha * B.w[t] * I.jx * I.jy;
#pragma unroll
  for (int l = 0; l < NP; ++l) {
    const long long n = vc.base + l * NP + t;
    const int nd = l * NP + t;
    const double amy_y = dot_row<NP>(B, l, am) * I.ijy, aE_y = dot_row<NP>(B, l, aE) * I.ijy;
    const double ir = a.invr[n];
    const double ux = a.mx[n] * ir, uy = a.my[n] * ir;
    const double v = fma(aE_y, uy, fma(s_d[1][e][nd], ux, s_d[0][e][nd] + amy_y));
    a.b[n] = v * (cw * B.w[l]);
  }
}

// Adjoint DG operator + sources + SSP-RK3 stage:
//   k = +(1/Jx) D fx + (1/Jy) D fy + face terms - C a + S_Sigma,
//   a_out = c0 a^n + c1 a_s + c2 dt k.
struct PdeRkArgs2D {
  const Tile2D* tiles; const Inst2D* inst; BasisDev B;
  const double *q[4], *S, *invr, *ws_x, *ws_y;   // snapshot
  const double* src[PDE_SRC];
  const double* nl[PDE_NL];
  const double* Pi;                              // nullptr: no nonlocal source (alpha = 0)
  const double *a[4];                            // stage input
  const double *an[4];                           // step start (read when c0 != 0)
  double c0, c1, c2;
  double* ao[4];                                 // stage output (may alias an, not a)
  double* k_out[4];                              // optional: the raw operator k
};

// Adjoint flux F_dag in both directions at one node (adjoint_pde.jl:41-80).
struct AdjFlux { double fx[4], fy[4]; };
__device__ __forceinline__ AdjFlux pde_adjoint_flux(double g, double mx, double my, double r, double E, double S,
                                                    double ir, const double a[4]) {
  const double gm = g - 1.0;
  const double ux = mx * ir, uy = my * ir;
  const double P = gm * (E - fma(mx, mx, my * my) * (0.5 * ir));
  const double Hr = (E + P + S) * ir;            // H_bar / rho
  const double Pr = gm * fma(ux, ux, uy * uy) * 0.5;
  const double amu = fma(a[0], ux, a[1] * uy);   // (a_mu . mu) / rho
  const double aEg = a[3] * gm;
  AdjFlux F;
  // x: P_mux = -gm ux, P_muy = -gm uy
  F.fx[0] = fma(a[3], Hr, amu + a[0] * ux - gm * ux * a[0] + a[2]) - aEg * ux * ux;
  F.fx[1] = a[1] * ux - gm * uy * a[0] - aEg * uy * ux;
  F.fx[2] = fma(a[3] * ux, Pr - Hr, Pr * a[0] - ux * amu);
  F.fx[3] = fma(gm, a[0], a[3] * g * ux);
  F.fy[0] = a[0] * uy - gm * ux * a[1] - aEg * ux * uy;
  F.fy[1] = fma(a[3], Hr, amu + a[1] * uy - gm * uy * a[1] + a[2]) - aEg * uy * uy;
  F.fy[2] = fma(a[3] * uy, Pr - Hr, Pr * a[1] - uy * amu);
  F.fy[3] = fma(gm, a[1], a[3] * g * uy);
  return F;
}

struct AdjFace { double a[4], f[4], ws; };

template <int NP>
__global__ void __launch_bounds__(Tiling2D<NP>::NT) k2_pde_rk(PdeRkArgs2D a) {
  using TL = Tiling2D<NP>;
  constexpr int TE = TL::TE, NN = TL::NN, L = TL::L, TX = TL::TX, TY = TL::TY;
  __shared__ double s_fy[4][TE][NN];    // adjoint y fluxes
  __shared__ double s_k[4][TE][NN];     // operator, x part
  __shared__ double s_a[4][TE][NN];     // adjoint stage input
  __shared__ double s_w[3][TE][NN];     // x-derivative parts of W_x, W_y, div C
  __shared__ AdjFace s_xf[TE][NP][2];   // x-face node data (left, right) per row
  const Tile2D tl = a.tiles[blockIdx.x];
  const Inst2D I = a.inst[tl.inst];
  const ElemView vr = elem_view<NP>(tl, I, 0), vc = elem_view<NP>(tl, I, 1);
  const BasisDev& B = a.B;
  const double g = I.gamma;
  const double invJx = I.ijx, invJy = I.ijy;
  const bool nonlocal = a.Pi != nullptr;

  // ---- phase 1 (row of vr): adjoint fluxes, x volume term, x-face data, x parts of the nonlocal source
  if (vr.valid) {
    const int t = vr.t, e = vr.e;
    double fx[4][NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const long long n = vr.base + t * NP + i;
      const double av[4] = {a.a[0][n], a.a[1][n], a.a[2][n], a.a[3][n]};
      const AdjFlux F = pde_adjoint_flux(g, a.q[0][n], a.q[1][n], a.q[2][n], a.q[3][n], a.S[n], a.invr[n], av);
#pragma unroll
      for (int c = 0; c < 4; ++c) { fx[c][i] = F.fx[c]; s_fy[c][e][t * NP + i] = F.fy[c]; s_a[c][e][t * NP + i] = av[c]; }
      if (i == 0 || i == L) {
        AdjFace& fs = s_xf[e][t][i == 0 ? 0 : 1];
#pragma unroll
        for (int c = 0; c < 4; ++c) { fs.a[c] = av[c]; fs.f[c] = F.fx[c]; }
        fs.ws = a.ws_x[n];
      }
    }
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
      for (int i = 0; i < NP; ++i) s_k[c][e][t * NP + i] = invJx * dot_row<NP>(B, i, fx[c]);
    if (nonlocal) {
      double pd[NP], pxx[NP], pxy[NP], cx[NP];
#pragma unroll
      for (int i = 0; i < NP; ++i) {
        const long long n = vr.base + t * NP + i;
        const double P = a.Pi[n], nxx = a.nl[0][n], nxy = a.nl[2][n], nyy = a.nl[3][n];
        pd[i] = P * (nxx + nyy); pxx[i] = P * nxx; pxy[i] = P * nxy; cx[i] = P * a.nl[4][n];
      }
#pragma unroll
      for (int i = 0; i < NP; ++i) {
        s_w[0][e][t * NP + i] = dot_row<NP>(B, i, pd) * invJx + dot_row<NP>(B, i, pxx) * invJx;
        s_w[1][e][t * NP + i] = dot_row<NP>(B, i, pxy) * invJx;
        s_w[2][e][t * NP + i] = dot_row<NP>(B, i, cx) * invJx;
      }
    }
  }
  __syncthreads();
  // ---- phase 2 (row of vr): x faces; adjoint LLF (adjoint_pde.jl:89-128) with the
  // forward's face signs flipped (:275-289); the owner computes its side
  if (vr.valid) {
    const int t = vr.t, e = vr.e;
    auto fetch = [&](int s) {
      int it;
      const long long pb = neighbour<NP>(tl, I, vr.ex, vr.ey, s == 0 ? -1 : 1, 0, &it);
      AdjFace pf;
      if (it >= 0) {
        pf = s_xf[it][t][s == 0 ? 1 : 0];
      } else {
        const long long n = pb + t * NP + (s == 0 ? L : 0);
#pragma unroll
        for (int c = 0; c < 4; ++c) pf.a[c] = a.a[c][n];
        const AdjFlux F = pde_adjoint_flux(g, a.q[0][n], a.q[1][n], a.q[2][n], a.q[3][n], a.S[n], a.invr[n], pf.a);
#pragma unroll
        for (int c = 0; c < 4; ++c) pf.f[c] = F.fx[c];
        pf.ws = a.ws_x[n];
      }
      return pf;
    };
    const int sf = first_side(vr.ext, TX);
    const AdjFace pA = fetch(sf), pB = fetch(1 - sf);
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const AdjFace& pf = (s == sf) ? pA : pB;
      const AdjFace& of = s_xf[e][t][s];
      const AdjFace& Ls = s == 0 ? pf : of;
      const AdjFace& Rs = s == 0 ? of : pf;
      const double lam = max_nonneg(Rs.ws, Ls.ws);
      const int io = s == 0 ? 0 : L;
      const double cf = s == 0 ? -invJx * B.iw0 : invJx * B.iwL;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const double fs = 0.5 * fma(-lam, Ls.a[c] - Rs.a[c], Ls.f[c] + Rs.f[c]);
        s_k[c][e][t * NP + io] = fma(cf, fs - of.f[c], s_k[c][e][t * NP + io]);
      }
    }
  }
  __syncthreads();
  if (!vc.valid) return;
  // ---- phase 3 (column of vc): y volume term, y faces, sources, RK combination
  const int t = vc.t, e = vc.e;
  double kc[4][NP];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    double fyc[NP];
#pragma unroll
    for (int l = 0; l < NP; ++l) fyc[l] = s_fy[c][e][l * NP + t];
#pragma unroll
    for (int l = 0; l < NP; ++l) kc[c][l] = fma(invJy, dot_row<NP>(B, l, fyc), s_k[c][e][l * NP + t]);
  }
  auto own_y = [&](int s) {
    const int nd = (s == 0 ? 0 : L) * NP + t;
    AdjFace f;
#pragma unroll
    for (int c = 0; c < 4; ++c) { f.a[c] = s_a[c][e][nd]; f.f[c] = s_fy[c][e][nd]; }
    f.ws = a.ws_y[vc.base + nd];
    return f;
  };
  auto fetchy = [&](int s) {
    int it;
    const long long pb = neighbour<NP>(tl, I, vc.ex, vc.ey, 0, s == 0 ? -1 : 1, &it);
    const int nd = (s == 0 ? L : 0) * NP + t;
    AdjFace pf;
    if (it >= 0) {
#pragma unroll
      for (int c = 0; c < 4; ++c) { pf.a[c] = s_a[c][it][nd]; pf.f[c] = s_fy[c][it][nd]; }
    } else {
      const long long n = pb + nd;
#pragma unroll
      for (int c = 0; c < 4; ++c) pf.a[c] = a.a[c][n];
      const AdjFlux F = pde_adjoint_flux(g, a.q[0][n], a.q[1][n], a.q[2][n], a.q[3][n], a.S[n], a.invr[n], pf.a);
#pragma unroll
      for (int c = 0; c < 4; ++c) pf.f[c] = F.fy[c];
    }
    pf.ws = a.ws_y[pb + nd];
    return pf;
  };
  const int sf = first_side(vc.eyt, TY);
  const AdjFace qA = fetchy(sf), qB = fetchy(1 - sf);
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const AdjFace& pf = (s == sf) ? qA : qB;
    const AdjFace of = own_y(s);
    const AdjFace& Ls = s == 0 ? pf : of;
    const AdjFace& Rs = s == 0 ? of : pf;
    const double lam = max_nonneg(Rs.ws, Ls.ws);
    const int lo = s == 0 ? 0 : L;
    const double cf = s == 0 ? -invJy * B.iw0 : invJy * B.iwL;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const double fs = 0.5 * fma(-lam, Ls.a[c] - Rs.a[c], Ls.f[c] + Rs.f[c]);
      kc[c][lo] = fma(cf, fs - of.f[c], kc[c][lo]);
    }
  }
  // nonlocal source, y parts (adjoint_pde.jl:420-466)
  double Wx[NP], Wy[NP], dC[NP];
  if (nonlocal) {
    double pd[NP], pyx[NP], pyy[NP], cy[NP];
#pragma unroll
    for (int l = 0; l < NP; ++l) {
      const long long n = vc.base + l * NP + t;
      const double P = a.Pi[n], nxx = a.nl[0][n], nyx = a.nl[1][n], nyy = a.nl[3][n];
      pd[l] = P * (nxx + nyy); pyx[l] = P * nyx; pyy[l] = P * nyy; cy[l] = P * a.nl[5][n];
    }
#pragma unroll
    for (int l = 0; l < NP; ++l) {
      const int nd = l * NP + t;
      Wx[l] = s_w[0][e][nd] + dot_row<NP>(B, l, pyx) * invJy;
      Wy[l] = (dot_row<NP>(B, l, pd) * invJy + s_w[1][e][nd]) + dot_row<NP>(B, l, pyy) * invJy;
      dC[l] = s_w[2][e][nd] + dot_row<NP>(B, l, cy) * invJy;
    }
  }
  const double c2dt = a.c2 * I.dt;
#pragma unroll
  for (int l = 0; l < NP; ++l) {
    const long long n = vc.base + l * NP + t;
    const int nd = l * NP + t;
    const double a0 = s_a[0][e][nd], a1 = s_a[1][e][nd], a2 = s_a[2][e][nd], a3 = s_a[3][e][nd];
    // minus the local source
    kc[0][l] -= fma(a0, a.src[0][n], fma(a1, a.src[1][n], a3 * a.src[2][n]));
    kc[1][l] -= fma(a0, a.src[3][n], fma(a1, a.src[4][n], a3 * a.src[5][n]));
    kc[2][l] -= fma(a0, a.src[6][n], fma(a1, a.src[7][n], a3 * a.src[8][n]));
    kc[3][l] -= a3 * a.src[9][n];
    if (nonlocal) {
      const double ir = a.invr[n];
      kc[0][l] += -2.0 * Wx[l] * ir;
      kc[1][l] += -2.0 * Wy[l] * ir;
      const double wm = fma(Wx[l], a.q[0][n], Wy[l] * a.q[1][n]);
      kc[2][l] += fma(a.Pi[n], a.nl[6][n], dC[l]) * ir + 2.0 * wm * (ir * ir);
    }
    const double as[4] = {a0, a1, a2, a3};
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      if (a.k_out[c]) a.k_out[c][n] = kc[c][l];
      double val = fma(c2dt, kc[c][l], a.c1 * as[c]);
      if (a.c0 != 0.0) val = fma(a.c0, a.an[c][n], val);
      if (a.ao[c]) a.ao[c][n] = val;
    }
  }
}

}  // namespace igrgpu
