// 2D discrete-adjoint (reverse-mode) kernels: the transpose of every forward
// kernel in igr2d_kernels.cuh, in the same tile / line-per-thread layout.
//
// What the reference gets from Enzyme (IGR_adjoints_2d/enzyme_adjoint.jl:270-296)
// is built here by hand, primitive by primitive:
//   k2_hyp_rev    reverse of the LLF/DG hyperbolic RHS and of the SSP-RK3
//                 stage combination; its epilogue starts the reverse of the
//                 fixed-count solver (the last iteration is pointwise);
//   k2_apply_rev  one reverse solver iteration: A u for the residual adjoint u
//                 (A is symmetric, elliptic.jl:30-145) plus the adjoint of the
//                 operator coefficients, d(u^T A(rho, alpha) x_k), against the
//                 taped iterate x_k;
//   k2_setup_rev  reverse of the IGR source (elliptic.jl:159-197) and of
//                 diag(A) (elliptic.jl:205-264), closing d/d rho and d/d alpha.
// Conventions at kinks follow the reference's Float64 Base functions:
// d|u|/du = +1 at u = +0.0, and max(a, b) differentiates into a on ties.
//
// Coefficient adjoints are carried as Z = (1/rho) * d(.)/d(1/rho) so that the
// stored coefficients (all proportional to 1/rho) are reused directly:
// Zm collects the mass part, Zs the alpha-proportional stiffness/face part;
// then d/d rho = -Z/rho and d/d alpha = Zs/alpha.
#pragma once
#include "igr2d_kernels.cuh"

namespace igrgpu {

// Reverse of node_flux (one direction) at one node: fb = adjoint of the 4 flux
// components; accumulates into qb[4], Sb and gb.
__device__ __forceinline__ void node_flux_rev(int dir, double g, double mx, double my, double E, double S, double ir,
                                              const double fb[4], double qb[4], double& Sb, double& gb) {
  const double ux = mx * ir, uy = my * ir;
  const double kin = fma(mx, mx, my * my) * (0.5 * ir);
  const double P = (g - 1.0) * (E - kin);
  const double pb = P + S;
  const double un = dir == 0 ? ux : uy;
  const double unb = fma(fb[0], mx, fma(fb[1], my, fb[3] * (E + pb)));
  double pbb;
  if (dir == 0) {
    pbb = fma(fb[3], un, fb[0]);
    qb[0] += fma(fb[0], un, fb[2]);
    qb[1] += fb[1] * un;
  } else {
    pbb = fma(fb[3], un, fb[1]);
    qb[0] += fb[0] * un;
    qb[1] += fma(fb[1], un, fb[2]);
  }
  qb[3] += fb[3] * un;
  Sb += pbb;
  // un = m_n / rho
  qb[dir] += unb * ir;
  qb[2] -= unb * un * ir;
  // P = (g-1)(E - kin), kin = |m|^2 / (2 rho)
  gb += pbb * (E - kin);
  const double gm1 = g - 1.0;
  qb[3] += pbb * gm1;
  const double kb = -pbb * gm1;
  qb[0] += kb * ux;
  qb[1] += kb * uy;
  qb[2] -= kb * kin * ir;
}

// Reverse of |u_n| + sqrt(g P / rho) at one node with adjoint wb.
__device__ __forceinline__ void wavespeed_rev(int dir, double g, double mx, double my, double E, double ir, double wb,
                                              double qb[4], double& gb) {
  const double ux = mx * ir, uy = my * ir;
  const double kin = fma(mx, mx, my * my) * (0.5 * ir);
  const double P = (g - 1.0) * (E - kin);
  const double un = dir == 0 ? ux : uy;
  const double unb = signbit(un) ? -wb : wb;
  qb[dir] += unb * ir;
  qb[2] -= unb * un * ir;
  const double X = g * P * ir;
  const double Xb = wb * 0.5 * rsqrt(X);
  gb += Xb * P * ir;
  const double Pb = Xb * g * ir;
  qb[2] -= Xb * X * ir;
  gb += Pb * (E - kin);
  qb[3] += Pb * (g - 1.0);
  const double kb = -Pb * (g - 1.0);
  qb[0] += kb * ux;
  qb[1] += kb * uy;
  qb[2] -= kb * kin * ir;
}

enum { SREV_NONE = 0, SREV_CHEB = 1, SREV_JACOBI = 2 };

// ---------------------------------------------------------------------------
// Reverse of k2_hyp_rk for one stage.
//   forward: q_out = c0 q^n + c1 q_s + c2 dt k(q_s, Sigma)
//   given A = adjoint of q_out:
//     Qn  (+)= c0 A                        (qn_mode: 0 skip, 1 write, 2 add)
//     Qs  (+)= c1 A + H_q^T(c2 dt A)        (qs_add: add instead of write)
//     Sb  (+)= H_S^T(c2 dt A)               (Sb_add)
//     gnode += d/dgamma
// Solver prologue (SREV_CHEB / SREV_JACOBI) with xb = Sb total: produces the
// residual adjoint u = rb_{n-1} for the first k2_apply_rev, initialises the
// diag(A) adjoint Mb, and (Chebyshev) the direction adjoint db.
// ---------------------------------------------------------------------------
struct HypRevArgs2D {
  const Tile2D* tiles; const Inst2D* inst; BasisDev B;
  const double *q[4], *invr, *S;     // taped stage input and Sigma_out
  const double *A[4];                // adjoint of the stage output
  double c0, c1, c2;
  double *Qn[4]; int qn_mode;
  double *Qs[4]; int qs_add;
  double *Sb; int Sb_add;
  double *gnode;                     // per-node dJ/dgamma accumulator
  // solver prologue
  int srev;
  const double *cinvM, *r_last;      // taped r_{n-1}
  double *u_out, *db, *Mb;
  double ca, cc, omega;              // Chebyshev a_n, c_n ; Jacobi omega
};

template <int NP>
__global__ void __launch_bounds__(Tiling2D<NP>::NT) k2_hyp_rev(HypRevArgs2D a) {
  using TL = Tiling2D<NP>;
  constexpr int TE = TL::TE, NN = TL::NN, L = TL::L;
  __shared__ double s_kb[4][TE][NN];      // kbar = c2 dt A
  __shared__ double s_pq[6][TE][NN];      // row-phase partials: q (4), S, gamma
  __shared__ double s_xw[TE][NP][2];      // x wave speed at x-face nodes
  __shared__ double s_yw[TE][NP][2];
  const Tile2D tl = a.tiles[blockIdx.x];
  const Inst2D I = a.inst[tl.inst];
  const ElemView v = elem_view<NP>(tl, I);
  const BasisDev& B = a.B;
  const int t = v.t, e = v.e;
  const double g = I.gamma;
  const double invJx = I.ijx, invJy = I.ijy;
  const double c2dt = a.c2 * I.dt;

  double q[4][NP], S[NP], ir[NP], kb[4][NP];
  if (v.valid) {
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const long long n = v.base + t * NP + i;
#pragma unroll
      for (int c = 0; c < 4; ++c) { q[c][i] = a.q[c][n]; kb[c][i] = c2dt * a.A[c][n]; s_kb[c][e][t * NP + i] = kb[c][i]; }
      S[i] = a.S[n]; ir[i] = a.invr[n];
    }
    {
      double f[4], ws;
      node_flux(0, g, q[0][0], q[1][0], q[2][0], q[3][0], S[0], ir[0], f, &ws); s_xw[e][t][0] = ws;
      node_flux(0, g, q[0][L], q[1][L], q[2][L], q[3][L], S[L], ir[L], f, &ws); s_xw[e][t][1] = ws;
    }
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const long long n = v.base + (s == 0 ? 0 : L) * NP + t;
      double f[4], ws;
      node_flux(1, g, a.q[0][n], a.q[1][n], a.q[2][n], a.q[3][n], a.S[n], a.invr[n], f, &ws);
      s_yw[e][t][s] = ws;
    }
  }
  __syncthreads();
  if (v.valid) {
    // ---- row t: F̄x = transpose of the x volume term, x-face LLF reverse, flux reverse
    double Fb[4][NP];
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
      for (int k = 0; k < NP; ++k) Fb[c][k] = -invJx * dot_col<NP>(B, k, kb[c], 0.0);
    double qbr[4][NP], Sbr[NP], gb = 0.0;
#pragma unroll
    for (int i = 0; i < NP; ++i) { Sbr[i] = 0.0;
#pragma unroll
      for (int c = 0; c < 4; ++c) qbr[c][i] = 0.0; }
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int io = s == 0 ? 0 : L;            // own face node
      int it;
      const long long pb = neighbour<NP>(tl, I, v.ex, v.ey, s == 0 ? -1 : 1, 0, &it);
      const int pi = s == 0 ? L : 0;
      const long long pn = pb + t * NP + pi;
      double pq[4], pkb[4], pws;
#pragma unroll
      for (int c = 0; c < 4; ++c) pq[c] = a.q[c][pn];
      if (it >= 0) {
#pragma unroll
        for (int c = 0; c < 4; ++c) pkb[c] = s_kb[c][it][t * NP + pi];
        pws = s_xw[it][t][s == 0 ? 1 : 0];
      } else {
#pragma unroll
        for (int c = 0; c < 4; ++c) pkb[c] = c2dt * a.A[c][pn];
        double f[4];
        node_flux(0, g, pq[0], pq[1], pq[2], pq[3], a.S[pn], a.invr[pn], f, &pws);
      }
      const double ows = s_xw[e][t][s];
      // correction coefficients: R side (node 0) +invJx/w0, L side (node L) -invJx/wL
      const double cfo = s == 0 ? invJx * B.iw0 : -invJx * B.iwL;
      const double cfp = s == 0 ? -invJx * B.iwL : invJx * B.iw0;
      const double wsL = s == 0 ? pws : ows, wsR = s == 0 ? ows : pws;
      const double lam = (wsR > wsL) ? wsR : wsL;
      const bool own_wins = (s == 0) ? (wsR > wsL) : !(wsR > wsL);
      double lamb = 0.0;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const double fsb = fma(cfo, kb[c][io], cfp * pkb[c]);
        Fb[c][io] = fma(-cfo, kb[c][io], Fb[c][io]) + 0.5 * fsb;
        const double qL = s == 0 ? pq[c] : q[c][io], qR = s == 0 ? q[c][io] : pq[c];
        qbr[c][io] += (s == 0 ? -0.5 : 0.5) * lam * fsb;
        lamb = fma(0.5 * fsb, qL - qR, lamb);
      }
      if (own_wins) {
        double qq[4] = {0, 0, 0, 0};
        wavespeed_rev(0, g, q[0][io], q[1][io], q[3][io], ir[io], lamb, qq, gb);
#pragma unroll
        for (int c = 0; c < 4; ++c) qbr[c][io] += qq[c];
      }
    }
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      double fb[4] = {Fb[0][i], Fb[1][i], Fb[2][i], Fb[3][i]};
      double qq[4] = {qbr[0][i], qbr[1][i], qbr[2][i], qbr[3][i]};
      node_flux_rev(0, g, q[0][i], q[1][i], q[3][i], S[i], ir[i], fb, qq, Sbr[i], gb);
#pragma unroll
      for (int c = 0; c < 4; ++c) s_pq[c][e][t * NP + i] = qq[c];
      s_pq[4][e][t * NP + i] = Sbr[i];
    }
#pragma unroll
    for (int i = 0; i < NP; ++i) s_pq[5][e][t * NP + i] = (i == 0) ? gb : 0.0;
  }
  __syncthreads();
  if (!v.valid) return;
  // ---- column t: F̄y, y-face LLF reverse, flux reverse, combination, outputs
  double cq[4][NP], cS[NP], cir[NP], ckb[4][NP];
#pragma unroll
  for (int l = 0; l < NP; ++l) {
    const long long n = v.base + l * NP + t;
#pragma unroll
    for (int c = 0; c < 4; ++c) { cq[c][l] = a.q[c][n]; ckb[c][l] = s_kb[c][e][l * NP + t]; }
    cS[l] = a.S[n]; cir[l] = a.invr[n];
  }
  double Fb[4][NP];
#pragma unroll
  for (int c = 0; c < 4; ++c)
#pragma unroll
    for (int k = 0; k < NP; ++k) Fb[c][k] = -invJy * dot_col<NP>(B, k, ckb[c], 0.0);
  double qbc[4][NP], gb = 0.0;
#pragma unroll
  for (int l = 0; l < NP; ++l)
#pragma unroll
    for (int c = 0; c < 4; ++c) qbc[c][l] = 0.0;
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const int lo = s == 0 ? 0 : L;
    int it;
    const long long pb = neighbour<NP>(tl, I, v.ex, v.ey, 0, s == 0 ? -1 : 1, &it);
    const int pl = s == 0 ? L : 0;
    const long long pn = pb + pl * NP + t;
    double pq[4], pkb[4], pws;
#pragma unroll
    for (int c = 0; c < 4; ++c) pq[c] = a.q[c][pn];
    if (it >= 0) {
#pragma unroll
      for (int c = 0; c < 4; ++c) pkb[c] = s_kb[c][it][pl * NP + t];
      pws = s_yw[it][t][s == 0 ? 1 : 0];
    } else {
#pragma unroll
      for (int c = 0; c < 4; ++c) pkb[c] = c2dt * a.A[c][pn];
      double f[4];
      node_flux(1, g, pq[0], pq[1], pq[2], pq[3], a.S[pn], a.invr[pn], f, &pws);
    }
    const double ows = s_yw[e][t][s];
    const double cfo = s == 0 ? invJy * B.iw0 : -invJy * B.iwL;
    const double cfp = s == 0 ? -invJy * B.iwL : invJy * B.iw0;
    const double wsL = s == 0 ? pws : ows, wsR = s == 0 ? ows : pws;
    const double lam = (wsR > wsL) ? wsR : wsL;
    const bool own_wins = (s == 0) ? (wsR > wsL) : !(wsR > wsL);
    double lamb = 0.0;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const double fsb = fma(cfo, ckb[c][lo], cfp * pkb[c]);
      Fb[c][lo] = fma(-cfo, ckb[c][lo], Fb[c][lo]) + 0.5 * fsb;
      const double qL = s == 0 ? pq[c] : cq[c][lo], qR = s == 0 ? cq[c][lo] : pq[c];
      qbc[c][lo] += (s == 0 ? -0.5 : 0.5) * lam * fsb;
      lamb = fma(0.5 * fsb, qL - qR, lamb);
    }
    if (own_wins) {
      double qq[4] = {0, 0, 0, 0};
      wavespeed_rev(1, g, cq[0][lo], cq[1][lo], cq[3][lo], cir[lo], lamb, qq, gb);
#pragma unroll
      for (int c = 0; c < 4; ++c) qbc[c][lo] += qq[c];
    }
  }
  double gsum = 0.0;
#pragma unroll
  for (int l = 0; l < NP; ++l) {
    const long long n = v.base + l * NP + t;
    double fb[4] = {Fb[0][l], Fb[1][l], Fb[2][l], Fb[3][l]};
    double qq[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) qq[c] = qbc[c][l] + s_pq[c][e][l * NP + t];
    double Sb = s_pq[4][e][l * NP + t];
    node_flux_rev(1, g, cq[0][l], cq[1][l], cq[3][l], cS[l], cir[l], fb, qq, Sb, gb);
    gsum += s_pq[5][e][l * NP + t];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const double Av = a.A[c][n];
      if (a.qn_mode == 1) a.Qn[c][n] = a.c0 * Av;
      else if (a.qn_mode == 2) a.Qn[c][n] = fma(a.c0, Av, a.Qn[c][n]);
      const double val = fma(a.c1, Av, qq[c]);
      a.Qs[c][n] = a.qs_add ? a.Qs[c][n] + val : val;
    }
    const double Sbt = a.Sb_add ? a.Sb[n] + Sb : Sb;
    a.Sb[n] = Sbt;
    if (a.srev == SREV_CHEB) {
      // x_n = x_{n-1} + d_n ; d_n = a_n d_{n-1} + c_n z_n ; z_n = M^-1 r_{n-1}
      const double zb = a.cc * Sbt;
      const double u = a.cinvM[n] * zb;
      a.u_out[n] = u;
      a.Mb[n] = -u * a.r_last[n] * a.cinvM[n];
      a.db[n] = a.ca * Sbt;
    } else if (a.srev == SREV_JACOBI) {
      // x_n = x_{n-1} + omega M^-1 r_{n-1}
      const double u = a.omega * Sbt * a.cinvM[n];
      a.u_out[n] = u;
      a.Mb[n] = -u * a.r_last[n] * a.cinvM[n];
    }
  }
  a.gnode[v.base + t] += gb + gsum;
}

// ---------------------------------------------------------------------------
// One reverse solver iteration m: u = residual adjoint r̄_m, x_m taped.
//   xb -= A u ; bb (+)= u ; Zm/Zs (+)= -(mass / stiffness+face parts of
//   d(u^T A x_m) in Z form); then the solver epilogue builds r̄_{m-1}.
// ---------------------------------------------------------------------------
struct ApplyRevArgs2D {
  const Tile2D* tiles; const Inst2D* inst; BasisDev B;
  const double *u, *xk;               // residual adjoint and taped iterate
  const double *cm, *ckx, *cky, *cpx, *cpy, *cinvM, *invr;
  double *xb, *bb, *Zm, *Zs;
  int first;                          // first reverse iteration of this solve: write bb, Zm, Zs
  double zscale;                      // -1 for r = b - A x terms
  // epilogue (when has_next): r̄_{m-1}
  int has_next;
  const double* r_prev;               // taped r_{m-1}
  double *u_out, *db, *Mb;
  double ca, cc, omega;
};

template <int NP, int SREV>
__global__ void __launch_bounds__(Tiling2D<NP>::NT) k2_apply_rev(ApplyRevArgs2D a) {
  using TL = Tiling2D<NP>;
  constexpr int TE = TL::TE, NN = TL::NN, L = TL::L;
  __shared__ double s_u[TE][NN], s_v[TE][NN], s_yx[TE][NN], s_zr[TE][NN];
  __shared__ double s_gxf[2][TE][NP][2], s_gyf[2][TE][NP][2];  // [u|v] face derivatives
  const Tile2D tl = a.tiles[blockIdx.x];
  const Inst2D I = a.inst[tl.inst];
  const ElemView v = elem_view<NP>(tl, I);
  const BasisDev& B = a.B;
  const int t = v.t, e = v.e;
  const double hw = B.hw;

  double ur[NP], vr[NP], gxu[NP], gxv[NP];
  double uc[NP], vc[NP], gyu[NP], gyv[NP];
  if (v.valid) {
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const long long n = v.base + t * NP + i;
      ur[i] = a.u[n]; vr[i] = a.xk[n];
      s_u[e][t * NP + i] = ur[i]; s_v[e][t * NP + i] = vr[i];
    }
#pragma unroll
    for (int i = 0; i < NP; ++i) { gxu[i] = dot_row<NP>(B, i, ur); gxv[i] = dot_row<NP>(B, i, vr); }
    s_gxf[0][e][t][0] = gxu[0]; s_gxf[0][e][t][1] = gxu[L];
    s_gxf[1][e][t][0] = gxv[0]; s_gxf[1][e][t][1] = gxv[L];
  }
  __syncthreads();
  if (v.valid) {
#pragma unroll
    for (int l = 0; l < NP; ++l) { uc[l] = s_u[e][l * NP + t]; vc[l] = s_v[e][l * NP + t]; }
#pragma unroll
    for (int l = 0; l < NP; ++l) { gyu[l] = dot_row<NP>(B, l, uc); gyv[l] = dot_row<NP>(B, l, vc); }
    s_gyf[0][e][t][0] = gyu[0]; s_gyf[0][e][t][1] = gyu[L];
    s_gyf[1][e][t][0] = gyv[0]; s_gyf[1][e][t][1] = gyv[L];

    // ---- row t: x faces
    double kxr[NP], zr[NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) { kxr[i] = a.ckx[v.base + t * NP + i]; zr[i] = kxr[i] * gxu[i] * gxv[i]; }
    double pu[2], pv[2], pdu[2], pdv[2], pk[2], pir[2];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      int it;
      const long long pb = neighbour<NP>(tl, I, v.ex, v.ey, s == 0 ? -1 : 1, 0, &it);
      const int pi = s == 0 ? L : 0;
      pk[s] = a.ckx[pb + t * NP + pi];
      pir[s] = a.invr[pb + t * NP + pi];
      if (it >= 0) {
        pu[s] = s_u[it][t * NP + pi]; pv[s] = s_v[it][t * NP + pi];
        pdu[s] = s_gxf[0][it][t][s == 0 ? 1 : 0]; pdv[s] = s_gxf[1][it][t][s == 0 ? 1 : 0];
      } else {
        double pr[NP], pw[NP];
#pragma unroll
        for (int k = 0; k < NP; ++k) { pr[k] = a.u[pb + t * NP + k]; pw[k] = a.xk[pb + t * NP + k]; }
        pu[s] = pr[pi]; pv[s] = pw[pi];
        pdu[s] = dot_row<NP>(B, pi, pr); pdv[s] = dot_row<NP>(B, pi, pw);
      }
    }
    const double irl0 = a.invr[v.base + t * NP], irlL = a.invr[v.base + t * NP + L];
    // left face (own R side, node 0)
    const double jul = pu[0] - ur[0], jvl = pv[0] - vr[0];
    const double pl_ = a.cpx[v.base + t * NP];
    const double Fl = fma(pl_, jul, hw * fma(pk[0], pdu[0], kxr[0] * gxu[0]));
    zr[0] = fma(hw * kxr[0], fma(gxv[0], jul, gxu[0] * jvl), zr[0]);
    if (irl0 > pir[0]) zr[0] = fma(pl_ * jvl, jul, zr[0]);  // R wins only when strictly larger
    // right face (own L side, node L)
    const double jur = ur[L] - pu[1], jvr = vr[L] - pv[1];
    const double pr_ = a.cpx[v.base + t * NP + L];
    const double Fr = fma(pr_, jur, hw * fma(kxr[L], gxu[L], pk[1] * pdu[1]));
    zr[L] = fma(hw * kxr[L], fma(gxv[L], jur, gxu[L] * jvr), zr[L]);
    if (!(pir[1] > irlL)) zr[L] = fma(pr_ * jvr, jur, zr[L]);
    double sx[NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) sx[i] = kxr[i] * gxu[i];
    sx[0] = kxr[0] * fma(hw, jul, gxu[0]);
    sx[L] = kxr[L] * fma(hw, jur, gxu[L]);
#pragma unroll
    for (int k = 0; k < NP; ++k) {
      const double acc = (k == 0) ? -Fl : ((k == L) ? Fr : 0.0);
      s_yx[e][t * NP + k] = dot_col<NP>(B, k, sx, acc);
      s_zr[e][t * NP + k] = zr[k];
    }
  }
  __syncthreads();
  if (!v.valid) return;
  // ---- column t: y faces, transposes, outputs
  double kyc[NP], zc[NP];
#pragma unroll
  for (int l = 0; l < NP; ++l) { kyc[l] = a.cky[v.base + l * NP + t]; zc[l] = kyc[l] * gyu[l] * gyv[l]; }
  double qu[2], qv[2], qdu[2], qdv[2], qk[2], qir[2];
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    int it;
    const long long pb = neighbour<NP>(tl, I, v.ex, v.ey, 0, s == 0 ? -1 : 1, &it);
    const int pl = s == 0 ? L : 0;
    qk[s] = a.cky[pb + pl * NP + t];
    qir[s] = a.invr[pb + pl * NP + t];
    if (it >= 0) {
      qu[s] = s_u[it][pl * NP + t]; qv[s] = s_v[it][pl * NP + t];
      qdu[s] = s_gyf[0][it][t][s == 0 ? 1 : 0]; qdv[s] = s_gyf[1][it][t][s == 0 ? 1 : 0];
    } else {
      double pc[NP], pw[NP];
#pragma unroll
      for (int k = 0; k < NP; ++k) { pc[k] = a.u[pb + k * NP + t]; pw[k] = a.xk[pb + k * NP + t]; }
      qu[s] = pc[pl]; qv[s] = pw[pl];
      qdu[s] = dot_row<NP>(B, pl, pc); qdv[s] = dot_row<NP>(B, pl, pw);
    }
  }
  const double ic0 = a.invr[v.base + t], icL = a.invr[v.base + L * NP + t];
  const double jub = qu[0] - uc[0], jvb = qv[0] - vc[0];
  const double pbot = a.cpy[v.base + t];
  const double Fb = fma(pbot, jub, hw * fma(qk[0], qdu[0], kyc[0] * gyu[0]));
  zc[0] = fma(hw * kyc[0], fma(gyv[0], jub, gyu[0] * jvb), zc[0]);
  if (ic0 > qir[0]) zc[0] = fma(pbot * jvb, jub, zc[0]);
  const double jut = uc[L] - qu[1], jvt = vc[L] - qv[1];
  const double ptop = a.cpy[v.base + L * NP + t];
  const double Ft = fma(ptop, jut, hw * fma(kyc[L], gyu[L], qk[1] * qdu[1]));
  zc[L] = fma(hw * kyc[L], fma(gyv[L], jut, gyu[L] * jvt), zc[L]);
  if (!(qir[1] > icL)) zc[L] = fma(ptop * jvt, jut, zc[L]);
  double sy[NP];
#pragma unroll
  for (int l = 0; l < NP; ++l) sy[l] = kyc[l] * gyu[l];
  sy[0] = kyc[0] * fma(hw, jub, gyu[0]);
  sy[L] = kyc[L] * fma(hw, jut, gyu[L]);
#pragma unroll
  for (int l = 0; l < NP; ++l) {
    const long long n = v.base + l * NP + t;
    const double cmn = a.cm[n];
    double w = fma(cmn, uc[l], s_yx[e][l * NP + t] + ((l == 0) ? -Fb : ((l == L) ? Ft : 0.0)));
    w = dot_col<NP>(B, l, sy, w);
    const double zm = a.zscale * (cmn * uc[l] * vc[l]);
    const double zs = a.zscale * (zc[l] + s_zr[e][l * NP + t]);
    const double xb = a.xb[n] - w;
    a.xb[n] = xb;
    if (a.first) { a.bb[n] = uc[l]; a.Zm[n] = zm; a.Zs[n] = zs; }
    else { a.bb[n] += uc[l]; a.Zm[n] += zm; a.Zs[n] += zs; }
    if (SREV == SREV_CHEB && a.has_next) {
      const double dbv = a.db[n] + xb;
      const double u = a.cinvM[n] * (a.cc * dbv);
      a.u_out[n] = u;
      a.Mb[n] -= u * a.r_prev[n] * a.cinvM[n];
      a.db[n] = a.ca * dbv;
    } else if (SREV == SREV_JACOBI && a.has_next) {
      const double u = a.omega * xb * a.cinvM[n];
      a.u_out[n] = u;
      a.Mb[n] -= u * a.r_prev[n] * a.cinvM[n];
    }
  }
}

// ---------------------------------------------------------------------------
// Reverse of the stage setup: IGR source b and diag(A), plus the conversion of
// the coefficient adjoints (Zm, Zs) into d/d rho and d/d alpha.
//   Qs[mx], Qs[my], Qs[rho] += ...      anode += dJ/dalpha contributions
// ---------------------------------------------------------------------------
struct SetupRevArgs2D {
  const Tile2D* tiles; const Inst2D* inst; BasisDev B;
  const double *mx, *my, *invr;       // taped stage input
  const double *b, *cm, *cM;          // taped source, mass coefficient, diag(A)
  const double *bb, *Mb, *Zm, *Zs;
  double *Qs[3];                      // adjoints of (mx, my, rho) of the stage input
  double *anode;
};

template <int NP>
__global__ void __launch_bounds__(Tiling2D<NP>::NT) k2_setup_rev(SetupRevArgs2D a) {
  using TL = Tiling2D<NP>;
  constexpr int TE = TL::TE, NN = TL::NN, L = TL::L;
  __shared__ double s_ux[TE][NN], s_uy[TE][NN], s_Mb[TE][NN];
  __shared__ double s_uxx[TE][NN], s_uyx[TE][NN];       // x derivatives (row phase)
  __shared__ double s_bxx[TE][NN], s_byx[TE][NN];       // adjoints of uxx, uyx (column phase)
  __shared__ double s_ir[TE][NN], s_ib[TE][NN];         // 1/rho; row-phase d/d(1/rho) from diag(A)
  const Tile2D tl = a.tiles[blockIdx.x];
  const Inst2D I = a.inst[tl.inst];
  const ElemView v = elem_view<NP>(tl, I);
  const BasisDev& B = a.B;
  const int t = v.t, e = v.e;
  const double invJx = I.ijx, invJy = I.ijy;
  const double alpha = I.alpha;
  if (alpha <= 0.0) return;
  const double eta = (double)(NP * NP);

  double ux[NP], uy[NP], Mbr[NP];
  if (v.valid) {
    const double cxs = alpha * B.w[t] * I.jy * invJx;
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const long long n = v.base + t * NP + i;
      const double ir = a.invr[n];
      ux[i] = a.mx[n] * ir; uy[i] = a.my[n] * ir; Mbr[i] = a.Mb[n];
      s_ux[e][t * NP + i] = ux[i]; s_uy[e][t * NP + i] = uy[i]; s_Mb[e][t * NP + i] = Mbr[i]; s_ir[e][t * NP + i] = ir;
    }
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      s_uxx[e][t * NP + i] = dot_row<NP>(B, i, ux) * invJx;
      s_uyx[e][t * NP + i] = dot_row<NP>(B, i, uy) * invJx;
      // x stiffness self-coupling of diag(A): d/d(1/rho[i,t]) = cxs * sum_k W2[i][k] Mb[k,t]
      double s = B.W2[i][0] * Mbr[0];
#pragma unroll
      for (int k = 1; k < NP; ++k) s = fma(B.W2[i][k], Mbr[k], s);
      s_ib[e][t * NP + i] = cxs * s;
    }
  }
  __syncthreads();
  // ---- column t: y derivatives, source adjoint, y transposes, diag(A) y part and faces
  double cux[NP], cuy[NP], cMb[NP], cir[NP];
  double uxb[NP], uyb[NP], ib[NP];
  if (v.valid) {
#pragma unroll
    for (int l = 0; l < NP; ++l) {
      cux[l] = s_ux[e][l * NP + t]; cuy[l] = s_uy[e][l * NP + t]; cMb[l] = s_Mb[e][l * NP + t]; cir[l] = s_ir[e][l * NP + t];
      uxb[l] = 0.0; uyb[l] = 0.0;
    }
    const double cys = alpha * B.w[t] * I.jx * invJy;
    double bxy[NP], byy[NP];
#pragma unroll
    for (int l = 0; l < NP; ++l) {
      const long long n = v.base + l * NP + t;
      const double uxy = dot_row<NP>(B, l, cux) * invJy, uyy = dot_row<NP>(B, l, cuy) * invJy;
      const double uxx = s_uxx[e][l * NP + t], uyx = s_uyx[e][l * NP + t];
      const double s = uxx + uyy;
      const double Qb = a.bb[n] * (B.w[t] * B.w[l] * I.jx * I.jy * alpha);
      s_bxx[e][l * NP + t] = Qb * 2.0 * (s + uxx);
      s_byx[e][l * NP + t] = Qb * 2.0 * uxy;
      bxy[l] = Qb * 2.0 * uyx * invJy;
      byy[l] = Qb * 2.0 * (s + uyy) * invJy;
      // y stiffness self-coupling of diag(A)
      double sm = B.W2[l][0] * cMb[0];
#pragma unroll
      for (int k = 1; k < NP; ++k) sm = fma(B.W2[l][k], cMb[k], sm);
      ib[l] = cys * sm;
    }
    // y transposes of the source adjoint: ux[t,k] gets D[l][k] * bxy[l]
#pragma unroll
    for (int k = 0; k < NP; ++k) { uxb[k] = dot_col<NP>(B, k, bxy, uxb[k]); uyb[k] = dot_col<NP>(B, k, byy, uyb[k]); }
    // diag(A) face terms, x faces (t == 0: own R side; t == L: own L side)
    if (t == 0 || t == L) {
      int it;
      const long long pb = neighbour<NP>(tl, I, v.ex, v.ey, t == 0 ? -1 : 1, 0, &it);
      const int pi = t == 0 ? L : 0;
#pragma unroll
      for (int l = 0; l < NP; ++l) {
        const double pir = it >= 0 ? s_ir[it][l * NP + pi] : a.invr[pb + l * NP + pi];
        const double pMb = it >= 0 ? s_Mb[it][l * NP + pi] : a.Mb[pb + l * NP + pi];
        const double wf = B.w[l] * I.jy;
        ib[l] += cMb[l] * (t == L ? -alpha * invJx * B.D[L][L] : alpha * invJx * B.D[0][0]) * wf;
        const double iL = t == L ? cir[l] : pir, iR = t == L ? pir : cir[l];
        const bool own_wins = (t == L) ? !(iR > iL) : (iR > iL);
        if (own_wins) ib[l] += (cMb[l] + pMb) * alpha * wf * eta * I.idx;
      }
    }
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int l = s == 0 ? 0 : L;
      int it;
      const long long pb = neighbour<NP>(tl, I, v.ex, v.ey, 0, s == 0 ? -1 : 1, &it);
      const int pl = s == 0 ? L : 0;
      const double pir = it >= 0 ? s_ir[it][pl * NP + t] : a.invr[pb + pl * NP + t];
      const double pMb = it >= 0 ? s_Mb[it][pl * NP + t] : a.Mb[pb + pl * NP + t];
      const double wf = B.w[t] * I.jx;
      ib[l] += cMb[l] * (l == L ? -alpha * invJy * B.D[L][L] : alpha * invJy * B.D[0][0]) * wf;
      const double iL = l == L ? cir[l] : pir, iR = l == L ? pir : cir[l];
      const bool own_wins = (l == L) ? !(iR > iL) : (iR > iL);
      if (own_wins) ib[l] += (cMb[l] + pMb) * alpha * wf * eta * I.idy;
    }
  }
  __syncthreads();
  if (!v.valid) return;
  // ---- column t, final: x transposes of the source adjoint (need row data),
  // mass part of diag(A), conversion to d/d rho and d/d alpha
#pragma unroll
  for (int l = 0; l < NP; ++l) {
    // ux[t,l] gets sum_i D[i][t] * bxx[i,l] * invJx (row l, x transpose at node t)
    double rx[NP], ry[NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) { rx[i] = s_bxx[e][l * NP + i]; ry[i] = s_byx[e][l * NP + i]; }
    double sxv = 0.0, syv = 0.0;
#pragma unroll
    for (int i = 0; i < NP; ++i) { sxv = fma(B.D[i][t], rx[i], sxv); syv = fma(B.D[i][t], ry[i], syv); }
    uxb[l] = fma(invJx, sxv, uxb[l]);
    uyb[l] = fma(invJx, syv, uyb[l]);
  }
#pragma unroll
  for (int l = 0; l < NP; ++l) {
    const long long n = v.base + l * NP + t;
    const double ir = cir[l];
    const double Mb = cMb[l];
    const double cmn = a.cm[n];
    // d/d(1/rho) of diag(A): mass + row-phase x stiffness + column-phase y stiffness and faces
    const double m0 = B.w[t] * B.w[l] * I.jx * I.jy;  // mass coefficient without 1/rho
    const double ibt = fma(Mb, m0, s_ib[e][l * NP + t] + ib[l]);
    const double zm = a.Zm[n], zs = a.Zs[n];
    a.Qs[0][n] += uxb[l] * ir;
    a.Qs[1][n] += uyb[l] * ir;
    const double rb = -(fma(uxb[l], cux[l], uyb[l] * cuy[l]) * ir) - ir * fma(ibt, ir, zm + zs);
    a.Qs[2][n] += rb;
    // d/dalpha: Zs/alpha + Mb (M - mass)/alpha + bb b/alpha
    a.anode[n] += fma(Mb, a.cM[n] - cmn, fma(a.bb[n], a.b[n], zs)) * I.ialpha;
  }
}

}  // namespace igrgpu
