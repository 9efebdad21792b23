// 2D discrete-adjoint (reverse-mode) kernels: the transpose of every forward
// kernel in igr2d_kernels.cuh, in the same tile / line-per-thread layout and
// with the same phase-dependent thread mapping (elem_view).
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
// Zm collects the mass part without its coefficient (the sum over the
// solve's reverse applies of +-u x, which k2_setup_rev multiplies by the mass
// coefficient once, instead of every apply), Zs the alpha-proportional
// stiffness/face part; then d/d rho = -Z/rho and d/d alpha = Zs/alpha.
#pragma once
#include "igr2d_kernels.cuh"

namespace igrgpu {

// Reverse of node_phys for both flux directions at one node: fbx, fby are
// the adjoints of the x and y flux components; accumulates into qb[4]
// (mx, my, rho, E), Sb and gb.
__device__ __forceinline__ void node_phys_rev(double g, double mx, double my, double E, double S, double ir,
                                              const double fbx[4], const double fby[4], double qb[4], double& Sb,
                                              double& gb) {
  const double ux = mx * ir, uy = my * ir;
  const double kin = fma(mx, mx, my * my) * (0.5 * ir);
  const double gm1 = g - 1.0;
  const double P = gm1 * (E - kin), pb = P + S, epb = E + pb;
  // fx = (mx ux + pb, my ux, mx, (E+pb) ux), fy = (mx uy, my uy + pb, my, (E+pb) uy)
  const double uxb = fma(fbx[0], mx, fma(fbx[1], my, fbx[3] * epb));
  const double uyb = fma(fby[0], mx, fma(fby[1], my, fby[3] * epb));
  const double e3 = fma(fbx[3], ux, fby[3] * uy);   // d/dE through E + pb, and part of d/d pb
  const double pbb = fbx[0] + fby[1] + e3;
  qb[0] += fma(fbx[0], ux, fma(fby[0], uy, fbx[2]));
  qb[1] += fma(fby[1], uy, fma(fbx[1], ux, fby[2]));
  qb[3] += e3;
  Sb += pbb;
  // u = m / rho
  qb[0] += uxb * ir;
  qb[1] += uyb * ir;
  qb[2] -= fma(uxb, ux, uyb * uy) * ir;
  // P = (g-1)(E - kin), kin = |m|^2 / (2 rho)
  gb = fma(pbb, E - kin, gb);
  qb[3] = fma(pbb, gm1, qb[3]);
  const double kb = -pbb * gm1;
  qb[0] = fma(kb, ux, qb[0]);
  qb[1] = fma(kb, uy, qb[1]);
  qb[2] -= kb * kin * ir;
}

// Reverse of |u_n| + sqrt(g P / rho) at one node with adjoint wb; c is the sound speed.
__device__ __forceinline__ void wavespeed_rev(int dir, double g, double mx, double my, double E, double ir, double c,
                                              double wb, double qb[4], double& gb) {
  const double ux = mx * ir, uy = my * ir;
  const double kin = fma(mx, mx, my * my) * (0.5 * ir);
  const double P = (g - 1.0) * (E - kin);
  const double un = dir == 0 ? ux : uy;
  const double unb = signbit(un) ? -wb : wb;
  qb[dir] += unb * ir;
  qb[2] -= unb * un * ir;
  // c = sqrt(X), X = g P / rho:  dX = wb / (2 c)
  const double Xb = wb * 0.5 / c;
  const double X = c * c;
  gb = fma(Xb, P * ir, gb);
  const double Pb = Xb * g * ir;
  qb[2] -= Xb * X * ir;
  gb = fma(Pb, E - kin, gb);
  qb[3] = fma(Pb, g - 1.0, qb[3]);
  const double kb = -Pb * (g - 1.0);
  qb[0] = fma(kb, ux, qb[0]);
  qb[1] = fma(kb, uy, qb[1]);
  qb[2] -= kb * kin * ir;
}

enum { SREV_NONE = 0, SREV_CHEB = 1, SREV_JACOBI = 2, SREV_PCG = 3 };

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
// adjoint iMb of 1/diag(A) (the forward multiplies by the stored reciprocal),
// and (Chebyshev) the direction adjoint db.
// ---------------------------------------------------------------------------
struct HypRevArgs2D {
  const Tile2D* tiles; const Inst2D* inst; BasisDev B;
  const double *q[4], *invr, *S;     // taped stage input and Sigma_out
  const double *ws_x, *ws_y;         // taped LLF wave speeds at face nodes
  const double *A[4];                // adjoint of the stage output
  double c0, c1, c2;
  double *Qn[4]; int qn_mode;
  double *Qs[4]; int qs_add;
  double *Sb; int Sb_add;
  double *gnode;                     // per-node dJ/dgamma accumulator
  // solver prologue
  int srev;
  const double *cinvM, *r_last;      // taped r_{n-1}
  double *u_out, *db, *iMb;
  double ca, cc, omega;              // Chebyshev a_n, c_n ; Jacobi omega
};

template <int NP>
__global__ void __launch_bounds__(Tiling2D<NP>::NT) k2_hyp_rev(HypRevArgs2D a) {
  using TL = Tiling2D<NP>;
  constexpr int TE = TL::TE, NN = TL::NN, L = TL::L, TX = TL::TX, TY = TL::TY;
  __shared__ double s_kb[4][TE][NN];      // kbar = c2 dt A
  __shared__ double s_q[4][TE][NN];       // taped stage state
  __shared__ double s_fbx[4][TE][NN];     // adjoint of the x fluxes (row phase)
  __shared__ double s_qbx[4][TE][NN];     // q adjoint from the x faces (row phase)
  __shared__ double s_xw[TE][NP][2];      // x wave speed at x-face nodes
  __shared__ double s_yw[TE][NP][2];
  __shared__ double s_grow[TE][NP];       // row-phase d/dgamma partials
  const Tile2D tl = a.tiles[blockIdx.x];
  const Inst2D I = a.inst[tl.inst];
  const ElemView vr = elem_view<NP>(tl, I, 0), vc = elem_view<NP>(tl, I, 1);
  const BasisDev& B = a.B;
  const double g = I.gamma;
  const double invJx = I.ijx, invJy = I.ijy;
  const double c2dt = a.c2 * I.dt;

  // ---- phase 1: row data of vr into smem; face wave speeds
  if (vr.valid) {
    const int t = vr.t, e = vr.e;
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const long long n = vr.base + t * NP + i;
#pragma unroll
      for (int c = 0; c < 4; ++c) { s_q[c][e][t * NP + i] = a.q[c][n]; s_kb[c][e][t * NP + i] = c2dt * a.A[c][n]; }
    }
    s_xw[e][t][0] = a.ws_x[vr.base + t * NP];
    s_xw[e][t][1] = a.ws_x[vr.base + t * NP + L];
  }
  if (vc.valid) {
    s_yw[vc.e][vc.t][0] = a.ws_y[vc.base + vc.t];
    s_yw[vc.e][vc.t][1] = a.ws_y[vc.base + L * NP + vc.t];
  }
  __syncthreads();
  // Reverse of one face's LLF flux for the own side: kb/pkb are the RHS
  // adjoints at the own and partner face nodes; returns the flux adjoint
  // increment and accumulates the own-state adjoint.
  auto face_rev = [&](int dir, int s, const double oq[4], const double okb[4], double ows, double pws, const double pq[4],
                      const double pkb[4], double ir_own, double fb[4], double qbo[4], double& gb) {
    const double invJ = dir == 0 ? invJx : invJy;
    // correction coefficients: R side (node 0) +invJ/w0, L side (node L) -invJ/wL
    const double cfo = s == 0 ? invJ * B.iw0 : -invJ * B.iwL;
    const double cfp = s == 0 ? -invJ * B.iwL : invJ * B.iw0;
    const double wsL = s == 0 ? pws : ows, wsR = s == 0 ? ows : pws;
    const double lam = max_nonneg(wsR, wsL);
    const bool own_wins = (s == 0) ? gt_nonneg(wsR, wsL) : !gt_nonneg(wsR, wsL);
    double lamb = 0.0;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const double fsb = fma(cfo, okb[c], cfp * pkb[c]);
      fb[c] = fma(-cfo, okb[c], fb[c]) + 0.5 * fsb;
      const double dq = s == 0 ? pq[c] - oq[c] : oq[c] - pq[c];  // q_L - q_R
      qbo[c] = fma((s == 0 ? -0.5 : 0.5) * lam, fsb, qbo[c]);
      lamb = fma(0.5 * fsb, dq, lamb);
    }
    if (own_wins) {
      const double un = (dir == 0 ? oq[0] : oq[1]) * ir_own;
      wavespeed_rev(dir, g, oq[0], oq[1], oq[3], ir_own, ows - fabs(un), lamb, qbo, gb);
    }
  };
  double gb = 0.0;
  // ---- phase 2a (row of vr): x flux adjoint = transpose of the x volume term + x-face LLF reverse
  if (vr.valid) {
    const int t = vr.t, e = vr.e;
    double kb[4][NP], fb[4][NP], qbo[4][NP];
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
      for (int i = 0; i < NP; ++i) { kb[c][i] = s_kb[c][e][t * NP + i]; qbo[c][i] = 0.0; }
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
      for (int k = 0; k < NP; ++k) fb[c][k] = -invJx * dot_col<NP>(B, k, kb[c], 0.0);
    struct PF { double q[4], kb[4], ws; };
    auto fetch = [&](int s) {
      PF P;
      int it;
      const long long pb = neighbour<NP>(tl, I, vr.ex, vr.ey, s == 0 ? -1 : 1, 0, &it);
      const int pi = s == 0 ? L : 0;
      if (it >= 0) {
#pragma unroll
        for (int c = 0; c < 4; ++c) { P.q[c] = s_q[c][it][t * NP + pi]; P.kb[c] = s_kb[c][it][t * NP + pi]; }
        P.ws = s_xw[it][t][s == 0 ? 1 : 0];
      } else {
        const long long pn = pb + t * NP + pi;
#pragma unroll
        for (int c = 0; c < 4; ++c) { P.q[c] = a.q[c][pn]; P.kb[c] = c2dt * a.A[c][pn]; }
        P.ws = a.ws_x[pn];
      }
      return P;
    };
    const int sf = first_side(vr.ext, TX);
    const PF pA = fetch(sf), pB = fetch(1 - sf);
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const PF& P = (s == sf) ? pA : pB;
      const int io = s == 0 ? 0 : L;
      double oq[4], okb[4], f4[4], q4[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) { oq[c] = s_q[c][e][t * NP + io]; okb[c] = kb[c][io]; f4[c] = fb[c][io]; q4[c] = qbo[c][io]; }
      face_rev(0, s, oq, okb, s_xw[e][t][s], P.ws, P.q, P.kb, a.invr[vr.base + t * NP + io], f4, q4, gb);
#pragma unroll
      for (int c = 0; c < 4; ++c) { fb[c][io] = f4[c]; qbo[c][io] = q4[c]; }
    }
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
      for (int i = 0; i < NP; ++i) { s_fbx[c][e][t * NP + i] = fb[c][i]; s_qbx[c][e][t * NP + i] = qbo[c][i]; }
    s_grow[e][t] = gb;
    gb = 0.0;
  }
  // ---- phase 2b (column of vc): y flux adjoint + y-face LLF reverse (registers)
  double fby[4][NP], qby[4][NP];
  if (vc.valid) {
    const int t = vc.t, e = vc.e;
    double kb[4][NP];
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
      for (int l = 0; l < NP; ++l) { kb[c][l] = s_kb[c][e][l * NP + t]; qby[c][l] = 0.0; }
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
      for (int k = 0; k < NP; ++k) fby[c][k] = -invJy * dot_col<NP>(B, k, kb[c], 0.0);
    struct PF { double q[4], kb[4], ws; };
    auto fetch = [&](int s) {
      PF P;
      int it;
      const long long pb = neighbour<NP>(tl, I, vc.ex, vc.ey, 0, s == 0 ? -1 : 1, &it);
      const int pl = s == 0 ? L : 0;
      if (it >= 0) {
#pragma unroll
        for (int c = 0; c < 4; ++c) { P.q[c] = s_q[c][it][pl * NP + t]; P.kb[c] = s_kb[c][it][pl * NP + t]; }
        P.ws = s_yw[it][t][s == 0 ? 1 : 0];
      } else {
        const long long pn = pb + pl * NP + t;
#pragma unroll
        for (int c = 0; c < 4; ++c) { P.q[c] = a.q[c][pn]; P.kb[c] = c2dt * a.A[c][pn]; }
        P.ws = a.ws_y[pn];
      }
      return P;
    };
    const int sf = first_side(vc.eyt, TY);
    const PF pA = fetch(sf), pB = fetch(1 - sf);
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const PF& P = (s == sf) ? pA : pB;
      const int lo = s == 0 ? 0 : L;
      double oq[4], okb[4], f4[4], q4[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) { oq[c] = s_q[c][e][lo * NP + t]; okb[c] = kb[c][lo]; f4[c] = fby[c][lo]; q4[c] = qby[c][lo]; }
      face_rev(1, s, oq, okb, s_yw[e][t][s], P.ws, P.q, P.kb, a.invr[vc.base + lo * NP + t], f4, q4, gb);
#pragma unroll
      for (int c = 0; c < 4; ++c) { fby[c][lo] = f4[c]; qby[c][lo] = q4[c]; }
    }
  }
  __syncthreads();
  if (!vc.valid) return;
  // ---- phase 3 (column of vc): merged flux reverse per node, combination, outputs
  const int t = vc.t, e = vc.e;
  gb += s_grow[e][t];
#pragma unroll
  for (int l = 0; l < NP; ++l) {
    const long long n = vc.base + l * NP + t;
    const int nd = l * NP + t;
    double fbx[4], fbyl[4], qq[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) { fbx[c] = s_fbx[c][e][nd]; fbyl[c] = fby[c][l]; qq[c] = qby[c][l] + s_qbx[c][e][nd]; }
    double Sb = 0.0;
    node_phys_rev(g, s_q[0][e][nd], s_q[1][e][nd], s_q[3][e][nd], a.S[n], a.invr[n], fbx, fbyl, qq, Sb, gb);
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
      // x_n = x_{n-1} + d_n ; d_n = a_n d_{n-1} + c_n z_n ; z_n = (1/M) r_{n-1}
      const double zb = a.cc * Sbt;
      a.u_out[n] = a.cinvM[n] * zb;
      a.iMb[n] = zb * a.r_last[n];
      a.db[n] = a.ca * Sbt;
    } else if (a.srev == SREV_JACOBI) {
      // x_n = x_{n-1} + (omega r_{n-1}) (1/M)
      const double tb = a.omega * Sbt;
      a.u_out[n] = tb * a.cinvM[n];
      a.iMb[n] = tb * a.r_last[n];
    }
  }
  a.gnode[vc.base + t] += gb;
}

// ---------------------------------------------------------------------------
// One reverse solver iteration m: u = residual adjoint r̄_m, x_m taped.
//   xb -= A u ; bb (+)= u ; Zm/Zs (+)= -(mass / stiffness+face parts of
//   d(u^T A x_m) in Z form); then the solver epilogue builds r̄_{m-1}.
// ---------------------------------------------------------------------------
struct ApplyRevArgs2D {
  const Tile2D* tiles; const Inst2D* inst; BasisDev B;
  const double *u, *xk;               // residual adjoint and taped iterate
  const double *gxk, *gyk;            // taped reference derivatives of x_k (null: recompute)
  const double *cm, *ckx, *cky, *cpx, *cpy, *cinvM, *invr;
  double *xb, *bb, *Zm, *Zs;
  int first;                          // first reverse apply of this solve: write Zm, Zs (else add)
  int bb_op;                          // bb: 0 untouched, 1 write u, 2 add u
  double zscale;                      // -1 for r = b - A x terms
  // epilogue (when has_next): r̄_{m-1}
  int has_next;
  const double* r_prev;               // taped r_{m-1}
  double *u_out, *db, *iMb;
  double ca, cc, omega;
  // SREV_PCG (reverse of A p_it, second half of the iteration reverse):
  //   u = -(adjoint of A p_it) = alpha_it rb - pApb p_it, formed on load from
  //   (u = rb, xk = p_it); xb = pb: pb += alpha_it xconst + pApb apk + A(adjoint of A p_it);
  //   with has_next, the tile's partial of pb . p_next (betab of the next reverse
  //   iteration) goes to partials[tile] and the instance's last block completes it (isum, mode 2)
  const double *al_it, *papb;  // per-instance alpha_it (tape) and the adjoint of pAp_it
  const double *xconst, *apk, *p_next;
  double* partials;
  InstSum isum;
};

// Partner data across one face for the reverse apply: values and end-node
// derivatives of u and of x_k, the partner's stiffness coefficient and 1/rho.
struct Partner2 { double u, v, du, dv, k, ir; };

template <int NP, int SREV>
__global__ void __launch_bounds__(Tiling2D<NP>::NT) k2_apply_rev(ApplyRevArgs2D a) {
  using TL = Tiling2D<NP>;
  constexpr int TE = TL::TE, NN = TL::NN, L = TL::L, TX = TL::TX, TY = TL::TY;
  constexpr bool PCG = SREV == SREV_PCG;
  constexpr int P2 = pow2_at_least(TL::NT);
  __shared__ double s_u[TE][NN], s_v[TE][NN], s_yx[TE][NN], s_zr[TE][NN];
  __shared__ double s_gxf[2][TE][NP][2], s_gyf[2][TE][NP][2];  // [u|v] face derivatives
  __shared__ double s_red[PCG ? P2 : 1];
  const Tile2D tl = a.tiles[blockIdx.x];
  const Inst2D I = a.inst[tl.inst];
  const ElemView vr = elem_view<NP>(tl, I, 0), vc = elem_view<NP>(tl, I, 1);
  const BasisDev& B = a.B;
  const double hw = B.hw;
  double pal = 0.0, ppb = 0.0;  // PCG: alpha_it and the adjoint of pAp_it
  if (PCG) {
    pal = a.al_it[tl.inst];
    ppb = a.papb[tl.inst];
  }
  // u at node n, given x_k there (PCG forms it from rb and p_it)
  auto ldu = [&](long long n, double xkv) -> double {
    if (PCG) return fma(pal, a.u[n], -ppb * xkv);
    return a.u[n];
  };

  double ur[NP], vr_[NP], gxu[NP], gxv[NP];
  const bool taped_g = !PCG && a.gxk != nullptr;
  if (vr.valid) {
    const int t = vr.t, e = vr.e;
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const long long n = vr.base + t * NP + i;
      vr_[i] = a.xk[n]; ur[i] = ldu(n, vr_[i]);
      s_u[e][t * NP + i] = ur[i]; s_v[e][t * NP + i] = vr_[i];
    }
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      gxu[i] = dot_row<NP>(B, i, ur);
      gxv[i] = taped_g ? a.gxk[vr.base + t * NP + i] : dot_row<NP>(B, i, vr_);
    }
    s_gxf[0][e][t][0] = gxu[0]; s_gxf[0][e][t][1] = gxu[L];
    s_gxf[1][e][t][0] = gxv[0]; s_gxf[1][e][t][1] = gxv[L];
  }
  __syncthreads();
  double uc[NP], vc_[NP], gyu[NP], gyv[NP];
  if (vc.valid) {
    const int t = vc.t, e = vc.e;
#pragma unroll
    for (int l = 0; l < NP; ++l) { uc[l] = s_u[e][l * NP + t]; vc_[l] = s_v[e][l * NP + t]; }
#pragma unroll
    for (int l = 0; l < NP; ++l) {
      gyu[l] = dot_row<NP>(B, l, uc);
      gyv[l] = taped_g ? a.gyk[vc.base + l * NP + t] : dot_row<NP>(B, l, vc_);
    }
    s_gyf[0][e][t][0] = gyu[0]; s_gyf[0][e][t][1] = gyu[L];
    s_gyf[1][e][t][0] = gyv[0]; s_gyf[1][e][t][1] = gyv[L];
  }
  if (vr.valid) {
    // ---- row of vr: x faces
    const int t = vr.t, e = vr.e;
    double kxr[NP], zr[NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) { kxr[i] = a.ckx[vr.base + t * NP + i]; zr[i] = kxr[i] * gxu[i] * gxv[i]; }
    auto fetch = [&](int s) {
      Partner2 P;
      int it;
      const long long pb = neighbour<NP>(tl, I, vr.ex, vr.ey, s == 0 ? -1 : 1, 0, &it);
      const int pi = s == 0 ? L : 0;
      P.k = a.ckx[pb + t * NP + pi];
      P.ir = a.invr[pb + t * NP + pi];
      if (it >= 0) {
        P.u = s_u[it][t * NP + pi]; P.v = s_v[it][t * NP + pi];
        P.du = s_gxf[0][it][t][s == 0 ? 1 : 0]; P.dv = s_gxf[1][it][t][s == 0 ? 1 : 0];
      } else {
        double pr[NP];
        if (taped_g) {
#pragma unroll
          for (int k = 0; k < NP; ++k) pr[k] = a.u[pb + t * NP + k];
          P.v = a.xk[pb + t * NP + pi];
          P.dv = a.gxk[pb + t * NP + pi];
        } else {
          double pw[NP];
#pragma unroll
          for (int k = 0; k < NP; ++k) { pw[k] = a.xk[pb + t * NP + k]; pr[k] = ldu(pb + t * NP + k, pw[k]); }
          P.v = s == 0 ? pw[L] : pw[0];
          P.dv = dot_end<NP>(B, s == 0, pw);
        }
        P.u = s == 0 ? pr[L] : pr[0];
        P.du = dot_end<NP>(B, s == 0, pr);
      }
      return P;
    };
    const int sf = first_side(vr.ext, TX);
    const Partner2 pA = fetch(sf), pB = fetch(1 - sf);
    const Partner2 pl = sf == 0 ? pA : pB, prt = sf == 0 ? pB : pA;
    const double irl0 = a.invr[vr.base + t * NP], irlL = a.invr[vr.base + t * NP + L];
    // left face (own R side, node 0)
    const double jul = pl.u - ur[0], jvl = pl.v - vr_[0];
    const double pl_ = a.cpx[vr.base + t * NP];
    const double Fl = fma(pl_, jul, hw * fma(pl.k, pl.du, kxr[0] * gxu[0]));
    zr[0] = fma(hw * kxr[0], fma(gxv[0], jul, gxu[0] * jvl), zr[0]);
    if (gt_nonneg(irl0, pl.ir)) zr[0] = fma(pl_ * jvl, jul, zr[0]);  // R wins only when strictly larger
    // right face (own L side, node L)
    const double jur = ur[L] - prt.u, jvr = vr_[L] - prt.v;
    const double pr_ = a.cpx[vr.base + t * NP + L];
    const double Fr = fma(pr_, jur, hw * fma(kxr[L], gxu[L], prt.k * prt.du));
    zr[L] = fma(hw * kxr[L], fma(gxv[L], jur, gxu[L] * jvr), zr[L]);
    if (!gt_nonneg(prt.ir, irlL)) zr[L] = fma(pr_ * jvr, jur, zr[L]);
    double sx[NP];
#pragma unroll
    for (int i = 1; i < L; ++i) sx[i] = kxr[i] * gxu[i];
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
  if (!PCG && !vc.valid) return;
  double part = 0.0;  // PCG: betab partial of this thread
  // ---- column of vc: y faces, transposes, outputs
  if (vc.valid) {
    const int t = vc.t, e = vc.e;
    double kyc[NP], zc[NP];
#pragma unroll
    for (int l = 0; l < NP; ++l) { kyc[l] = a.cky[vc.base + l * NP + t]; zc[l] = kyc[l] * gyu[l] * gyv[l]; }
    auto fetchy = [&](int s) {
      Partner2 P;
      int it;
      const long long pb = neighbour<NP>(tl, I, vc.ex, vc.ey, 0, s == 0 ? -1 : 1, &it);
      const int pl = s == 0 ? L : 0;
      P.k = a.cky[pb + pl * NP + t];
      P.ir = a.invr[pb + pl * NP + t];
      if (it >= 0) {
        P.u = s_u[it][pl * NP + t]; P.v = s_v[it][pl * NP + t];
        P.du = s_gyf[0][it][t][s == 0 ? 1 : 0]; P.dv = s_gyf[1][it][t][s == 0 ? 1 : 0];
      } else {
        double pc[NP];
        if (taped_g) {
#pragma unroll
          for (int k = 0; k < NP; ++k) pc[k] = a.u[pb + k * NP + t];
          P.v = a.xk[pb + pl * NP + t];
          P.dv = a.gyk[pb + pl * NP + t];
        } else {
          double pw[NP];
#pragma unroll
          for (int k = 0; k < NP; ++k) { pw[k] = a.xk[pb + k * NP + t]; pc[k] = ldu(pb + k * NP + t, pw[k]); }
          P.v = s == 0 ? pw[L] : pw[0];
          P.dv = dot_end<NP>(B, s == 0, pw);
        }
        P.u = s == 0 ? pc[L] : pc[0];
        P.du = dot_end<NP>(B, s == 0, pc);
      }
      return P;
    };
    const int sf = first_side(vc.eyt, TY);
    const Partner2 qA = fetchy(sf), qB = fetchy(1 - sf);
    const Partner2 qb = sf == 0 ? qA : qB, qt = sf == 0 ? qB : qA;
    const double ic0 = a.invr[vc.base + t], icL = a.invr[vc.base + L * NP + t];
    const double jub = qb.u - uc[0], jvb = qb.v - vc_[0];
    const double pbot = a.cpy[vc.base + t];
    const double Fb = fma(pbot, jub, hw * fma(qb.k, qb.du, kyc[0] * gyu[0]));
    zc[0] = fma(hw * kyc[0], fma(gyv[0], jub, gyu[0] * jvb), zc[0]);
    if (gt_nonneg(ic0, qb.ir)) zc[0] = fma(pbot * jvb, jub, zc[0]);
    const double jut = uc[L] - qt.u, jvt = vc_[L] - qt.v;
    const double ptop = a.cpy[vc.base + L * NP + t];
    const double Ft = fma(ptop, jut, hw * fma(kyc[L], gyu[L], qt.k * qt.du));
    zc[L] = fma(hw * kyc[L], fma(gyv[L], jut, gyu[L] * jvt), zc[L]);
    if (!gt_nonneg(qt.ir, icL)) zc[L] = fma(ptop * jvt, jut, zc[L]);
    double sy[NP];
#pragma unroll
    for (int l = 1; l < L; ++l) sy[l] = kyc[l] * gyu[l];
    sy[0] = kyc[0] * fma(hw, jub, gyu[0]);
    sy[L] = kyc[L] * fma(hw, jut, gyu[L]);
#pragma unroll
    for (int l = 0; l < NP; ++l) {
      const long long n = vc.base + l * NP + t;
      const double cmn = a.cm[n];
      const double syx = s_yx[e][l * NP + t];  // y-face flux at the end nodes only (l is compile-time)
      double w = fma(cmn, uc[l], (l == 0) ? syx - Fb : ((l == L) ? syx + Ft : syx));
      w = dot_col<NP>(B, l, sy, w);
      // zscale is -1 (r = b - A x) or +1 (A p): applied through operand signs, not a multiply
      const double uz = a.zscale > 0 ? uc[l] : -uc[l];
      const double zs = a.zscale > 0 ? zc[l] + s_zr[e][l * NP + t] : -(zc[l] + s_zr[e][l * NP + t]);
      double xb = a.xb[n] - w;
      if (PCG) xb = fma(ppb, a.apk[n], fma(pal, a.xconst[n], xb));
      a.xb[n] = xb;
      if (a.bb_op == 1) a.bb[n] = uc[l];
      else if (a.bb_op == 2) a.bb[n] += uc[l];
      if (a.first) { a.Zm[n] = uz * vc_[l]; a.Zs[n] = zs; }
      else { a.Zm[n] = fma(uz, vc_[l], a.Zm[n]); a.Zs[n] += zs; }
      if (PCG && a.has_next) part = fma(xb, a.p_next[n], part);
      if (SREV == SREV_CHEB && a.has_next) {
        const double dbv = a.db[n] + xb;
        const double zb = a.cc * dbv;
        a.u_out[n] = a.cinvM[n] * zb;
        a.iMb[n] = fma(zb, a.r_prev[n], a.iMb[n]);
        a.db[n] = a.ca * dbv;
      } else if (SREV == SREV_JACOBI && a.has_next) {
        const double tb = a.omega * xb;
        a.u_out[n] = tb * a.cinvM[n];
        a.iMb[n] = fma(tb, a.r_prev[n], a.iMb[n]);
      }
    }
  }
  if (PCG && a.has_next) {
    const double tot = block_sum<P2>(part, s_red);
    inst_sum_last_block(a.isum, tl.inst, I.ntiles, tot, a.partials, blockIdx.x, I.tile0, I.ntiles);
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
  const double *b, *cm, *cM, *cinvM;  // taped source, mass coefficient, diag(A), 1/diag(A)
  const double *bb, *iMb, *Zm, *Zs;   // iMb: adjoint of 1/diag(A)
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
  const ElemView vr = elem_view<NP>(tl, I, 0), vc = elem_view<NP>(tl, I, 1);
  const BasisDev& B = a.B;
  const double invJx = I.ijx, invJy = I.ijy;
  const double alpha = I.alpha;
  if (alpha <= 0.0) return;
  const double eta = (double)(NP * NP);

  if (vr.valid) {
    const int t = vr.t, e = vr.e;
    double ux[NP], uy[NP], Mbr[NP];
    const double cxs = alpha * B.w[t] * I.jy * invJx;
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const long long n = vr.base + t * NP + i;
      const double ir = a.invr[n];
      const double im = a.cinvM[n];
      ux[i] = a.mx[n] * ir; uy[i] = a.my[n] * ir; Mbr[i] = -(a.iMb[n] * im) * im;  // d/dM = -d/d(1/M) / M^2
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
  // ---- column of vc: y derivatives, source adjoint, y transposes, diag(A) y part and faces
  double cux[NP], cuy[NP], cMb[NP], cir[NP];
  double uxb[NP], uyb[NP], ib[NP];
  if (vc.valid) {
    const int t = vc.t, e = vc.e;
#pragma unroll
    for (int l = 0; l < NP; ++l) {
      cux[l] = s_ux[e][l * NP + t]; cuy[l] = s_uy[e][l * NP + t]; cMb[l] = s_Mb[e][l * NP + t]; cir[l] = s_ir[e][l * NP + t];
    }
    const double cys = alpha * B.w[t] * I.jx * invJy;
    double bxy[NP], byy[NP];
#pragma unroll
    for (int l = 0; l < NP; ++l) {
      const long long n = vc.base + l * NP + t;
      const double uxy = dot_row<NP>(B, l, cux) * invJy, uyy = dot_row<NP>(B, l, cuy) * invJy;
      const double uxx = s_uxx[e][l * NP + t], uyx = s_uyx[e][l * NP + t];
      const double s = uxx + uyy;
      const double Qb2 = 2.0 * a.bb[n] * (B.w[t] * B.w[l] * I.jx * I.jy * alpha);
      s_bxx[e][l * NP + t] = Qb2 * (s + uxx);
      s_byx[e][l * NP + t] = Qb2 * uxy;
      bxy[l] = Qb2 * uyx * invJy;
      byy[l] = Qb2 * (s + uyy) * invJy;
      // y stiffness self-coupling of diag(A)
      double sm = B.W2[l][0] * cMb[0];
#pragma unroll
      for (int k = 1; k < NP; ++k) sm = fma(B.W2[l][k], cMb[k], sm);
      ib[l] = cys * sm;
    }
    // y transposes of the source adjoint: ux[t,k] gets D[l][k] * bxy[l]
#pragma unroll
    for (int k = 0; k < NP; ++k) { uxb[k] = dot_col<NP>(B, k, bxy, 0.0); uyb[k] = dot_col<NP>(B, k, byy, 0.0); }
    // diag(A) face terms, x faces (t == 0: own R side; t == L: own L side)
    if (t == 0 || t == L) {
      int it;
      const long long pb = neighbour<NP>(tl, I, vc.ex, vc.ey, t == 0 ? -1 : 1, 0, &it);
      const int pi = t == 0 ? L : 0;
      const double cself = (t == L ? -alpha * invJx * B.D[L][L] : alpha * invJx * B.D[0][0]);
#pragma unroll
      for (int l = 0; l < NP; ++l) {
        const double pir = it >= 0 ? s_ir[it][l * NP + pi] : a.invr[pb + l * NP + pi];
        const long long pn = pb + l * NP + pi;
        const double pMb = it >= 0 ? s_Mb[it][l * NP + pi] : -(a.iMb[pn] * a.cinvM[pn]) * a.cinvM[pn];
        const double wf = B.w[l] * I.jy;
        ib[l] = fma(cMb[l] * cself, wf, ib[l]);
        const double iL = t == L ? cir[l] : pir, iR = t == L ? pir : cir[l];
        const bool own_wins = (t == L) ? !gt_nonneg(iR, iL) : gt_nonneg(iR, iL);
        if (own_wins) ib[l] = fma((cMb[l] + pMb) * alpha * wf, eta * I.idx, ib[l]);
      }
    }
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int l = s == 0 ? 0 : L;
      int it;
      const long long pb = neighbour<NP>(tl, I, vc.ex, vc.ey, 0, s == 0 ? -1 : 1, &it);
      const int pl = s == 0 ? L : 0;
      const double pir = it >= 0 ? s_ir[it][pl * NP + t] : a.invr[pb + pl * NP + t];
      const long long pn = pb + pl * NP + t;
      const double pMb = it >= 0 ? s_Mb[it][pl * NP + t] : -(a.iMb[pn] * a.cinvM[pn]) * a.cinvM[pn];
      const double wf = B.w[t] * I.jx;
      ib[l] = fma(cMb[l] * (l == L ? -alpha * invJy * B.D[L][L] : alpha * invJy * B.D[0][0]), wf, ib[l]);
      const double iL = l == L ? cir[l] : pir, iR = l == L ? pir : cir[l];
      const bool own_wins = (l == L) ? !gt_nonneg(iR, iL) : gt_nonneg(iR, iL);
      if (own_wins) ib[l] = fma((cMb[l] + pMb) * alpha * wf, eta * I.idy, ib[l]);
    }
  }
  __syncthreads();
  if (!vc.valid) return;
  // ---- column of vc, final: x transposes of the source adjoint (need row data),
  // mass part of diag(A), conversion to d/d rho and d/d alpha
  const int t = vc.t, e = vc.e;
#pragma unroll
  for (int l = 0; l < NP; ++l) {
    // ux[t,l] gets sum_i D[i][t] * bxx[i,l] * invJx (row l, x transpose at node t)
    double sxv = 0.0, syv = 0.0;
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      sxv = fma(B.D[i][t], s_bxx[e][l * NP + i], sxv);
      syv = fma(B.D[i][t], s_byx[e][l * NP + i], syv);
    }
    uxb[l] = fma(invJx, sxv, uxb[l]);
    uyb[l] = fma(invJx, syv, uyb[l]);
  }
#pragma unroll
  for (int l = 0; l < NP; ++l) {
    const long long n = vc.base + l * NP + t;
    const double ir = cir[l];
    const double Mb = cMb[l];
    const double cmn = a.cm[n];
    // d/d(1/rho) of diag(A): mass + row-phase x stiffness + column-phase y stiffness and faces
    const double m0 = B.w[t] * B.w[l] * I.jx * I.jy;  // mass coefficient without 1/rho
    const double ibt = fma(Mb, m0, s_ib[e][l * NP + t] + ib[l]);
    const double zs = a.Zs[n], zms = fma(cmn, a.Zm[n], zs);  // Zm + Zs, with Zm's mass coefficient
    a.Qs[0][n] += uxb[l] * ir;
    a.Qs[1][n] += uyb[l] * ir;
    const double rb = -(fma(uxb[l], cux[l], uyb[l] * cuy[l]) * ir) - ir * fma(ibt, ir, zms);
    a.Qs[2][n] += rb;
    // d/dalpha: Zs/alpha + Mb (M - mass)/alpha + bb b/alpha
    a.anode[n] += fma(Mb, a.cM[n] - cmn, fma(a.bb[n], a.b[n], zs)) * I.ialpha;
  }
}

}  // namespace igrgpu
