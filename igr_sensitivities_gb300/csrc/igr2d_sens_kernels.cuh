// 2D tangent (forward sensitivity) kernels: run_sensitivity of
// IGR_adjoints_2d/sensitivity.jl:353-413.
//
// Per RK stage the tangent needs, besides the primal stage:
//   k2_sens_rhs      the tangent elliptic source b_s (form 2,
//                    compute_sensitivity_elliptic_rhs!, sensitivity.jl:236-292),
//                    solved with the primal stage's operator (same rho, alpha)
//                    by the ordinary solver kernels;
//   k2_sens_hyp_rk   the tangent DG right-hand side
//                    (compute_sensitivity_hyperbolic_rhs!, sensitivity.jl:131-215)
//                    fused with the SSP-RK3 stage combination of the tangent.
// The tangent LLF flux uses the primal wave speed (sensitivity_llf_flux_x/_y,
// sensitivity.jl:85-118: no d lambda term); it is read from the face-node wave
// speeds the primal k2_hyp_rk of the same stage wrote.
// Same thread mapping as the primal kernels (one thread per element line).
#pragma once
#include "igr2d_kernels.cuh"

namespace igrgpu {

// ---------------------------------------------------------------------------
// Tangent elliptic source, form 2 (sensitivity.jl:236-292). Per node, with
// u = mu/rho, s_u = (zeta - u sigma)/rho (tangent velocity), r_s = sigma/rho:
//   Rp = alpha (div u^2 + ux_x^2 + 2 ux_y uy_x + uy_y^2)
//   Rs = alpha (2 div u div s_u + 2 (ux_x sx_x + ux_y sy_x + uy_x sx_y + uy_y sy_y))
//   b  = w_i w_j Jx Jy (Rs + r_s Rp - alpha (d_x r_s d_x Sigma + d_y r_s d_y Sigma) / rho)
// ---------------------------------------------------------------------------
struct SensRhsArgs2D {
  const Tile2D* tiles; const Inst2D* inst; BasisDev B;
  const double *q[3], *invr, *S;   // mu_x, mu_y, rho of the stage; 1/rho; solved Sigma
  const double *s[3];              // zeta_x, zeta_y, sigma (tangent of mu_x, mu_y, rho)
  double* b_out;
};

template <int NP>
__global__ void __launch_bounds__(Tiling2D<NP>::NT) k2_sens_rhs(SensRhsArgs2D a) {
  using TL = Tiling2D<NP>;
  constexpr int TE = TL::TE, NN = TL::NN;
  constexpr int NQ = 6;  // u_x, u_y, s_x, s_y, Sigma, sigma/rho
  __shared__ double s_v[NQ][TE][NN];
  __shared__ double s_dx[NQ][TE][NN];
  const Tile2D tl = a.tiles[blockIdx.x];
  const Inst2D I = a.inst[tl.inst];
  const ElemView vr = elem_view<NP>(tl, I, 0), vc = elem_view<NP>(tl, I, 1);
  const BasisDev& B = a.B;
  if (vr.valid) {
    const int t = vr.t, e = vr.e;
    double v[NQ][NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const long long n = vr.base + t * NP + i;
      const double ir = a.invr[n];
      const double ux = a.q[0][n] * ir, uy = a.q[1][n] * ir, sr = a.s[2][n];
      v[0][i] = ux; v[1][i] = uy;
      v[2][i] = (a.s[0][n] - ux * sr) * ir;
      v[3][i] = (a.s[1][n] - uy * sr) * ir;
      v[4][i] = a.S[n];
      v[5][i] = sr * ir;
#pragma unroll
      for (int c = 0; c < NQ; ++c) s_v[c][e][t * NP + i] = v[c][i];
    }
#pragma unroll
    for (int c = 0; c < NQ; ++c)
#pragma unroll
      for (int i = 0; i < NP; ++i) s_dx[c][e][t * NP + i] = I.ijx * dot_row<NP>(B, i, v[c]);
  }
  __syncthreads();
  if (!vc.valid) return;
  const int t = vc.t, e = vc.e;
  double dy[NQ][NP];
#pragma unroll
  for (int c = 0; c < NQ; ++c) {
    double col[NP];
#pragma unroll
    for (int l = 0; l < NP; ++l) col[l] = s_v[c][e][l * NP + t];
#pragma unroll
    for (int l = 0; l < NP; ++l) dy[c][l] = I.ijy * dot_row<NP>(B, l, col);
  }
  const double al = I.alpha;
#pragma unroll
  for (int l = 0; l < NP; ++l) {
    const int nd = l * NP + t;
    const long long n = vc.base + nd;
    const double uxx = s_dx[0][e][nd], uyx = s_dx[1][e][nd], sxx = s_dx[2][e][nd], syx = s_dx[3][e][nd];
    const double Sx = s_dx[4][e][nd], dxs = s_dx[5][e][nd];
    const double uxy = dy[0][l], uyy = dy[1][l], sxy = dy[2][l], syy = dy[3][l], Sy = dy[4][l], dys = dy[5][l];
    const double divu = uxx + uyy, divs = sxx + syy;
    const double Rp = al * (divu * divu + uxx * uxx + 2.0 * uxy * uyx + uyy * uyy);
    const double Rs = al * (2.0 * divu * divs + 2.0 * (uxx * sxx + uxy * syx + uyx * sxy + uyy * syy));
    const double bp = Rs + s_v[5][e][nd] * Rp - al * (dxs * Sx + dys * Sy) * a.invr[n];
    a.b_out[n] = (B.w[t] * B.w[l]) * (I.jx * I.jy) * bp;
  }
}

// ---------------------------------------------------------------------------
// Tangent fluxes at one node (sensitivity_flux_x/_y, sensitivity.jl:43-76):
//   Phi = (gamma-1) (eta - sigma |u|^2/2 - rho u . s_u)  [+ s_gamma rho e]
//   P~  = Phi + varsigma
//   fx  = (zx ux + mx sux + P~, zx uy + mx suy, zx, (eta + P~) ux + (E + P + Sigma) sux)
//   fy  = (zx uy + mx suy, zy uy + my suy + P~, zy, (eta + P~) uy + (E + P + Sigma) suy)
// The s_gamma term (direct dP/dgamma source, zero in the reference's 2D
// package) follows the 1D package (IGR_adjoints_1d/sensitivity.jl:36-41).
// ---------------------------------------------------------------------------
struct SensNode { double fx[4], fy[4]; };

__device__ __forceinline__ SensNode sens_phys(double g, double sg, double mx, double my, double r, double E, double S,
                                              double ir, double zx, double zy, double sr, double et, double vs) {
  SensNode o;
  const double ux = mx * ir, uy = my * ir;
  const double sux = (zx - ux * sr) * ir, suy = (zy - uy * sr) * ir;
  const double u2h = 0.5 * fma(ux, ux, uy * uy);
  const double P = (g - 1.0) * (E - r * u2h);
  double Phi = (g - 1.0) * (et - sr * u2h - r * fma(ux, sux, uy * suy));
  if (sg != 0.0) Phi = fma(sg, r * (E * ir - u2h), Phi);
  const double Pt = Phi + vs;
  const double etp = et + Pt, eps = E + P + S;
  const double f1 = fma(zx, uy, mx * suy);
  o.fx[0] = fma(zx, ux, mx * sux) + Pt; o.fx[1] = f1; o.fx[2] = zx; o.fx[3] = fma(etp, ux, eps * sux);
  o.fy[0] = f1; o.fy[1] = fma(zy, uy, my * suy) + Pt; o.fy[2] = zy; o.fy[3] = fma(etp, uy, eps * suy);
  return o;
}

struct SensHypArgs2D {
  const Tile2D* tiles; const Inst2D* inst; BasisDev B;
  const double *q[4], *invr, *S;   // primal stage input and its Sigma
  const double *s[4], *vs;         // tangent stage input and varsigma
  const double *sn[4];             // tangent at the step start (stages 2 and 3)
  const double *ws_x, *ws_y;       // primal |u_n| + c at x-face / y-face nodes of this stage
  double c0, c1, c2, s_gamma;
  double *so[4];                   // tangent stage output (may alias sn: pointwise)
  double *k_out[4];                // optional: raw tangent RHS
  int* status;
};

struct SensFace { double s[4], f[4], ws; };

template <int NP>
__global__ void __launch_bounds__(Tiling2D<NP>::NT) k2_sens_hyp_rk(SensHypArgs2D a) {
  using TL = Tiling2D<NP>;
  constexpr int TE = TL::TE, NN = TL::NN, L = TL::L, TX = TL::TX, TY = TL::TY;
  __shared__ double s_fy[4][TE][NN];
  __shared__ double s_k[4][TE][NN];
  __shared__ double s_s[4][TE][NN];
  __shared__ SensFace s_xf[TE][NP][2];
  __shared__ SensFace s_yf[TE][NP][2];
  const Tile2D tl = a.tiles[blockIdx.x];
  const Inst2D I = a.inst[tl.inst];
  const ElemView vr = elem_view<NP>(tl, I, 0), vc = elem_view<NP>(tl, I, 1);
  const BasisDev& B = a.B;
  const double g = I.gamma, sg = a.s_gamma;
  const double invJx = I.ijx, invJy = I.ijy;
  auto node = [&](long long n) {
    return sens_phys(g, sg, a.q[0][n], a.q[1][n], a.q[2][n], a.q[3][n], a.S[n], a.invr[n], a.s[0][n], a.s[1][n],
                     a.s[2][n], a.s[3][n], a.vs[n]);
  };

  // ---- phase 1 (rows): tangent fluxes, x volume term, x-face node data
  if (vr.valid) {
    const int t = vr.t, e = vr.e;
    double fx[4][NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const long long n = vr.base + t * NP + i;
      const SensNode sp = node(n);
#pragma unroll
      for (int c = 0; c < 4; ++c) { fx[c][i] = sp.fx[c]; s_fy[c][e][t * NP + i] = sp.fy[c]; s_s[c][e][t * NP + i] = a.s[c][n]; }
      if (i == 0 || i == L) {
        SensFace& fs = s_xf[e][t][i == 0 ? 0 : 1];
#pragma unroll
        for (int c = 0; c < 4; ++c) { fs.s[c] = a.s[c][n]; fs.f[c] = sp.fx[c]; }
        fs.ws = a.ws_x[n];
      }
    }
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
      for (int i = 0; i < NP; ++i) s_k[c][e][t * NP + i] = -invJx * dot_row<NP>(B, i, fx[c]);
  }
  __syncthreads();
  // ---- phase 2 (columns): y-face node data
  if (vc.valid) {
    const int t = vc.t, e = vc.e;
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int nd = (s == 0 ? 0 : L) * NP + t;
      SensFace& fs = s_yf[e][t][s];
#pragma unroll
      for (int c = 0; c < 4; ++c) { fs.s[c] = s_s[c][e][nd]; fs.f[c] = s_fy[c][e][nd]; }
      fs.ws = a.ws_y[vc.base + nd];
    }
  }
  __syncthreads();
  // ---- phase 3 (rows): x faces
  if (vr.valid) {
    const int t = vr.t, e = vr.e;
    auto fetch = [&](int s) {
      int it;
      const long long pb = neighbour<NP>(tl, I, vr.ex, vr.ey, s == 0 ? -1 : 1, 0, &it);
      SensFace pf;
      if (it >= 0) {
        pf = s_xf[it][t][s == 0 ? 1 : 0];
      } else {
        const long long n = pb + t * NP + (s == 0 ? L : 0);
        const SensNode sp = node(n);
#pragma unroll
        for (int c = 0; c < 4; ++c) { pf.s[c] = a.s[c][n]; pf.f[c] = sp.fx[c]; }
        pf.ws = a.ws_x[n];
      }
      return pf;
    };
    const int sf = first_side(vr.ext, TX);
    const SensFace pA = fetch(sf), pB = fetch(1 - sf);
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const SensFace& pf = (s == sf) ? pA : pB;
      const SensFace& of = s_xf[e][t][s];
      const SensFace& Ls = s == 0 ? pf : of;
      const SensFace& Rs = s == 0 ? of : pf;
      const double lam = max_nonneg(Rs.ws, Ls.ws);
      const int io = s == 0 ? 0 : L;
      const double cf = s == 0 ? invJx * B.iw0 : -invJx * B.iwL;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const double fs = 0.5 * fma(lam, Ls.s[c] - Rs.s[c], Ls.f[c] + Rs.f[c]);
        s_k[c][e][t * NP + io] = fma(cf, fs - of.f[c], s_k[c][e][t * NP + io]);
      }
    }
  }
  __syncthreads();
  if (!vc.valid) return;
  // ---- phase 4 (columns): y volume term, y faces, RK combination
  const int t = vc.t, e = vc.e;
  double kc[4][NP];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    double fyc[NP];
#pragma unroll
    for (int l = 0; l < NP; ++l) fyc[l] = s_fy[c][e][l * NP + t];
#pragma unroll
    for (int l = 0; l < NP; ++l) kc[c][l] = fma(-invJy, dot_row<NP>(B, l, fyc), s_k[c][e][l * NP + t]);
  }
  auto fetchy = [&](int s) {
    int it;
    const long long pb = neighbour<NP>(tl, I, vc.ex, vc.ey, 0, s == 0 ? -1 : 1, &it);
    SensFace pf;
    if (it >= 0) {
      pf = s_yf[it][t][s == 0 ? 1 : 0];
    } else {
      const long long n = pb + (s == 0 ? L : 0) * NP + t;
      const SensNode sp = node(n);
#pragma unroll
      for (int c = 0; c < 4; ++c) { pf.s[c] = a.s[c][n]; pf.f[c] = sp.fy[c]; }
      pf.ws = a.ws_y[n];
    }
    return pf;
  };
  const int sf = first_side(vc.eyt, TY);
  const SensFace qA = fetchy(sf), qB = fetchy(1 - sf);
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const SensFace& pf = (s == sf) ? qA : qB;
    const SensFace& of = s_yf[e][t][s];
    const SensFace& Ls = s == 0 ? pf : of;
    const SensFace& Rs = s == 0 ? of : pf;
    const double lam = max_nonneg(Rs.ws, Ls.ws);
    const int lo = s == 0 ? 0 : L;
    const double cf = s == 0 ? invJy * B.iw0 : -invJy * B.iwL;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const double fs = 0.5 * fma(lam, Ls.s[c] - Rs.s[c], Ls.f[c] + Rs.f[c]);
      kc[c][lo] = fma(cf, fs - of.f[c], kc[c][lo]);
    }
  }
  const double c2dt = a.c2 * I.dt;
  bool bad = false;
#pragma unroll
  for (int l = 0; l < NP; ++l) {
    const long long n = vc.base + l * NP + t;
    double so[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      if (a.k_out[c]) a.k_out[c][n] = kc[c][l];
      double val = fma(c2dt, kc[c][l], a.c1 * s_s[c][e][l * NP + t]);
      if (a.c0 != 0.0) val = fma(a.c0, a.sn[c][n], val);
      so[c] = val;
      bad |= nonfinite_bits(val);
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) if (a.so[c]) a.so[c][n] = so[c];
  }
  if (bad) flag_nonfinite(a.status);
}

}  // namespace igrgpu
