// 1D tangent (run_sensitivity, IGR_adjoints_1d/sensitivity.jl:401-515): the
// coupled primal + tangent SSP-RK3, one CTA per instance.
//
// Stepping follows ssp_rk3_coupled (sensitivity.jl:419-420): `while t < T -
// 1e-14`, h = min(dt, T - t), with no re-rounding of dt. Per stage: the primal
// Sigma solve, the tangent elliptic source (form 1 or form 2) solved with the
// same operator for varsigma, the primal DG RHS and the tangent DG RHS, whose
// LLF flux uses the primal wave speed (no d lambda term).
#pragma once
#include "igr1d_kernels.cuh"

namespace igrgpu {

// Tangent fluxes at one node (sensitivity_flux, sensitivity.jl:36-48):
//   su = (s_mu - u s_rho)/rho,  sP = (gamma-1)(sE - s_rho u^2/2 - rho u su) + s_gamma rho e
//   f = (s_mu u + mu su + sP + sS,  s_mu,  su (E + P + Sigma) + u (sE + sP + sS))
__device__ __forceinline__ void sens_flux1(double g, double sg, double mu, double r, double E, double S, double ir,
                                           double smu, double sr, double sE, double sS, double f[3]) {
  const double u = mu * ir, su = (smu - u * sr) * ir;
  const double u2h = 0.5 * u * u;
  const double P = (g - 1.0) * (E - r * u2h);
  double sP = (g - 1.0) * (sE - sr * u2h - r * u * su);
  if (sg != 0.0) sP = fma(sg, r * (E * ir - u2h), sP);
  f[0] = fma(smu, u, mu * su) + sP + sS;
  f[1] = smu;
  f[2] = fma(su, E + P + S, u * (sE + sP + sS));
}

// Tangent DG RHS (compute_sensitivity_hyperbolic_rhs!, sensitivity.jl:90-152)
// fused with the RK combination s_out = c0 s^n + c1 s_s + c2 dt k.
template <int NP>
__device__ void d1_sens_hyp_rk(const View1<NP>& v, const BasisDev& B, double sg, const double* const q[3], const double* ir,
                               const double* S, const double* const s[3], const double* vs, const double* const sn[3],
                               double c0, double c1, double c2, double dt, double* const so[3], int* status) {
  constexpr int L = NP - 1;
  const Inst1D& I = v.I;
  const double g = I.gamma, iJ = I.iJ, c2dt = c2 * dt;
  bool bad = false;
  auto flux = [&](int m, double f[3]) {
    sens_flux1(g, sg, q[0][m], q[1][m], q[2][m], S[m], ir[m], s[0][m], s[1][m], s[2][m], vs[m], f);
  };
  auto wsp = [&](int m) { return ws1(g, node1(g, q[0][m], q[2][m], S[m], ir[m]), ir[m]); };
  for (int e = v.e0 + threadIdx.x; e < v.e1; e += blockDim.x) {
    const int eL = wrap_left(e, I.ne), eR = wrap_right(e, I.ne);
    const int base = e * NP;
    double f[3][NP], k[3][NP], ss[3][NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      double fi[3];
      flux(base + i, fi);
#pragma unroll
      for (int c = 0; c < 3; ++c) { f[c][i] = fi[c]; ss[c][i] = s[c][base + i]; }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int i = 0; i < NP; ++i) k[c][i] = -iJ * dot_row<NP>(B, i, f[c]);
    {  // right face
      const int m = eR * NP;
      double fp[3];
      flux(m, fp);
      const double wl = wsp(base + L), wr = wsp(m);
      const double lam = max_nonneg(wr, wl);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const double fs = 0.5 * fma(lam, ss[c][L] - s[c][m], f[c][L] + fp[c]);
        k[c][L] = fma(-iJ * B.iwL, fs - f[c][L], k[c][L]);
      }
    }
    {  // left face
      const int m = eL * NP + L;
      double fp[3];
      flux(m, fp);
      const double wl = wsp(m), wr = wsp(base);
      const double lam = max_nonneg(wr, wl);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const double fs = 0.5 * fma(lam, s[c][m] - ss[c][0], fp[c] + f[c][0]);
        k[c][0] = fma(iJ * B.iw0, fs - f[c][0], k[c][0]);
      }
    }
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const int m = base + i;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        double val = fma(c2dt, k[c][i], c1 * ss[c][i]);
        if (c0 != 0.0) val = fma(c0, sn[c][m], val);
        so[c][m] = val;
        bad |= nonfinite_bits(val);
      }
    }
  }
  if (bad) flag_nonfinite(status);
  v.sync();
}

// Tangent elliptic source.
// form 2 (sensitivity.jl:272-314): b = w J alpha (2 u_x (2 su_x + r_s u_x) - (r_s)_x Sigma_x / rho),
//   r_s = s_rho / rho;
// form 1 (sensitivity.jl:168-256): b = w J 4 alpha u_x su_x + A_k Sigma, where
//   A_k is the SIP operator with 1/rho replaced by k = s_rho / rho^2 (mass,
//   stiffness and face terms). cm/ck/cpR: scratch for A_k's coefficients.
template <int NP>
__device__ void d1_sens_rhs(const View1<NP>& v, const BasisDev& B, int form, const double* const q[3], const double* ir,
                            const double* S, const double* const s[3], double* b, double* cm, double* ck, double* cpR) {
  constexpr int L = NP - 1;
  const Inst1D& I = v.I;
  const double al = I.alpha, iJ = I.iJ, eta = (double)(NP * NP);
  for (int e = v.e0 + threadIdx.x; e < v.e1; e += blockDim.x) {
    const int eR = wrap_right(e, I.ne);
    const int base = e * NP;
    double u[NP], su[NP], rs[NP], Sv[NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const int m = base + i;
      const double r = ir[m];
      u[i] = q[0][m] * r;
      su[i] = (s[0][m] - u[i] * s[1][m]) * r;
      rs[i] = s[1][m] * r;
      Sv[i] = S[m];
    }
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const double ux = iJ * dot_row<NP>(B, i, u), sux = iJ * dot_row<NP>(B, i, su);
      const double c = B.w[i] * I.J;
      if (form == 2) {
        const double dso = iJ * dot_row<NP>(B, i, rs), dS = iJ * dot_row<NP>(B, i, Sv);
        b[base + i] = c * (al * (2.0 * ux * fma(rs[i], ux, 2.0 * sux) - dso * dS * ir[base + i]));
      } else {
        b[base + i] = c * (4.0 * al * ux * sux);
        const double kk = rs[i] * ir[base + i];  // s_rho / rho^2
        cm[base + i] = c * kk;
        ck[base + i] = (al * B.w[i] * iJ) * kk;
      }
    }
    if (form != 2) {
      const double kL = rs[L] * ir[base + L], kR = s[1][eR * NP] * ir[eR * NP] * ir[eR * NP];
      cpR[e] = al * eta * I.idx * ((kR > kL) ? kR : kL);
    }
  }
  v.sync();
  if (form == 2) return;
  d1_apply<NP>(v, B, [&](int m) { return S[m]; }, cm, ck, cpR, [&](int e, const double*, const double* y) {
#pragma unroll
    for (int i = 0; i < NP; ++i) b[e * NP + i] += y[i];
  });
  v.sync();
}

// Scratch of the tangent kernel (fields of N doubles, after the step work).
enum : int {
  T1_IR0 = F1_STEP_FIELDS, T1_SA = T1_IR0 + 1, T1_VA = T1_SA + 1, T1_S1 = T1_VA + 1, T1_S2 = T1_S1 + 3,
  T1_BS = T1_S2 + 3, T1_KM = T1_BS + 1, T1_KK = T1_KM + 1, T1_KP = T1_KK + 1, T1_FIELDS = T1_KP + 1
};

struct Tan1DArgs {
  const Inst1D* inst; const int* order; BasisDev B;
  double* q;      // batch state [inst][3][N], in place
  double* s;      // batch tangent, same layout, in place
  double* sig;    // batch Sigma out
  double* vs;     // batch varsigma out
  double* scr;
  int solver, n_iter, form;
  double s_gamma;
  int cs;         // CTAs per instance (cluster size)
  int* status;
};

template <int NP>
__global__ void __launch_bounds__(T1, 2) k1_tangent(Tan1DArgs a) {
  __shared__ double s_red[T1];
  int inst;
  const View1<NP> v = make_view1<NP>(a.inst, a.order, a.scr, a.cs, &inst);
  const BasisDev& B = a.B;
  const Inst1D& I = v.I;
  const int N = v.N;
  const bool apos = I.alpha > 0;
  double* q[3] = {a.q + 3 * I.off, a.q + 3 * I.off + N, a.q + 3 * I.off + 2 * N};
  double* s[3] = {a.s + 3 * I.off, a.s + 3 * I.off + N, a.s + 3 * I.off + 2 * N};
  auto W = [&](int k) { return v.f(k); };
  double* q1[3] = {W(F1_Q1), W(F1_Q1 + 1), W(F1_Q1 + 2)};
  double* q2[3] = {W(F1_Q2), W(F1_Q2 + 1), W(F1_Q2 + 2)};
  double* s1[3] = {W(T1_S1), W(T1_S1 + 1), W(T1_S1 + 2)};
  double* s2[3] = {W(T1_S2), W(T1_S2 + 1), W(T1_S2 + 2)};
  double* irs[3] = {W(T1_IR0), W(F1_IR1), W(F1_IR2)};
  double* sig = a.sig + I.off;
  double* vsg = a.vs + I.off;
  double* Sx = sig; double* Sy = W(T1_SA);
  double* Vx = vsg; double* Vy = W(T1_VA);
  const SolveTape1 none;
  d1_zero(v, Sx);
  d1_zero(v, Vx);
  d1_recip(v, q[1], irs[0]);
  auto solve_pair = [&](double* const* qs, double* irq, double* const* ss) {
    d1_setup(v, B, qs[0], irq, W(F1_B), W(F1_CM), W(F1_CK), W(F1_CPR), W(F1_CINVM), nullptr);
    d1_solve(v, B, a.solver, a.n_iter, W(F1_B), Sx, Sy, W(F1_CM), W(F1_CK), W(F1_CPR), W(F1_CINVM), W(F1_W0), W(F1_W1),
             W(F1_W2), W(F1_W3), none, s_red);
    double* t = Sx; Sx = Sy; Sy = t;
    const double* qc[3] = {qs[0], qs[1], qs[2]};
    const double* sc[3] = {ss[0], ss[1], ss[2]};
    d1_sens_rhs(v, B, a.form, qc, irq, Sx, sc, W(T1_BS), W(T1_KM), W(T1_KK), W(T1_KP));
    d1_solve(v, B, a.solver, a.n_iter, W(T1_BS), Vx, Vy, W(F1_CM), W(F1_CK), W(F1_CPR), W(F1_CINVM), W(F1_W0), W(F1_W1),
             W(F1_W2), W(F1_W3), none, s_red);
    t = Vx; Vx = Vy; Vy = t;
  };
  double t = 0.0;
  while (t < I.t_end - 1e-14) {
    const double h = fmin(I.dt, I.t_end - t);
    for (int k = 0; k < 3; ++k) {
      double* const* qs = k == 0 ? q : (k == 1 ? q1 : q2);
      double* const* ss = k == 0 ? s : (k == 1 ? s1 : s2);
      if (apos) solve_pair(qs, irs[k], ss);
      double c0, c1, c2;
      rk1_coef(k, &c0, &c1, &c2);
      const double* qsc[3] = {qs[0], qs[1], qs[2]};
      const double* qnc[3] = {q[0], q[1], q[2]};
      const double* ssc[3] = {ss[0], ss[1], ss[2]};
      const double* snc[3] = {s[0], s[1], s[2]};
      // tangent first: it reads the primal stage input, which the stage-3 primal update overwrites only for q^n
      d1_sens_hyp_rk(v, B, a.s_gamma, qsc, irs[k], Sx, ssc, Vx, snc, c0, c1, c2, h, k == 0 ? s1 : (k == 1 ? s2 : s),
                     a.status);
      d1_hyp_rk(v, B, qsc, irs[k], Sx, qnc, c0, c1, c2, h, k == 0 ? q1 : (k == 1 ? q2 : q), k < 2 ? irs[k + 1] : irs[0],
                nullptr, a.status);
    }
    t += h;
  }
  if (apos) solve_pair(q, irs[0], s);
  if (Sx != sig) d1_copy(v, Sx, sig);
  if (Vx != vsg) d1_copy(v, Vx, vsg);
}

}  // namespace igrgpu
