// 1D discrete adjoint (the gradient enzyme_adjoint_ic returns,
// IGR_adjoints_1d/enzyme_adjoint.jl:267-314, computed by hand-written reverse
// code instead of Enzyme): one CTA per instance, like the forward.
//
// Reverse conventions (the derivative the reverse takes where the forward is
// not differentiable): max(a, b) passes the derivative to the first argument
// on ties, |x| has derivative +1 at +0.0 (sign bit), as the CPU reverse does.
// Every element's thread accumulates into its own nodes only ("owner
// computes"): face terms that touch two elements are evaluated by both, so no
// atomics are needed and results do not depend on scheduling. The gamma and
// alpha derivatives accumulate per element (View1::gbe / abe) and are reduced
// at the end in a fixed order.
#pragma once
#include "igr1d_kernels.cuh"

namespace igrgpu {

// ---------------------------------------------------------------------------
// Pointwise reverses (IGR_adjoints_1d/euler.jl:46-111)
// ---------------------------------------------------------------------------
// Adjoint of f = (mu^2/rho + P_bar, mu, (E + P_bar) mu/rho) given fb.
__device__ __forceinline__ void flux1_rev(double g, double mu, double ir, double E, double S, const double fb[3],
                                          double qb[3], double& Sb, double& gb) {
  const double u = mu * ir, K = 0.5 * mu * u, P = (g - 1.0) * (E - K), pb = P + S;
  const double pbb = fma(fb[2], u, fb[0]);
  qb[0] += fma(fb[0], 2.0 * u, fb[1]) + fb[2] * (E + pb) * ir;
  qb[1] += -(fb[0] * u * u) - fb[2] * (E + pb) * u * ir;
  qb[2] += fb[2] * u;
  Sb += pbb;
  gb += pbb * (E - K);
  qb[2] += pbb * (g - 1.0);
  const double Kb = -pbb * (g - 1.0);
  qb[0] += Kb * u;
  qb[1] += -Kb * K * ir;
}
// Adjoint of |u| + sqrt(gamma P / rho) given wb.
__device__ __forceinline__ void ws1_rev(double g, double mu, double ir, double E, double wb, double qb[3], double& gb) {
  const double u = mu * ir, K = 0.5 * mu * u, P = (g - 1.0) * (E - K);
  const double ub = signbit(u) ? -wb : wb;
  qb[0] += ub * ir;
  qb[1] += -ub * u * ir;
  const double X = g * P * ir, c = sqrt(X), Xb = wb / (2.0 * c);
  gb += Xb * P * ir;
  const double Pb = Xb * g * ir;
  qb[1] += -Xb * X * ir;
  gb += Pb * (E - K);
  qb[2] += Pb * (g - 1.0);
  const double Kb = -Pb * (g - 1.0);
  qb[0] += Kb * u;
  qb[1] += -Kb * K * ir;
}

// ---------------------------------------------------------------------------
// Reverse of d1_hyp_rk for one stage (hyperbolic.jl:134-194 + the RK
// combination). Given A = adjoint of the stage output:
//   Qn (+)= c0 A  (qn_mode 0 skip / 1 write / 2 add),  kb = c2 dt A,
//   Qs  = c1 A + H_q^T kb (qs_add: add instead of write),  Sb += H_S^T kb,
//   gb += d/dgamma.
// Each face flux is used by both of its elements; its adjoint is the sum of
// the two uses, evaluated identically by both owners.
// ---------------------------------------------------------------------------
template <int NP>
__device__ void d1_hyp_rev(const View1<NP>& v, const BasisDev& B, const double* const q[3], const double* ir,
                           const double* S, const double* const A[3], double c0, double c1, double c2, double* const Qn[3],
                           int qn_mode, double* const Qs[3], int qs_add, double* Sb) {
  constexpr int L = NP - 1;
  const Inst1D& I = v.I;
  const double g = I.gamma, iJ = I.iJ, c2dt = c2 * I.dt;
  for (int e = v.e0 + threadIdx.x; e < v.e1; e += blockDim.x) {
    const int eL = wrap_left(e, I.ne), eR = wrap_right(e, I.ne);
    const int base = e * NP;
    double gb = 0.0;  // this element's d/dgamma
    double kb[3][NP], Fb[3][NP], qb[3][NP];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int i = 0; i < NP; ++i) { kb[c][i] = c2dt * A[c][base + i]; qb[c][i] = 0.0; }
    // volume term: k = -iJ D F  ->  Fb = -iJ D^T kb ; face-local parts of k
#pragma unroll
    for (int c = 0; c < 3; ++c) {
#pragma unroll
      for (int j = 0; j < NP; ++j) Fb[c][j] = -iJ * dot_col<NP>(B, j, kb[c], 0.0);
      Fb[c][L] = fma(iJ * B.iwL, kb[c][L], Fb[c][L]);
      Fb[c][0] = fma(-iJ * B.iw0, kb[c][0], Fb[c][0]);
    }
    // right face (own node L | node 0 of eR)
    {
      const int m = eR * NP, o = base + L;
      double fsb[3], jq[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        fsb[c] = fma(-iJ * B.iwL, kb[c][L], iJ * B.iw0 * (c2dt * A[c][m]));
        jq[c] = q[c][o] - q[c][m];
      }
      const Node1 nl = node1(g, q[0][o], q[2][o], S[o], ir[o]);
      const Node1 nr = node1(g, q[0][m], q[2][m], S[m], ir[m]);
      const double wl = ws1(g, nl, ir[o]), wr = ws1(g, nr, ir[m]);
      const double lam = max_nonneg(wr, wl);
      double lamb = 0.0;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        Fb[c][L] = fma(0.5, fsb[c], Fb[c][L]);
        qb[c][L] = fma(0.5 * lam, fsb[c], qb[c][L]);
        lamb = fma(0.5 * fsb[c], jq[c], lamb);
      }
      if (!gt_nonneg(wr, wl)) {
        double t[3] = {0.0, 0.0, 0.0};
        ws1_rev(g, q[0][o], ir[o], q[2][o], lamb, t, gb);
#pragma unroll
        for (int c = 0; c < 3; ++c) qb[c][L] += t[c];
      }
    }
    // left face (node L of eL | own node 0)
    {
      const int m = eL * NP + L, o = base;
      double fsb[3], jq[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        fsb[c] = fma(-iJ * B.iwL, c2dt * A[c][m], iJ * B.iw0 * kb[c][0]);
        jq[c] = q[c][m] - q[c][o];
      }
      const Node1 nl = node1(g, q[0][m], q[2][m], S[m], ir[m]);
      const Node1 nr = node1(g, q[0][o], q[2][o], S[o], ir[o]);
      const double wl = ws1(g, nl, ir[m]), wr = ws1(g, nr, ir[o]);
      const double lam = max_nonneg(wr, wl);
      double lamb = 0.0;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        Fb[c][0] = fma(0.5, fsb[c], Fb[c][0]);
        qb[c][0] = fma(-0.5 * lam, fsb[c], qb[c][0]);
        lamb = fma(0.5 * fsb[c], jq[c], lamb);
      }
      if (gt_nonneg(wr, wl)) {
        double t[3] = {0.0, 0.0, 0.0};
        ws1_rev(g, q[0][o], ir[o], q[2][o], lamb, t, gb);
#pragma unroll
        for (int c = 0; c < 3; ++c) qb[c][0] += t[c];
      }
    }
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const int m = base + i;
      const double fb[3] = {Fb[0][i], Fb[1][i], Fb[2][i]};
      double t[3] = {qb[0][i], qb[1][i], qb[2][i]};
      double sb = 0.0;
      flux1_rev(g, q[0][m], ir[m], q[2][m], S[m], fb, t, sb, gb);
      Sb[m] += sb;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const double Av = A[c][m];
        if (qn_mode == 1) Qn[c][m] = c0 * Av;
        else if (qn_mode == 2) Qn[c][m] = fma(c0, Av, Qn[c][m]);
        const double val = fma(c1, Av, t[c]);
        Qs[c][m] = qs_add ? Qs[c][m] + val : val;
      }
    }
    v.gbe()[e] += gb;
  }
  v.sync();
}

// ---------------------------------------------------------------------------
// Reverse operator application with the coefficient adjoints
// (sip_param_adj of the CPU reverse, 1D): for the forward term u^T A(rho, alpha) v,
//   out -= A u (A is symmetric),
//   Zinv += zscale d(u^T A v)/d(1/rho)   per node,  ab += zscale d(u^T A v)/d alpha.
// ldu(n, v_n) supplies u at node n (given v there). epi(e, u[], y[]) consumes A u.
// ---------------------------------------------------------------------------
template <int NP, class LDU, class EPI>
__device__ __forceinline__ void d1_apply_rev(const View1<NP>& v, const BasisDev& B, LDU ldu, const double* vt,
                                             const double* ir, const double* cm, const double* ck, const double* cpR,
                                             double zscale, double* Zinv, int z_first, EPI epi) {
  constexpr int L = NP - 1;
  const Inst1D& I = v.I;
  const int ne = I.ne;
  const double hw = B.hw, al = I.alpha, iJ = I.iJ;
  const double eta = (double)(NP * NP);
  for (int e = v.e0 + threadIdx.x; e < v.e1; e += blockDim.x) {
    const int eL = wrap_left(e, ne), eR = wrap_right(e, ne);
    const int base = e * NP;
    double u[NP], w[NP], ul[NP], ur[NP], wl[NP], wr[NP], kc[NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      w[i] = vt[base + i]; u[i] = ldu(base + i, w[i]); kc[i] = ck[base + i];
      wl[i] = vt[eL * NP + i]; ul[i] = ldu(eL * NP + i, wl[i]);
      wr[i] = vt[eR * NP + i]; ur[i] = ldu(eR * NP + i, wr[i]);
    }
    double gu[NP], gw[NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) { gu[i] = dot_row<NP>(B, i, u); gw[i] = dot_row<NP>(B, i, w); }
    const double gul = dot_end<NP>(B, true, ul), gur = dot_end<NP>(B, false, ur);
    const double gwl = dot_end<NP>(B, true, wl), gwr = dot_end<NP>(B, false, wr);
    // A u (same folding as d1_apply)
    {
      const double ckl = ck[eL * NP + L], ckr = ck[eR * NP];
      const double jl = ul[L] - u[0];
      const double Fl = fma(cpR[eL], jl, hw * fma(ckl, gul, kc[0] * gu[0]));
      const double jr = u[L] - ur[0];
      const double Fr = fma(cpR[e], jr, hw * fma(kc[L], gu[L], ckr * gur));
      double sx[NP];
#pragma unroll
      for (int i = 1; i < L; ++i) sx[i] = kc[i] * gu[i];
      sx[0] = kc[0] * fma(hw, jl, gu[0]);
      sx[L] = kc[L] * fma(hw, jr, gu[L]);
      double y[NP];
#pragma unroll
      for (int k = 0; k < NP; ++k)
        y[k] = dot_col<NP>(B, k, sx, fma(cm[base + k], u[k], (k == 0) ? -Fl : ((k == L) ? Fr : 0.0)));
      epi(e, u, y);
    }
    // coefficient adjoints
    double z[NP];
    double abl = 0.0;
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const double st = B.w[i] * iJ * gw[i] * gu[i];
      z[i] = fma(B.w[i] * I.J, u[i] * w[i], al * st);
      abl = fma(st, ir[base + i], abl);
    }
    {  // right face (e | eR), counted for alpha by e
      const double iL = ir[base + L], iR = ir[eR * NP];
      const double ju = u[L] - ur[0], jw = w[L] - wr[0];
      const double cL = fma(gw[L], ju, gu[L] * jw), cR = fma(gwr, ju, gur * jw);
      z[L] += -al * iJ * 0.5 * cL;
      if (!gt_nonneg(iR, iL)) z[L] += al * eta * I.idx * jw * ju;
      abl += -iJ * 0.5 * fma(iL, cL, iR * cR) + eta * max_nonneg(iR, iL) * I.idx * jw * ju;
    }
    {  // left face (eL | e)
      const double iL = ir[eL * NP + L], iR = ir[base];
      const double ju = ul[L] - u[0], jw = wl[L] - w[0];
      const double cR = fma(gw[0], ju, gu[0] * jw);
      z[0] += -al * iJ * 0.5 * cR;
      if (gt_nonneg(iR, iL)) z[0] += al * eta * I.idx * jw * ju;
    }
#pragma unroll
    for (int i = 0; i < NP; ++i) Zinv[base + i] = z_first ? zscale * z[i] : fma(zscale, z[i], Zinv[base + i]);
    v.abe()[e] = fma(zscale, abl, v.abe()[e]);
  }
}

// ---------------------------------------------------------------------------
// Reverse of d1_solve (solve_rev of the CPU reverse: Chebyshev, Jacobi, PCG).
// xb: in = adjoint of the solution, out = adjoint of the warm start x_0.
// Writes bb (adjoint of b), iMb (adjoint of 1/diag(A)), Zinv (coefficient
// adjoint per node) and adds to ab. w0..w4: scratch fields. All threads call it.
// ---------------------------------------------------------------------------
template <int NP>
__device__ void d1_solve_rev(const View1<NP>& v, const BasisDev& B, int solver, int n, const StageTape1& t, double* xb,
                             double* bb, double* iMb, double* Zinv, double* w0, double* w1, double* w2, double* w3,
                             double* s_red) {
  const int N = v.N;
  const SolveTape1& tp = t.st;
  const double* cinvM = t.cinvM;
  if (solver == 2 || solver == 1) {
    // u = residual adjoint r̄ (w0/w1 ping-pong), db = direction adjoint (w2, Chebyshev)
    double* U[2] = {w0, w1};
    double* db = w2;
    // Chebyshev coefficients of iteration it: a table built by one thread when
    // it fits, else recomputed from the recurrence
    constexpr int CHEB_TAB = 128;
    __shared__ double s_ct[2][CHEB_TAB];
    const bool tab = solver == 2 && n < CHEB_TAB;
    if (tab) {
      if (threadIdx.x == 0) {
        double rc = 0.0;
        for (int j = 1; j <= n; ++j) cheb_coef(B, j, rc, &s_ct[0][j], &s_ct[1][j]);
      }
      __syncthreads();
    }
    auto coef = [&](int it, double* ca, double* cc) {
      if (tab) { *ca = s_ct[0][it]; *cc = s_ct[1][it]; return; }
      double rc = 0.0;
      for (int j = 1; j <= it; ++j) cheb_coef(B, j, rc, ca, cc);
    };
    double can = 0.0, ccn = 0.0;
    if (solver == 2) coef(n, &can, &ccn);
    // last iteration's x_n = x_{n-1} + (...) r_{n-1}: r̄_{n-1} from xb
    for (int m = v.m0() + threadIdx.x; m < v.m1(); m += blockDim.x) {
      const double xbv = xb[m];
      if (solver == 2) {
        const double zb = ccn * xbv;
        U[0][m] = cinvM[m] * zb;
        iMb[m] = zb * tp.r(n - 1)[m];
        db[m] = can * xbv;
      } else {
        const double tb = (2.0 / 3.0) * xbv;
        U[0][m] = tb * cinvM[m];
        iMb[m] = tb * tp.r(n - 1)[m];
      }
    }
    v.sync();
    int cur = 0;
    for (int k = n - 1; k >= 0; --k) {
      // r_k = b - A x_k : bb += u, xb -= A u, Z += -(u, x_k); then r̄_{k-1}
      double* u = U[cur];
      double* un = U[1 - cur];
      const bool first = k == n - 1;
      double cak = 0.0, cck = 0.0;
      if (solver == 2 && k > 0) coef(k, &cak, &cck);
      d1_apply_rev<NP>(v, B, [&](int m, double) { return u[m]; }, tp.x(k), t.ir, t.cm, t.ck, t.cpR, -1.0, Zinv,
                       first ? 1 : 0, [&](int e, const double* uu, const double* y) {
#pragma unroll
        for (int i = 0; i < NP; ++i) {
          const int m = e * NP + i;
          const double xbv = xb[m] - y[i];
          xb[m] = xbv;
          bb[m] = first ? uu[i] : bb[m] + uu[i];
          if (k > 0) {
            if (solver == 2) {
              const double dbv = db[m] + xbv;
              const double zb = cck * dbv;
              un[m] = cinvM[m] * zb;
              iMb[m] = fma(zb, tp.r(k - 1)[m], iMb[m]);
              db[m] = cak * dbv;
            } else {
              const double tb = (2.0 / 3.0) * xbv;
              un[m] = tb * cinvM[m];
              iMb[m] = fma(tb, tp.r(k - 1)[m], iMb[m]);
            }
          }
        }
      });
      v.sync();
      cur = 1 - cur;
    }
    return;
  }
  // ---- PCG (reverse of pcg_fixed!, elliptic.jl:307-339 in 1D): w0 = pb, w1 = rb
  double* pb = w0;
  double* rb = w1;
  const double* RZ = tp.scal();
  const double* PAP = tp.scal() + n + 1;
  double rzb = 0.0;   // running adjoint of rz_{it+1} (then rz_it)
  double betab = 0.0; // pb . p_it from the previous reverse apply
  for (int m = v.m0() + threadIdx.x; m < v.m1(); m += blockDim.x) { pb[m] = 0.0; rb[m] = 0.0; }
  v.sync();
  bool first_z = true;
  __shared__ double s_sc[3];
  for (int it = n - 1; it >= 0; --it) {
    const double rz0 = RZ[it], rz1 = RZ[it + 1], pap = PAP[it];
    const double e0 = rz0 + 1e-30, den = pap + 1e-30;
    if (threadIdx.x == 0) {  // the iteration's quotients, once per CTA (see cta_div)
      s_sc[0] = rz1 / e0;           // beta
      s_sc[1] = rz0 / den;          // alpha
      s_sc[2] = rzb + betab / e0;   // adjoint of rz_{it+1}
    }
    __syncthreads();
    const double beta = s_sc[0], al = s_sc[1], rzb1 = s_sc[2];
    __syncthreads();
    const double* r1 = tp.r(it + 1);
    const double* ap = tp.ap(it);
    const double* p = tp.p(it);
    double* red = v.slot();
    for (int e = v.e0 + threadIdx.x; e < v.e1; e += blockDim.x) {
      double pe = 0.0;
#pragma unroll
      for (int i = 0; i < NP; ++i) {
        const int m = e * NP + i;
        const double pbv = pb[m], im = cinvM[m], rr = r1[m];
        pb[m] = beta * pbv;
        const double zb = fma(rzb1, rr, pbv);
        double rbv = fma(rzb1, rr * im, rb[m]);
        rbv = fma(zb, im, rbv);
        rb[m] = rbv;
        iMb[m] = (it == n - 1) ? zb * rr : fma(zb, rr, iMb[m]);
        pe = fma(xb[m], p[m], fma(-rbv, ap[m], pe));
      }
      red[e] = pe;
    }
    const double abv = v.reduce(s_red);
    if (threadIdx.x == 0) {
      s_sc[0] = -betab * rz1 / (e0 * e0) + abv / den;   // adjoint of rz_it
      s_sc[1] = -abv * rz0 / (den * den);               // adjoint of pAp_it
    }
    __syncthreads();
    rzb = s_sc[0];
    const double papb = s_sc[1];
    __syncthreads();
    // Ap = A p: pb += alpha xb + papb Ap + A (adjoint of Ap); u = -(adjoint of Ap) = alpha rb - papb p
    const double* pn = it > 0 ? tp.p(it - 1) : nullptr;
    red = v.slot();
    d1_apply_rev<NP>(v, B, [&](int m, double pv) { return fma(al, rb[m], -papb * pv); }, p, t.ir, t.cm, t.ck, t.cpR, -1.0,
                     Zinv, first_z ? 1 : 0, [&](int e, const double*, const double* y) {
      double pe = 0.0;
#pragma unroll
      for (int i = 0; i < NP; ++i) {
        const int m = e * NP + i;
        const double pbv = fma(papb, ap[m], fma(al, xb[m], pb[m] - y[i]));
        pb[m] = pbv;
        if (pn) pe = fma(pbv, pn[m], pe);
      }
      red[e] = pe;
    });
    first_z = false;
    betab = v.reduce(s_red);  // also synchronises the pb / rb updates
  }
  // p_0 = z_0, rz_0 = r_0 . z_0, z_0 = M^-1 r_0
  const double* r0 = tp.r(0);
  for (int m = v.m0() + threadIdx.x; m < v.m1(); m += blockDim.x) {
    const double rr = r0[m], im = cinvM[m];
    const double z0b = fma(rzb, rr, pb[m]);
    rb[m] = rb[m] + fma(rzb, rr * im, z0b * im);
    iMb[m] = fma(z0b, rr, iMb[m]);
  }
  v.sync();
  // r_0 = b - A x_0
  d1_apply_rev<NP>(v, B, [&](int m, double) { return rb[m]; }, tp.x(0), t.ir, t.cm, t.ck, t.cpR, -1.0, Zinv, 0,
                   [&](int e, const double* uu, const double* y) {
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const int m = e * NP + i;
      xb[m] -= y[i];
      bb[m] = uu[i];
    }
  });
  v.sync();
}

// ---------------------------------------------------------------------------
// Reverse of the stage setup: IGR source (igr_rhs1d), diag(A)
// (sip_diagonal1d) and the coefficient adjoints, into the adjoints of the
// stage input (Qs[0] = mu, Qs[1] = rho) and ab.
// ---------------------------------------------------------------------------
template <int NP>
__device__ void d1_setup_rev(const View1<NP>& v, const BasisDev& B, const StageTape1& t, const double* bb,
                             const double* iMb, const double* Zinv, double* const Qs[3]) {
  constexpr int L = NP - 1;
  const Inst1D& I = v.I;
  const double al = I.alpha, iJ = I.iJ, eta = (double)(NP * NP);
  auto Mb = [&](int m) { const double im = t.cinvM[m]; return -(iMb[m] * im) * im; };
  for (int e = v.e0 + threadIdx.x; e < v.e1; e += blockDim.x) {
    const int eL = wrap_left(e, I.ne), eR = wrap_right(e, I.ne);
    const int base = e * NP;
    double ab = 0.0;  // this element's d/dalpha
    double r[NP], mu[NP], u[NP], mb[NP], invb[NP], dub[NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      r[i] = t.ir[base + i]; mu[i] = t.q[0][base + i]; u[i] = mu[i] * r[i];
      mb[i] = Mb(base + i);
      invb[i] = Zinv[base + i];
    }
    // igr_rhs1d: b_i = w_i J 2 alpha du_i^2, du = iJ D u
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const double du = iJ * dot_row<NP>(B, i, u);
      const double c = B.w[i] * I.J;
      ab = fma(bb[base + i] * c * 2.0, du * du, ab);
      dub[i] = bb[base + i] * c * 2.0 * al * 2.0 * du;
    }
    // sip_diagonal1d: mass, stiffness self terms
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      invb[i] = fma(mb[i], B.w[i] * I.J, invb[i]);
#pragma unroll
      for (int k = 0; k < NP; ++k) {
        const double c = B.w[i] * iJ * (B.D[i][k] * B.D[i][k]);
        invb[i] = fma(mb[k] * al, c, invb[i]);
        ab = fma(mb[k] * c, r[i], ab);
      }
    }
    invb[L] = fma(mb[L] * (-al), iJ * B.D[L][L], invb[L]);
    invb[0] = fma(mb[0] * al, iJ * B.D[0][0], invb[0]);
    {  // right face: penalty self terms (alpha counted by e)
      const double iL = r[L], iR = t.ir[eR * NP];
      const double mR = Mb(eR * NP);
      const double sigb = (mb[L] + mR) * al;
      if (!(iR > iL)) invb[L] = fma(sigb, eta * I.idx, invb[L]);
      const double sig = eta * max_nonneg(iR, iL) * I.idx;
      ab += mb[L] * (-iJ * B.D[L][L] * iL + sig) + mR * (iJ * B.D[0][0] * iR + sig);
    }
    {  // left face
      const double iL = t.ir[eL * NP + L], iR = r[0];
      const double sigb = (Mb(eL * NP + L) + mb[0]) * al;
      if (iR > iL) invb[0] = fma(sigb, eta * I.idx, invb[0]);
    }
#pragma unroll
    for (int j = 0; j < NP; ++j) {
      const double ub = iJ * dot_col<NP>(B, j, dub, 0.0);
      Qs[0][base + j] += ub * r[j];
      Qs[1][base + j] += -(ub * mu[j]) * r[j] * r[j] - invb[j] * r[j] * r[j];
    }
    v.abe()[e] += ab;
  }
  v.sync();
}

// ---------------------------------------------------------------------------
// Objectives (IGR_adjoints_1d/enzyme_adjoint.jl:34-215 and the nodal interval
// extension) and their gradients. Objective codes as igr_objective.
// ---------------------------------------------------------------------------
template <int NP>
__device__ double d1_objective(const View1<NP>& v, const BasisDev& B, int obj, const double* prm, const double* const q[3],
                               double* s_red, double* ke_out, double* ms_out) {
  const Inst1D& I = v.I;
  const double g = I.gamma, pi = 3.14159265358979323846;
  double* red = v.slot();
  double* red2 = v.gbe();  // unused until the reverse starts: holds the mass partials
  for (int e = v.e0 + threadIdx.x; e < v.e1; e += blockDim.x) {
    double acc = 0.0, ms = 0.0;
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const int m = e * NP + i;
      const double c = B.w[i] * I.J;
      const double x = e * I.dx + I.J * (1.0 + B.xi[i]);
      const double mu = q[0][m], r = q[1][m], E = q[2][m];
      switch (obj) {
        case 0: acc = fma(c, r * r, acc); break;
        case 1: { const double P = (g - 1.0) * (E - mu * mu / (2.0 * r)); acc = fma(c, P * P, acc); break; }
        case 2: acc += c * (mu * mu) / (2.0 * r); ms = fma(c, r, ms); break;
        case 4: acc += c * mu * sin(2.0 * pi * x / (I.ne * I.dx)); break;
        case 6: acc += (x >= prm[0] && x <= prm[1]) ? c * r : 0.0; break;
        default: break;
      }
    }
    red[e] = acc;
    red2[e] = ms;
  }
  const double J = v.reduce(s_red);
  const double M = obj == 2 ? v.esum(red2, s_red) : 1.0;
  *ke_out = J;
  *ms_out = M;
  v.sync();  // every CTA has read the partials before they are overwritten
  return obj == 2 ? J / M : J;
}

template <int NP>
__device__ void d1_objective_grad(const View1<NP>& v, const BasisDev& B, int obj, const double* prm, const double* const q[3],
                                  double KE, double Ms, double* const qb[3]) {
  const Inst1D& I = v.I;
  const double g = I.gamma, pi = 3.14159265358979323846;
  for (int e = v.e0 + threadIdx.x; e < v.e1; e += blockDim.x) {
    double gb = 0.0;
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const int m = e * NP + i;
      const double c = B.w[i] * I.J;
      const double x = e * I.dx + I.J * (1.0 + B.xi[i]);
      const double mu = q[0][m], r = q[1][m], E = q[2][m];
      double b0 = 0.0, b1 = 0.0, b2 = 0.0;
      switch (obj) {
        case 0: b1 = 2.0 * c * r; break;
        case 1: {
          const double K = mu * mu / (2.0 * r), P = (g - 1.0) * (E - K), Pb = 2.0 * c * P, Kb = -Pb * (g - 1.0);
          gb += Pb * (E - K); b2 = Pb * (g - 1.0); b0 = Kb * mu / r; b1 = -Kb * K / r; break;
        }
        case 2: {
          const double KEb = 1.0 / Ms, Mb = -KE / (Ms * Ms);
          b0 = KEb * c * mu / r; b1 = -KEb * c * mu * mu / (2.0 * r * r) + Mb * c; break;
        }
        case 4: b0 = c * sin(2.0 * pi * x / (I.ne * I.dx)); break;
        case 6: b1 = (x >= prm[0] && x <= prm[1]) ? c : 0.0; break;
        default: break;
      }
      qb[0][m] = b0; qb[1][m] = b1; qb[2][m] = b2;
    }
    v.gbe()[e] = gb;  // starts the per-element d/dgamma accumulators
    v.abe()[e] = 0.0;
  }
  v.sync();
}

// ---------------------------------------------------------------------------
// Reverse of one RK stage: hyperbolic reverse, solver reverse, setup reverse.
// Sb: in = adjoint of Sigma carried from the later stages (adjoint of this
// stage's Sigma_out besides the RHS), out = adjoint of this stage's warm start.
// ---------------------------------------------------------------------------
template <int NP>
__device__ void d1_stage_rev(const View1<NP>& v, const BasisDev& B, int solver, int n, const StageTape1& t,
                             const double* const A[3], double c0, double c1, double c2, double* const Qn[3], int qn_mode,
                             double* const Qs[3], int qs_add, double* Sb, double* wk, double* s_red) {
  auto W = [&](int k) { return wk + (long long)k * v.N; };
  const double* qc[3] = {t.q[0], t.q[1], t.q[2]};
  d1_hyp_rev(v, B, qc, t.ir, t.sout, A, c0, c1, c2, Qn, qn_mode, Qs, qs_add, Sb);
  if (!(v.I.alpha > 0)) {
    d1_zero(v, Sb);  // Sigma = 0: nothing flows to the warm start
    return;
  }
  double* bb = W(0);
  double* iMb = W(1);
  double* Zinv = W(2);
  d1_solve_rev(v, B, solver, n, t, Sb, bb, iMb, Zinv, W(3), W(4), W(5), W(6), s_red);
  d1_setup_rev(v, B, t, bb, iMb, Zinv, Qs);
}

// ---------------------------------------------------------------------------
// The adjoint kernel. Scratch per instance (fields of N doubles):
//   state X (3), 1/rho, Sigma chain (2), step work, reverse buffers,
//   three stage tapes, `seg` step snapshots (level 2) and ceil(n_steps/seg)
//   segment snapshots (level 1). The forward runs once storing level-1
//   snapshots; each segment is re-run storing every step's state, and each
//   step is re-run once more with full stage tapes before its reverse.
// ---------------------------------------------------------------------------
enum : int {
  A1_X = 0, A1_IR = 3, A1_SA = 4, A1_SB = 5, A1_WK = 6,
  A1_QB = A1_WK + F1_STEP_FIELDS, A1_QN = A1_QB + 3, A1_Q2B = A1_QN + 3, A1_Q1B = A1_Q2B + 3, A1_SBAR = A1_Q1B + 3,
  A1_RW = A1_SBAR + 1, A1_TAPE = A1_RW + 7
};
__host__ __device__ inline long long adjoint1d_fields(int solver, int n_iter, int N, int n_steps, int seg) {
  const int nseg = seg > 0 ? (n_steps + seg - 1) / seg : 0;
  return (long long)A1_TAPE + 3LL * (STAGE1_FIELDS + solve_tape_fields1(solver, n_iter, N)) + 4LL * seg + 4LL * nseg;
}

struct Adj1DArgs {
  const Inst1D* inst; const int* order; BasisDev B;
  const double* q0;     // batch initial states [inst][3][N_i]
  double* dq0;          // batch gradients, same layout
  double *J, *dgamma, *dalpha;  // per instance
  double* scr;
  int solver, n_iter, objective, seg;
  double prm[4];
  int cs;               // CTAs per instance (cluster size)
  int* status;
};

template <int NP>
__global__ void __launch_bounds__(T1, 2) k1_adjoint(Adj1DArgs a) {
  __shared__ double s_red[T1];
  int inst;
  const View1<NP> v = make_view1<NP>(a.inst, a.order, a.scr, a.cs, &inst);
  const BasisDev& B = a.B;
  const Inst1D& I = v.I;
  const int N = v.N, n = I.n_steps, seg = a.seg;
  const int nseg = seg > 0 ? (n + seg - 1) / seg : 0;
  double* X[3] = {v.f(A1_X), v.f(A1_X + 1), v.f(A1_X + 2)};
  double* ir = v.f(A1_IR);
  double* wk = v.f(A1_WK);
  StageTape1 tp[3];
  const int tf = STAGE1_FIELDS + solve_tape_fields1(a.solver, a.n_iter, N);
  for (int s = 0; s < 3; ++s) tp[s] = stage_tape1(v, v.f(A1_TAPE + s * tf), a.solver, a.n_iter);
  double* ck2 = v.f(A1_TAPE + 3 * tf);
  double* ck1 = ck2 + 4LL * seg * N;
  auto snap = [&](double* dst, const double* S) {
    for (int m = v.m0() + threadIdx.x; m < v.m1(); m += blockDim.x) {
      dst[m] = X[0][m]; dst[N + m] = X[1][m]; dst[2 * N + m] = X[2][m]; dst[3 * N + m] = S[m];
    }
    v.sync();
  };
  double* Sx = v.f(A1_SA);
  double* Sy = v.f(A1_SB);
  auto restore = [&](const double* src) {
    Sx = v.f(A1_SA); Sy = v.f(A1_SB);
    for (int m = v.m0() + threadIdx.x; m < v.m1(); m += blockDim.x) {
      X[0][m] = src[m]; X[1][m] = src[N + m]; X[2][m] = src[2 * N + m]; Sx[m] = src[3 * N + m];
      ir[m] = 1.0 / src[N + m];
    }
    v.sync();
  };
  // ---- forward with level-1 snapshots
  const double* q0 = a.q0 + 3 * I.off;
  for (int m = v.m0() + threadIdx.x; m < v.m1(); m += blockDim.x) {
    X[0][m] = q0[m]; X[1][m] = q0[N + m]; X[2][m] = q0[2 * N + m]; ir[m] = 1.0 / q0[N + m]; Sx[m] = 0.0;
  }
  v.sync();
  for (int s = 0; s < n; ++s) {
    if (s % seg == 0) snap(ck1 + 4LL * (s / seg) * N, Sx);
    d1_step(v, B, a.solver, a.n_iter, X, ir, Sx, Sy, wk, nullptr, a.status, s_red);
  }
  // ---- objective and its gradient
  double KE = 0.0, Ms = 0.0;
  const double* Xc[3] = {X[0], X[1], X[2]};
  const double J = d1_objective(v, B, a.objective, a.prm, Xc, s_red, &KE, &Ms);
  double* QB[3] = {v.f(A1_QB), v.f(A1_QB + 1), v.f(A1_QB + 2)};
  double* QN[3] = {v.f(A1_QN), v.f(A1_QN + 1), v.f(A1_QN + 2)};
  double* Q2b[3] = {v.f(A1_Q2B), v.f(A1_Q2B + 1), v.f(A1_Q2B + 2)};
  double* Q1b[3] = {v.f(A1_Q1B), v.f(A1_Q1B + 1), v.f(A1_Q1B + 2)};
  double* Sb = v.f(A1_SBAR);
  d1_objective_grad(v, B, a.objective, a.prm, Xc, KE, Ms, QB);
  d1_zero(v, Sb);
  // ---- reverse, segment by segment
  for (int j = nseg - 1; j >= 0; --j) {
    const int s0 = j * seg, s1 = min(n, s0 + seg);
    restore(ck1 + 4LL * j * N);
    for (int s = s0; s < s1; ++s) {
      snap(ck2 + 4LL * (s - s0) * N, Sx);
      if (s + 1 < s1) d1_step(v, B, a.solver, a.n_iter, X, ir, Sx, Sy, wk, nullptr, a.status, s_red);
    }
    for (int s = s1 - 1; s >= s0; --s) {
      restore(ck2 + 4LL * (s - s0) * N);
      d1_step(v, B, a.solver, a.n_iter, X, ir, Sx, Sy, wk, tp, a.status, s_red);
      const double* A2[3] = {QB[0], QB[1], QB[2]};
      d1_stage_rev(v, B, a.solver, a.n_iter, tp[2], A2, 1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0, QN, 1, Q2b, 0, Sb, v.f(A1_RW),
                   s_red);
      const double* A1[3] = {Q2b[0], Q2b[1], Q2b[2]};
      d1_stage_rev(v, B, a.solver, a.n_iter, tp[1], A1, 0.75, 0.25, 0.25, QN, 2, Q1b, 0, Sb, v.f(A1_RW), s_red);
      const double* A0[3] = {Q1b[0], Q1b[1], Q1b[2]};
      d1_stage_rev(v, B, a.solver, a.n_iter, tp[0], A0, 0.0, 1.0, 1.0, QN, 0, QN, 1, Sb, v.f(A1_RW), s_red);
      for (int c = 0; c < 3; ++c) { double* t = QB[c]; QB[c] = QN[c]; QN[c] = t; }
    }
  }
  double* dq = a.dq0 + 3 * I.off;
  for (int m = v.m0() + threadIdx.x; m < v.m1(); m += blockDim.x) { dq[m] = QB[0][m]; dq[N + m] = QB[1][m]; dq[2 * N + m] = QB[2][m]; }
  const double gsum = v.esum(v.gbe(), s_red);
  const double asum = v.esum(v.abe(), s_red);
  if (threadIdx.x == 0 && v.e0 == 0) {
    a.J[inst] = J;
    a.dgamma[inst] = gsum;
    a.dalpha[inst] = asum;
  }
}

}  // namespace igrgpu
