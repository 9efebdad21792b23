// 1D continuous adjoint (optimise-then-discretise, conservative Pi form,
// IGR_adjoints_1d/adjoint_pde.jl:48-551) and run_forward_store
// (IGR_adjoints_1d/forward.jl:137-186) as one persistent kernel per instance,
// on the 1D engine's per-instance view (one CTA or a cluster per instance).
//
// Modes: 0 = store + adjoint (snapshots kept in the instance's scratch: all
// of them, or checkpoints every `seg` steps and one recomputed segment);
// 1 = store only (every snapshot written to a caller buffer); 2 = adjoint
// only (snapshots read from a caller buffer); 3 = one evaluation of the
// adjoint operator (compute_adjoint_rhs_conservative!).
//
// Per adjoint step the snapshot-only quantities are prepared once
// (d1_pde_prep: five local-source coefficients, the nodal d_x u, d_x Sigma /
// rho, 1/rho, the LLF wave speed) and each RK stage runs the Pi right-hand
// side, the Pi solve (the forward's d1_setup / d1_solve on the snapshot's
// density, warm-started) and the adjoint operator fused with the stage
// combination (d1_pde_rk).
#pragma once
#include "igr1d_rev_kernels.cuh"

namespace igrgpu {

// Scratch fields (after the E1_FIELDS per-element work) of k1_pde_adjoint.
enum : int {
  P1_X = F1_STEP_FIELDS, P1_IR = P1_X + 3, P1_SA = P1_IR + 1, P1_SB = P1_SA + 1,
  P1_A = P1_SB + 1, P1_A1 = P1_A + 3, P1_A2 = P1_A1 + 3, P1_PI = P1_A2 + 3,
  P1_B = P1_PI + 2, P1_CM = P1_B + 1, P1_CK = P1_CM + 1, P1_CPR = P1_CK + 1, P1_CINVM = P1_CPR + 1,
  P1_PP = P1_CINVM + 1, P1_SNAP = P1_PP + 9  // P1_PP: the 9 prepared fields of d1_pde_prep
};
// Snapshot fields (4 per snapshot) of mode 0: all n+1 snapshots when seg >= n,
// else n/seg + 1 checkpoints and a segment of seg snapshots.
__host__ __device__ inline long long pde1_snap_fields(int n, int seg) {
  if (seg >= n) return 4LL * (n + 1);
  return 4LL * (n / seg + 1) + 4LL * seg;
}

// Adjoint flux F_dag at one node (adjoint_pde.jl:48-68), linear in a.
__device__ __forceinline__ void pde1_flux(double g, double mu, double E, double S, double ir, const double a[3], double f[3]) {
  const double gm = g - 1.0;
  const double u = mu * ir;
  const double P = gm * (E - 0.5 * mu * u);
  const double Er = (E + P + S) * ir;       // (E + P_bar) / rho
  const double dPdmu = -gm * u, dPdr = 0.5 * gm * u * u;
  f[0] = fma(a[0], 2.0 * u + dPdmu, a[1]) + a[2] * fma(dPdmu, u, Er);
  f[1] = a[0] * (dPdr - u * u) + a[2] * u * (dPdr - Er);
  f[2] = fma(a[0], gm, a[2] * g * u);
}

// Per-step preparation from one snapshot (mu, rho, E, Sigma): the local-source
// coefficients of compute_adjoint_source_local! (adjoint_pde.jl:106-185),
//   S_mu = a_mu C0 + a_E C1,  S_rho = a_mu C2 + a_E C3,  S_E = a_E C4,
// the nodal d_x u and d_x Sigma / rho of the nonlocal source (:323-391), 1/rho
// and |u| + c. All threads call it; ends synchronised.
// s: snapshot (mu, rho, E, Sigma: 4 consecutive fields of N); pp: the prepared
// fields, consecutive: 1/rho, C0..C4, d_x u, d_x Sigma / rho, |u| + c.
constexpr int PP_IRS = 0, PP_SRC = 1, PP_NL = 6, PP_WS = 8, PP_FIELDS = 9;

template <int NP>
__device__ void d1_pde_prep(const View1<NP>& v, const BasisDev& B, const double* s, double* pp) {
  const Inst1D& I = v.I;
  const int N = v.N;
  const double* sq[4] = {s, s + N, s + 2 * N, s + 3 * N};
  double* irS = pp + PP_IRS * N;
  double* ws = pp + PP_WS * N;
  auto src = [&](int k) { return pp + (PP_SRC + k) * N; };
  auto nl = [&](int k) { return pp + (PP_NL + k) * N; };
  const double g = I.gamma, gm = g - 1.0, iJ = I.iJ;
  for (int e = v.e0 + threadIdx.x; e < v.e1; e += blockDim.x) {
    const int base = e * NP;
    double mu[NP], r[NP], E[NP], S[NP], ir[NP], u[NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const int m = base + i;
      mu[i] = sq[0][m]; r[i] = sq[1][m]; E[i] = sq[2][m]; S[i] = sq[3][m];
      ir[i] = 1.0 / r[i];
      u[i] = mu[i] * ir[i];
    }
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const int m = base + i;
      const double mu_x = iJ * dot_row<NP>(B, i, mu), r_x = iJ * dot_row<NP>(B, i, r);
      const double E_x = iJ * dot_row<NP>(B, i, E), S_x = iJ * dot_row<NP>(B, i, S);
      const double unx = iJ * dot_row<NP>(B, i, u);
      const double iri = ir[i], ir2 = iri * iri, ir3 = ir2 * iri;
      const double ui = u[i], mui = mu[i];
      const double P = gm * (E[i] - 0.5 * mui * ui);
      const double Pb = P + S[i];
      const double uxq = (mu_x - ui * r_x) * iri;
      const double dPdmu = -gm * ui, dPdr = 0.5 * gm * ui * ui;
      const double P_x = gm * (E_x - mui * mu_x * iri + 0.5 * mui * mui * r_x * ir2);
      const double drP_x = gm * (mui * mu_x * ir2 - mui * mui * r_x * ir3);
      const double dmuP_x = -gm * uxq;
      const double EPx = E_x + P_x + S_x, EP = E[i] + Pb;
      const double dmu_ux = -r_x * ir2;
      const double dr_u = -ui * iri;
      const double dr_ux = 2.0 * mui * r_x * ir3 - mu_x * ir2;
      src(0)[m] = mu_x * iri + uxq + mui * dmu_ux + dmuP_x;
      src(1)[m] = dmuP_x * ui + EPx * iri + dPdmu * uxq + EP * dmu_ux;
      src(2)[m] = mu_x * dr_u + mui * dr_ux + drP_x;
      src(3)[m] = drP_x * ui + EPx * dr_u + dPdr * uxq + EP * dr_ux;
      src(4)[m] = g * uxq;
      irS[m] = iri;
      ws[m] = fabs(ui) + sqrt(g * P * iri);
      nl(0)[m] = unx;
      nl(1)[m] = S_x * iri;
    }
  }
  v.sync();
}

// Pi right-hand side (adjoint_pde.jl:280-302, :424-429):
// b = alpha w_i J (d_x a_mu + u d_x a_E). All threads call it; ends synchronised.
template <int NP>
__device__ void d1_pde_b(const View1<NP>& v, const BasisDev& B, const double* a, const double* mu, const double* irS,
                         double* b) {
  const Inst1D& I = v.I;
  const double* a0 = a;
  const double* a2 = a + 2 * v.N;
  for (int e = v.e0 + threadIdx.x; e < v.e1; e += blockDim.x) {
    const int base = e * NP;
    double am[NP], aE[NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) { am[i] = a0[base + i]; aE[i] = a2[base + i]; }
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const int m = base + i;
      const double u = mu[m] * irS[m];
      const double v0 = I.iJ * fma(u, dot_row<NP>(B, i, aE), dot_row<NP>(B, i, am));
      b[m] = v0 * (I.alpha * B.w[i] * I.J);
    }
  }
  v.sync();
}

// Adjoint operator + RK stage: k = +(1/J) D f_dag + flipped LLF faces - S_loc a
// + S_Sigma(Pi) (adjoint_pde.jl:198-265, :323-391), a_out = c0 a^n + c1 a_s +
// c2 h k. Adjoint states are 3 consecutive fields of N (asb: stage input,
// anb: step start, aob: output, may alias anb but not asb); pp: prepared
// fields; Pi == nullptr: no nonlocal source; kb: optional raw k. All threads
// call it; ends synchronised.
template <int NP>
__device__ void d1_pde_rk(const View1<NP>& v, const BasisDev& B, const double* s, const double* pp, const double* Pi,
                          const double* asb, const double* anb, double c0, double c1, double c2, double h, double* aob,
                          double* kb) {
  constexpr int L = NP - 1;
  const Inst1D& I = v.I;
  const int N = v.N;
  const double* sq[4] = {s, s + N, s + 2 * N, s + 3 * N};
  const double* irS = pp + PP_IRS * N;
  const double* ws = pp + PP_WS * N;
  auto src = [&](int k) { return pp + (PP_SRC + k) * N; };
  auto nl = [&](int k) { return pp + (PP_NL + k) * N; };
  auto as = [&](int c) { return asb + c * N; };
  auto an = [&](int c) { return anb + c * N; };
  const double g = I.gamma, iJ = I.iJ, c2h = c2 * h;
  for (int e = v.e0 + threadIdx.x; e < v.e1; e += blockDim.x) {
    const int eL = wrap_left(e, I.ne), eR = wrap_right(e, I.ne);
    const int base = e * NP;
    double aa[3][NP], f[3][NP], k[3][NP];
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const int m = base + i;
      double av[3] = {as(0)[m], as(1)[m], as(2)[m]};
      double fv[3];
      pde1_flux(g, sq[0][m], sq[2][m], sq[3][m], irS[m], av, fv);
#pragma unroll
      for (int c = 0; c < 3; ++c) { aa[c][i] = av[c]; f[c][i] = fv[c]; }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int i = 0; i < NP; ++i) k[c][i] = iJ * dot_row<NP>(B, i, f[c]);
    // right face (own node L | node 0 of eR), correction with + sign
    {
      const int m = eR * NP;
      const double pa[3] = {as(0)[m], as(1)[m], as(2)[m]};
      double pf[3];
      pde1_flux(g, sq[0][m], sq[2][m], sq[3][m], irS[m], pa, pf);
      const double wl = ws[base + L], wr = ws[m];
      const double lam = max_nonneg(wr, wl);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const double fs = 0.5 * fma(-lam, aa[c][L] - pa[c], f[c][L] + pf[c]);
        k[c][L] = fma(iJ * B.iwL, fs - f[c][L], k[c][L]);
      }
    }
    // left face (node L of eL | own node 0), correction with - sign
    {
      const int m = eL * NP + L;
      const double pa[3] = {as(0)[m], as(1)[m], as(2)[m]};
      double pf[3];
      pde1_flux(g, sq[0][m], sq[2][m], sq[3][m], irS[m], pa, pf);
      const double wl = ws[m], wr = ws[base];
      const double lam = max_nonneg(wr, wl);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const double fs = 0.5 * fma(-lam, pa[c] - aa[c][0], pf[c] + f[c][0]);
        k[c][0] = fma(-iJ * B.iw0, fs - f[c][0], k[c][0]);
      }
    }
    // minus the local source
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const int m = base + i;
      k[0][i] -= fma(aa[0][i], src(0)[m], aa[2][i] * src(1)[m]);
      k[1][i] -= fma(aa[0][i], src(2)[m], aa[2][i] * src(3)[m]);
      k[2][i] -= aa[2][i] * src(4)[m];
    }
    // plus the nonlocal source
    if (Pi) {
      double pux[NP], psr[NP], P[NP];
#pragma unroll
      for (int i = 0; i < NP; ++i) {
        const int m = base + i;
        P[i] = Pi[m];
        pux[i] = P[i] * nl(0)[m];
        psr[i] = P[i] * nl(1)[m];
      }
#pragma unroll
      for (int i = 0; i < NP; ++i) {
        const int m = base + i;
        const double dpux = iJ * dot_row<NP>(B, i, pux), dpsr = iJ * dot_row<NP>(B, i, psr);
        const double ir = irS[m], ux = nl(0)[m];
        k[0][i] += -4.0 * dpux * ir;
        k[1][i] += fma(2.0 * P[i] * ux, ux, dpsr) * ir + 4.0 * dpux * sq[0][m] * (ir * ir);
      }
    }
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const int m = base + i;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        if (kb) kb[c * N + m] = k[c][i];
        if (aob) {
          double val = fma(c2h, k[c][i], c1 * aa[c][i]);
          if (c0 != 0.0) val = fma(c0, an(c)[m], val);
          aob[c * N + m] = val;
        }
      }
    }
  }
  v.sync();
}

// Terminal condition (adjoint_pde.jl:487-525): the L2 gradient density of J at
// the final state q; objectives 0 l2_density, 1 l2_pressure, 2 kinetic_energy,
// 4 weighted_momentum (L = N_e dx), 6 interval_rho (a_rho = chi_[a, b]).
template <int NP>
__device__ void d1_pde_terminal(const View1<NP>& v, const BasisDev& B, int obj, const double* prm, const double* const q[3],
                                double* const a[3], double* s_red) {
  const Inst1D& I = v.I;
  const double g = I.gamma, gm = g - 1.0, pi = 3.14159265358979323846;
  double KE = 0.0, M = 1.0;
  if (obj == 2) d1_objective(v, B, 2, prm, q, s_red, &KE, &M);
  for (int e = v.e0 + threadIdx.x; e < v.e1; e += blockDim.x) {
#pragma unroll
    for (int i = 0; i < NP; ++i) {
      const int m = e * NP + i;
      const double x = e * I.dx + I.J * (1.0 + B.xi[i]);
      const double mu = q[0][m], r = q[1][m], E = q[2][m];
      double b0 = 0.0, b1 = 0.0, b2 = 0.0;
      switch (obj) {
        case 0: b1 = 2.0 * r; break;
        case 1: {
          const double u = mu / r, p = gm * (E - mu * mu / (2.0 * r));
          b0 = -2.0 * gm * p * u; b1 = gm * p * (u * u); b2 = 2.0 * gm * p;
          break;
        }
        case 2: b0 = (mu / r) / M; b1 = -(mu * mu) / (2.0 * (r * r)) / M - KE / (M * M); break;
        case 4: b0 = sin(2.0 * pi * x / (I.ne * I.dx)); break;
        case 6: b1 = (x >= prm[0] && x <= prm[1]) ? 1.0 : 0.0; break;
        default: break;
      }
      a[0][m] = b0; a[1][m] = b1; a[2][m] = b2;
    }
  }
  v.sync();
}

// Batch layout: instance i's fields start at 3 off_i (q0, a0, as in the other
// 1D kernels) and its snapshots (modes 1, 2) at 4 (n_i + 1) off_i... given per
// instance by snap_off[i] (doubles).
struct Pde1DArgs {
  const Inst1D* inst; const int* order; BasisDev B;
  const double* q0;        // mode 0/1: initial states; mode 3: (mu, rho, E, Sigma) per instance at 4 off_i
  const double* ain;       // mode 3: the adjoint a (3 fields per instance)
  double* a0;              // modes 0/2: adjoint at t = 0; mode 3: the operator k
  double* pi;              // mode 3: Pi warm start in, solution out (N_i per instance at off_i)
  double* snaps;           // modes 1/2: snapshots, instance i at snap_off[i]
  const long long* snap_off;
  double* scr;
  int mode, solver, n_iter, objective, seg;
  double prm[4];
  int cs;
  int* status;
};

template <int NP>
__global__ void __launch_bounds__(T1, 2) k1_pde_adjoint(Pde1DArgs a) {
  __shared__ double s_red[T1];
  int inst;
  const View1<NP> v = make_view1<NP>(a.inst, a.order, a.scr, a.cs, &inst);
  const BasisDev& B = a.B;
  const Inst1D& I = v.I;
  const int N = v.N, n = I.n_steps;
  const bool apos = I.alpha > 0;
  const SolveTape1 none;
  double* X[3] = {v.f(P1_X), v.f(P1_X + 1), v.f(P1_X + 2)};
  double* ir = v.f(P1_IR);
  double* Sx = v.f(P1_SA);
  double* Sy = v.f(P1_SB);
  int cur = 0;

  // Sigma solve on the working state X (1/rho in ir): x0 = Sx, result swapped into Sx.
  auto solve_sigma = [&]() {
    d1_setup(v, B, X[0], ir, v.f(F1_B), v.f(F1_CM), v.f(F1_CK), v.f(F1_CPR), v.f(F1_CINVM), nullptr);
    d1_solve(v, B, a.solver, a.n_iter, v.f(F1_B), Sx, Sy, v.f(F1_CM), v.f(F1_CK), v.f(F1_CPR), v.f(F1_CINVM),
             v.f(F1_W0), v.f(F1_W1), v.f(F1_W2), v.f(F1_W3), none, s_red);
    double* t = Sx; Sx = Sy; Sy = t;
  };
  auto put = [&](double* dst) {  // snapshot (X, Sx) -> dst
    for (int m = v.m0() + threadIdx.x; m < v.m1(); m += blockDim.x) {
      dst[m] = X[0][m]; dst[N + m] = X[1][m]; dst[2 * N + m] = X[2][m]; dst[3 * N + m] = Sx[m];
    }
    v.sync();
  };
  auto get = [&](const double* src_) {  // working state <- snapshot
    Sx = v.f(P1_SA); Sy = v.f(P1_SB);
    for (int m = v.m0() + threadIdx.x; m < v.m1(); m += blockDim.x) {
      X[0][m] = src_[m]; X[1][m] = src_[N + m]; X[2][m] = src_[2 * N + m]; Sx[m] = src_[3 * N + m];
      ir[m] = 1.0 / src_[N + m];
    }
    v.sync();
  };
  // one forward step of run_forward_store: the RK step, then the post-step solve
  auto store_step = [&]() {
    d1_step(v, B, a.solver, a.n_iter, X, ir, Sx, Sy, v.scr, nullptr, a.status, s_red);
    if (apos) solve_sigma();
  };
  // the Pi solve of one stage on the prepared snapshot s (adjoint_pde.jl:424-441): b from the
  // stage input ain, warm start = the current Pi, result in x (!= x0)
  auto pi_solve = [&](const double* s, const double* ain, const double* x0, double* x) {
    d1_pde_b(v, B, ain, s, v.f(P1_PP + PP_IRS), v.f(P1_B));
    d1_solve(v, B, a.solver, a.n_iter, v.f(P1_B), x0, x, v.f(P1_CM), v.f(P1_CK), v.f(P1_CPR), v.f(P1_CINVM),
             v.f(F1_W0), v.f(F1_W1), v.f(F1_W2), v.f(F1_W3), none, s_red);
  };
  auto prep = [&](const double* s) {
    d1_pde_prep(v, B, s, v.f(P1_PP));
    if (apos) d1_setup(v, B, s, v.f(P1_PP + PP_IRS), v.f(F1_B), v.f(P1_CM), v.f(P1_CK), v.f(P1_CPR), v.f(P1_CINVM), nullptr);
  };
  // one backward SSP-RK3 step over snapshot s (adjoint_pde.jl:530-548): A -> A1 -> A2 -> A
  auto adjoint_step = [&](const double* s) {
    prep(s);
#pragma unroll 1
    for (int st = 0; st < 3; ++st) {
      const double* ain = v.f(st == 0 ? P1_A : (st == 1 ? P1_A1 : P1_A2));
      double* aout = v.f(st == 0 ? P1_A1 : (st == 1 ? P1_A2 : P1_A));
      if (apos) {
        pi_solve(s, ain, v.f(P1_PI + cur), v.f(P1_PI + 1 - cur));
        cur = 1 - cur;
      }
      double c0, c1, c2;
      rk1_coef(st, &c0, &c1, &c2);
      d1_pde_rk(v, B, s, v.f(P1_PP), apos ? v.f(P1_PI + cur) : nullptr, ain, v.f(P1_A), c0, c1, c2, I.h, aout, nullptr);
    }
  };

  if (a.mode == 3) {  // compute_adjoint_rhs_conservative! at one state
    const double* s = a.q0 + 4 * I.off;
    const double* ain = a.ain + 3 * I.off;
    double* pio = a.pi + I.off;
    prep(s);
    if (apos) pi_solve(s, ain, pio, v.f(P1_PI));
    d1_pde_rk(v, B, s, v.f(P1_PP), apos ? v.f(P1_PI) : nullptr, ain, ain, 0.0, 1.0, 0.0, 0.0, nullptr, a.a0 + 3 * I.off);
    if (apos) d1_copy(v, v.f(P1_PI), pio);
    return;
  }

  double* ext = (a.mode == 1 || a.mode == 2) ? a.snaps + a.snap_off[inst] : nullptr;
  const bool all = a.mode != 0 || a.seg >= n;
  double* sn = v.f(P1_SNAP);
  auto snap = [&](int k) -> double* { return (ext ? ext : sn) + 4LL * k * N; };  // all resident

  if (a.mode != 2) {
    // ---- forward store: snapshot 0 = q0 and its Sigma solve from zero (forward.jl:140-152)
    const double* q0 = a.q0 + 3 * I.off;
    for (int m = v.m0() + threadIdx.x; m < v.m1(); m += blockDim.x) {
      X[0][m] = q0[m]; X[1][m] = q0[N + m]; X[2][m] = q0[2 * N + m]; ir[m] = 1.0 / q0[N + m]; Sx[m] = 0.0;
    }
    v.sync();
    if (apos) solve_sigma();
    put(snap(0));
    for (int k = 0; k < n; ++k) {
      store_step();
      if (all) put(snap(k + 1));
      else if ((k + 1) % a.seg == 0) put(sn + 4LL * ((k + 1) / a.seg) * N);
    }
    if (a.mode == 1) return;
  }
  // ---- terminal condition at T and the backward integration
  {
    const double* sT = snap(n);
    const double* qT[3] = {all ? sT : X[0], all ? sT + N : X[1], all ? sT + 2 * N : X[2]};
    double* Ab[3] = {v.f(P1_A), v.f(P1_A + 1), v.f(P1_A + 2)};
    d1_pde_terminal(v, B, a.objective, a.prm, qT, Ab, s_red);
  }
  d1_zero(v, v.f(P1_PI));
  if (all) {
    for (int k = n; k >= 1; --k) adjoint_step(snap(k));
  } else {
    const int seg = a.seg, nseg = (n + seg - 1) / seg;
    double* sb = sn + 4LL * (n / seg + 1) * N;  // segment snapshots k0+1 .. k1
    for (int j = nseg - 1; j >= 0; --j) {
      const int k0 = j * seg, k1 = min(n, k0 + seg);
      get(sn + 4LL * j * N);
      for (int k = k0; k < k1; ++k) {
        store_step();
        put(sb + 4LL * (k - k0) * N);
      }
      for (int k = k1; k > k0; --k) adjoint_step(sb + 4LL * (k - k0 - 1) * N);
    }
  }
  double* out = a.a0 + 3 * I.off;
  const double* A = v.f(P1_A);
  for (int m = v.m0() + threadIdx.x; m < v.m1(); m += blockDim.x) {
    out[m] = A[m]; out[N + m] = A[N + m]; out[2 * N + m] = A[2 * N + m];
  }
}

}  // namespace igrgpu
