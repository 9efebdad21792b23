// ORACLE — test infrastructure only (see igr_common.hpp for the parity status).
// Continuous (optimise-then-discretise) adjoint of the 1D IGR-Euler system,
// conservative Pi formulation: run_forward_store (IGR_adjoints_1d/forward.jl:
// 137-186) and IGR_adjoints_1d/adjoint_pde.jl:48-551, restated expression by
// expression (left-to-right evaluation, no FMA contraction).
//
// Parity pin: the reference's own test of this path
// (IGR_adjoints_1d/tests/run_adjoint_conservative_test.jl) compares dJ/dA
// assembled from the adjoint at t = 0 with central finite differences of
// J(A) (tolerance 1e-2 at alpha = 0, 5e-2 at alpha > 0); tests/test_oracle.py
// runs it on this restatement.
#pragma once
#include "igr1d.hpp"

namespace igr {

// adjoint_flux_local, adjoint_pde.jl:48-68
inline void pde1_flux(double g, double mu, double r, double E, double S, const double a[3], double f[3]) {
  const double u = mu / r;
  const double P = pressure1d(g, mu, r, E);
  const double Pb = P + S;
  const double dP_dE = g - 1;
  const double dP_dmu = -(g - 1) * u;
  const double dP_dr = (g - 1) * (u * u) / 2;
  f[0] = a[0] * (2 * u + dP_dmu) + a[1] + a[2] * ((E + Pb) / r + dP_dmu * u);
  f[1] = a[0] * (-(u * u) + dP_dr) + a[2] * (dP_dr * u - (E + Pb) * u / r);
  f[2] = a[0] * dP_dE + a[2] * (1 + dP_dE) * u;
}

// adjoint_llf_flux_local, adjoint_pde.jl:77-91
inline void pde1_llf(double g, const double qL[4], const double qR[4], const double aL[3], const double aR[3], double fs[3]) {
  const double lam = jmax(wavespeed1d(g, qL[0], qL[1], qL[2]), wavespeed1d(g, qR[0], qR[1], qR[2]));
  double fL[3], fR[3];
  pde1_flux(g, qL[0], qL[1], qL[2], qL[3], aL, fL);
  pde1_flux(g, qR[0], qR[1], qR[2], qR[3], aR, fR);
  for (int v = 0; v < 3; ++v) fs[v] = (fL[v] + fR[v]) / 2 - lam * (aL[v] - aR[v]) / 2;
}

// compute_adjoint_source_local!, adjoint_pde.jl:106-185
inline void pde1_source_local(const Grid1D& G, double g, const double* const q[3], const double* Sig,
                              const double* const a[3], double* const Sv[3]) {
  const int np = G.np;
  const double invJ = 1 / G.m.J;
  for (int e = 0; e < G.m.Ne; ++e)
    for (int i = 0; i < np; ++i) {
      double mu_x = 0.0, r_x = 0.0, E_x = 0.0, S_x = 0.0;
      for (int j = 0; j < np; ++j) {
        const size_t k = G.id(j, e);
        mu_x += G.b.Dik(i, j) * q[0][k];
        r_x += G.b.Dik(i, j) * q[1][k];
        E_x += G.b.Dik(i, j) * q[2][k];
        S_x += G.b.Dik(i, j) * Sig[k];
      }
      mu_x *= invJ; r_x *= invJ; E_x *= invJ; S_x *= invJ;
      const size_t n = G.id(i, e);
      const double r = q[1][n], mu = q[0][n], E = q[2][n];
      const double u = mu / r;
      const double P = pressure1d(g, mu, r, E);
      const double Pb = P + Sig[n];
      const double u_x = (mu_x - u * r_x) / r;
      const double dP_dE = g - 1;
      const double dP_dmu = -(g - 1) * u;
      const double dP_dr = (g - 1) * (u * u) / 2;
      const double P_x = (g - 1) * (E_x - mu * mu_x / r + (mu * mu) * r_x / (2 * (r * r)));
      const double drP_x = (g - 1) * (mu * mu_x / (r * r) - (mu * mu) * r_x / (r * r * r));
      const double dmuP_x = -(g - 1) * u_x;
      const double Pb_x = P_x + S_x;
      const double amu = a[0][n], aE = a[2][n];
      const double dmu_u = 1 / r;
      const double dmu_ux = -r_x / (r * r);
      const double dr_u = -u / r;
      const double dr_ux = -mu_x / (r * r) + 2 * mu * r_x / (r * r * r);
      const double dmu_divFmu = mu_x * dmu_u + u_x + mu * dmu_ux + dmuP_x;
      const double dmu_divFE = dmuP_x * u + (E_x + Pb_x) * dmu_u + dP_dmu * u_x + (E + Pb) * dmu_ux;
      Sv[0][n] = amu * dmu_divFmu + aE * dmu_divFE;
      const double dr_divFmu = mu_x * dr_u + mu * dr_ux + drP_x;
      const double dr_divFE = drP_x * u + (E_x + Pb_x) * dr_u + dP_dr * u_x + (E + Pb) * dr_ux;
      Sv[1][n] = amu * dr_divFmu + aE * dr_divFE;
      const double dE_divFE = (1 + dP_dE) * u_x;
      Sv[2][n] = aE * dE_divFE;
    }
}

// compute_adjoint_hyperbolic_rhs_local!, adjoint_pde.jl:198-265
inline void pde1_hyperbolic_rhs_local(const Grid1D& G, double g, const double* const q[3], const double* Sig,
                                      const double* const a[3], double* const da[3]) {
  const int np = G.np, Ne = G.m.Ne, L = np - 1;
  const double invJ = 1 / G.m.J;
  std::vector<double> F[3];
  for (int v = 0; v < 3; ++v) F[v].resize(G.N);
  for (size_t n = 0; n < G.N; ++n) {
    const double an[3] = {a[0][n], a[1][n], a[2][n]};
    double f[3];
    pde1_flux(g, q[0][n], q[1][n], q[2][n], Sig[n], an, f);
    for (int v = 0; v < 3; ++v) F[v][n] = f[v];
  }
  for (int e = 0; e < Ne; ++e)
    for (int i = 0; i < np; ++i) {
      const size_t n = G.id(i, e);
      for (int v = 0; v < 3; ++v) da[v][n] = 0.0;
      for (int j = 0; j < np; ++j)
        for (int v = 0; v < 3; ++v) da[v][n] += invJ * G.b.Dik(i, j) * F[v][G.id(j, e)];
    }
  auto face = [&](size_t nl, size_t nr, double fs[3]) {
    const double qL[4] = {q[0][nl], q[1][nl], q[2][nl], Sig[nl]};
    const double qR[4] = {q[0][nr], q[1][nr], q[2][nr], Sig[nr]};
    const double aL[3] = {a[0][nl], a[1][nl], a[2][nl]};
    const double aR[3] = {a[0][nr], a[1][nr], a[2][nr]};
    pde1_llf(g, qL, qR, aL, aR, fs);
  };
  for (int e = 0; e < Ne; ++e) {
    const int eL = e == 0 ? Ne - 1 : e - 1, eR = e == Ne - 1 ? 0 : e + 1;
    double fR[3], fL[3];
    face(G.id(L, e), G.id(0, eR), fR);
    face(G.id(L, eL), G.id(0, e), fL);
    for (int v = 0; v < 3; ++v) { const size_t n = G.id(L, e); da[v][n] += invJ * (fR[v] - F[v][n]) / G.b.w[L]; }
    for (int v = 0; v < 3; ++v) { const size_t n = G.id(0, e); da[v][n] -= invJ * (fL[v] - F[v][n]) / G.b.w[0]; }
  }
  std::vector<double> Sb[3];
  for (int v = 0; v < 3; ++v) Sb[v].resize(G.N);
  double* Sv[3] = {Sb[0].data(), Sb[1].data(), Sb[2].data()};
  pde1_source_local(G, g, q, Sig, a, Sv);
  for (int v = 0; v < 3; ++v) for (size_t n = 0; n < G.N; ++n) da[v][n] -= Sv[v][n];
}

// compute_adjoint_elliptic_rhs!, adjoint_pde.jl:280-302: d_x a_mu + d_x a_E u
inline void pde1_elliptic_rhs(const Grid1D& G, double* b, const double* const a[3], const double* const q[3]) {
  const int np = G.np;
  const double invJ = 1 / G.m.J;
  for (int e = 0; e < G.m.Ne; ++e)
    for (int i = 0; i < np; ++i) {
      double amu_x = 0.0, aE_x = 0.0;
      for (int j = 0; j < np; ++j) {
        amu_x += G.b.Dik(i, j) * a[0][G.id(j, e)];
        aE_x += G.b.Dik(i, j) * a[2][G.id(j, e)];
      }
      amu_x *= invJ;
      aE_x *= invJ;
      const size_t n = G.id(i, e);
      const double u = q[0][n] / q[1][n];
      b[n] = amu_x + aE_x * u;
    }
}

// compute_nonlocal_source!, adjoint_pde.jl:323-391 (d = 1):
//   S_mu = -4 d_x(Pi u_x) / rho,
//   S_rho = [2 Pi u_x^2 + d_x(Pi Sigma_x / rho)] / rho + 4 d_x(Pi u_x) mu / rho^2,  S_E = 0.
inline void pde1_nonlocal_source(const Grid1D& G, const double* Pi, const double* const q[3], const double* Sig,
                                 double* const Sv[3]) {
  const int np = G.np;
  const double invJ = 1 / G.m.J;
  std::vector<double> Pux(G.N), PSr(G.N);
  auto ux_at = [&](int i, int e) {
    double s = 0.0;
    for (int j = 0; j < np; ++j) s += G.b.Dik(i, j) * (q[0][G.id(j, e)] / q[1][G.id(j, e)]);
    return s * invJ;
  };
  for (int e = 0; e < G.m.Ne; ++e)
    for (int i = 0; i < np; ++i) {
      double ux = 0.0, Sx = 0.0;
      for (int j = 0; j < np; ++j) {
        const size_t k = G.id(j, e);
        const double uj = q[0][k] / q[1][k];
        ux += G.b.Dik(i, j) * uj;
        Sx += G.b.Dik(i, j) * Sig[k];
      }
      ux *= invJ;
      Sx *= invJ;
      const size_t n = G.id(i, e);
      Pux[n] = Pi[n] * ux;
      PSr[n] = Pi[n] * Sx / q[1][n];
    }
  for (int e = 0; e < G.m.Ne; ++e)
    for (int i = 0; i < np; ++i) {
      double dPux = 0.0, dPSr = 0.0;
      for (int j = 0; j < np; ++j) {
        dPux += G.b.Dik(i, j) * Pux[G.id(j, e)];
        dPSr += G.b.Dik(i, j) * PSr[G.id(j, e)];
      }
      dPux *= invJ;
      dPSr *= invJ;
      const double ux = ux_at(i, e);
      const size_t n = G.id(i, e);
      const double r = q[1][n], mu = q[0][n];
      Sv[0][n] = -4 * dPux / r;
      Sv[1][n] = (2 * Pi[n] * (ux * ux) + dPSr) / r + 4 * dPux * mu / (r * r);
      Sv[2][n] = 0.0;
    }
}

// compute_adjoint_rhs_conservative!, adjoint_pde.jl:410-456 (Pi in-out).
inline void pde1_adjoint_rhs(const Grid1D& G, double g, double alpha, int n_iter, int solver, const double* const q[3],
                             const double* Sig, double* Pi, const double* const a[3], double* const da[3],
                             Work2D<double>& W) {
  pde1_hyperbolic_rhs_local(G, g, q, Sig, a, da);
  if (alpha > 0) {
    double* b = W.b.data();
    pde1_elliptic_rhs(G, b, a, q);
    for (int e = 0; e < G.m.Ne; ++e)
      for (int i = 0; i < G.np; ++i) b[G.id(i, e)] *= alpha * G.b.w[i] * G.m.J;
    sip_diagonal1d(G, W.M.data(), q[1], alpha);
    if (solver == SOLVER_PCG) pcg_fixed(G, Pi, b, W.M.data(), n_iter, q[1], alpha, W);
    else if (solver == SOLVER_JACOBI) jacobi_fixed(G, Pi, b, W.M.data(), n_iter, q[1], alpha, 2.0 / 3.0, W);
    else if (solver == SOLVER_CHEBYSHEV) chebyshev_fixed(G, Pi, b, W.M.data(), n_iter, q[1], alpha, W);
    std::vector<double> Sb[3];
    for (int v = 0; v < 3; ++v) Sb[v].resize(G.N);
    double* Sv[3] = {Sb[0].data(), Sb[1].data(), Sb[2].data()};
    pde1_nonlocal_source(G, Pi, q, Sig, Sv);
    for (int v = 0; v < 3; ++v) for (size_t n = 0; n < G.N; ++n) da[v][n] += Sv[v][n];
  }
}

// run_forward_store, IGR_adjoints_1d/forward.jl:137-186: snapshot k holds
// (mu, rho, E, Sigma) after step k; snaps: (n_steps + 1) * 4 * N doubles.
inline int run_forward_store1d(const Grid1D& G, const double* const q0[3], double dt, double T_end, double g,
                               double alpha, int n_iter, int solver, std::vector<double>& snaps) {
  const size_t N = G.N;
  std::vector<double> qv[3], Sig(N, 0.0);
  for (int v = 0; v < 3; ++v) qv[v].assign(q0[v], q0[v] + N);
  double* q[3] = {qv[0].data(), qv[1].data(), qv[2].data()};
  const double* qc[3] = {q[0], q[1], q[2]};
  Work2D<double> W; W.alloc(N);
  if (alpha > 0) solve_elliptic1d(G, Sig.data(), qc, alpha, n_iter, solver, W);
  double dtr;
  const int n_steps = rerounded_steps(dt, T_end, &dtr);
  snaps.assign((size_t)(n_steps + 1) * 4 * N, 0.0);
  auto push = [&](int k) {
    double* s = snaps.data() + (size_t)k * 4 * N;
    for (int v = 0; v < 3; ++v) std::copy(q[v], q[v] + N, s + v * N);
    std::copy(Sig.begin(), Sig.end(), s + 3 * N);
  };
  push(0);
  for (int s = 0; s < n_steps; ++s) {
    rk3_step1d(G, q, Sig.data(), g, alpha, dtr, n_iter, solver, W);
    if (alpha > 0) solve_elliptic1d(G, Sig.data(), qc, alpha, n_iter, solver, W);
    push(s + 1);
  }
  return n_steps;
}

// Terminal condition, adjoint_pde.jl:487-525 (l2_density, l2_pressure,
// weighted_momentum with L = N_e dx, kinetic_energy) plus the nodal interval
// objective (a_rho = chi_[a, b], no reference counterpart); others raise.
inline void pde1_terminal(const Grid1D& G, int obj, const double* const q[3], double g, const double* prm,
                          double* const a[3]) {
  const size_t N = G.N;
  const double pi = 3.14159265358979323846;
  for (int v = 0; v < 3; ++v) std::fill(a[v], a[v] + N, 0.0);
  if (obj == OBJ1_KINETIC_ENERGY) {
    double KE = 0.0, M = 0.0;
    for (int e = 0; e < G.m.Ne; ++e)
      for (int i = 0; i < G.np; ++i) {
        const size_t n = G.id(i, e);
        const double wJ = G.b.w[i] * G.m.J;
        KE += wJ * (q[0][n] * q[0][n]) / (2 * q[1][n]);
        M += wJ * q[1][n];
      }
    for (size_t n = 0; n < N; ++n) {
      a[0][n] = (q[0][n] / q[1][n]) / M;
      a[1][n] = -(q[0][n] * q[0][n]) / (2 * (q[1][n] * q[1][n])) / M - KE / (M * M);
    }
    return;
  }
  const double Ld = G.m.Ne * G.m.dx;
  for (int e = 0; e < G.m.Ne; ++e)
    for (int i = 0; i < G.np; ++i) {
      const size_t n = G.id(i, e);
      const double mu = q[0][n], r = q[1][n], E = q[2][n];
      switch (obj) {
        case OBJ1_L2_DENSITY: a[1][n] = 2 * r; break;
        case OBJ1_L2_PRESSURE: {
          const double u = mu / r;
          const double p = (g - 1) * (E - (mu * mu) / (2 * r));
          a[0][n] = -2 * (g - 1) * p * u;
          a[1][n] = (g - 1) * p * (u * u);
          a[2][n] = 2 * (g - 1) * p;
          break;
        }
        case OBJ1_WEIGHTED_MOMENTUM: a[0][n] = std::sin(2 * pi * G.x(i, e) / Ld); break;
        case OBJ1_INTERVAL_RHO: a[1][n] = interval_indicator(G.x(i, e), prm); break;
        default: throw std::invalid_argument("Unknown objective (use :l2_density, :l2_pressure, or :kinetic_energy)");
      }
    }
}

// run_adjoint_conservative, adjoint_pde.jl:474-551.
inline void run_adjoint_conservative1d(const Grid1D& G, const double* snaps, int n_steps, double dt, double T_end,
                                       double g, double alpha, int n_iter, int objective, int solver, const double* prm,
                                       double* const a_out[3]) {
  const size_t N = G.N;
  const double* qT[3];
  for (int v = 0; v < 3; ++v) qT[v] = snaps + (size_t)n_steps * 4 * N + v * N;
  std::vector<double> av[3], a1v[3], a2v[3], dav[3], Pi(N, 0.0);
  for (int v = 0; v < 3; ++v) { av[v].resize(N); a1v[v].resize(N); a2v[v].resize(N); dav[v].resize(N); }
  double* a[3] = {av[0].data(), av[1].data(), av[2].data()};
  double* a1[3] = {a1v[0].data(), a1v[1].data(), a1v[2].data()};
  double* a2[3] = {a2v[0].data(), a2v[1].data(), a2v[2].data()};
  double* da[3] = {dav[0].data(), dav[1].data(), dav[2].data()};
  pde1_terminal(G, objective, qT, g, prm, a);
  Work2D<double> W; W.alloc(N);
  const double h = std::min(dt, T_end);
  for (int n = n_steps; n >= 1; --n) {
    const double* s = snaps + (size_t)n * 4 * N;
    const double* q[3] = {s, s + N, s + 2 * N};
    const double* Sig = s + 3 * N;
    const double* ac[3] = {a[0], a[1], a[2]};
    pde1_adjoint_rhs(G, g, alpha, n_iter, solver, q, Sig, Pi.data(), ac, da, W);
    for (int v = 0; v < 3; ++v) for (size_t k = 0; k < N; ++k) a1[v][k] = a[v][k] + h * da[v][k];
    const double* a1c[3] = {a1[0], a1[1], a1[2]};
    pde1_adjoint_rhs(G, g, alpha, n_iter, solver, q, Sig, Pi.data(), a1c, da, W);
    for (int v = 0; v < 3; ++v) for (size_t k = 0; k < N; ++k)
      a2[v][k] = 3.0 / 4 * a[v][k] + 1.0 / 4 * a1[v][k] + 1.0 / 4 * h * da[v][k];
    const double* a2c[3] = {a2[0], a2[1], a2[2]};
    pde1_adjoint_rhs(G, g, alpha, n_iter, solver, q, Sig, Pi.data(), a2c, da, W);
    for (int v = 0; v < 3; ++v) for (size_t k = 0; k < N; ++k)
      a[v][k] = 1.0 / 3 * a[v][k] + 2.0 / 3 * a2[v][k] + 2.0 / 3 * h * da[v][k];
  }
  for (int v = 0; v < 3; ++v) std::copy(a[v], a[v] + N, a_out[v]);
}

}  // namespace igr
