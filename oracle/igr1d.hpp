// ORACLE — test infrastructure only (see igr_common.hpp for the parity status).
// 1D restatement of IGR_adjoints_1d: euler.jl, hyperbolic.jl, elliptic.jl,
// forward.jl, sensitivity.jl, enzyme_adjoint.jl objectives, plus the
// hand-written reverse of the objective loop.
// Field layout: Julia column-major (n_p, N_e): idx(i, e) = i + np*e.
// State ordering (mu, rho, E), IGR_adjoints_1d/euler.jl:23.
#pragma once
#include "igr2d_adjoint.hpp"

namespace igr {

struct Mesh1D { int Ne = 1; double L = 1.0, dx = 1.0, J = 0.5; };
// IGR_adjoints_1d/mesh.jl:21-33
inline Mesh1D make_mesh1d(int Ne, double L) { Mesh1D m; m.Ne = Ne; m.L = L; m.dx = L / Ne; m.J = m.dx / 2.0; return m; }

struct Grid1D {
  Basis b; Mesh1D m; int np; size_t N;
  Grid1D(const Basis& b_, const Mesh1D& m_) : b(b_), m(m_), np(b_.np), N((size_t)b_.np * m_.Ne) {}
  size_t id(int i, int e) const { return (size_t)i + (size_t)np * e; }
  double x(int i, int e) const { return (e * m.dx) + m.J * (1.0 + b.xi[i]); }
};

// euler.jl:46-111
template <class T> inline T pressure1d(const T& g, const T& mu, const T& r, const T& E) { return (g - 1.0) * (E - mu * mu / (2.0 * r)); }
template <class T> inline void flux1d(const T& g, const T& mu, const T& r, const T& E, const T& S, T f[3]) {
  T p = pressure1d(g, mu, r, E); T pb = p + S;
  f[0] = mu * mu / r + pb; f[1] = mu; f[2] = (E + pb) * mu / r;
}
template <class T> inline T wavespeed1d(const T& g, const T& mu, const T& r, const T& E) {
  T u = mu / r; T c = jsqrt(g * pressure1d(g, mu, r, E) / r); return jabs(u) + c;
}

// hyperbolic.jl:134-194
template <class T>
void hyperbolic_rhs1d(const Grid1D& G, const T& g, const T* const q[3], const T* S, T* const dq[3]) {
  const int np = G.np, Ne = G.m.Ne, L = np - 1; const Basis& B = G.b;
  std::vector<T> F[3];
  for (int v = 0; v < 3; ++v) F[v].resize(G.N);
  for (size_t n = 0; n < G.N; ++n) { T f[3]; flux1d(g, q[0][n], q[1][n], q[2][n], S[n], f); for (int v = 0; v < 3; ++v) F[v][n] = f[v]; }
  const double invJ = 1 / G.m.J;
  for (int e = 0; e < Ne; ++e) for (int i = 0; i < np; ++i) {
    const size_t n = G.id(i, e);
    for (int v = 0; v < 3; ++v) dq[v][n] = T(0.0);
    for (int j = 0; j < np; ++j) for (int v = 0; v < 3; ++v) dq[v][n] = dq[v][n] - invJ * B.Dik(i, j) * F[v][G.id(j, e)];
  }
  auto llf = [&](size_t nl, size_t nr, T fs[3]) {
    T lam = jmax(wavespeed1d(g, q[0][nl], q[1][nl], q[2][nl]), wavespeed1d(g, q[0][nr], q[1][nr], q[2][nr]));
    lam = 1.0 * lam;
    for (int v = 0; v < 3; ++v) fs[v] = (F[v][nl] + F[v][nr]) / 2.0 + lam * (q[v][nl] - q[v][nr]) / 2.0;
  };
  for (int e = 0; e < Ne; ++e) {
    const int eL = e == 0 ? Ne - 1 : e - 1, eR = e == Ne - 1 ? 0 : e + 1;
    T fR[3], fL[3];
    llf(G.id(L, e), G.id(0, eR), fR);
    llf(G.id(L, eL), G.id(0, e), fL);
    for (int v = 0; v < 3; ++v) { const size_t n = G.id(L, e); dq[v][n] = dq[v][n] - invJ * (fR[v] - F[v][n]) / B.w[L]; }
    for (int v = 0; v < 3; ++v) { const size_t n = G.id(0, e); dq[v][n] = dq[v][n] + invJ * (fL[v] - F[v][n]) / B.w[0]; }
  }
}

// elliptic.jl:32-116
template <class T>
void apply_sip(const Grid1D& G, T* y, const T* x, const T* rho, const T& alpha) {
  const int np = G.np, Ne = G.m.Ne, L = np - 1; const Basis& B = G.b; const double J = G.m.J, invJ = 1 / J;
  const int eta = (B.p + 1) * (B.p + 1);
  for (size_t n = 0; n < G.N; ++n) y[n] = T(0.0);
  for (int e = 0; e < Ne; ++e) for (int i = 0; i < np; ++i) {
    const size_t n = G.id(i, e);
    y[n] = y[n] + B.w[i] * J * x[n] / rho[n];
    T dxi(0.0);
    for (int j = 0; j < np; ++j) dxi = dxi + B.Dik(i, j) * x[G.id(j, e)];
    for (int k = 0; k < np; ++k) { const size_t m = G.id(k, e); y[m] = y[m] + alpha * B.w[i] * invJ * dxi / rho[n] * B.Dik(i, k); }
  }
  for (int e = 0; e < Ne; ++e) {
    const int eR = e == Ne - 1 ? 0 : e + 1;
    const size_t nl = G.id(L, e), nr = G.id(0, eR);
    T SL = x[nl], SR = x[nr], rL = rho[nl], rR = rho[nr];
    T jump = SL - SR;
    T dL(0.0), dR(0.0);
    for (int j = 0; j < np; ++j) { dL = dL + B.Dik(L, j) * x[G.id(j, e)]; dR = dR + B.Dik(0, j) * x[G.id(j, eR)]; }
    T avg = invJ * ((1.0 / rL) * dL + (1.0 / rR) * dR) / 2.0;
    T kap = jmax(T(1.0 / rL), T(1.0 / rR));
    T sig = (double)eta * kap / G.m.dx;
    y[nl] = y[nl] + (-alpha) * avg * 1.0;
    y[nr] = y[nr] + (-alpha) * avg * (-1.0);
    for (int k = 0; k < np; ++k) {
      const size_t a = G.id(k, e), c = G.id(k, eR);
      y[a] = y[a] + (-alpha) * (1.0 / (2.0 * rL)) * invJ * B.Dik(L, k) * 1.0 * jump;
      y[c] = y[c] + (-alpha) * (1.0 / (2.0 * rR)) * invJ * B.Dik(0, k) * 1.0 * jump;
    }
    y[nl] = y[nl] + alpha * sig * jump;
    y[nr] = y[nr] - alpha * sig * jump;
  }
}
template <class T> void apply_sip1d(const Grid1D& G, T* y, const T* x, const T* rho, const T& alpha) { apply_sip(G, y, x, rho, alpha); }

// elliptic.jl:126-154
template <class T>
void igr_rhs1d(const Grid1D& G, T* b, const T* mu, const T* rho, const T& alpha) {
  const int np = G.np; const Basis& B = G.b; const double J = G.m.J, invJ = 1 / J;
  for (int e = 0; e < G.m.Ne; ++e) for (int i = 0; i < np; ++i) {
    T du(0.0);
    for (int j = 0; j < np; ++j) { const size_t m = G.id(j, e); du = du + B.Dik(i, j) * (mu[m] / rho[m]); }
    du = du * invJ;
    T R = 2.0 * alpha * (du * du);
    b[G.id(i, e)] = B.w[i] * J * R;
  }
}

// elliptic.jl:206-253
template <class T>
void sip_diagonal1d(const Grid1D& G, T* M, const T* rho, const T& alpha) {
  const int np = G.np, L = np - 1; const Basis& B = G.b; const double J = G.m.J, invJ = 1 / J;
  const int eta = np * np;
  for (size_t n = 0; n < G.N; ++n) M[n] = T(0.0);
  for (int e = 0; e < G.m.Ne; ++e) for (int i = 0; i < np; ++i) { const size_t n = G.id(i, e); M[n] = M[n] + B.w[i] * J / rho[n]; }
  for (int e = 0; e < G.m.Ne; ++e) for (int k = 0; k < np; ++k) {
    const size_t n = G.id(k, e);
    for (int i = 0; i < np; ++i) { const double d = B.Dik(i, k); M[n] = M[n] + alpha * B.w[i] * invJ * (d * d) / rho[G.id(i, e)]; }
  }
  for (int e = 0; e < G.m.Ne; ++e) {
    const int eR = e == G.m.Ne - 1 ? 0 : e + 1;
    const size_t nl = G.id(L, e), nr = G.id(0, eR);
    T rL = rho[nl], rR = rho[nr];
    T sig = (double)eta * jmax(T(1.0 / rL), T(1.0 / rR)) / G.m.dx;
    M[nl] = M[nl] + (-alpha) * invJ * B.Dik(L, L) / rL;
    M[nl] = M[nl] + alpha * sig;
    M[nr] = M[nr] + alpha * invJ * B.Dik(0, 0) / rR;
    M[nr] = M[nr] + alpha * sig;
  }
}

template <class T>
void solve_elliptic1d(const Grid1D& G, T* Sig, const T* const q[3], const T& alpha, int n_iter, int solver, Work2D<T>& W) {
  igr_rhs1d(G, W.b.data(), q[0], q[1], alpha);
  sip_diagonal1d(G, W.M.data(), q[1], alpha);
  if (solver == SOLVER_PCG) pcg_fixed(G, Sig, W.b.data(), W.M.data(), n_iter, q[1], alpha, W);
  else if (solver == SOLVER_JACOBI) jacobi_fixed(G, Sig, W.b.data(), W.M.data(), n_iter, q[1], alpha, 2.0 / 3.0, W);
  else if (solver == SOLVER_CHEBYSHEV) chebyshev_fixed(G, Sig, W.b.data(), W.M.data(), n_iter, q[1], alpha, W);
  else throw std::invalid_argument("Unknown solver (use :pcg, :jacobi, or :chebyshev)");
}

template <class T>
void igr_euler_rhs1d(const Grid1D& G, const T* const q[3], T* Sig, const T& g, const T& alpha, int n_iter, int solver, Work2D<T>& W) {
  if (value(alpha) > 0) solve_elliptic1d(G, Sig, q, alpha, n_iter, solver, W);
  else for (size_t k = 0; k < G.N; ++k) Sig[k] = T(0.0);
  T* dq[3] = {W.dq[0].data(), W.dq[1].data(), W.dq[2].data()};
  hyperbolic_rhs1d(G, g, q, Sig, dq);
}

// forward.jl:61-79 (one SSP-RK3 step)
template <class T>
void rk3_step1d(const Grid1D& G, T* const q[3], T* Sig, const T& g, const T& alpha, double dt, int n_iter, int solver, Work2D<T>& W) {
  const size_t N = G.N;
  const T* qc[3] = {q[0], q[1], q[2]};
  igr_euler_rhs1d(G, qc, Sig, g, alpha, n_iter, solver, W);
  for (int v = 0; v < 3; ++v) for (size_t k = 0; k < N; ++k) W.q1[v][k] = q[v][k] + dt * W.dq[v][k];
  const T* q1[3] = {W.q1[0].data(), W.q1[1].data(), W.q1[2].data()};
  igr_euler_rhs1d(G, q1, Sig, g, alpha, n_iter, solver, W);
  for (int v = 0; v < 3; ++v) for (size_t k = 0; k < N; ++k) W.q2[v][k] = 3.0 / 4 * q[v][k] + 1.0 / 4 * W.q1[v][k] + 1.0 / 4 * dt * W.dq[v][k];
  const T* q2[3] = {W.q2[0].data(), W.q2[1].data(), W.q2[2].data()};
  igr_euler_rhs1d(G, q2, Sig, g, alpha, n_iter, solver, W);
  for (int v = 0; v < 3; ++v) for (size_t k = 0; k < N; ++k) q[v][k] = 1.0 / 3 * q[v][k] + 2.0 / 3 * W.q2[v][k] + 2.0 / 3 * dt * W.dq[v][k];
}

// run_forward!, forward.jl:50-87
template <class T>
void run_forward1d(const Grid1D& G, T* const q[3], T* Sig, double dt, double T_end, const T& g, const T& alpha, int n_iter, int solver) {
  for (size_t k = 0; k < G.N; ++k) Sig[k] = T(0.0);
  Work2D<T> W; W.alloc(G.N);
  double dtr; int n_steps = rerounded_steps(dt, T_end, &dtr);
  for (int s = 0; s < n_steps; ++s) rk3_step1d(G, q, Sig, g, alpha, dtr, n_iter, solver, W);
  if (value(alpha) > 0) { const T* qc[3] = {q[0], q[1], q[2]}; solve_elliptic1d(G, Sig, qc, alpha, n_iter, solver, W); }
}

// Objectives: enzyme_adjoint.jl:34-215 (l2_density, l2_pressure, weighted_momentum,
// kinetic_energy) plus the nodal interval extension (prm = (a, b)).
enum Objective1D { OBJ1_L2_DENSITY = 0, OBJ1_L2_PRESSURE = 1, OBJ1_KINETIC_ENERGY = 2, OBJ1_WEIGHTED_MOMENTUM = 4, OBJ1_INTERVAL_RHO = 6 };
inline double interval_indicator(double x, const double* prm) { return (x >= prm[0] && x <= prm[1]) ? 1.0 : 0.0; }

template <class T>
T objective1d(const Grid1D& G, int obj, const T* const q[3], const T& g, const double* prm) {
  const int np = G.np; const Basis& B = G.b; const double J = G.m.J;
  const double pi = 3.14159265358979323846;
  T acc(0.0), Ms(0.0);
  for (int e = 0; e < G.m.Ne; ++e) for (int i = 0; i < np; ++i) {
    const size_t n = G.id(i, e);
    const T &mu = q[0][n], &r = q[1][n], &E = q[2][n];
    switch (obj) {
      case OBJ1_L2_DENSITY: acc = acc + B.w[i] * J * (r * r); break;
      case OBJ1_L2_PRESSURE: { T p = (g - 1.0) * (E - mu * mu / (2.0 * r)); acc = acc + B.w[i] * J * (p * p); break; }
      case OBJ1_KINETIC_ENERGY: { const double wJ = B.w[i] * J; acc = acc + wJ * (mu * mu) / (2.0 * r); Ms = Ms + wJ * r; break; }
      case OBJ1_WEIGHTED_MOMENTUM: {
        const double Ld = G.m.Ne * G.m.dx;
        acc = acc + B.w[i] * J * mu * std::sin(2 * pi * G.x(i, e) / Ld); break;
      }
      case OBJ1_INTERVAL_RHO: acc = acc + B.w[i] * J * r * interval_indicator(G.x(i, e), prm); break;
      default: throw std::invalid_argument("Unknown objective");
    }
  }
  if (obj == OBJ1_KINETIC_ENERGY) return acc / Ms;
  return acc;
}

template <class T>
T objective_run1d(const Grid1D& G, int obj, T* const q[3], int n_steps, double dt, const T& g, const T& alpha, int n_iter, int solver, const double* prm) {
  std::vector<T> Sig(G.N, T(0.0));
  Work2D<T> W; W.alloc(G.N);
  for (int s = 0; s < n_steps; ++s) rk3_step1d(G, q, Sig.data(), g, alpha, dt, n_iter, solver, W);
  const T* qc[3] = {q[0], q[1], q[2]};
  return objective1d(G, obj, qc, g, prm);
}

// --------------------------- tangent (sensitivity.jl) ---------------------------
// sensitivity_flux, sensitivity.jl:36-48
template <class T>
inline void sens_flux1d(const T& g, const T& mu, const T& r, const T& E, const T& S, const T& smu, const T& sr, const T& sE, const T& sS,
                        double sg, T f[3]) {
  T u = mu / r; T su = (smu - u * sr) / r; T P = pressure1d(g, mu, r, E);
  T e = E / r - u * u / 2.0;
  T sP = (g - 1.0) * (sE - sr * (u * u) / 2.0 - r * u * su) + sg * r * e;
  f[0] = smu * u + mu * su + sP + sS; f[1] = smu; f[2] = su * (E + P + S) + u * (sE + sP + sS);
}

// compute_sensitivity_hyperbolic_rhs!, sensitivity.jl:90-152
template <class T>
void sens_hyperbolic_rhs1d(const Grid1D& G, const T& g, const T* const q[3], const T* S, const T* const s[3], const T* sS, double sg, T* const ds[3]) {
  const int np = G.np, Ne = G.m.Ne, L = np - 1; const Basis& B = G.b; const double invJ = 1 / G.m.J;
  std::vector<T> F[3];
  for (int v = 0; v < 3; ++v) F[v].resize(G.N);
  for (size_t n = 0; n < G.N; ++n) { T f[3]; sens_flux1d(g, q[0][n], q[1][n], q[2][n], S[n], s[0][n], s[1][n], s[2][n], sS[n], sg, f); for (int v = 0; v < 3; ++v) F[v][n] = f[v]; }
  for (int e = 0; e < Ne; ++e) for (int i = 0; i < np; ++i) {
    const size_t n = G.id(i, e);
    for (int v = 0; v < 3; ++v) ds[v][n] = T(0.0);
    for (int j = 0; j < np; ++j) for (int v = 0; v < 3; ++v) ds[v][n] = ds[v][n] - invJ * B.Dik(i, j) * F[v][G.id(j, e)];
  }
  auto llf = [&](size_t nl, size_t nr, T fs[3]) {
    T lam = jmax(wavespeed1d(g, q[0][nl], q[1][nl], q[2][nl]), wavespeed1d(g, q[0][nr], q[1][nr], q[2][nr]));
    for (int v = 0; v < 3; ++v) fs[v] = (F[v][nl] + F[v][nr]) / 2.0 + lam * (s[v][nl] - s[v][nr]) / 2.0;
  };
  for (int e = 0; e < Ne; ++e) {
    const int eL = e == 0 ? Ne - 1 : e - 1, eR = e == Ne - 1 ? 0 : e + 1;
    T fR[3], fL[3];
    llf(G.id(L, e), G.id(0, eR), fR);
    llf(G.id(L, eL), G.id(0, e), fL);
    for (int v = 0; v < 3; ++v) { const size_t n = G.id(L, e); ds[v][n] = ds[v][n] - invJ * (fR[v] - F[v][n]) / B.w[L]; }
    for (int v = 0; v < 3; ++v) { const size_t n = G.id(0, e); ds[v][n] = ds[v][n] + invJ * (fL[v] - F[v][n]) / B.w[0]; }
  }
}

// Form 1 RHS, sensitivity.jl:168-256
template <class T>
void sens_elliptic_rhs1d_form1(const Grid1D& G, T* b, const T* const q[3], const T* S, const T* const s[3], const T& alpha) {
  const int np = G.np, L = np - 1; const Basis& B = G.b; const double J = G.m.J, invJ = 1 / J;
  const int eta = np * np;
  const T *mu = q[0], *rho = q[1], *smu = s[0], *sr = s[1];
  for (size_t n = 0; n < G.N; ++n) b[n] = T(0.0);
  for (int e = 0; e < G.m.Ne; ++e) for (int i = 0; i < np; ++i) {
    T ux(0.0), sux(0.0);
    for (int j = 0; j < np; ++j) {
      const size_t m = G.id(j, e);
      T uj = mu[m] / rho[m]; T suj = (smu[m] - uj * sr[m]) / rho[m];
      ux = ux + B.Dik(i, j) * uj; sux = sux + B.Dik(i, j) * suj;
    }
    ux = ux * invJ; sux = sux * invJ;
    const size_t n = G.id(i, e);
    T src = 4.0 * alpha * ux * sux + sr[n] * S[n] / (rho[n] * rho[n]);
    b[n] = b[n] + B.w[i] * J * src;
    T ki = sr[n] / (rho[n] * rho[n]);
    T dS(0.0);
    for (int j = 0; j < np; ++j) dS = dS + B.Dik(i, j) * S[G.id(j, e)];
    for (int k = 0; k < np; ++k) { const size_t m = G.id(k, e); b[m] = b[m] + alpha * B.w[i] * invJ * ki * dS * B.Dik(i, k); }
  }
  for (int e = 0; e < G.m.Ne; ++e) {
    const int eR = e == G.m.Ne - 1 ? 0 : e + 1;
    const size_t nl = G.id(L, e), nr = G.id(0, eR);
    T SL = S[nl], SR = S[nr];
    T kL = sr[nl] / (rho[nl] * rho[nl]), kR = sr[nr] / (rho[nr] * rho[nr]);
    T jump = SL - SR;
    T dL(0.0), dR(0.0);
    for (int j = 0; j < np; ++j) { dL = dL + B.Dik(L, j) * S[G.id(j, e)]; dR = dR + B.Dik(0, j) * S[G.id(j, eR)]; }
    T avg = invJ * (kL * dL + kR * dR) / 2.0;
    T kmax = jmax(kL, kR);
    T sig = (double)eta * kmax / G.m.dx;
    b[nl] = b[nl] + (-alpha) * avg * 1.0;
    b[nr] = b[nr] + (-alpha) * avg * (-1.0);
    for (int k = 0; k < np; ++k) {
      const size_t a = G.id(k, e), c = G.id(k, eR);
      b[a] = b[a] + (-alpha) * (kL / 2.0) * invJ * B.Dik(L, k) * 1.0 * jump;
      b[c] = b[c] + (-alpha) * (kR / 2.0) * invJ * B.Dik(0, k) * 1.0 * jump;
    }
    b[nl] = b[nl] + alpha * sig * jump;
    b[nr] = b[nr] - alpha * sig * jump;
  }
}

// Form 2 RHS, sensitivity.jl:272-314
template <class T>
void sens_elliptic_rhs1d_form2(const Grid1D& G, T* b, const T* const q[3], const T* S, const T* const s[3], const T& alpha) {
  const int np = G.np; const Basis& B = G.b; const double J = G.m.J, invJ = 1 / J;
  const T *mu = q[0], *rho = q[1], *smu = s[0], *sr = s[1];
  for (int e = 0; e < G.m.Ne; ++e) for (int i = 0; i < np; ++i) {
    T ux(0.0), sux(0.0), dso(0.0), dS(0.0);
    for (int j = 0; j < np; ++j) {
      const size_t m = G.id(j, e);
      T uj = mu[m] / rho[m]; T suj = (smu[m] - uj * sr[m]) / rho[m];
      ux = ux + B.Dik(i, j) * uj; sux = sux + B.Dik(i, j) * suj;
      dso = dso + B.Dik(i, j) * (sr[m] / rho[m]); dS = dS + B.Dik(i, j) * S[m];
    }
    ux = ux * invJ; sux = sux * invJ; dso = dso * invJ; dS = dS * invJ;
    const size_t n = G.id(i, e);
    T so = sr[n] / rho[n];
    T R = alpha * (2.0 * ux * (2.0 * sux + so * ux) - dso * dS / rho[n]);
    b[n] = B.w[i] * J * R;
  }
}

// run_sensitivity + ssp_rk3_coupled, sensitivity.jl:401-515: the step loop is
// `while t < T - 1e-14; dt = min(dt, T - t)` with no dt re-rounding.
template <class T>
void run_sensitivity1d(const Grid1D& G, T* const q[3], T* const s[3], T* Sig, T* sSig, double dt, double T_end, const T& g,
                       const T& alpha, int n_iter, int solver, int form, double sg) {
  const size_t N = G.N;
  for (size_t k = 0; k < N; ++k) { Sig[k] = T(0.0); sSig[k] = T(0.0); }
  Work2D<T> W; W.alloc(N);
  std::vector<T> s1[3], s2[3], dsv[3], dqs[3];
  for (int v = 0; v < 3; ++v) { s1[v].resize(N); s2[v].resize(N); dsv[v].resize(N); dqs[v].resize(N); }
  auto sens_solve = [&](const T* const qq[3], const T* const ss[3]) {
    if (form == 1) sens_elliptic_rhs1d_form1(G, W.b.data(), qq, Sig, ss, alpha);
    else if (form == 2) sens_elliptic_rhs1d_form2(G, W.b.data(), qq, Sig, ss, alpha);
    else throw std::invalid_argument("Unknown elliptic_rhs (use :form1 or :form2)");
    sip_diagonal1d(G, W.M.data(), qq[1], alpha);
    if (solver == SOLVER_PCG) pcg_fixed(G, sSig, W.b.data(), W.M.data(), n_iter, qq[1], alpha, W);
    else if (solver == SOLVER_JACOBI) jacobi_fixed(G, sSig, W.b.data(), W.M.data(), n_iter, qq[1], alpha, 2.0 / 3.0, W);
    else chebyshev_fixed(G, sSig, W.b.data(), W.M.data(), n_iter, qq[1], alpha, W);
  };
  auto stage = [&](const T* const qq[3], const T* const ss[3]) {
    igr_euler_rhs1d(G, qq, Sig, g, alpha, n_iter, solver, W);
    for (int v = 0; v < 3; ++v) dqs[v] = W.dq[v];
    if (value(alpha) > 0) sens_solve(qq, ss);
    else for (size_t k = 0; k < N; ++k) sSig[k] = T(0.0);
    T* dsp[3] = {dsv[0].data(), dsv[1].data(), dsv[2].data()};
    sens_hyperbolic_rhs1d(G, g, qq, Sig, ss, sSig, sg, dsp);
  };
  double t = 0.0;
  while (t < T_end - 1e-14) {
    const double h = std::min(dt, T_end - t);
    { const T* qq[3] = {q[0], q[1], q[2]}; const T* ss[3] = {s[0], s[1], s[2]}; stage(qq, ss); }
    for (int v = 0; v < 3; ++v) for (size_t k = 0; k < N; ++k) { W.q1[v][k] = q[v][k] + h * dqs[v][k]; s1[v][k] = s[v][k] + h * dsv[v][k]; }
    { const T* qq[3] = {W.q1[0].data(), W.q1[1].data(), W.q1[2].data()}; const T* ss[3] = {s1[0].data(), s1[1].data(), s1[2].data()}; stage(qq, ss); }
    for (int v = 0; v < 3; ++v) for (size_t k = 0; k < N; ++k) {
      W.q2[v][k] = 3.0 / 4 * q[v][k] + 1.0 / 4 * W.q1[v][k] + 1.0 / 4 * h * dqs[v][k];
      s2[v][k] = 3.0 / 4 * s[v][k] + 1.0 / 4 * s1[v][k] + 1.0 / 4 * h * dsv[v][k];
    }
    { const T* qq[3] = {W.q2[0].data(), W.q2[1].data(), W.q2[2].data()}; const T* ss[3] = {s2[0].data(), s2[1].data(), s2[2].data()}; stage(qq, ss); }
    for (int v = 0; v < 3; ++v) for (size_t k = 0; k < N; ++k) {
      q[v][k] = 1.0 / 3 * q[v][k] + 2.0 / 3 * W.q2[v][k] + 2.0 / 3 * h * dqs[v][k];
      s[v][k] = 1.0 / 3 * s[v][k] + 2.0 / 3 * s2[v][k] + 2.0 / 3 * h * dsv[v][k];
    }
    t += h;
  }
  if (value(alpha) > 0) {
    const T* qq[3] = {q[0], q[1], q[2]}; const T* ss[3] = {s[0], s[1], s[2]};
    solve_elliptic1d(G, Sig, qq, alpha, n_iter, solver, W);
    sens_solve(qq, ss);
  }
}

// ------------------------------- 1D reverse -------------------------------
inline void flux1d_rev(double g, double mu, double r, double E, double S, const double fb[3], double qb[3], double& Sb, double& gb) {
  // f = (mu^2/r + pb, mu, (E + pb) mu / r), pb = (g-1)(E - mu^2/(2r)) + S
  const double K = mu * mu / (2.0 * r), P = (g - 1.0) * (E - K), pb = P + S, u = mu / r;
  const double pbb = fb[0] + fb[2] * u;
  qb[0] += fb[0] * 2.0 * mu / r + fb[1] + fb[2] * (E + pb) / r;
  qb[1] += -fb[0] * mu * mu / (r * r) - fb[2] * (E + pb) * mu / (r * r);
  qb[2] += fb[2] * u;
  Sb += pbb;
  gb += pbb * (E - K); qb[2] += pbb * (g - 1.0);
  const double Kb = -pbb * (g - 1.0);
  qb[0] += Kb * mu / r; qb[1] += -Kb * K / r;
}
inline void wavespeed1d_rev(double g, double mu, double r, double E, double wb, double qb[3], double& gb) {
  const double K = mu * mu / (2.0 * r), P = (g - 1.0) * (E - K), u = mu / r;
  const double ub = std::signbit(u) ? -wb : wb;
  qb[0] += ub / r; qb[1] += -ub * u / r;
  const double X = g * P / r, c = std::sqrt(X), Xb = wb / (2.0 * c);
  gb += Xb * P / r; const double Pb = Xb * g / r; qb[1] += -Xb * X / r;
  gb += Pb * (E - K); qb[2] += Pb * (g - 1.0);
  const double Kb = -Pb * (g - 1.0);
  qb[0] += Kb * mu / r; qb[1] += -Kb * K / r;
}

inline void hyperbolic_rhs1d_rev(const Grid1D& G, double g, const double* const q[3], const double* S, const double* const kb[3],
                                 double* const qb[3], double* Sb, double& gb) {
  const int np = G.np, Ne = G.m.Ne, L = np - 1; const Basis& B = G.b; const double invJ = 1 / G.m.J;
  std::vector<double> Fb[3];
  for (int v = 0; v < 3; ++v) Fb[v].assign(G.N, 0.0);
  for (int e = 0; e < Ne; ++e) for (int i = 0; i < np; ++i)
    for (int j = 0; j < np; ++j) for (int v = 0; v < 3; ++v) Fb[v][G.id(j, e)] -= invJ * B.Dik(i, j) * kb[v][G.id(i, e)];
  // Each face's LLF flux is computed twice in the forward (once per side); each copy feeds one side.
  auto llf_rev = [&](size_t nl, size_t nr, const double fsb[3]) {
    const double wL = wavespeed1d(g, q[0][nl], q[1][nl], q[2][nl]), wR = wavespeed1d(g, q[0][nr], q[1][nr], q[2][nr]);
    const double lam = jmax(wL, wR);
    double lamb = 0.0;
    for (int v = 0; v < 3; ++v) {
      Fb[v][nl] += fsb[v] / 2.0; Fb[v][nr] += fsb[v] / 2.0;
      qb[v][nl] += lam * fsb[v] / 2.0; qb[v][nr] -= lam * fsb[v] / 2.0;
      lamb += fsb[v] * (q[v][nl] - q[v][nr]) / 2.0;
    }
    double qq[3] = {0, 0, 0};
    if (wR > wL) { wavespeed1d_rev(g, q[0][nr], q[1][nr], q[2][nr], lamb, qq, gb); for (int v = 0; v < 3; ++v) qb[v][nr] += qq[v]; }
    else { wavespeed1d_rev(g, q[0][nl], q[1][nl], q[2][nl], lamb, qq, gb); for (int v = 0; v < 3; ++v) qb[v][nl] += qq[v]; }
  };
  for (int e = 0; e < Ne; ++e) {
    const int eL = e == 0 ? Ne - 1 : e - 1, eR = e == Ne - 1 ? 0 : e + 1;
    const size_t nR = G.id(L, e), n0 = G.id(0, e);
    double fRb[3], fLb[3];
    for (int v = 0; v < 3; ++v) {
      fRb[v] = -invJ / B.w[L] * kb[v][nR]; Fb[v][nR] += invJ / B.w[L] * kb[v][nR];
      fLb[v] = invJ / B.w[0] * kb[v][n0]; Fb[v][n0] -= invJ / B.w[0] * kb[v][n0];
    }
    llf_rev(G.id(L, e), G.id(0, eR), fRb);
    llf_rev(G.id(L, eL), G.id(0, e), fLb);
  }
  for (size_t n = 0; n < G.N; ++n) {
    double qq[3] = {0, 0, 0}, Sbn = 0.0; const double fb[3] = {Fb[0][n], Fb[1][n], Fb[2][n]};
    flux1d_rev(g, q[0][n], q[1][n], q[2][n], S[n], fb, qq, Sbn, gb);
    for (int v = 0; v < 3; ++v) qb[v][n] += qq[v];
    Sb[n] += Sbn;
  }
}

// Gradient of scale * u^T A(rho, alpha) v for the 1D SIP operator.
inline void sip_param_adj(const Grid1D& G, double scale, const double* u, const double* v, const double* rho, double alpha, double* rhob, double& alphab) {
  const int np = G.np, Ne = G.m.Ne, L = np - 1; const Basis& B = G.b; const double J = G.m.J, invJ = 1 / J;
  const double eta = (double)((B.p + 1) * (B.p + 1));
  std::vector<double> invb(G.N, 0.0); double ab = 0.0;
  for (int e = 0; e < Ne; ++e) for (int i = 0; i < np; ++i) {
    const size_t n = G.id(i, e);
    double dv = 0, du = 0;
    for (int j = 0; j < np; ++j) { dv += B.Dik(i, j) * v[G.id(j, e)]; du += B.Dik(i, j) * u[G.id(j, e)]; }
    invb[n] += B.w[i] * J * u[n] * v[n];
    const double st = B.w[i] * invJ * dv * du;
    invb[n] += alpha * st; ab += st / rho[n];
  }
  for (int e = 0; e < Ne; ++e) {
    const int eR = e == Ne - 1 ? 0 : e + 1;
    const size_t nl = G.id(L, e), nr = G.id(0, eR);
    double dvL = 0, dvR = 0, duL = 0, duR = 0;
    for (int j = 0; j < np; ++j) {
      dvL += B.Dik(L, j) * v[G.id(j, e)]; dvR += B.Dik(0, j) * v[G.id(j, eR)];
      duL += B.Dik(L, j) * u[G.id(j, e)]; duR += B.Dik(0, j) * u[G.id(j, eR)];
    }
    const double iL = 1.0 / rho[nl], iR = 1.0 / rho[nr];
    const double jv = v[nl] - v[nr], ju = u[nl] - u[nr];
    const double cL = dvL * ju + duL * jv, cR = dvR * ju + duR * jv;
    invb[nl] += -alpha * invJ / 2.0 * cL; invb[nr] += -alpha * invJ / 2.0 * cR;
    const double pen = alpha * eta / G.m.dx * jv * ju;
    if (iR > iL) invb[nr] += pen; else invb[nl] += pen;
    ab += -invJ / 2.0 * (iL * cL + iR * cR) + eta * jmax(iL, iR) / G.m.dx * jv * ju;
  }
  for (size_t n = 0; n < G.N; ++n) rhob[n] += scale * (-invb[n] / (rho[n] * rho[n]));
  alphab += scale * ab;
}

inline void sip_diagonal1d_rev(const Grid1D& G, const double* Mb, const double* rho, double alpha, double* rhob, double& alphab) {
  const int np = G.np, L = np - 1; const Basis& B = G.b; const double J = G.m.J, invJ = 1 / J;
  const double eta = (double)(np * np);
  std::vector<double> invb(G.N, 0.0); double ab = 0.0;
  for (int e = 0; e < G.m.Ne; ++e) {
    for (int i = 0; i < np; ++i) invb[G.id(i, e)] += Mb[G.id(i, e)] * B.w[i] * J;
    for (int k = 0; k < np; ++k) for (int i = 0; i < np; ++i) {
      const double d = B.Dik(i, k), c = B.w[i] * invJ * (d * d); const size_t m = G.id(i, e);
      invb[m] += Mb[G.id(k, e)] * alpha * c; ab += Mb[G.id(k, e)] * c / rho[m];
    }
  }
  for (int e = 0; e < G.m.Ne; ++e) {
    const int eR = e == G.m.Ne - 1 ? 0 : e + 1;
    const size_t nl = G.id(L, e), nr = G.id(0, eR);
    const double iL = 1.0 / rho[nl], iR = 1.0 / rho[nr];
    invb[nl] += Mb[nl] * (-alpha) * invJ * B.Dik(L, L);
    invb[nr] += Mb[nr] * alpha * invJ * B.Dik(0, 0);
    const double sigb = (Mb[nl] + Mb[nr]) * alpha;
    if (iR > iL) invb[nr] += sigb * eta / G.m.dx; else invb[nl] += sigb * eta / G.m.dx;
    const double sig = eta * jmax(iL, iR) / G.m.dx;
    ab += Mb[nl] * (-invJ * B.Dik(L, L) * iL + sig) + Mb[nr] * (invJ * B.Dik(0, 0) * iR + sig);
  }
  for (size_t n = 0; n < G.N; ++n) rhob[n] += -invb[n] / (rho[n] * rho[n]);
  alphab += ab;
}

inline void igr_rhs1d_rev(const Grid1D& G, const double* bb, const double* mu, const double* rho, double alpha, double* mub, double* rhob, double& alphab) {
  const int np = G.np; const Basis& B = G.b; const double J = G.m.J, invJ = 1 / J;
  std::vector<double> ub(G.N, 0.0);
  for (int e = 0; e < G.m.Ne; ++e) for (int i = 0; i < np; ++i) {
    double du = 0;
    for (int j = 0; j < np; ++j) { const size_t m = G.id(j, e); du += B.Dik(i, j) * (mu[m] / rho[m]); }
    du *= invJ;
    const size_t n = G.id(i, e);
    const double c = B.w[i] * J;
    alphab += bb[n] * c * 2.0 * du * du;
    const double dub = bb[n] * c * 2.0 * alpha * 2.0 * du;
    for (int j = 0; j < np; ++j) ub[G.id(j, e)] += invJ * B.Dik(i, j) * dub;
  }
  for (size_t n = 0; n < G.N; ++n) { mub[n] += ub[n] / rho[n]; rhob[n] += -ub[n] * mu[n] / (rho[n] * rho[n]); }
}

struct StageTape1D { std::vector<double> q[3], Sin, Sout, b, M; SolverTape st; };
struct StepTape1D { StageTape1D s[3]; };

inline void stage_forward1d(const Grid1D& G, StageTape1D& T, const double* const q[3], double* Sig, double g, double alpha, int n_iter,
                            int solver, double* const dq[3]) {
  for (int v = 0; v < 3; ++v) T.q[v].assign(q[v], q[v] + G.N);
  T.Sin.assign(Sig, Sig + G.N);
  if (alpha > 0) {
    T.b.resize(G.N); T.M.resize(G.N);
    igr_rhs1d(G, T.b.data(), q[0], q[1], alpha);
    sip_diagonal1d(G, T.M.data(), q[1], alpha);
    solve_tape(G, Sig, T.b.data(), T.M.data(), n_iter, q[1], alpha, solver, T.st);
  } else for (size_t k = 0; k < G.N; ++k) Sig[k] = 0.0;
  T.Sout.assign(Sig, Sig + G.N);
  hyperbolic_rhs1d(G, g, q, Sig, dq);
}

inline void stage_reverse1d(const Grid1D& G, const StageTape1D& T, const double* const kb[3], double* Sb, double* const qb[3], double g,
                            double alpha, int n_iter, int solver, double& gb, double& alphab) {
  const double* q[3] = {T.q[0].data(), T.q[1].data(), T.q[2].data()};
  hyperbolic_rhs1d_rev(G, g, q, T.Sout.data(), kb, qb, Sb, gb);
  if (alpha > 0) {
    std::vector<double> bb(G.N, 0.0), Mb(G.N, 0.0);
    solve_rev(G, Sb, T.b.data(), T.M.data(), n_iter, q[1], alpha, solver, T.st, bb.data(), Mb.data(), qb[1], alphab);
    igr_rhs1d_rev(G, bb.data(), q[0], q[1], alpha, qb[0], qb[1], alphab);
    sip_diagonal1d_rev(G, Mb.data(), q[1], alpha, qb[1], alphab);
  } else for (size_t k = 0; k < G.N; ++k) Sb[k] = 0.0;
}

inline void objective1d_grad(const Grid1D& G, int obj, const double* const q[3], double g, const double* prm, double* const qb[3], double& gb) {
  const int np = G.np; const Basis& B = G.b; const double J = G.m.J; const double pi = 3.14159265358979323846;
  for (int v = 0; v < 3; ++v) for (size_t n = 0; n < G.N; ++n) qb[v][n] = 0.0;
  double KE = 0, Ms = 0;
  if (obj == OBJ1_KINETIC_ENERGY)
    for (int e = 0; e < G.m.Ne; ++e) for (int i = 0; i < np; ++i) {
      const size_t n = G.id(i, e); const double wJ = B.w[i] * J;
      KE += wJ * q[0][n] * q[0][n] / (2.0 * q[1][n]); Ms += wJ * q[1][n];
    }
  for (int e = 0; e < G.m.Ne; ++e) for (int i = 0; i < np; ++i) {
    const size_t n = G.id(i, e); const double c = B.w[i] * J;
    const double mu = q[0][n], r = q[1][n], E = q[2][n];
    switch (obj) {
      case OBJ1_L2_DENSITY: qb[1][n] += 2.0 * c * r; break;
      case OBJ1_L2_PRESSURE: {
        const double K = mu * mu / (2.0 * r), p = (g - 1.0) * (E - K), pb = 2.0 * c * p, Kb = -pb * (g - 1.0);
        gb += pb * (E - K); qb[2][n] += pb * (g - 1.0); qb[0][n] += Kb * mu / r; qb[1][n] += -Kb * K / r; break;
      }
      case OBJ1_KINETIC_ENERGY: {
        const double KEb = 1.0 / Ms, Mb = -KE / (Ms * Ms);
        qb[0][n] += KEb * c * mu / r; qb[1][n] += -KEb * c * mu * mu / (2.0 * r * r) + Mb * c; break;
      }
      case OBJ1_WEIGHTED_MOMENTUM: qb[0][n] += c * std::sin(2 * pi * G.x(i, e) / (G.m.Ne * G.m.dx)); break;
      case OBJ1_INTERVAL_RHO: qb[1][n] += c * interval_indicator(G.x(i, e), prm); break;
      default: throw std::invalid_argument("Unknown objective");
    }
  }
}

inline double adjoint_ic1d(const Grid1D& G, int obj, const double* prm, const double* const q0[3], int n_steps, double dt, double g,
                           double alpha, int n_iter, int solver, double* const dq0[3], double* dgamma, double* dalpha) {
  const size_t N = G.N;
  std::vector<std::vector<double>> qs((size_t)(n_steps + 1) * 3), Ss(n_steps + 1);
  std::vector<double> q[3], Sig(N, 0.0);
  for (int v = 0; v < 3; ++v) q[v].assign(q0[v], q0[v] + N);
  double* qp[3] = {q[0].data(), q[1].data(), q[2].data()};
  Work2D<double> W; W.alloc(N);
  for (int s = 0; s < n_steps; ++s) {
    for (int v = 0; v < 3; ++v) qs[(size_t)s * 3 + v] = q[v];
    Ss[s] = Sig;
    rk3_step1d(G, qp, Sig.data(), g, alpha, dt, n_iter, solver, W);
  }
  const double* qc[3] = {q[0].data(), q[1].data(), q[2].data()};
  const double J = objective1d(G, obj, qc, g, prm);
  std::vector<double> qbv[3], Sb(N, 0.0);
  for (int v = 0; v < 3; ++v) qbv[v].assign(N, 0.0);
  double* qb[3] = {qbv[0].data(), qbv[1].data(), qbv[2].data()};
  double gb = 0.0, ab = 0.0;
  objective1d_grad(G, obj, qc, g, prm, qb, gb);
  StepTape1D tape;
  std::vector<double> dqv[3], q1[3], q2[3], kbv[3], q1b[3], q2b[3], qnb[3];
  for (int v = 0; v < 3; ++v) { dqv[v].resize(N); q1[v].resize(N); q2[v].resize(N); kbv[v].resize(N); q1b[v].resize(N); q2b[v].resize(N); qnb[v].resize(N); }
  double* dq[3] = {dqv[0].data(), dqv[1].data(), dqv[2].data()};
  const double* kb[3] = {kbv[0].data(), kbv[1].data(), kbv[2].data()};
  double* q1p[3] = {q1b[0].data(), q1b[1].data(), q1b[2].data()};
  double* q2p[3] = {q2b[0].data(), q2b[1].data(), q2b[2].data()};
  double* qnp[3] = {qnb[0].data(), qnb[1].data(), qnb[2].data()};
  for (int s = n_steps - 1; s >= 0; --s) {
    for (int v = 0; v < 3; ++v) q[v] = qs[(size_t)s * 3 + v];
    Sig = Ss[s];
    const double* qn[3] = {q[0].data(), q[1].data(), q[2].data()};
    stage_forward1d(G, tape.s[0], qn, Sig.data(), g, alpha, n_iter, solver, dq);
    for (int v = 0; v < 3; ++v) for (size_t k = 0; k < N; ++k) q1[v][k] = q[v][k] + dt * dq[v][k];
    const double* q1c[3] = {q1[0].data(), q1[1].data(), q1[2].data()};
    stage_forward1d(G, tape.s[1], q1c, Sig.data(), g, alpha, n_iter, solver, dq);
    for (int v = 0; v < 3; ++v) for (size_t k = 0; k < N; ++k) q2[v][k] = 3.0 / 4 * q[v][k] + 1.0 / 4 * q1[v][k] + 1.0 / 4 * dt * dq[v][k];
    const double* q2c[3] = {q2[0].data(), q2[1].data(), q2[2].data()};
    stage_forward1d(G, tape.s[2], q2c, Sig.data(), g, alpha, n_iter, solver, dq);
    for (int v = 0; v < 3; ++v) for (size_t k = 0; k < N; ++k) { qnb[v][k] = 1.0 / 3 * qb[v][k]; q2b[v][k] = 2.0 / 3 * qb[v][k]; kbv[v][k] = 2.0 / 3 * dt * qb[v][k]; q1b[v][k] = 0.0; }
    stage_reverse1d(G, tape.s[2], kb, Sb.data(), q2p, g, alpha, n_iter, solver, gb, ab);
    for (int v = 0; v < 3; ++v) for (size_t k = 0; k < N; ++k) { qnb[v][k] += 3.0 / 4 * q2b[v][k]; q1b[v][k] = 1.0 / 4 * q2b[v][k]; kbv[v][k] = 1.0 / 4 * dt * q2b[v][k]; }
    stage_reverse1d(G, tape.s[1], kb, Sb.data(), q1p, g, alpha, n_iter, solver, gb, ab);
    for (int v = 0; v < 3; ++v) for (size_t k = 0; k < N; ++k) { qnb[v][k] += q1b[v][k]; kbv[v][k] = dt * q1b[v][k]; }
    stage_reverse1d(G, tape.s[0], kb, Sb.data(), qnp, g, alpha, n_iter, solver, gb, ab);
    for (int v = 0; v < 3; ++v) for (size_t k = 0; k < N; ++k) qb[v][k] = qnb[v][k];
  }
  for (int v = 0; v < 3; ++v) for (size_t k = 0; k < N; ++k) dq0[v][k] = qb[v][k];
  if (dgamma) *dgamma = gb;
  if (dalpha) *dalpha = ab;
  return J;
}

}  // namespace igr
