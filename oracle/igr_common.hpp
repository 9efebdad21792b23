// ORACLE — test infrastructure only. CPU restatement of the Julia reference
// f-t-s/IGR_sensitivities used as the parity checker for the CUDA path and as
// the timed CPU baseline. Nothing in the product library links or calls this.
//
// Parity status: no golden vectors ship with the reference and the Julia
// reference cannot run in this environment (no Julia). The restatement is
// pinned to the reference's own known-answer tests, ported in tests/:
// free-stream preservation (IGR_adjoints_2d/tests/run_euler_test.jl:15-33),
// quasi-1D 2D==1D (IGR_adjoints_2d/tests/run_quasi1d_test.jl:1-179),
// SIP manufactured-solution order, tangent vs FD
// (IGR_adjoints_2d/tests/run_sensitivity_test.jl), reverse vs FD
// (IGR_adjoints_2d/tests/run_enzyme_test.jl) and reverse == forward-mode
// dual (IGR_adjoints_1d/tests/run_enzyme_test.jl:24-91, Enzyme == ForwardDiff).
//
// Arithmetic follows the reference expression by expression (left-to-right
// evaluation, no FMA contraction: build with -ffp-contract=off), so that the
// oracle is the reference's IEEE-double computation up to summation order
// where noted.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <vector>

namespace igr {

// ---------------------------------------------------------------------------
// Forward-mode dual numbers (the role ForwardDiff.Dual plays in the
// reference's tests). Derivative conventions at kinks follow Julia:
//   abs(x):  signbit(x) ? -x : x           (derivative +1 at +0.0)
//   max(a,b): b > a ? b : a                (ties take the first argument;
//             Base.max for Float64, julia/base/math.jl)
// ---------------------------------------------------------------------------
template <int N>
struct Dual {
  double v;
  double d[N];
  Dual() : v(0.0) { for (int k = 0; k < N; ++k) d[k] = 0.0; }
  Dual(double x) : v(x) { for (int k = 0; k < N; ++k) d[k] = 0.0; }  // NOLINT
};

template <int N> inline Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v + b.v; for (int k = 0; k < N; ++k) r.d[k] = a.d[k] + b.d[k]; return r;
}
template <int N> inline Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v - b.v; for (int k = 0; k < N; ++k) r.d[k] = a.d[k] - b.d[k]; return r;
}
template <int N> inline Dual<N> operator-(const Dual<N>& a) {
  Dual<N> r; r.v = -a.v; for (int k = 0; k < N; ++k) r.d[k] = -a.d[k]; return r;
}
template <int N> inline Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v * b.v; for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k]; return r;
}
template <int N> inline Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v / b.v;
  for (int k = 0; k < N; ++k) r.d[k] = (a.d[k] * b.v - a.v * b.d[k]) / (b.v * b.v);
  return r;
}
template <int N> inline Dual<N> operator+(const Dual<N>& a, double b) { return a + Dual<N>(b); }
template <int N> inline Dual<N> operator+(double a, const Dual<N>& b) { return Dual<N>(a) + b; }
template <int N> inline Dual<N> operator-(const Dual<N>& a, double b) { return a - Dual<N>(b); }
template <int N> inline Dual<N> operator-(double a, const Dual<N>& b) { return Dual<N>(a) - b; }
template <int N> inline Dual<N> operator*(const Dual<N>& a, double b) {
  Dual<N> r; r.v = a.v * b; for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * b; return r;
}
template <int N> inline Dual<N> operator*(double a, const Dual<N>& b) {
  Dual<N> r; r.v = a * b.v; for (int k = 0; k < N; ++k) r.d[k] = a * b.d[k]; return r;
}
template <int N> inline Dual<N> operator/(const Dual<N>& a, double b) {
  Dual<N> r; r.v = a.v / b; for (int k = 0; k < N; ++k) r.d[k] = a.d[k] / b; return r;
}
template <int N> inline Dual<N> operator/(double a, const Dual<N>& b) { return Dual<N>(a) / b; }
template <int N> inline Dual<N>& operator+=(Dual<N>& a, const Dual<N>& b) { a = a + b; return a; }
template <int N> inline Dual<N>& operator-=(Dual<N>& a, const Dual<N>& b) { a = a - b; return a; }
template <int N> inline Dual<N>& operator*=(Dual<N>& a, const Dual<N>& b) { a = a * b; return a; }
template <int N> inline Dual<N>& operator+=(Dual<N>& a, double b) { a = a + b; return a; }
template <int N> inline Dual<N>& operator-=(Dual<N>& a, double b) { a = a - b; return a; }
template <int N> inline Dual<N>& operator*=(Dual<N>& a, double b) { a = a * b; return a; }
template <int N> inline bool operator<(const Dual<N>& a, const Dual<N>& b) { return a.v < b.v; }
template <int N> inline bool operator>(const Dual<N>& a, const Dual<N>& b) { return a.v > b.v; }
template <int N> inline bool operator>(const Dual<N>& a, double b) { return a.v > b; }
template <int N> inline bool operator<(const Dual<N>& a, double b) { return a.v < b; }
template <int N> inline Dual<N> sqrt(const Dual<N>& a) {
  Dual<N> r; r.v = std::sqrt(a.v); double h = 0.5 / r.v;
  for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * h;
  return r;
}
template <int N> inline Dual<N> abs(const Dual<N>& a) { return std::signbit(a.v) ? -a : a; }

inline double value(double x) { return x; }
template <int N> inline double value(const Dual<N>& x) { return x.v; }

// Julia's Base.max for floats on finite inputs: the first argument wins ties.
template <class T> inline T jmax(const T& a, const T& b) { return (value(b) > value(a)) ? b : a; }
template <class T> inline T jabs(const T& a) { using std::abs; using igr::abs; return abs(a); }
inline double jabs(double a) { return std::fabs(a); }
template <class T> inline T jsqrt(const T& a) { using std::sqrt; using igr::sqrt; return sqrt(a); }
inline double jsqrt(double a) { return std::sqrt(a); }

// ---------------------------------------------------------------------------
// DG basis: LGL nodes, weights and differentiation matrix.
// Follows IGR_adjoints_2d/basis.jl:19-68 (barycentric weights :19-30,
// differentiation matrix :38-49). Nodes and weights come from
// FastGaussQuadrature.gausslobatto (v1.1.0) in the reference; here they are
// the closed forms for p <= 4 and Newton iteration on (1-x^2)P_p'(x) above.
// ---------------------------------------------------------------------------
struct Basis {
  int p = 0, np = 1;
  std::vector<double> xi, w, D;  // D row-major: D[i*np + k]
  double Dik(int i, int k) const { return D[(size_t)i * np + k]; }
};

inline void lgl_nodes_weights(int p, std::vector<double>& xi, std::vector<double>& w) {
  const int n = p + 1;
  xi.assign(n, 0.0); w.assign(n, 0.0);
  if (p == 1) { xi = {-1.0, 1.0}; w = {1.0, 1.0}; return; }
  if (p == 2) { xi = {-1.0, 0.0, 1.0}; w = {1.0 / 3.0, 4.0 / 3.0, 1.0 / 3.0}; return; }
  if (p == 3) {
    const double a = std::sqrt(1.0 / 5.0);
    xi = {-1.0, -a, a, 1.0}; w = {1.0 / 6.0, 5.0 / 6.0, 5.0 / 6.0, 1.0 / 6.0}; return;
  }
  if (p == 4) {
    const double a = std::sqrt(3.0 / 7.0);
    xi = {-1.0, -a, 0.0, a, 1.0};
    w = {1.0 / 10.0, 49.0 / 90.0, 32.0 / 45.0, 49.0 / 90.0, 1.0 / 10.0}; return;
  }
  // General p: Newton on the Legendre-Gauss-Lobatto condition, Chebyshev-Gauss-Lobatto start.
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < n; ++i) {
    double x = -std::cos(pi * i / p), xold = 2.0, Pn = 0.0;
    for (int it = 0; it < 100 && std::fabs(x - xold) > 1e-16; ++it) {
      double P0 = 1.0, P1 = x;
      for (int k = 2; k <= p; ++k) { double P2 = ((2.0 * k - 1.0) * x * P1 - (k - 1.0) * P0) / k; P0 = P1; P1 = P2; }
      Pn = P1; double Pm1 = P0;
      xold = x;
      x = x - (x * Pn - Pm1) / (n * Pn);
    }
    double P0 = 1.0, P1 = x;
    for (int k = 2; k <= p; ++k) { double P2 = ((2.0 * k - 1.0) * x * P1 - (k - 1.0) * P0) / k; P0 = P1; P1 = P2; }
    xi[i] = x; w[i] = 2.0 / (p * n * P1 * P1);
  }
}

inline Basis make_basis(int p) {
  Basis b; b.p = p; b.np = p + 1;
  if (p == 0) { b.xi = {0.0}; b.w = {2.0}; b.D = {0.0}; return b; }
  lgl_nodes_weights(p, b.xi, b.w);
  const int n = b.np;
  std::vector<double> lam(n, 1.0);  // barycentric weights, basis.jl:19-30
  for (int j = 0; j < n; ++j) {
    for (int i = 0; i < n; ++i) { if (i == j) continue; lam[j] *= (b.xi[j] - b.xi[i]); }
    lam[j] = 1.0 / lam[j];
  }
  b.D.assign((size_t)n * n, 0.0);  // basis.jl:38-49
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      if (i == j) continue;
      b.D[(size_t)i * n + j] = (lam[j] / lam[i]) / (b.xi[i] - b.xi[j]);
      b.D[(size_t)i * n + i] -= b.D[(size_t)i * n + j];
    }
  return b;
}

inline Basis basis_from_arrays(int p, const double* xi, const double* w, const double* D_colmajor) {
  // Caller-supplied basis in Julia's column-major D layout (D[i,k] at i + k*np).
  Basis b; b.p = p; b.np = p + 1; const int n = b.np;
  b.xi.assign(xi, xi + n); b.w.assign(w, w + n); b.D.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) for (int k = 0; k < n; ++k) b.D[(size_t)i * n + k] = D_colmajor[i + (size_t)k * n];
  return b;
}

enum Solver { SOLVER_PCG = 0, SOLVER_JACOBI = 1, SOLVER_CHEBYSHEV = 2 };

// Chebyshev eigenvalue bounds of the Jacobi-preconditioned SIP operator,
// IGR_adjoints_2d/elliptic.jl:373-378 (lambda_max table indexed by min(p,4)).
struct ChebParams { double theta, delta, sigma; };
inline ChebParams cheb_params(int p) {
  const double lmin = 1.0;
  const double table[4] = {1.5, 2.0, 2.1, 2.2};
  int idx = std::min(p, 4);
  if (idx < 1) throw std::invalid_argument("chebyshev solver needs p >= 1");
  const double lmax = table[idx - 1];
  ChebParams c;
  c.theta = (lmax + lmin) / 2;
  c.delta = (lmax - lmin) / 2;
  c.sigma = c.theta / std::max(c.delta, 1e-10);
  return c;
}

}  // namespace igr
