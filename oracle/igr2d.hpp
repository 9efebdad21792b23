// ORACLE — test infrastructure only (see igr_common.hpp for the parity status).
// 2D restatement of IGR_adjoints_2d: euler.jl, hyperbolic.jl, elliptic.jl,
// forward.jl, sensitivity.jl and the objective tails of enzyme_adjoint.jl.
// Templated on the state scalar T (double, or Dual<N> for exact directional
// derivatives of the discrete map).
//
// Field layout: Julia column-major (n_p, n_p, N_ex, N_ey), i (x-node) fastest:
//   idx(i, j, ex, ey) = i + np*(j + np*(ex + N_ex*ey))       (0-based here)
#pragma once
#include "igr_common.hpp"

namespace igr {

struct Mesh2D {
  int Nex = 1, Ney = 1;
  double Lx = 1.0, Ly = 1.0, dx = 1.0, dy = 1.0, Jx = 0.5, Jy = 0.5;
};

// IGR_adjoints_2d/mesh.jl:108-125
inline Mesh2D make_mesh2d(int Nex, int Ney, double Lx, double Ly) {
  Mesh2D m; m.Nex = Nex; m.Ney = Ney; m.Lx = Lx; m.Ly = Ly;
  m.dx = Lx / Nex; m.dy = Ly / Ney; m.Jx = m.dx / 2.0; m.Jy = m.dy / 2.0;
  return m;
}
inline double node_x(const Basis& b, const Mesh2D& m, int i, int ex) { return ex * m.dx + m.Jx * (1.0 + b.xi[i]); }
inline double node_y(const Basis& b, const Mesh2D& m, int j, int ey) { return ey * m.dy + m.Jy * (1.0 + b.xi[j]); }

struct Grid2D {
  Basis b; Mesh2D m; int np; size_t N;
  Grid2D(const Basis& b_, const Mesh2D& m_) : b(b_), m(m_), np(b_.np), N((size_t)b_.np * b_.np * m_.Nex * m_.Ney) {}
  size_t id(int i, int j, int ex, int ey) const { return (size_t)i + np * ((size_t)j + np * ((size_t)ex + (size_t)m.Nex * ey)); }
};

// ---------------------------------------------------------------------------
// Pointwise physics, IGR_adjoints_2d/euler.jl:20-133
// ---------------------------------------------------------------------------
template <class T> inline T pressure2d(const T& g, const T& mx, const T& my, const T& r, const T& E) {
  return (g - 1.0) * (E - (mx * mx + my * my) / (2.0 * r));
}
template <class T> inline void flux_x(const T& g, const T& mx, const T& my, const T& r, const T& E, const T& S, T f[4]) {
  T P = pressure2d(g, mx, my, r, E); T pb = P + S; T ux = mx / r;
  f[0] = mx * ux + pb; f[1] = my * ux; f[2] = mx; f[3] = (E + pb) * ux;
}
template <class T> inline void flux_y(const T& g, const T& mx, const T& my, const T& r, const T& E, const T& S, T f[4]) {
  T P = pressure2d(g, mx, my, r, E); T pb = P + S; T uy = my / r;
  f[0] = mx * uy; f[1] = my * uy + pb; f[2] = my; f[3] = (E + pb) * uy;
}
template <class T> inline T sound_speed2d(const T& g, const T& mx, const T& my, const T& r, const T& E) {
  T P = pressure2d(g, mx, my, r, E); return jsqrt(g * P / r);
}
template <class T> inline T wavespeed_x(const T& g, const T& mx, const T& my, const T& r, const T& E) {
  return jabs(mx / r) + sound_speed2d(g, mx, my, r, E);
}
template <class T> inline T wavespeed_y(const T& g, const T& mx, const T& my, const T& r, const T& E) {
  return jabs(my / r) + sound_speed2d(g, mx, my, r, E);
}
// LLF flux across an x- (dir=0) or y-normal (dir=1) face, euler.jl:222-258 (beta = 1).
template <class T> inline void llf_flux(int dir, const T& g, const T qL[5], const T qR[5], T fs[4]) {
  T lam = dir == 0 ? jmax(wavespeed_x(g, qL[0], qL[1], qL[2], qL[3]), wavespeed_x(g, qR[0], qR[1], qR[2], qR[3]))
                   : jmax(wavespeed_y(g, qL[0], qL[1], qL[2], qL[3]), wavespeed_y(g, qR[0], qR[1], qR[2], qR[3]));
  lam = 1.0 * lam;
  T fL[4], fR[4];
  if (dir == 0) { flux_x(g, qL[0], qL[1], qL[2], qL[3], qL[4], fL); flux_x(g, qR[0], qR[1], qR[2], qR[3], qR[4], fR); }
  else { flux_y(g, qL[0], qL[1], qL[2], qL[3], qL[4], fL); flux_y(g, qR[0], qR[1], qR[2], qR[3], qR[4], fR); }
  for (int v = 0; v < 4; ++v) fs[v] = (fL[v] + fR[v]) / 2.0 + lam * (qL[v] - qR[v]) / 2.0;
}

// ---------------------------------------------------------------------------
// Hyperbolic DG RHS, IGR_adjoints_2d/hyperbolic.jl:27-119.
// q[0..3] = (mux, muy, rho, E); dq likewise. Fx/Fy: 8 workspace arrays of N.
// ---------------------------------------------------------------------------
template <class T>
void hyperbolic_rhs(const Grid2D& G, const T& g, const T* const q[4], const T* S, T* const dq[4], std::vector<T>* F /*[8]*/) {
  const int np = G.np, Nex = G.m.Nex, Ney = G.m.Ney;
  const Basis& B = G.b;
  const double invJx = 1 / G.m.Jx, invJy = 1 / G.m.Jy;
  for (int v = 0; v < 8; ++v) F[v].resize(G.N);
  for (size_t n = 0; n < G.N; ++n) {
    T fx[4], fy[4];
    flux_x(g, q[0][n], q[1][n], q[2][n], q[3][n], S[n], fx);
    flux_y(g, q[0][n], q[1][n], q[2][n], q[3][n], S[n], fy);
    for (int v = 0; v < 4; ++v) { F[v][n] = fx[v]; F[4 + v][n] = fy[v]; }
  }
  for (int ey = 0; ey < Ney; ++ey) for (int ex = 0; ex < Nex; ++ex)
    for (int j = 0; j < np; ++j) for (int i = 0; i < np; ++i) {
      T a[4] = {T(0.0), T(0.0), T(0.0), T(0.0)};
      for (int k = 0; k < np; ++k) {
        const size_t nx = G.id(k, j, ex, ey), ny = G.id(i, k, ex, ey);
        for (int v = 0; v < 4; ++v) a[v] = a[v] - (invJx * B.Dik(i, k)) * F[v][nx];
        for (int v = 0; v < 4; ++v) a[v] = a[v] - (invJy * B.Dik(j, k)) * F[4 + v][ny];
      }
      // hyperbolic.jl:55-66 interleaves x and y per k and per variable; each
      // variable's accumulation order (x_k then y_k for k = 1..np) is kept.
      const size_t n = G.id(i, j, ex, ey);
      for (int v = 0; v < 4; ++v) dq[v][n] = a[v];
    }
  const int L = np - 1;
  for (int ey = 0; ey < Ney; ++ey) for (int ex = 0; ex < Nex; ++ex) {
    const int exR = ex == Nex - 1 ? 0 : ex + 1;
    for (int j = 0; j < np; ++j) {
      const size_t nl = G.id(L, j, ex, ey), nr = G.id(0, j, exR, ey);
      T qL[5] = {q[0][nl], q[1][nl], q[2][nl], q[3][nl], S[nl]};
      T qR[5] = {q[0][nr], q[1][nr], q[2][nr], q[3][nr], S[nr]};
      T fs[4]; llf_flux(0, g, qL, qR, fs);
      for (int v = 0; v < 4; ++v) dq[v][nl] = dq[v][nl] - invJx * (fs[v] - F[v][nl]) / B.w[L];
      for (int v = 0; v < 4; ++v) dq[v][nr] = dq[v][nr] + invJx * (fs[v] - F[v][nr]) / B.w[0];
    }
  }
  for (int ey = 0; ey < Ney; ++ey) for (int ex = 0; ex < Nex; ++ex) {
    const int eyR = ey == Ney - 1 ? 0 : ey + 1;
    for (int i = 0; i < np; ++i) {
      const size_t nl = G.id(i, L, ex, ey), nr = G.id(i, 0, ex, eyR);
      T qL[5] = {q[0][nl], q[1][nl], q[2][nl], q[3][nl], S[nl]};
      T qR[5] = {q[0][nr], q[1][nr], q[2][nr], q[3][nr], S[nr]};
      T fs[4]; llf_flux(1, g, qL, qR, fs);
      for (int v = 0; v < 4; ++v) dq[v][nl] = dq[v][nl] - invJy * (fs[v] - F[4 + v][nl]) / B.w[L];
      for (int v = 0; v < 4; ++v) dq[v][nr] = dq[v][nr] + invJy * (fs[v] - F[4 + v][nr]) / B.w[0];
    }
  }
}

// ---------------------------------------------------------------------------
// SIP operator y = A(rho, alpha) x, IGR_adjoints_2d/elliptic.jl:30-145.
// TA is the coefficient scalar (rho, alpha); TX the vector scalar.
// ---------------------------------------------------------------------------
template <class T>
void apply_sip(const Grid2D& G, T* y, const T* x, const T* rho, const T& alpha) {
  const int np = G.np, Nex = G.m.Nex, Ney = G.m.Ney, L = np - 1;
  const Basis& B = G.b; const double Jx = G.m.Jx, Jy = G.m.Jy, invJx = 1 / Jx, invJy = 1 / Jy;
  const int eta = (B.p + 1) * (B.p + 1);
  for (size_t n = 0; n < G.N; ++n) y[n] = T(0.0);
  for (int ey = 0; ey < Ney; ++ey) for (int ex = 0; ex < Nex; ++ex)
    for (int j = 0; j < np; ++j) for (int i = 0; i < np; ++i) {
      const size_t n = G.id(i, j, ex, ey);
      y[n] = y[n] + B.w[i] * B.w[j] * Jx * Jy * x[n] / rho[n];
      T dxi(0.0), deta(0.0);
      for (int k = 0; k < np; ++k) { dxi = dxi + B.Dik(i, k) * x[G.id(k, j, ex, ey)]; deta = deta + B.Dik(j, k) * x[G.id(i, k, ex, ey)]; }
      T invr = 1.0 / rho[n];
      T cx = alpha * B.w[i] * B.w[j] * Jy * invJx * invr * dxi;
      T cy = alpha * B.w[i] * B.w[j] * Jx * invJy * invr * deta;
      for (int k = 0; k < np; ++k) {
        const size_t a = G.id(k, j, ex, ey), c = G.id(i, k, ex, ey);
        y[a] = y[a] + cx * B.Dik(i, k);
        y[c] = y[c] + cy * B.Dik(j, k);
      }
    }
  for (int ey = 0; ey < Ney; ++ey) for (int ex = 0; ex < Nex; ++ex) {
    const int exR = ex == Nex - 1 ? 0 : ex + 1;
    for (int j = 0; j < np; ++j) {
      const double wf = B.w[j] * Jy;
      const size_t nl = G.id(L, j, ex, ey), nr = G.id(0, j, exR, ey);
      T SL = x[nl], SR = x[nr], rL = rho[nl], rR = rho[nr];
      T jump = SL - SR;
      T dL(0.0), dR(0.0);
      for (int k = 0; k < np; ++k) { dL = dL + B.Dik(L, k) * x[G.id(k, j, ex, ey)]; dR = dR + B.Dik(0, k) * x[G.id(k, j, exR, ey)]; }
      T avg = invJx * ((1.0 / rL) * dL + (1.0 / rR) * dR) / 2.0;
      T sig = (double)eta * jmax(T(1.0 / rL), T(1.0 / rR)) / G.m.dx;
      y[nl] = y[nl] + (-alpha) * avg * wf;
      y[nr] = y[nr] + alpha * avg * wf;
      for (int k = 0; k < np; ++k) {
        const size_t a = G.id(k, j, ex, ey), c = G.id(k, j, exR, ey);
        y[a] = y[a] + (-alpha) * (1.0 / (2.0 * rL)) * invJx * B.Dik(L, k) * jump * wf;
        y[c] = y[c] + (-alpha) * (1.0 / (2.0 * rR)) * invJx * B.Dik(0, k) * jump * wf;
      }
      y[nl] = y[nl] + alpha * sig * jump * wf;
      y[nr] = y[nr] - alpha * sig * jump * wf;
    }
  }
  for (int ey = 0; ey < Ney; ++ey) for (int ex = 0; ex < Nex; ++ex) {
    const int eyR = ey == Ney - 1 ? 0 : ey + 1;
    for (int i = 0; i < np; ++i) {
      const double wf = B.w[i] * Jx;
      const size_t nl = G.id(i, L, ex, ey), nr = G.id(i, 0, ex, eyR);
      T SL = x[nl], SR = x[nr], rL = rho[nl], rR = rho[nr];
      T jump = SL - SR;
      T dL(0.0), dR(0.0);
      for (int k = 0; k < np; ++k) { dL = dL + B.Dik(L, k) * x[G.id(i, k, ex, ey)]; dR = dR + B.Dik(0, k) * x[G.id(i, k, ex, eyR)]; }
      T avg = invJy * ((1.0 / rL) * dL + (1.0 / rR) * dR) / 2.0;
      T sig = (double)eta * jmax(T(1.0 / rL), T(1.0 / rR)) / G.m.dy;
      y[nl] = y[nl] + (-alpha) * avg * wf;
      y[nr] = y[nr] + alpha * avg * wf;
      for (int k = 0; k < np; ++k) {
        const size_t a = G.id(i, k, ex, ey), c = G.id(i, k, ex, eyR);
        y[a] = y[a] + (-alpha) * (1.0 / (2.0 * rL)) * invJy * B.Dik(L, k) * jump * wf;
        y[c] = y[c] + (-alpha) * (1.0 / (2.0 * rR)) * invJy * B.Dik(0, k) * jump * wf;
      }
      y[nl] = y[nl] + alpha * sig * jump * wf;
      y[nr] = y[nr] - alpha * sig * jump * wf;
    }
  }
}

// IGR source b = w_i w_j Jx Jy alpha[(div u)^2 + tr((Du)^2)], elliptic.jl:159-197
template <class T>
void igr_rhs(const Grid2D& G, T* b, const T* mx, const T* my, const T* rho, const T& alpha) {
  const int np = G.np; const Basis& B = G.b;
  const double invJx = 1 / G.m.Jx, invJy = 1 / G.m.Jy;
  for (int ey = 0; ey < G.m.Ney; ++ey) for (int ex = 0; ex < G.m.Nex; ++ex)
    for (int j = 0; j < np; ++j) for (int i = 0; i < np; ++i) {
      T uxx(0.0), uxy(0.0), uyx(0.0), uyy(0.0);
      for (int k = 0; k < np; ++k) {
        const size_t a = G.id(k, j, ex, ey), c = G.id(i, k, ex, ey);
        T ux_kj = mx[a] / rho[a], uy_kj = my[a] / rho[a], ux_ik = mx[c] / rho[c], uy_ik = my[c] / rho[c];
        uxx = uxx + B.Dik(i, k) * ux_kj; uyx = uyx + B.Dik(i, k) * uy_kj;
        uxy = uxy + B.Dik(j, k) * ux_ik; uyy = uyy + B.Dik(j, k) * uy_ik;
      }
      uxx = uxx * invJx; uyx = uyx * invJx; uxy = uxy * invJy; uyy = uyy * invJy;
      T s = uxx + uyy;
      T R = alpha * (s * s + uxx * uxx + 2.0 * uxy * uyx + uyy * uyy);
      b[G.id(i, j, ex, ey)] = B.w[i] * B.w[j] * G.m.Jx * G.m.Jy * R;
    }
}

// diag(A), elliptic.jl:205-264
template <class T>
void sip_diagonal(const Grid2D& G, T* M, const T* rho, const T& alpha) {
  const int np = G.np, L = np - 1; const Basis& B = G.b;
  const double Jx = G.m.Jx, Jy = G.m.Jy, invJx = 1 / Jx, invJy = 1 / Jy;
  const int eta = np * np;
  for (size_t n = 0; n < G.N; ++n) M[n] = T(0.0);
  for (int ey = 0; ey < G.m.Ney; ++ey) for (int ex = 0; ex < G.m.Nex; ++ex) {
    for (int j = 0; j < np; ++j) for (int i = 0; i < np; ++i) {
      const size_t n = G.id(i, j, ex, ey);
      M[n] = M[n] + B.w[i] * B.w[j] * Jx * Jy / rho[n];
    }
    for (int l = 0; l < np; ++l) for (int k = 0; k < np; ++k) {
      const size_t n = G.id(k, l, ex, ey);
      for (int i = 0; i < np; ++i) { double d = B.Dik(i, k); M[n] = M[n] + alpha * B.w[i] * B.w[l] * Jy * invJx * (d * d) / rho[G.id(i, l, ex, ey)]; }
      for (int j = 0; j < np; ++j) { double d = B.Dik(j, l); M[n] = M[n] + alpha * B.w[k] * B.w[j] * Jx * invJy * (d * d) / rho[G.id(k, j, ex, ey)]; }
    }
  }
  for (int ey = 0; ey < G.m.Ney; ++ey) for (int ex = 0; ex < G.m.Nex; ++ex) {
    const int exR = ex == G.m.Nex - 1 ? 0 : ex + 1;
    for (int j = 0; j < np; ++j) {
      const double wf = B.w[j] * Jy;
      const size_t nl = G.id(L, j, ex, ey), nr = G.id(0, j, exR, ey);
      T rL = rho[nl], rR = rho[nr];
      T sig = (double)eta * jmax(T(1.0 / rL), T(1.0 / rR)) / G.m.dx;
      M[nl] = M[nl] + ((-alpha) * invJx * B.Dik(L, L) / rL + alpha * sig) * wf;
      M[nr] = M[nr] + (alpha * invJx * B.Dik(0, 0) / rR + alpha * sig) * wf;
    }
  }
  for (int ey = 0; ey < G.m.Ney; ++ey) for (int ex = 0; ex < G.m.Nex; ++ex) {
    const int eyR = ey == G.m.Ney - 1 ? 0 : ey + 1;
    for (int i = 0; i < np; ++i) {
      const double wf = B.w[i] * Jx;
      const size_t nl = G.id(i, L, ex, ey), nr = G.id(i, 0, ex, eyR);
      T rL = rho[nl], rR = rho[nr];
      T sig = (double)eta * jmax(T(1.0 / rL), T(1.0 / rR)) / G.m.dy;
      M[nl] = M[nl] + ((-alpha) * invJy * B.Dik(L, L) / rL + alpha * sig) * wf;
      M[nr] = M[nr] + (alpha * invJy * B.Dik(0, 0) / rR + alpha * sig) * wf;
    }
  }
}

// Summation order of dotv: 0 = sequential (the default), 1 = reversed, 2 =
// pairwise (a binary tree over halves). The tests switch orders to measure how
// far a result moves under a change of inner-product summation order alone,
// the size of the difference between two correct implementations (the GPU
// sums in a fixed tree order).
inline int& dot_order() { static int o = 0; return o; }

template <class T> inline T dot_pairwise(const T* a, const T* b, size_t n) {
  if (n <= 8) {
    T s(0.0);
    for (size_t k = 0; k < n; ++k) s = s + a[k] * b[k];
    return s;
  }
  const size_t h = n / 2;
  return dot_pairwise(a, b, h) + dot_pairwise(a + h, b + h, n - h);
}

template <class T> inline T dotv(const T* a, const T* b, size_t n) {
  // LinearAlgebra.dot on Vector{Float64} is a BLAS ddot in the reference; the
  // summation order there is implementation-defined, here it is sequential.
  if (dot_order() == 2) return dot_pairwise(a, b, n);
  T s(0.0);
  if (dot_order() == 1) {
    for (size_t k = n; k-- > 0;) s = s + a[k] * b[k];
  } else {
    for (size_t k = 0; k < n; ++k) s = s + a[k] * b[k];
  }
  return s;
}

// Workspace for the solvers and the RK loop.
template <class T> struct Work2D {
  std::vector<T> b, M, r, z, p, Ap, d, F[8];
  std::vector<T> q1[4], q2[4], dq[4];
  void alloc(size_t N) {
    b.resize(N); M.resize(N); r.resize(N); z.resize(N); p.resize(N); Ap.resize(N); d.resize(N);
    for (int v = 0; v < 4; ++v) { q1[v].resize(N); q2[v].resize(N); dq[v].resize(N); }
  }
};

// pcg_fixed!, elliptic.jl:329-347
template <class T, class GridT>
void pcg_fixed(const GridT& G, T* x, const T* b, const T* M, int n_iter, const T* rho, const T& alpha, Work2D<T>& W) {
  const size_t N = G.N; T *r = W.r.data(), *z = W.z.data(), *p = W.p.data(), *Ap = W.Ap.data();
  apply_sip(G, Ap, x, rho, alpha);
  for (size_t k = 0; k < N; ++k) r[k] = b[k] - Ap[k];
  for (size_t k = 0; k < N; ++k) z[k] = r[k] / M[k];
  for (size_t k = 0; k < N; ++k) p[k] = z[k];
  T rz_old = dotv(r, z, N);
  for (int it = 0; it < n_iter; ++it) {
    apply_sip(G, Ap, p, rho, alpha);
    T a = rz_old / (dotv(p, Ap, N) + 1e-30);
    for (size_t k = 0; k < N; ++k) x[k] = x[k] + a * p[k];
    for (size_t k = 0; k < N; ++k) r[k] = r[k] - a * Ap[k];
    for (size_t k = 0; k < N; ++k) z[k] = r[k] / M[k];
    T rz_new = dotv(r, z, N);
    T beta = rz_new / (rz_old + 1e-30);
    for (size_t k = 0; k < N; ++k) p[k] = z[k] + beta * p[k];
    rz_old = rz_new;
  }
}

// jacobi_fixed!, elliptic.jl:354-361 (omega = 2/3, elliptic.jl:420)
template <class T, class GridT>
void jacobi_fixed(const GridT& G, T* x, const T* b, const T* M, int n_iter, const T* rho, const T& alpha, double omega, Work2D<T>& W) {
  const size_t N = G.N; T* Ax = W.Ap.data();
  for (int it = 0; it < n_iter; ++it) {
    apply_sip(G, Ax, x, rho, alpha);
    for (size_t k = 0; k < N; ++k) x[k] = x[k] + omega * (b[k] - Ax[k]) / M[k];
  }
}

// chebyshev_fixed!, elliptic.jl:370-397
template <class T, class GridT>
void chebyshev_fixed(const GridT& G, T* x, const T* b, const T* M, int n_iter, const T* rho, const T& alpha, Work2D<T>& W) {
  const size_t N = G.N; T *Ax = W.Ap.data(), *r = W.r.data(), *z = W.z.data(), *d = W.d.data();
  const ChebParams c = cheb_params(G.b.p);
  apply_sip(G, Ax, x, rho, alpha);
  for (size_t k = 0; k < N; ++k) r[k] = b[k] - Ax[k];
  double rc = 1 / c.sigma;
  for (int it = 1; it <= n_iter; ++it) {
    for (size_t k = 0; k < N; ++k) z[k] = r[k] / M[k];
    if (it == 1) {
      for (size_t k = 0; k < N; ++k) d[k] = z[k] / c.theta;
    } else {
      double rn = 1 / (2 * c.sigma - rc);
      for (size_t k = 0; k < N; ++k) d[k] = rn * rc * d[k] + (2 * rn / c.delta) * z[k];
      rc = rn;
    }
    for (size_t k = 0; k < N; ++k) x[k] = x[k] + d[k];
    apply_sip(G, Ax, x, rho, alpha);
    for (size_t k = 0; k < N; ++k) r[k] = b[k] - Ax[k];
  }
}

// cg_fixed! (unpreconditioned, elliptic.jl:304-320) and cg_solve! (tolerance exit, :278-297)
template <class T, class GridT>
int cg_solve(const GridT& G, T* x, const T* b, const T* rho, const T& alpha, double tol, int maxiter, bool fixed, Work2D<T>& W) {
  const size_t N = G.N; T *r = W.r.data(), *p = W.p.data(), *Ap = W.Ap.data();
  apply_sip(G, Ap, x, rho, alpha);
  for (size_t k = 0; k < N; ++k) r[k] = b[k] - Ap[k];
  for (size_t k = 0; k < N; ++k) p[k] = r[k];
  T rs_old = dotv(r, r, N);
  for (int it = 1; it <= maxiter; ++it) {
    if (!fixed && std::sqrt(value(rs_old)) < tol) return it;
    apply_sip(G, Ap, p, rho, alpha);
    T a = fixed ? rs_old / (dotv(p, Ap, N) + 1e-30) : rs_old / dotv(p, Ap, N);
    for (size_t k = 0; k < N; ++k) x[k] = x[k] + a * p[k];
    for (size_t k = 0; k < N; ++k) r[k] = r[k] - a * Ap[k];
    T rs_new = dotv(r, r, N);
    T beta = fixed ? rs_new / (rs_old + 1e-30) : rs_new / rs_old;
    for (size_t k = 0; k < N; ++k) p[k] = r[k] + beta * p[k];
    rs_old = rs_new;
  }
  return maxiter;
}

// solve_elliptic!, elliptic.jl:413-427 (Sigma is the warm start, in-out)
template <class T>
void solve_elliptic(const Grid2D& G, T* Sig, const T* const q[4], const T& alpha, int n_iter, int solver, Work2D<T>& W) {
  igr_rhs(G, W.b.data(), q[0], q[1], q[2], alpha);
  sip_diagonal(G, W.M.data(), q[2], alpha);
  if (solver == SOLVER_PCG) pcg_fixed(G, Sig, W.b.data(), W.M.data(), n_iter, q[2], alpha, W);
  else if (solver == SOLVER_JACOBI) jacobi_fixed(G, Sig, W.b.data(), W.M.data(), n_iter, q[2], alpha, 2.0 / 3.0, W);
  else if (solver == SOLVER_CHEBYSHEV) chebyshev_fixed(G, Sig, W.b.data(), W.M.data(), n_iter, q[2], alpha, W);
  else throw std::invalid_argument("Unknown solver (use :pcg, :jacobi, or :chebyshev)");
}

// compute_igr_euler_rhs!, forward.jl:22-31
template <class T>
void igr_euler_rhs(const Grid2D& G, const T* const q[4], T* Sig, const T& g, const T& alpha, int n_iter, int solver, Work2D<T>& W) {
  if (value(alpha) > 0) solve_elliptic(G, Sig, q, alpha, n_iter, solver, W);
  else for (size_t k = 0; k < G.N; ++k) Sig[k] = T(0.0);
  T* dq[4] = {W.dq[0].data(), W.dq[1].data(), W.dq[2].data(), W.dq[3].data()};
  hyperbolic_rhs(G, g, q, Sig, dq, W.F);
}

// One SSP-RK3 step, forward.jl:51-69 (state q in-out, Sigma in-out warm start).
template <class T>
void rk3_step(const Grid2D& G, T* const q[4], T* Sig, const T& g, const T& alpha, double dt, int n_iter, int solver, Work2D<T>& W) {
  const size_t N = G.N;
  const T* qc[4] = {q[0], q[1], q[2], q[3]};
  igr_euler_rhs(G, qc, Sig, g, alpha, n_iter, solver, W);
  for (int v = 0; v < 4; ++v) for (size_t k = 0; k < N; ++k) W.q1[v][k] = q[v][k] + dt * W.dq[v][k];
  const T* q1[4] = {W.q1[0].data(), W.q1[1].data(), W.q1[2].data(), W.q1[3].data()};
  igr_euler_rhs(G, q1, Sig, g, alpha, n_iter, solver, W);
  for (int v = 0; v < 4; ++v) for (size_t k = 0; k < N; ++k)
    W.q2[v][k] = 3.0 / 4 * q[v][k] + 1.0 / 4 * W.q1[v][k] + 1.0 / 4 * dt * W.dq[v][k];
  const T* q2[4] = {W.q2[0].data(), W.q2[1].data(), W.q2[2].data(), W.q2[3].data()};
  igr_euler_rhs(G, q2, Sig, g, alpha, n_iter, solver, W);
  for (int v = 0; v < 4; ++v) for (size_t k = 0; k < N; ++k)
    q[v][k] = 1.0 / 3 * q[v][k] + 2.0 / 3 * W.q2[v][k] + 2.0 / 3 * dt * W.dq[v][k];
}

inline int rerounded_steps(double dt, double T_end, double* dt_out) {
  // forward.jl:48-49: n_steps = ceil(Int, T/dt); dt = T/n_steps
  int n = (int)std::ceil(T_end / dt);
  *dt_out = T_end / n;
  return n;
}

// run_forward!, forward.jl:41-75
template <class T>
void run_forward(const Grid2D& G, T* const q[4], T* Sig, double dt, double T_end, const T& g, const T& alpha, int n_iter, int solver) {
  for (size_t k = 0; k < G.N; ++k) Sig[k] = T(0.0);
  Work2D<T> W; W.alloc(G.N);
  double dtr; int n_steps = rerounded_steps(dt, T_end, &dtr);
  for (int s = 0; s < n_steps; ++s) rk3_step(G, q, Sig, g, alpha, dtr, n_iter, solver, W);
  if (value(alpha) > 0) { const T* qc[4] = {q[0], q[1], q[2], q[3]}; solve_elliptic(G, Sig, qc, alpha, n_iter, solver, W); }
}

// ---------------------------------------------------------------------------
// Objectives (enzyme_adjoint.jl:48-229) plus the nodal-window extensions.
// ---------------------------------------------------------------------------
enum Objective2D {
  OBJ_L2_DENSITY = 0, OBJ_L2_PRESSURE = 1, OBJ_KINETIC_ENERGY = 2, OBJ_WINDOWED_KE = 3,
  OBJ_WEIGHTED_MOMENTUM = 4, OBJ_WINDOW_RHO2 = 5, OBJ_INTERVAL_RHO = 6
};
// KE_WINDOW constants, enzyme_adjoint.jl:26-31
constexpr double KE_XC = 0.55, KE_YC = 0.50, KE_SIG = 0.15;

// Square-window indicator used by OBJ_WINDOW_RHO2: params = (x0, y0, side).
inline double window_indicator(double x, double y, const double* prm) {
  return (x >= prm[0] && x <= prm[0] + prm[2] && y >= prm[1] && y <= prm[1] + prm[2]) ? 1.0 : 0.0;
}

template <class T>
T objective2d(const Grid2D& G, int obj, const T* const q[4], const T& g, const double* prm) {
  const int np = G.np; const Basis& B = G.b; const double Jx = G.m.Jx, Jy = G.m.Jy;
  const double pi = 3.14159265358979323846;
  if (obj == OBJ_KINETIC_ENERGY) {
    T KE(0.0), Ms(0.0);
    for (int ey = 0; ey < G.m.Ney; ++ey) for (int ex = 0; ex < G.m.Nex; ++ex) for (int j = 0; j < np; ++j) for (int i = 0; i < np; ++i) {
      const size_t n = G.id(i, j, ex, ey); const double wJ = B.w[i] * B.w[j] * Jx * Jy;
      KE = KE + wJ * (q[0][n] * q[0][n] + q[1][n] * q[1][n]) / (2.0 * q[2][n]);
      Ms = Ms + wJ * q[2][n];
    }
    return KE / Ms;
  }
  T J(0.0);
  for (int ey = 0; ey < G.m.Ney; ++ey) for (int ex = 0; ex < G.m.Nex; ++ex) for (int j = 0; j < np; ++j) for (int i = 0; i < np; ++i) {
    const size_t n = G.id(i, j, ex, ey);
    const double c = B.w[i] * B.w[j] * Jx * Jy;
    const double x = node_x(B, G.m, i, ex), y = node_y(B, G.m, j, ey);
    switch (obj) {
      case OBJ_L2_DENSITY: J = J + c * (q[2][n] * q[2][n]); break;
      case OBJ_L2_PRESSURE: {
        T P = (g - 1.0) * (q[3][n] - (q[0][n] * q[0][n] + q[1][n] * q[1][n]) / (2.0 * q[2][n]));
        J = J + c * (P * P); break;
      }
      case OBJ_WINDOWED_KE: {
        const double wx = std::exp(-((x - KE_XC) * (x - KE_XC) + (y - KE_YC) * (y - KE_YC)) / (KE_SIG * KE_SIG));
        J = J + c * wx * (q[0][n] * q[0][n] + q[1][n] * q[1][n]) / (2.0 * q[2][n]); break;
      }
      case OBJ_WEIGHTED_MOMENTUM: {
        const double gg = std::sin(2 * pi * x / G.m.Lx) * std::sin(2 * pi * y / G.m.Ly);
        J = J + c * q[0][n] * gg; break;
      }
      case OBJ_WINDOW_RHO2: J = J + c * (q[2][n] * q[2][n]) * window_indicator(x, y, prm); break;
      default: throw std::invalid_argument("Unknown objective");
    }
  }
  return J;
}

// Inlined SSP-RK3 objective loop of enzyme_adjoint.jl:56-71 (no dt re-rounding,
// Sigma warm start from zero). Leaves the final state in q.
template <class T>
T objective_run(const Grid2D& G, int obj, T* const q[4], int n_steps, double dt, const T& g, const T& alpha, int n_iter, int solver, const double* prm) {
  std::vector<T> Sig(G.N, T(0.0));
  Work2D<T> W; W.alloc(G.N);
  for (int s = 0; s < n_steps; ++s) rk3_step(G, q, Sig.data(), g, alpha, dt, n_iter, solver, W);
  const T* qc[4] = {q[0], q[1], q[2], q[3]};
  return objective2d(G, obj, qc, g, prm);
}

// ---------------------------------------------------------------------------
// Tangent (forward sensitivity), IGR_adjoints_2d/sensitivity.jl:34-413.
// s_gamma != 0 adds the direct dP/dgamma source by analogy with the 1D
// package (IGR_adjoints_1d/sensitivity.jl:36-41): sP += s_gamma * rho * e,
// e = E/rho - |u|^2/2. The 2D reference has no such term (sensitivity.jl:15-16).
// ---------------------------------------------------------------------------
template <class T>
inline void sens_flux(int dir, const T& g, const T& mx, const T& my, const T& r, const T& E, const T& S,
                      const T& zx, const T& zy, const T& sr, const T& et, const T& vs, double sg, T f[4]) {
  T ux = mx / r, uy = my / r;
  T sux = (zx - ux * sr) / r, suy = (zy - uy * sr) / r;
  T P = pressure2d(g, mx, my, r, E);
  T Phi = (g - 1.0) * (et - sr * (ux * ux + uy * uy) / 2.0 - r * (ux * sux + uy * suy));
  if (sg != 0.0) Phi = Phi + sg * r * (E / r - (ux * ux + uy * uy) / 2.0);
  T Pt = Phi + vs;
  if (dir == 0) {
    f[0] = zx * ux + mx * sux + Pt; f[1] = zx * uy + mx * suy; f[2] = zx; f[3] = (et + Pt) * ux + (E + P + S) * sux;
  } else {
    f[0] = zx * uy + mx * suy; f[1] = zy * uy + my * suy + Pt; f[2] = zy; f[3] = (et + Pt) * uy + (E + P + S) * suy;
  }
}

template <class T>
void sens_hyperbolic_rhs(const Grid2D& G, const T& g, const T* const q[4], const T* S, const T* const s[4], const T* vs,
                         double sg, T* const ds[4], std::vector<T>* F) {
  const int np = G.np, Nex = G.m.Nex, Ney = G.m.Ney, L = np - 1; const Basis& B = G.b;
  const double invJx = 1 / G.m.Jx, invJy = 1 / G.m.Jy;
  for (int v = 0; v < 8; ++v) F[v].resize(G.N);
  for (size_t n = 0; n < G.N; ++n) {
    T fx[4], fy[4];
    sens_flux(0, g, q[0][n], q[1][n], q[2][n], q[3][n], S[n], s[0][n], s[1][n], s[2][n], s[3][n], vs[n], sg, fx);
    sens_flux(1, g, q[0][n], q[1][n], q[2][n], q[3][n], S[n], s[0][n], s[1][n], s[2][n], s[3][n], vs[n], sg, fy);
    for (int v = 0; v < 4; ++v) { F[v][n] = fx[v]; F[4 + v][n] = fy[v]; }
  }
  for (int ey = 0; ey < Ney; ++ey) for (int ex = 0; ex < Nex; ++ex)
    for (int j = 0; j < np; ++j) for (int i = 0; i < np; ++i) {
      T a[4] = {T(0.0), T(0.0), T(0.0), T(0.0)};
      for (int k = 0; k < np; ++k) {
        const size_t nx = G.id(k, j, ex, ey), ny = G.id(i, k, ex, ey);
        for (int v = 0; v < 4; ++v) a[v] = a[v] - (invJx * B.Dik(i, k) * F[v][nx] + invJy * B.Dik(j, k) * F[4 + v][ny]);
      }
      const size_t n = G.id(i, j, ex, ey);
      for (int v = 0; v < 4; ++v) ds[v][n] = a[v];
    }
  for (int dir = 0; dir < 2; ++dir)
    for (int ey = 0; ey < Ney; ++ey) for (int ex = 0; ex < Nex; ++ex)
      for (int t = 0; t < np; ++t) {
        size_t nl, nr;
        if (dir == 0) { const int exR = ex == Nex - 1 ? 0 : ex + 1; nl = G.id(L, t, ex, ey); nr = G.id(0, t, exR, ey); }
        else { const int eyR = ey == Ney - 1 ? 0 : ey + 1; nl = G.id(t, L, ex, ey); nr = G.id(t, 0, ex, eyR); }
        const double invJ = dir == 0 ? invJx : invJy;
        T lam = dir == 0 ? jmax(wavespeed_x(g, q[0][nl], q[1][nl], q[2][nl], q[3][nl]), wavespeed_x(g, q[0][nr], q[1][nr], q[2][nr], q[3][nr]))
                         : jmax(wavespeed_y(g, q[0][nl], q[1][nl], q[2][nl], q[3][nl]), wavespeed_y(g, q[0][nr], q[1][nr], q[2][nr], q[3][nr]));
        T fL[4], fR[4];
        sens_flux(dir, g, q[0][nl], q[1][nl], q[2][nl], q[3][nl], S[nl], s[0][nl], s[1][nl], s[2][nl], s[3][nl], vs[nl], sg, fL);
        sens_flux(dir, g, q[0][nr], q[1][nr], q[2][nr], q[3][nr], S[nr], s[0][nr], s[1][nr], s[2][nr], s[3][nr], vs[nr], sg, fR);
        for (int v = 0; v < 4; ++v) {
          T fs = (fL[v] + fR[v]) / 2.0 + lam * (s[v][nl] - s[v][nr]) / 2.0;
          ds[v][nl] = ds[v][nl] - invJ * (fs - F[4 * dir + v][nl]) / B.w[L];
          ds[v][nr] = ds[v][nr] + invJ * (fs - F[4 * dir + v][nr]) / B.w[0];
        }
      }
}

// compute_sensitivity_elliptic_rhs! (form 2), sensitivity.jl:236-292
template <class T>
void sens_elliptic_rhs(const Grid2D& G, T* b, const T* const q[4], const T* S, const T* const s[4], const T& alpha) {
  const int np = G.np; const Basis& B = G.b;
  const double invJx = 1 / G.m.Jx, invJy = 1 / G.m.Jy;
  const T *mx = q[0], *my = q[1], *rho = q[2], *zx = s[0], *zy = s[1], *sr = s[2];
  for (int ey = 0; ey < G.m.Ney; ++ey) for (int ex = 0; ex < G.m.Nex; ++ex)
    for (int j = 0; j < np; ++j) for (int i = 0; i < np; ++i) {
      T uxx(0.0), uxy(0.0), uyx(0.0), uyy(0.0), sxx(0.0), sxy(0.0), syx(0.0), syy(0.0), Sx(0.0), Sy(0.0), dxs(0.0), dys(0.0);
      for (int k = 0; k < np; ++k) {
        const size_t a = G.id(k, j, ex, ey), c = G.id(i, k, ex, ey);
        T uxkj = mx[a] / rho[a], uykj = my[a] / rho[a], uxik = mx[c] / rho[c], uyik = my[c] / rho[c];
        T sxkj = (zx[a] - uxkj * sr[a]) / rho[a], sykj = (zy[a] - uykj * sr[a]) / rho[a];
        T sxik = (zx[c] - uxik * sr[c]) / rho[c], syik = (zy[c] - uyik * sr[c]) / rho[c];
        const double Di = B.Dik(i, k), Dj = B.Dik(j, k);
        uxx = uxx + Di * uxkj; uyx = uyx + Di * uykj; uxy = uxy + Dj * uxik; uyy = uyy + Dj * uyik;
        sxx = sxx + Di * sxkj; syx = syx + Di * sykj; sxy = sxy + Dj * sxik; syy = syy + Dj * syik;
        Sx = Sx + Di * S[a]; Sy = Sy + Dj * S[c];
        dxs = dxs + Di * (sr[a] / rho[a]); dys = dys + Dj * (sr[c] / rho[c]);
      }
      uxx = uxx * invJx; uyx = uyx * invJx; uxy = uxy * invJy; uyy = uyy * invJy;
      sxx = sxx * invJx; syx = syx * invJx; sxy = sxy * invJy; syy = syy * invJy;
      Sx = Sx * invJx; Sy = Sy * invJy; dxs = dxs * invJx; dys = dys * invJy;
      T divu = uxx + uyy, divs = sxx + syy;
      T Rp = alpha * (divu * divu + uxx * uxx + 2.0 * uxy * uyx + uyy * uyy);
      T Rs = alpha * (2.0 * divu * divs + 2.0 * (uxx * sxx + uxy * syx + uyx * sxy + uyy * syy));
      const size_t n = G.id(i, j, ex, ey);
      T r = rho[n]; T srr = sr[n] / r;
      T bp = Rs + srr * Rp - alpha * (dxs * Sx + dys * Sy) / r;
      b[n] = B.w[i] * B.w[j] * G.m.Jx * G.m.Jy * bp;
    }
}

template <class T, class GridT>
void solve_with(const GridT& G, T* x, const T* rho, const T& alpha, int n_iter, int solver, Work2D<T>& W) {
  sip_diagonal(G, W.M.data(), rho, alpha);
  if (solver == SOLVER_PCG) pcg_fixed(G, x, W.b.data(), W.M.data(), n_iter, rho, alpha, W);
  else if (solver == SOLVER_JACOBI) jacobi_fixed(G, x, W.b.data(), W.M.data(), n_iter, rho, alpha, 2.0 / 3.0, W);
  else if (solver == SOLVER_CHEBYSHEV) chebyshev_fixed(G, x, W.b.data(), W.M.data(), n_iter, rho, alpha, W);
  else throw std::invalid_argument("Unknown solver");
}

// run_sensitivity, sensitivity.jl:353-413. q, s in-out; Sig, vs out.
template <class T>
void run_sensitivity(const Grid2D& G, T* const q[4], T* const s[4], T* Sig, T* vs, double dt, double T_end,
                     const T& g, const T& alpha, int n_iter, int solver, double s_gamma) {
  const size_t N = G.N;
  for (size_t k = 0; k < N; ++k) { Sig[k] = T(0.0); vs[k] = T(0.0); }
  Work2D<T> W; W.alloc(N);
  std::vector<T> s1[4], s2[4], dsv[4], dqs[4];
  for (int v = 0; v < 4; ++v) { s1[v].resize(N); s2[v].resize(N); dsv[v].resize(N); dqs[v].resize(N); }
  double dtr; int n_steps = rerounded_steps(dt, T_end, &dtr);
  auto stage = [&](const T* const qq[4], const T* const ss[4]) {
    igr_euler_rhs(G, qq, Sig, g, alpha, n_iter, solver, W);
    for (int v = 0; v < 4; ++v) dqs[v] = W.dq[v];
    if (value(alpha) > 0) {
      sens_elliptic_rhs(G, W.b.data(), qq, Sig, ss, alpha);
      solve_with(G, vs, qq[2], alpha, n_iter, solver, W);
    } else for (size_t k = 0; k < N; ++k) vs[k] = T(0.0);
    T* dsp[4] = {dsv[0].data(), dsv[1].data(), dsv[2].data(), dsv[3].data()};
    sens_hyperbolic_rhs(G, g, qq, Sig, ss, vs, s_gamma, dsp, W.F);
  };
  for (int st = 0; st < n_steps; ++st) {
    { const T* qq[4] = {q[0], q[1], q[2], q[3]}; const T* ss[4] = {s[0], s[1], s[2], s[3]}; stage(qq, ss); }
    for (int v = 0; v < 4; ++v) for (size_t k = 0; k < N; ++k) {
      W.q1[v][k] = q[v][k] + dtr * dqs[v][k]; s1[v][k] = s[v][k] + dtr * dsv[v][k];
    }
    { const T* qq[4] = {W.q1[0].data(), W.q1[1].data(), W.q1[2].data(), W.q1[3].data()};
      const T* ss[4] = {s1[0].data(), s1[1].data(), s1[2].data(), s1[3].data()}; stage(qq, ss); }
    for (int v = 0; v < 4; ++v) for (size_t k = 0; k < N; ++k) {
      W.q2[v][k] = 3.0 / 4 * q[v][k] + 1.0 / 4 * W.q1[v][k] + 1.0 / 4 * dtr * dqs[v][k];
      s2[v][k] = 3.0 / 4 * s[v][k] + 1.0 / 4 * s1[v][k] + 1.0 / 4 * dtr * dsv[v][k];
    }
    { const T* qq[4] = {W.q2[0].data(), W.q2[1].data(), W.q2[2].data(), W.q2[3].data()};
      const T* ss[4] = {s2[0].data(), s2[1].data(), s2[2].data(), s2[3].data()}; stage(qq, ss); }
    for (int v = 0; v < 4; ++v) for (size_t k = 0; k < N; ++k) {
      q[v][k] = 1.0 / 3 * q[v][k] + 2.0 / 3 * W.q2[v][k] + 2.0 / 3 * dtr * dqs[v][k];
      s[v][k] = 1.0 / 3 * s[v][k] + 2.0 / 3 * s2[v][k] + 2.0 / 3 * dtr * dsv[v][k];
    }
  }
  if (value(alpha) > 0) {
    const T* qq[4] = {q[0], q[1], q[2], q[3]}; const T* ss[4] = {s[0], s[1], s[2], s[3]};
    solve_elliptic(G, Sig, qq, alpha, n_iter, solver, W);
    sens_elliptic_rhs(G, W.b.data(), qq, Sig, ss, alpha);
    solve_with(G, vs, q[2], alpha, n_iter, solver, W);
  }
}

}  // namespace igr
