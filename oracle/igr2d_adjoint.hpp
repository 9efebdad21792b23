// ORACLE — test infrastructure only (see igr_common.hpp for the parity status).
// Hand-written discrete adjoint (reverse mode) of the 2D IGR-Euler map that
// IGR_adjoints_2d/enzyme_adjoint.jl:270-296 differentiates with Enzyme:
// J(q_T) after n_steps inlined SSP-RK3 steps (enzyme_adjoint.jl:56-71), with
// the gradient taken w.r.t. the initial conservative state q0 and, as an
// extension the reference lacks, w.r.t. gamma and alpha.
//
// Every forward primitive of igr2d.hpp has its transpose here. Conventions at
// kinks match the forward dual numbers: d|u|/du = +1 at u = +0.0, and
// max(a, b) sends the derivative to the first argument on ties.
#pragma once
#include "igr2d.hpp"

namespace igr {

// Reverse of flux_x (dir 0) / flux_y (dir 1) at one node: fb = adjoint of f[4];
// accumulates into qb[4] (mx, my, rho, E), Sb and gb.
inline void flux_rev(int dir, double g, double mx, double my, double r, double E, double S, const double fb[4],
                     double qb[4], double& Sb, double& gb) {
  const double K = (mx * mx + my * my) / (2.0 * r);
  const double P = (g - 1.0) * (E - K);
  const double pb = P + S;
  const double mn = dir == 0 ? mx : my;          // normal momentum
  const double un = mn / r;
  double unb, pbb;
  if (dir == 0) {
    // f = (mx*ux + pb, my*ux, mx, (E+pb)*ux)
    unb = fb[0] * mx + fb[1] * my + fb[3] * (E + pb);
    pbb = fb[0] + fb[3] * un;
    qb[0] += fb[0] * un + fb[2];
    qb[1] += fb[1] * un;
  } else {
    // f = (mx*uy, my*uy + pb, my, (E+pb)*uy)
    unb = fb[0] * mx + fb[1] * my + fb[3] * (E + pb);
    pbb = fb[1] + fb[3] * un;
    qb[0] += fb[0] * un;
    qb[1] += fb[1] * un + fb[2];
  }
  qb[3] += fb[3] * un;
  Sb += pbb;
  const double Pb = pbb;
  // un = mn / r
  qb[dir] += unb / r;
  qb[2] += -unb * un / r;
  // P = (g-1)(E - K)
  gb += Pb * (E - K);
  qb[3] += Pb * (g - 1.0);
  const double Kb = -Pb * (g - 1.0);
  qb[0] += Kb * mx / r;
  qb[1] += Kb * my / r;
  qb[2] += -Kb * K / r;
}

// Reverse of wavespeed_{x,y} = |u_n| + sqrt(g P / r).
inline void wavespeed_rev(int dir, double g, double mx, double my, double r, double E, double wb, double qb[4], double& gb) {
  const double K = (mx * mx + my * my) / (2.0 * r);
  const double P = (g - 1.0) * (E - K);
  const double un = (dir == 0 ? mx : my) / r;
  const double unb = std::signbit(un) ? -wb : wb;
  qb[dir] += unb / r;
  qb[2] += -unb * un / r;
  const double X = g * P / r;
  const double c = std::sqrt(X);
  const double Xb = wb / (2.0 * c);
  gb += Xb * P / r;
  const double Pb = Xb * g / r;
  qb[2] += -Xb * X / r;
  gb += Pb * (E - K);
  qb[3] += Pb * (g - 1.0);
  const double Kb = -Pb * (g - 1.0);
  qb[0] += Kb * mx / r;
  qb[1] += Kb * my / r;
  qb[2] += -Kb * K / r;
}

// Reverse of hyperbolic_rhs: kb = adjoint of dq[4]; accumulates qb[4], Sb, gb.
inline void hyperbolic_rhs_rev(const Grid2D& G, double g, const double* const q[4], const double* S,
                               const double* const kb[4], double* const qb[4], double* Sb, double& gb) {
  const int np = G.np, Nex = G.m.Nex, Ney = G.m.Ney, L = np - 1; const Basis& B = G.b;
  const double invJx = 1 / G.m.Jx, invJy = 1 / G.m.Jy;
  std::vector<double> Fb[8];
  for (int v = 0; v < 8; ++v) Fb[v].assign(G.N, 0.0);
  // volume: dq_ij -= invJx D_ik Fx_kj + invJy D_jk Fy_ik
  for (int ey = 0; ey < Ney; ++ey) for (int ex = 0; ex < Nex; ++ex)
    for (int j = 0; j < np; ++j) for (int i = 0; i < np; ++i) {
      const size_t n = G.id(i, j, ex, ey);
      for (int k = 0; k < np; ++k) {
        const size_t nx = G.id(k, j, ex, ey), ny = G.id(i, k, ex, ey);
        for (int v = 0; v < 4; ++v) {
          Fb[v][nx] -= invJx * B.Dik(i, k) * kb[v][n];
          Fb[4 + v][ny] -= invJy * B.Dik(j, k) * kb[v][n];
        }
      }
    }
  for (int dir = 0; dir < 2; ++dir)
    for (int ey = 0; ey < Ney; ++ey) for (int ex = 0; ex < Nex; ++ex)
      for (int t = 0; t < np; ++t) {
        size_t nl, nr;
        if (dir == 0) { const int exR = ex == Nex - 1 ? 0 : ex + 1; nl = G.id(L, t, ex, ey); nr = G.id(0, t, exR, ey); }
        else { const int eyR = ey == Ney - 1 ? 0 : ey + 1; nl = G.id(t, L, ex, ey); nr = G.id(t, 0, ex, eyR); }
        const double invJ = dir == 0 ? invJx : invJy;
        double fsb[4];
        for (int v = 0; v < 4; ++v) {
          fsb[v] = -invJ / B.w[L] * kb[v][nl] + invJ / B.w[0] * kb[v][nr];
          Fb[4 * dir + v][nl] += invJ / B.w[L] * kb[v][nl];
          Fb[4 * dir + v][nr] -= invJ / B.w[0] * kb[v][nr];
        }
        const double qL[4] = {q[0][nl], q[1][nl], q[2][nl], q[3][nl]};
        const double qR[4] = {q[0][nr], q[1][nr], q[2][nr], q[3][nr]};
        const double wL = dir == 0 ? wavespeed_x(g, qL[0], qL[1], qL[2], qL[3]) : wavespeed_y(g, qL[0], qL[1], qL[2], qL[3]);
        const double wR = dir == 0 ? wavespeed_x(g, qR[0], qR[1], qR[2], qR[3]) : wavespeed_y(g, qR[0], qR[1], qR[2], qR[3]);
        const double lam = jmax(wL, wR);
        double lamb = 0.0, fLb[4], fRb[4], qLb[4] = {0, 0, 0, 0}, qRb[4] = {0, 0, 0, 0};
        for (int v = 0; v < 4; ++v) {
          fLb[v] = fsb[v] / 2.0; fRb[v] = fsb[v] / 2.0;
          qLb[v] += lam * fsb[v] / 2.0; qRb[v] -= lam * fsb[v] / 2.0;
          lamb += fsb[v] * (qL[v] - qR[v]) / 2.0;
        }
        double SLb = 0.0, SRb = 0.0;
        flux_rev(dir, g, qL[0], qL[1], qL[2], qL[3], S[nl], fLb, qLb, SLb, gb);
        flux_rev(dir, g, qR[0], qR[1], qR[2], qR[3], S[nr], fRb, qRb, SRb, gb);
        if (wR > wL) wavespeed_rev(dir, g, qR[0], qR[1], qR[2], qR[3], lamb, qRb, gb);
        else wavespeed_rev(dir, g, qL[0], qL[1], qL[2], qL[3], lamb, qLb, gb);
        for (int v = 0; v < 4; ++v) { qb[v][nl] += qLb[v]; qb[v][nr] += qRb[v]; }
        Sb[nl] += SLb; Sb[nr] += SRb;
      }
  for (size_t n = 0; n < G.N; ++n) {
    double qbn[4] = {0, 0, 0, 0}, Sbn = 0.0;
    const double fxb[4] = {Fb[0][n], Fb[1][n], Fb[2][n], Fb[3][n]};
    const double fyb[4] = {Fb[4][n], Fb[5][n], Fb[6][n], Fb[7][n]};
    flux_rev(0, g, q[0][n], q[1][n], q[2][n], q[3][n], S[n], fxb, qbn, Sbn, gb);
    flux_rev(1, g, q[0][n], q[1][n], q[2][n], q[3][n], S[n], fyb, qbn, Sbn, gb);
    for (int v = 0; v < 4; ++v) qb[v][n] += qbn[v];
    Sb[n] += Sbn;
  }
}

// Gradient of scale * u^T A(rho, alpha) v w.r.t. rho (accumulated in rhob) and alpha.
inline void sip_param_adj(const Grid2D& G, double scale, const double* u, const double* v, const double* rho, double alpha,
                          double* rhob, double& alphab) {
  const int np = G.np, Nex = G.m.Nex, Ney = G.m.Ney, L = np - 1; const Basis& B = G.b;
  const double Jx = G.m.Jx, Jy = G.m.Jy, invJx = 1 / Jx, invJy = 1 / Jy;
  const double eta = (double)((B.p + 1) * (B.p + 1));
  std::vector<double> invb(G.N, 0.0);
  double ab = 0.0;
  for (int ey = 0; ey < Ney; ++ey) for (int ex = 0; ex < Nex; ++ex)
    for (int j = 0; j < np; ++j) for (int i = 0; i < np; ++i) {
      const size_t n = G.id(i, j, ex, ey);
      double dvx = 0, dvy = 0, dux = 0, duy = 0;
      for (int k = 0; k < np; ++k) {
        const size_t a = G.id(k, j, ex, ey), c = G.id(i, k, ex, ey);
        dvx += B.Dik(i, k) * v[a]; dux += B.Dik(i, k) * u[a];
        dvy += B.Dik(j, k) * v[c]; duy += B.Dik(j, k) * u[c];
      }
      const double ww = B.w[i] * B.w[j];
      invb[n] += ww * Jx * Jy * u[n] * v[n];
      const double st = ww * Jy * invJx * dvx * dux + ww * Jx * invJy * dvy * duy;
      invb[n] += alpha * st;
      ab += st / rho[n];
    }
  for (int dir = 0; dir < 2; ++dir)
    for (int ey = 0; ey < Ney; ++ey) for (int ex = 0; ex < Nex; ++ex)
      for (int t = 0; t < np; ++t) {
        double wf, invJ, h; size_t nl, nr; double dvL = 0, dvR = 0, duL = 0, duR = 0;
        if (dir == 0) {
          const int exR = ex == Nex - 1 ? 0 : ex + 1; wf = B.w[t] * Jy; invJ = invJx; h = G.m.dx;
          nl = G.id(L, t, ex, ey); nr = G.id(0, t, exR, ey);
          for (int k = 0; k < np; ++k) {
            dvL += B.Dik(L, k) * v[G.id(k, t, ex, ey)]; dvR += B.Dik(0, k) * v[G.id(k, t, exR, ey)];
            duL += B.Dik(L, k) * u[G.id(k, t, ex, ey)]; duR += B.Dik(0, k) * u[G.id(k, t, exR, ey)];
          }
        } else {
          const int eyR = ey == Ney - 1 ? 0 : ey + 1; wf = B.w[t] * Jx; invJ = invJy; h = G.m.dy;
          nl = G.id(t, L, ex, ey); nr = G.id(t, 0, ex, eyR);
          for (int k = 0; k < np; ++k) {
            dvL += B.Dik(L, k) * v[G.id(t, k, ex, ey)]; dvR += B.Dik(0, k) * v[G.id(t, k, ex, eyR)];
            duL += B.Dik(L, k) * u[G.id(t, k, ex, ey)]; duR += B.Dik(0, k) * u[G.id(t, k, ex, eyR)];
          }
        }
        const double iL = 1.0 / rho[nl], iR = 1.0 / rho[nr];
        const double jv = v[nl] - v[nr], ju = u[nl] - u[nr];
        const double cL = dvL * ju + duL * jv, cR = dvR * ju + duR * jv;
        const double imax = jmax(iL, iR);
        // face form: -alpha wf invJ/2 (iL cL + iR cR) + alpha wf eta max(iL,iR)/h jv ju
        invb[nl] += -alpha * wf * invJ / 2.0 * cL;
        invb[nr] += -alpha * wf * invJ / 2.0 * cR;
        const double pen = alpha * wf * eta / h * jv * ju;
        if (iR > iL) invb[nr] += pen; else invb[nl] += pen;
        ab += -wf * invJ / 2.0 * (iL * cL + iR * cR) + wf * eta * imax / h * jv * ju;
      }
  for (size_t n = 0; n < G.N; ++n) rhob[n] += scale * (-invb[n] / (rho[n] * rho[n]));
  alphab += scale * ab;
}

// Reverse of sip_diagonal: Mb = adjoint of M.
inline void sip_diagonal_rev(const Grid2D& G, const double* Mb, const double* rho, double alpha, double* rhob, double& alphab) {
  const int np = G.np, L = np - 1; const Basis& B = G.b;
  const double Jx = G.m.Jx, Jy = G.m.Jy, invJx = 1 / Jx, invJy = 1 / Jy;
  const double eta = (double)(np * np);
  std::vector<double> invb(G.N, 0.0);
  double ab = 0.0;
  for (int ey = 0; ey < G.m.Ney; ++ey) for (int ex = 0; ex < G.m.Nex; ++ex) {
    for (int j = 0; j < np; ++j) for (int i = 0; i < np; ++i) {
      const size_t n = G.id(i, j, ex, ey);
      invb[n] += Mb[n] * B.w[i] * B.w[j] * Jx * Jy;
    }
    for (int l = 0; l < np; ++l) for (int k = 0; k < np; ++k) {
      const size_t n = G.id(k, l, ex, ey);
      for (int i = 0; i < np; ++i) {
        const double d = B.Dik(i, k); const size_t m = G.id(i, l, ex, ey);
        const double c = B.w[i] * B.w[l] * Jy * invJx * (d * d);
        invb[m] += Mb[n] * alpha * c; ab += Mb[n] * c / rho[m];
      }
      for (int j = 0; j < np; ++j) {
        const double d = B.Dik(j, l); const size_t m = G.id(k, j, ex, ey);
        const double c = B.w[k] * B.w[j] * Jx * invJy * (d * d);
        invb[m] += Mb[n] * alpha * c; ab += Mb[n] * c / rho[m];
      }
    }
  }
  for (int dir = 0; dir < 2; ++dir)
    for (int ey = 0; ey < G.m.Ney; ++ey) for (int ex = 0; ex < G.m.Nex; ++ex)
      for (int t = 0; t < np; ++t) {
        double wf, invJ, h; size_t nl, nr;
        if (dir == 0) { const int exR = ex == G.m.Nex - 1 ? 0 : ex + 1; wf = B.w[t] * Jy; invJ = invJx; h = G.m.dx; nl = G.id(L, t, ex, ey); nr = G.id(0, t, exR, ey); }
        else { const int eyR = ey == G.m.Ney - 1 ? 0 : ey + 1; wf = B.w[t] * Jx; invJ = invJy; h = G.m.dy; nl = G.id(t, L, ex, ey); nr = G.id(t, 0, ex, eyR); }
        const double iL = 1.0 / rho[nl], iR = 1.0 / rho[nr];
        // M[nl] += (-alpha invJ D_LL iL + alpha sig) wf ; M[nr] += (alpha invJ D_00 iR + alpha sig) wf
        invb[nl] += Mb[nl] * (-alpha) * invJ * B.Dik(L, L) * wf;
        invb[nr] += Mb[nr] * alpha * invJ * B.Dik(0, 0) * wf;
        const double sigb = (Mb[nl] + Mb[nr]) * alpha * wf;
        const double imax = jmax(iL, iR);
        if (iR > iL) invb[nr] += sigb * eta / h; else invb[nl] += sigb * eta / h;
        ab += Mb[nl] * (-invJ * B.Dik(L, L) * iL + eta * imax / h) * wf + Mb[nr] * (invJ * B.Dik(0, 0) * iR + eta * imax / h) * wf;
      }
  for (size_t n = 0; n < G.N; ++n) rhob[n] += -invb[n] / (rho[n] * rho[n]);
  alphab += ab;
}

// Reverse of igr_rhs: bb = adjoint of b.
inline void igr_rhs_rev(const Grid2D& G, const double* bb, const double* mx, const double* my, const double* rho, double alpha,
                        double* mxb, double* myb, double* rhob, double& alphab) {
  const int np = G.np; const Basis& B = G.b;
  const double invJx = 1 / G.m.Jx, invJy = 1 / G.m.Jy;
  std::vector<double> uxb(G.N, 0.0), uyb(G.N, 0.0);
  for (int ey = 0; ey < G.m.Ney; ++ey) for (int ex = 0; ex < G.m.Nex; ++ex)
    for (int j = 0; j < np; ++j) for (int i = 0; i < np; ++i) {
      double uxx = 0, uxy = 0, uyx = 0, uyy = 0;
      for (int k = 0; k < np; ++k) {
        const size_t a = G.id(k, j, ex, ey), c = G.id(i, k, ex, ey);
        uxx += B.Dik(i, k) * (mx[a] / rho[a]); uyx += B.Dik(i, k) * (my[a] / rho[a]);
        uxy += B.Dik(j, k) * (mx[c] / rho[c]); uyy += B.Dik(j, k) * (my[c] / rho[c]);
      }
      uxx *= invJx; uyx *= invJx; uxy *= invJy; uyy *= invJy;
      const size_t n = G.id(i, j, ex, ey);
      const double c = B.w[i] * B.w[j] * G.m.Jx * G.m.Jy;
      const double s = uxx + uyy;
      const double Q = s * s + uxx * uxx + 2.0 * uxy * uyx + uyy * uyy;
      alphab += bb[n] * c * Q;
      const double Qb = bb[n] * c * alpha;
      const double uxxb = Qb * (2.0 * s + 2.0 * uxx), uyyb = Qb * (2.0 * s + 2.0 * uyy);
      const double uxyb = Qb * 2.0 * uyx, uyxb = Qb * 2.0 * uxy;
      for (int k = 0; k < np; ++k) {
        const size_t a = G.id(k, j, ex, ey), cc = G.id(i, k, ex, ey);
        uxb[a] += invJx * B.Dik(i, k) * uxxb; uyb[a] += invJx * B.Dik(i, k) * uyxb;
        uxb[cc] += invJy * B.Dik(j, k) * uxyb; uyb[cc] += invJy * B.Dik(j, k) * uyyb;
      }
    }
  for (size_t n = 0; n < G.N; ++n) {
    mxb[n] += uxb[n] / rho[n]; myb[n] += uyb[n] / rho[n];
    rhob[n] += -(uxb[n] * mx[n] + uyb[n] * my[n]) / (rho[n] * rho[n]);
  }
}

// ---------------------------------------------------------------------------
// Solver tapes and reverses (elliptic.jl:329-397)
// ---------------------------------------------------------------------------
struct SolverTape {
  std::vector<std::vector<double>> x, r, p, Ap;  // per-iteration vectors
  std::vector<double> rz, pAp, a, beta;          // PCG scalars
};

// Forward solve recording the tape. x in-out (warm start).
template <class GridT>
inline void solve_tape(const GridT& G, double* x, const double* b, const double* M, int n_iter, const double* rho, double alpha,
                       int solver, SolverTape& tp) {
  const size_t N = G.N;
  std::vector<double> Ax(N), r(N), z(N), d(N), p(N), Ap(N);
  tp = SolverTape();
  if (solver == SOLVER_CHEBYSHEV) {
    const ChebParams c = cheb_params(G.b.p);
    apply_sip(G, Ax.data(), x, rho, alpha);
    for (size_t k = 0; k < N; ++k) r[k] = b[k] - Ax[k];
    double rc = 1 / c.sigma;
    for (int it = 1; it <= n_iter; ++it) {
      tp.x.emplace_back(x, x + N); tp.r.push_back(r);
      for (size_t k = 0; k < N; ++k) z[k] = r[k] / M[k];
      if (it == 1) { for (size_t k = 0; k < N; ++k) d[k] = z[k] / c.theta; }
      else { double rn = 1 / (2 * c.sigma - rc); for (size_t k = 0; k < N; ++k) d[k] = rn * rc * d[k] + (2 * rn / c.delta) * z[k]; rc = rn; }
      for (size_t k = 0; k < N; ++k) x[k] = x[k] + d[k];
      apply_sip(G, Ax.data(), x, rho, alpha);
      for (size_t k = 0; k < N; ++k) r[k] = b[k] - Ax[k];
    }
  } else if (solver == SOLVER_JACOBI) {
    for (int it = 0; it < n_iter; ++it) {
      tp.x.emplace_back(x, x + N);
      apply_sip(G, Ax.data(), x, rho, alpha);
      for (size_t k = 0; k < N; ++k) r[k] = b[k] - Ax[k];
      tp.r.push_back(r);
      for (size_t k = 0; k < N; ++k) x[k] = x[k] + 2.0 / 3.0 * (b[k] - Ax[k]) / M[k];
    }
  } else if (solver == SOLVER_PCG) {
    tp.x.emplace_back(x, x + N);
    apply_sip(G, Ap.data(), x, rho, alpha);
    for (size_t k = 0; k < N; ++k) r[k] = b[k] - Ap[k];
    for (size_t k = 0; k < N; ++k) z[k] = r[k] / M[k];
    p = z;
    double rz = dotv(r.data(), z.data(), N);
    tp.r.push_back(r); tp.rz.push_back(rz);
    for (int it = 0; it < n_iter; ++it) {
      apply_sip(G, Ap.data(), p.data(), rho, alpha);
      double pAp = dotv(p.data(), Ap.data(), N);
      double a = rz / (pAp + 1e-30);
      tp.p.push_back(p); tp.Ap.push_back(Ap); tp.pAp.push_back(pAp); tp.a.push_back(a);
      for (size_t k = 0; k < N; ++k) x[k] = x[k] + a * p[k];
      for (size_t k = 0; k < N; ++k) r[k] = r[k] - a * Ap[k];
      for (size_t k = 0; k < N; ++k) z[k] = r[k] / M[k];
      double rzn = dotv(r.data(), z.data(), N);
      double beta = rzn / (rz + 1e-30);
      for (size_t k = 0; k < N; ++k) p[k] = z[k] + beta * p[k];
      tp.r.push_back(r); tp.rz.push_back(rzn); tp.beta.push_back(beta);
      rz = rzn;
    }
  } else throw std::invalid_argument("Unknown solver");
}

// Reverse of the solve. xb: in = adjoint of the output x, out = adjoint of the
// warm start x0. Accumulates bb, Mb, rhob (through A) and alphab (through A).
template <class GridT>
inline void solve_rev(const GridT& G, double* xb, const double* b, const double* M, int n_iter, const double* rho, double alpha,
                      int solver, const SolverTape& tp, double* bb, double* Mb, double* rhob, double& alphab) {
  const size_t N = G.N;
  std::vector<double> t(N), Au(N);
  if (solver == SOLVER_CHEBYSHEV) {
    const ChebParams c = cheb_params(G.b.p);
    std::vector<double> coef_a(n_iter + 1, 0.0), coef_c(n_iter + 1, 0.0);
    double rc = 1 / c.sigma;
    for (int it = 1; it <= n_iter; ++it) {
      if (it == 1) { coef_a[it] = 0.0; coef_c[it] = 1.0 / c.theta; }
      else { double rn = 1 / (2 * c.sigma - rc); coef_a[it] = rn * rc; coef_c[it] = 2 * rn / c.delta; rc = rn; }
    }
    std::vector<double> db(N, 0.0), rb(N, 0.0);  // r_n is never read: its adjoint is zero
    for (int it = n_iter; it >= 1; --it) {
      // r_it = b - A x_it (only for it < n_iter is r_it read, by z_{it+1})
      if (it < n_iter) {
        for (size_t k = 0; k < N; ++k) bb[k] += rb[k];
        apply_sip(G, Au.data(), rb.data(), rho, alpha);
        for (size_t k = 0; k < N; ++k) xb[k] -= Au[k];
        sip_param_adj(G, -1.0, rb.data(), tp.x[it].data(), rho, alpha, rhob, alphab);
      }
      // x_it = x_{it-1} + d_it
      for (size_t k = 0; k < N; ++k) db[k] += xb[k];
      // d_it = a d_{it-1} + c z_it ; z_it = r_{it-1} / M
      for (size_t k = 0; k < N; ++k) {
        const double zb = coef_c[it] * db[k];
        rb[k] = zb / M[k];
        Mb[k] += -zb * tp.r[it - 1][k] / (M[k] * M[k]);
        db[k] = coef_a[it] * db[k];
      }
    }
    // r_0 = b - A x_0
    for (size_t k = 0; k < N; ++k) bb[k] += rb[k];
    apply_sip(G, Au.data(), rb.data(), rho, alpha);
    for (size_t k = 0; k < N; ++k) xb[k] -= Au[k];
    sip_param_adj(G, -1.0, rb.data(), tp.x[0].data(), rho, alpha, rhob, alphab);
  } else if (solver == SOLVER_JACOBI) {
    const double om = 2.0 / 3.0;
    for (int it = n_iter - 1; it >= 0; --it) {
      // x_{it+1} = x_it + om (b - A x_it) / M
      for (size_t k = 0; k < N; ++k) {
        t[k] = om * xb[k] / M[k];
        Mb[k] += -xb[k] * om * tp.r[it][k] / (M[k] * M[k]);
        bb[k] += t[k];
      }
      apply_sip(G, Au.data(), t.data(), rho, alpha);
      for (size_t k = 0; k < N; ++k) xb[k] -= Au[k];
      sip_param_adj(G, -1.0, t.data(), tp.x[it].data(), rho, alpha, rhob, alphab);
    }
  } else if (solver == SOLVER_PCG) {
    std::vector<double> pb(N, 0.0), rb(N, 0.0), zb(N, 0.0), Apb(N);
    std::vector<double> rzb(n_iter + 1, 0.0);
    for (int it = n_iter - 1; it >= 0; --it) {
      const std::vector<double>& r1 = tp.r[it + 1];
      // p_{it+1} = z_{it+1} + beta p_it
      double betab = dotv(pb.data(), tp.p[it].data(), N);
      for (size_t k = 0; k < N; ++k) { zb[k] = pb[k]; pb[k] = tp.beta[it] * pb[k]; }
      // beta = rz_{it+1} / (rz_it + eps)
      rzb[it + 1] += betab / (tp.rz[it] + 1e-30);
      rzb[it] += -betab * tp.rz[it + 1] / ((tp.rz[it] + 1e-30) * (tp.rz[it] + 1e-30));
      // rz_{it+1} = r_{it+1} . z_{it+1} ; z_{it+1} = r_{it+1} / M
      for (size_t k = 0; k < N; ++k) {
        const double z1 = r1[k] / M[k];
        rb[k] += rzb[it + 1] * z1;
        zb[k] += rzb[it + 1] * r1[k];
        rb[k] += zb[k] / M[k];
        Mb[k] += -zb[k] * r1[k] / (M[k] * M[k]);
      }
      // r_{it+1} = r_it - a Ap_it ; x_{it+1} = x_it + a p_it
      double ab = -dotv(rb.data(), tp.Ap[it].data(), N) + dotv(xb, tp.p[it].data(), N);
      for (size_t k = 0; k < N; ++k) { Apb[k] = -tp.a[it] * rb[k]; pb[k] += tp.a[it] * xb[k]; }
      // a = rz_it / (pAp + eps)
      const double den = tp.pAp[it] + 1e-30;
      rzb[it] += ab / den;
      const double pApb = -ab * tp.rz[it] / (den * den);
      for (size_t k = 0; k < N; ++k) { pb[k] += pApb * tp.Ap[it][k]; Apb[k] += pApb * tp.p[it][k]; }
      // Ap = A p
      apply_sip(G, Au.data(), Apb.data(), rho, alpha);
      for (size_t k = 0; k < N; ++k) pb[k] += Au[k];
      sip_param_adj(G, 1.0, Apb.data(), tp.p[it].data(), rho, alpha, rhob, alphab);
    }
    // p_0 = z_0 ; rz_0 = r_0 . z_0 ; z_0 = r_0 / M ; r_0 = b - A x_0
    const std::vector<double>& r0 = tp.r[0];
    for (size_t k = 0; k < N; ++k) {
      const double z0 = r0[k] / M[k];
      double z0b = pb[k] + rzb[0] * r0[k];
      rb[k] += rzb[0] * z0 + z0b / M[k];
      Mb[k] += -z0b * r0[k] / (M[k] * M[k]);
      bb[k] += rb[k];
    }
    apply_sip(G, Au.data(), rb.data(), rho, alpha);
    for (size_t k = 0; k < N; ++k) xb[k] -= Au[k];
    sip_param_adj(G, -1.0, rb.data(), tp.x[0].data(), rho, alpha, rhob, alphab);
  } else throw std::invalid_argument("Unknown solver");
}

// ---------------------------------------------------------------------------
// One RK3 step with a tape, and its reverse.
// ---------------------------------------------------------------------------
struct StageTape {
  std::vector<double> q[4], Sin, Sout, b, M;
  SolverTape st;
};

struct StepTape { StageTape s[3]; };

inline void stage_forward(const Grid2D& G, StageTape& T, const double* const q[4], double* Sig, double g, double alpha,
                          int n_iter, int solver, double* const dq[4], std::vector<double>* F) {
  for (int v = 0; v < 4; ++v) T.q[v].assign(q[v], q[v] + G.N);
  T.Sin.assign(Sig, Sig + G.N);
  if (alpha > 0) {
    T.b.resize(G.N); T.M.resize(G.N);
    igr_rhs(G, T.b.data(), q[0], q[1], q[2], alpha);
    sip_diagonal(G, T.M.data(), q[2], alpha);
    solve_tape(G, Sig, T.b.data(), T.M.data(), n_iter, q[2], alpha, solver, T.st);
  } else {
    for (size_t k = 0; k < G.N; ++k) Sig[k] = 0.0;
  }
  T.Sout.assign(Sig, Sig + G.N);
  hyperbolic_rhs(G, g, q, Sig, dq, F);
}

// Reverse of one stage: kb = adjoint of the stage RHS k; Sb: in = adjoint of
// Sigma_out, out = adjoint of Sigma_in. Accumulates qb, gb, alphab.
inline void stage_reverse(const Grid2D& G, const StageTape& T, const double* const kb[4], double* Sb, double* const qb[4],
                          double g, double alpha, int n_iter, int solver, double& gb, double& alphab) {
  const double* q[4] = {T.q[0].data(), T.q[1].data(), T.q[2].data(), T.q[3].data()};
  hyperbolic_rhs_rev(G, g, q, T.Sout.data(), kb, qb, Sb, gb);
  if (alpha > 0) {
    std::vector<double> bb(G.N, 0.0), Mb(G.N, 0.0);
    solve_rev(G, Sb, T.b.data(), T.M.data(), n_iter, q[2], alpha, solver, T.st, bb.data(), Mb.data(), qb[2], alphab);
    igr_rhs_rev(G, bb.data(), q[0], q[1], q[2], alpha, qb[0], qb[1], qb[2], alphab);
    sip_diagonal_rev(G, Mb.data(), q[2], alpha, qb[2], alphab);
  } else {
    for (size_t k = 0; k < G.N; ++k) Sb[k] = 0.0;
  }
}

inline void step_forward_tape(const Grid2D& G, StepTape& tape, double* const q[4], double* Sig, double g, double alpha,
                              double dt, int n_iter, int solver) {
  const size_t N = G.N;
  std::vector<double> dqv[4], q1[4], q2[4], F[8];
  for (int v = 0; v < 4; ++v) { dqv[v].resize(N); q1[v].resize(N); q2[v].resize(N); }
  double* dq[4] = {dqv[0].data(), dqv[1].data(), dqv[2].data(), dqv[3].data()};
  const double* qc[4] = {q[0], q[1], q[2], q[3]};
  stage_forward(G, tape.s[0], qc, Sig, g, alpha, n_iter, solver, dq, F);
  for (int v = 0; v < 4; ++v) for (size_t k = 0; k < N; ++k) q1[v][k] = q[v][k] + dt * dq[v][k];
  const double* q1c[4] = {q1[0].data(), q1[1].data(), q1[2].data(), q1[3].data()};
  stage_forward(G, tape.s[1], q1c, Sig, g, alpha, n_iter, solver, dq, F);
  for (int v = 0; v < 4; ++v) for (size_t k = 0; k < N; ++k) q2[v][k] = 3.0 / 4 * q[v][k] + 1.0 / 4 * q1[v][k] + 1.0 / 4 * dt * dq[v][k];
  const double* q2c[4] = {q2[0].data(), q2[1].data(), q2[2].data(), q2[3].data()};
  stage_forward(G, tape.s[2], q2c, Sig, g, alpha, n_iter, solver, dq, F);
  for (int v = 0; v < 4; ++v) for (size_t k = 0; k < N; ++k) q[v][k] = 1.0 / 3 * q[v][k] + 2.0 / 3 * q2[v][k] + 2.0 / 3 * dt * dq[v][k];
}

// qb: in = adjoint of q^{n+1}, out = adjoint of q^n. Sb likewise for Sigma.
inline void step_reverse(const Grid2D& G, const StepTape& tape, double* const qb[4], double* Sb, double g, double alpha,
                         double dt, int n_iter, int solver, double& gb, double& alphab) {
  const size_t N = G.N;
  std::vector<double> kbv[4], q1b[4], q2b[4], qnb[4];
  for (int v = 0; v < 4; ++v) { kbv[v].resize(N); q1b[v].assign(N, 0.0); q2b[v].assign(N, 0.0); qnb[v].assign(N, 0.0); }
  const double* kb[4] = {kbv[0].data(), kbv[1].data(), kbv[2].data(), kbv[3].data()};
  double* q1p[4] = {q1b[0].data(), q1b[1].data(), q1b[2].data(), q1b[3].data()};
  double* q2p[4] = {q2b[0].data(), q2b[1].data(), q2b[2].data(), q2b[3].data()};
  double* qnp[4] = {qnb[0].data(), qnb[1].data(), qnb[2].data(), qnb[3].data()};
  // q^{n+1} = 1/3 q^n + 2/3 q2 + 2/3 dt k3
  for (int v = 0; v < 4; ++v) for (size_t k = 0; k < N; ++k) {
    qnb[v][k] = 1.0 / 3 * qb[v][k]; q2b[v][k] = 2.0 / 3 * qb[v][k]; kbv[v][k] = 2.0 / 3 * dt * qb[v][k];
  }
  stage_reverse(G, tape.s[2], kb, Sb, q2p, g, alpha, n_iter, solver, gb, alphab);
  // q2 = 3/4 q^n + 1/4 q1 + 1/4 dt k2
  for (int v = 0; v < 4; ++v) for (size_t k = 0; k < N; ++k) {
    qnb[v][k] += 3.0 / 4 * q2b[v][k]; q1b[v][k] = 1.0 / 4 * q2b[v][k]; kbv[v][k] = 1.0 / 4 * dt * q2b[v][k];
  }
  stage_reverse(G, tape.s[1], kb, Sb, q1p, g, alpha, n_iter, solver, gb, alphab);
  // q1 = q^n + dt k1
  for (int v = 0; v < 4; ++v) for (size_t k = 0; k < N; ++k) { qnb[v][k] += q1b[v][k]; kbv[v][k] = dt * q1b[v][k]; }
  stage_reverse(G, tape.s[0], kb, Sb, qnp, g, alpha, n_iter, solver, gb, alphab);
  for (int v = 0; v < 4; ++v) for (size_t k = 0; k < N; ++k) qb[v][k] = qnb[v][k];
}

// Gradient of objective2d w.r.t. the final state (and gamma).
inline void objective2d_grad(const Grid2D& G, int obj, const double* const q[4], double g, const double* prm,
                             double* const qb[4], double& gb) {
  const int np = G.np; const Basis& B = G.b; const double Jx = G.m.Jx, Jy = G.m.Jy;
  const double pi = 3.14159265358979323846;
  for (int v = 0; v < 4; ++v) for (size_t n = 0; n < G.N; ++n) qb[v][n] = 0.0;
  if (obj == OBJ_KINETIC_ENERGY) {
    double KE = 0, Ms = 0;
    for (int ey = 0; ey < G.m.Ney; ++ey) for (int ex = 0; ex < G.m.Nex; ++ex) for (int j = 0; j < np; ++j) for (int i = 0; i < np; ++i) {
      const size_t n = G.id(i, j, ex, ey); const double wJ = B.w[i] * B.w[j] * Jx * Jy;
      KE += wJ * (q[0][n] * q[0][n] + q[1][n] * q[1][n]) / (2.0 * q[2][n]); Ms += wJ * q[2][n];
    }
    const double KEb = 1.0 / Ms, Mb = -KE / (Ms * Ms);
    for (int ey = 0; ey < G.m.Ney; ++ey) for (int ex = 0; ex < G.m.Nex; ++ex) for (int j = 0; j < np; ++j) for (int i = 0; i < np; ++i) {
      const size_t n = G.id(i, j, ex, ey); const double wJ = B.w[i] * B.w[j] * Jx * Jy;
      const double r = q[2][n];
      qb[0][n] += KEb * wJ * q[0][n] / r; qb[1][n] += KEb * wJ * q[1][n] / r;
      qb[2][n] += -KEb * wJ * (q[0][n] * q[0][n] + q[1][n] * q[1][n]) / (2.0 * r * r) + Mb * wJ;
    }
    return;
  }
  for (int ey = 0; ey < G.m.Ney; ++ey) for (int ex = 0; ex < G.m.Nex; ++ex) for (int j = 0; j < np; ++j) for (int i = 0; i < np; ++i) {
    const size_t n = G.id(i, j, ex, ey);
    const double c = B.w[i] * B.w[j] * Jx * Jy;
    const double x = node_x(B, G.m, i, ex), y = node_y(B, G.m, j, ey);
    const double mx = q[0][n], my = q[1][n], r = q[2][n], E = q[3][n];
    switch (obj) {
      case OBJ_L2_DENSITY: qb[2][n] += 2.0 * c * r; break;
      case OBJ_L2_PRESSURE: {
        const double K = (mx * mx + my * my) / (2.0 * r), P = (g - 1.0) * (E - K);
        const double Pb = 2.0 * c * P, Kb = -Pb * (g - 1.0);
        gb += Pb * (E - K); qb[3][n] += Pb * (g - 1.0);
        qb[0][n] += Kb * mx / r; qb[1][n] += Kb * my / r; qb[2][n] += -Kb * K / r; break;
      }
      case OBJ_WINDOWED_KE: {
        const double wx = std::exp(-((x - KE_XC) * (x - KE_XC) + (y - KE_YC) * (y - KE_YC)) / (KE_SIG * KE_SIG));
        qb[0][n] += c * wx * mx / r; qb[1][n] += c * wx * my / r;
        qb[2][n] += -c * wx * (mx * mx + my * my) / (2.0 * r * r); break;
      }
      case OBJ_WEIGHTED_MOMENTUM:
        qb[0][n] += c * std::sin(2 * pi * x / G.m.Lx) * std::sin(2 * pi * y / G.m.Ly); break;
      case OBJ_WINDOW_RHO2: qb[2][n] += 2.0 * c * r * window_indicator(x, y, prm); break;
      default: throw std::invalid_argument("Unknown objective");
    }
  }
}

// enzyme_adjoint_ic equivalent: J and dJ/dq0 (+ dJ/dgamma, dJ/dalpha).
// Stores every step state (q, Sigma) and recomputes each step with a tape.
inline double adjoint_ic(const Grid2D& G, int obj, const double* prm, const double* const q0[4], int n_steps, double dt,
                         double g, double alpha, int n_iter, int solver, double* const dq0[4], double* dgamma, double* dalpha) {
  const size_t N = G.N;
  std::vector<std::vector<double>> qs((size_t)(n_steps + 1) * 4), Ss(n_steps + 1);
  std::vector<double> q[4], Sig(N, 0.0);
  for (int v = 0; v < 4; ++v) q[v].assign(q0[v], q0[v] + N);
  double* qp[4] = {q[0].data(), q[1].data(), q[2].data(), q[3].data()};
  Work2D<double> W; W.alloc(N);
  for (int s = 0; s < n_steps; ++s) {
    for (int v = 0; v < 4; ++v) qs[(size_t)s * 4 + v] = q[v];
    Ss[s] = Sig;
    rk3_step(G, qp, Sig.data(), g, alpha, dt, n_iter, solver, W);
  }
  const double* qc[4] = {q[0].data(), q[1].data(), q[2].data(), q[3].data()};
  const double J = objective2d(G, obj, qc, g, prm);
  std::vector<double> qbv[4], Sb(N, 0.0);
  for (int v = 0; v < 4; ++v) qbv[v].assign(N, 0.0);
  double* qb[4] = {qbv[0].data(), qbv[1].data(), qbv[2].data(), qbv[3].data()};
  double gb = 0.0, ab = 0.0;
  objective2d_grad(G, obj, qc, g, prm, qb, gb);
  StepTape tape;
  for (int s = n_steps - 1; s >= 0; --s) {
    for (int v = 0; v < 4; ++v) q[v] = qs[(size_t)s * 4 + v];
    Sig = Ss[s];
    step_forward_tape(G, tape, qp, Sig.data(), g, alpha, dt, n_iter, solver);
    step_reverse(G, tape, qb, Sb.data(), g, alpha, dt, n_iter, solver, gb, ab);
  }
  for (int v = 0; v < 4; ++v) for (size_t k = 0; k < N; ++k) dq0[v][k] = qb[v][k];
  if (dgamma) *dgamma = gb;
  if (dalpha) *dalpha = ab;
  return J;
}

}  // namespace igr
