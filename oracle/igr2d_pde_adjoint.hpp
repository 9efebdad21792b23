// ORACLE — test infrastructure only (see igr_common.hpp for the parity status).
// Continuous (optimise-then-discretise) adjoint of the 2D IGR-Euler system,
// conservative Pi formulation: run_forward_store (IGR_adjoints_2d/forward.jl:
// 111-158) and IGR_adjoints_2d/adjoint_pde.jl:41-611, restated expression by
// expression (left-to-right evaluation, no FMA contraction).
//
// Reversing time (tau = T - t) the adjoint q_dag = (a_mux, a_muy, a_rho, a_E)
// obeys  d_tau q_dag = +div F_dag_loc(q, q_dag) - S_loc + S_Sigma,  with the
// nonlocal source S_Sigma from one SIP solve for Pi per RK stage (the same
// operator A(rho, alpha) as the forward Sigma solve, warm-started from the
// previous stage's Pi).
//
// Parity pin: the reference's own test of this path
// (IGR_adjoints_2d/tests/run_adjoint_test.jl:15-99) compares the PDE adjoint
// with the discrete (Enzyme) gradient divided by the nodal mass, combined
// relative L2 < 0.2, and checks that the gap does not grow under refinement;
// tests/test_oracle.py runs the same comparison against this oracle's
// hand-written discrete reverse (itself pinned to forward-mode duals).
#pragma once
#include "igr2d.hpp"

namespace igr {

// adjoint_flux_local_x (dir 0) / adjoint_flux_local_y (dir 1), adjoint_pde.jl:41-80:
// the transposed flux Jacobian applied to the adjoint, Sigma frozen.
inline void pde_adjoint_flux(int dir, double g, double mx, double my, double r, double E, double S, const double a[4],
                             double f[4]) {
  const double ux = mx / r, uy = my / r;
  const double P = pressure2d(g, mx, my, r, E);
  const double Hb = E + P + S;
  const double Pmx = -(g - 1) * ux;
  const double Pmy = -(g - 1) * uy;
  const double Pr = (g - 1) * (ux * ux + uy * uy) / 2;
  const double PE = g - 1;
  const double amu = a[0] * mx + a[1] * my;
  if (dir == 0) {
    f[0] = amu / r + a[0] * ux + Pmx * a[0] + a[2] + a[3] * (Hb / r) + a[3] * Pmx * mx / r;
    f[1] = a[1] * ux + Pmy * a[0] + a[3] * Pmy * mx / r;
    f[2] = -ux * amu / r + Pr * a[0] + a[3] * mx * (Pr / r - Hb / (r * r));
    f[3] = PE * a[0] + a[3] * (1 + PE) * ux;
  } else {
    f[0] = a[0] * uy + Pmx * a[1] + a[3] * Pmx * my / r;
    f[1] = amu / r + a[1] * uy + Pmy * a[1] + a[2] + a[3] * (Hb / r) + a[3] * Pmy * my / r;
    f[2] = -uy * amu / r + Pr * a[1] + a[3] * my * (Pr / r - Hb / (r * r));
    f[3] = PE * a[1] + a[3] * (1 + PE) * uy;
  }
}

// adjoint_llf_flux_x / _y, adjoint_pde.jl:89-128: primal LLF wave speed, the
// dissipation with the opposite sign of the forward flux.
inline void pde_adjoint_llf(int dir, double g, const double qL[5], const double qR[5], const double aL[4],
                            const double aR[4], double fs[4]) {
  const double lam = dir == 0 ? jmax(wavespeed_x(g, qL[0], qL[1], qL[2], qL[3]), wavespeed_x(g, qR[0], qR[1], qR[2], qR[3]))
                              : jmax(wavespeed_y(g, qL[0], qL[1], qL[2], qL[3]), wavespeed_y(g, qR[0], qR[1], qR[2], qR[3]));
  double fL[4], fR[4];
  pde_adjoint_flux(dir, g, qL[0], qL[1], qL[2], qL[3], qL[4], aL, fL);
  pde_adjoint_flux(dir, g, qR[0], qR[1], qR[2], qR[3], qR[4], aR, fR);
  for (int v = 0; v < 4; ++v) fs[v] = (fL[v] + fR[v]) / 2 - lam * (aL[v] - aR[v]) / 2;
}

// Reference derivatives of field f at node (i, j) of element (ex, ey):
// dx = sum_k D[i,k] f[k,j], dy = sum_k D[j,k] f[i,k] (unscaled).
inline void ref_grad(const Grid2D& G, const double* f, int i, int j, int ex, int ey, double* dx, double* dy) {
  double sx = 0.0, sy = 0.0;
  for (int k = 0; k < G.np; ++k) {
    sx += G.b.Dik(i, k) * f[G.id(k, j, ex, ey)];
    sy += G.b.Dik(j, k) * f[G.id(i, k, ex, ey)];
  }
  *dx = sx; *dy = sy;
}

// compute_adjoint_source_local!, adjoint_pde.jl:138-217.
inline void pde_source_local(const Grid2D& G, double g, const double* const q[4], const double* Sig,
                             const double* const a[4], double* const Sv[4]) {
  const int np = G.np;
  const double invJx = 1 / G.m.Jx, invJy = 1 / G.m.Jy;
  const double gm = g - 1;
  for (int ey = 0; ey < G.m.Ney; ++ey) for (int ex = 0; ex < G.m.Nex; ++ex)
    for (int j = 0; j < np; ++j) for (int i = 0; i < np; ++i) {
      double mxx, mxy, myx, myy, rx, ry, Ex, Ey, Sx, Sy;
      ref_grad(G, q[0], i, j, ex, ey, &mxx, &mxy);
      ref_grad(G, q[1], i, j, ex, ey, &myx, &myy);
      ref_grad(G, q[2], i, j, ex, ey, &rx, &ry);
      ref_grad(G, q[3], i, j, ex, ey, &Ex, &Ey);
      ref_grad(G, Sig, i, j, ex, ey, &Sx, &Sy);
      mxx *= invJx; myx *= invJx; rx *= invJx; Ex *= invJx; Sx *= invJx;
      mxy *= invJy; myy *= invJy; ry *= invJy; Ey *= invJy; Sy *= invJy;
      const size_t n = G.id(i, j, ex, ey);
      const double r = q[2][n], mx = q[0][n], my = q[1][n], en = q[3][n];
      const double ux = mx / r, uy = my / r;
      // The reference also forms the cross gradients d_y u_x and d_x u_y here;
      // no source term uses them.
      const double uxx = (mxx - ux * rx) / r;
      const double uyy = (myy - uy * ry) / r;
      const double P = gm * (en - (mx * mx + my * my) / (2 * r));
      const double Hb = en + P + Sig[n];
      const double Pr = gm * (ux * ux + uy * uy) / 2;
      const double Pbx = gm * (Ex - (mx * mxx + my * myx) / r + (mx * mx + my * my) * rx / (2 * (r * r))) + Sx;
      const double Pby = gm * (Ey - (mx * mxy + my * myy) / r + (mx * mx + my * my) * ry / (2 * (r * r))) + Sy;
      const double dPx_dmx = gm * (-mxx / r + mx * rx / (r * r));
      const double dPx_dmy = gm * (-myx / r + my * rx / (r * r));
      const double dPx_dr = gm * ((mx * mxx + my * myx) / (r * r) - (mx * mx + my * my) * rx / (r * r * r));
      const double dPy_dmx = gm * (-mxy / r + mx * ry / (r * r));
      const double dPy_dmy = gm * (-myy / r + my * ry / (r * r));
      const double dPy_dr = gm * ((mx * mxy + my * myy) / (r * r) - (mx * mx + my * my) * ry / (r * r * r));
      const double HEx = Ex + Pbx, HEy = Ey + Pby;
      const double dmx_mx = mxx / r + uxx - mx * rx / (r * r) + dPx_dmx + uyy;
      const double dmx_my = dPx_dmy + mxy / r - mx * ry / (r * r);
      const double dmx_r = mxx * (-ux / r) + mx * (ux * rx / (r * r) - uxx / r) + dPx_dr + mxy * (-uy / r) +
                           mx * (uy * ry / (r * r) - uyy / r);
      const double dmy_mx = myx / r - my * rx / (r * r) + dPy_dmx;
      const double dmy_my = uxx + myy / r + uyy - my * ry / (r * r) + dPy_dmy;
      const double dmy_r = myx * (-ux / r) + my * (ux * rx / (r * r) - uxx / r) + myy * (-uy / r) +
                           my * (uy * ry / (r * r) - uyy / r) + dPy_dr;
      const double dE_mx = dPx_dmx * ux + HEx / r + (-gm * ux) * uxx + Hb * (-rx / (r * r)) + dPy_dmx * uy + (-gm * ux) * uyy;
      const double dE_my = dPx_dmy * ux + (-gm * uy) * uxx + dPy_dmy * uy + HEy / r + (-gm * uy) * uyy + Hb * (-ry / (r * r));
      const double dE_r = dPx_dr * ux + HEx * (-ux / r) + Pr * uxx + Hb * (ux * rx / (r * r) - uxx / r) + dPy_dr * uy +
                          HEy * (-uy / r) + Pr * uyy + Hb * (uy * ry / (r * r) - uyy / r);
      const double dE_E = g * (uxx + uyy);
      const double axx = a[0][n], ayy = a[1][n], aEE = a[3][n];
      Sv[0][n] = axx * dmx_mx + ayy * dmy_mx + aEE * dE_mx;
      Sv[1][n] = axx * dmx_my + ayy * dmy_my + aEE * dE_my;
      Sv[2][n] = axx * dmx_r + ayy * dmy_r + aEE * dE_r;
      Sv[3][n] = aEE * dE_E;
    }
}

// compute_adjoint_hyperbolic_rhs_local!, adjoint_pde.jl:231-325: +div F_dag
// (volume), adjoint LLF faces with flipped signs, minus the local source.
inline void pde_hyperbolic_rhs_local(const Grid2D& G, double g, const double* const q[4], const double* Sig,
                                     const double* const a[4], double* const da[4]) {
  const int np = G.np, Nex = G.m.Nex, Ney = G.m.Ney, L = np - 1;
  const Basis& B = G.b;
  const double invJx = 1 / G.m.Jx, invJy = 1 / G.m.Jy;
  std::vector<double> F[8];
  for (int v = 0; v < 8; ++v) F[v].resize(G.N);
  for (size_t n = 0; n < G.N; ++n) {
    const double an[4] = {a[0][n], a[1][n], a[2][n], a[3][n]};
    double fx[4], fy[4];
    pde_adjoint_flux(0, g, q[0][n], q[1][n], q[2][n], q[3][n], Sig[n], an, fx);
    pde_adjoint_flux(1, g, q[0][n], q[1][n], q[2][n], q[3][n], Sig[n], an, fy);
    for (int v = 0; v < 4; ++v) { F[v][n] = fx[v]; F[4 + v][n] = fy[v]; }
  }
  for (int ey = 0; ey < Ney; ++ey) for (int ex = 0; ex < Nex; ++ex)
    for (int j = 0; j < np; ++j) for (int i = 0; i < np; ++i) {
      double acc[4] = {0.0, 0.0, 0.0, 0.0};
      for (int k = 0; k < np; ++k) {
        const size_t nx = G.id(k, j, ex, ey), ny = G.id(i, k, ex, ey);
        for (int v = 0; v < 4; ++v) acc[v] += invJx * B.Dik(i, k) * F[v][nx] + invJy * B.Dik(j, k) * F[4 + v][ny];
      }
      const size_t n = G.id(i, j, ex, ey);
      for (int v = 0; v < 4; ++v) da[v][n] = acc[v];
    }
  for (int ey = 0; ey < Ney; ++ey) for (int ex = 0; ex < Nex; ++ex) {
    const int exR = ex == Nex - 1 ? 0 : ex + 1;
    for (int j = 0; j < np; ++j) {
      const size_t nl = G.id(L, j, ex, ey), nr = G.id(0, j, exR, ey);
      const double qL[5] = {q[0][nl], q[1][nl], q[2][nl], q[3][nl], Sig[nl]};
      const double qR[5] = {q[0][nr], q[1][nr], q[2][nr], q[3][nr], Sig[nr]};
      const double aL[4] = {a[0][nl], a[1][nl], a[2][nl], a[3][nl]};
      const double aR[4] = {a[0][nr], a[1][nr], a[2][nr], a[3][nr]};
      double fs[4];
      pde_adjoint_llf(0, g, qL, qR, aL, aR, fs);
      for (int v = 0; v < 4; ++v) da[v][nl] += invJx * (fs[v] - F[v][nl]) / B.w[L];
      for (int v = 0; v < 4; ++v) da[v][nr] -= invJx * (fs[v] - F[v][nr]) / B.w[0];
    }
  }
  for (int ey = 0; ey < Ney; ++ey) for (int ex = 0; ex < Nex; ++ex) {
    const int eyR = ey == Ney - 1 ? 0 : ey + 1;
    for (int i = 0; i < np; ++i) {
      const size_t nl = G.id(i, L, ex, ey), nr = G.id(i, 0, ex, eyR);
      const double qL[5] = {q[0][nl], q[1][nl], q[2][nl], q[3][nl], Sig[nl]};
      const double qR[5] = {q[0][nr], q[1][nr], q[2][nr], q[3][nr], Sig[nr]};
      const double aL[4] = {a[0][nl], a[1][nl], a[2][nl], a[3][nl]};
      const double aR[4] = {a[0][nr], a[1][nr], a[2][nr], a[3][nr]};
      double fs[4];
      pde_adjoint_llf(1, g, qL, qR, aL, aR, fs);
      for (int v = 0; v < 4; ++v) da[v][nl] += invJy * (fs[v] - F[4 + v][nl]) / B.w[L];
      for (int v = 0; v < 4; ++v) da[v][nr] -= invJy * (fs[v] - F[4 + v][nr]) / B.w[0];
    }
  }
  std::vector<double> Sb[4];
  for (int v = 0; v < 4; ++v) Sb[v].resize(G.N);
  double* Sv[4] = {Sb[0].data(), Sb[1].data(), Sb[2].data(), Sb[3].data()};
  pde_source_local(G, g, q, Sig, a, Sv);
  for (int v = 0; v < 4; ++v) for (size_t n = 0; n < G.N; ++n) da[v][n] -= Sv[v][n];
}

// compute_adjoint_elliptic_rhs!, adjoint_pde.jl:337-364: div(a_mu) + grad(a_E) . u
inline void pde_elliptic_rhs(const Grid2D& G, double* b, const double* const a[4], const double* const q[4]) {
  const int np = G.np;
  const double invJx = 1 / G.m.Jx, invJy = 1 / G.m.Jy;
  for (int ey = 0; ey < G.m.Ney; ++ey) for (int ex = 0; ex < G.m.Nex; ++ex)
    for (int j = 0; j < np; ++j) for (int i = 0; i < np; ++i) {
      double amx_x = 0.0, amy_y = 0.0, aE_x = 0.0, aE_y = 0.0;
      for (int k = 0; k < np; ++k) {
        amx_x += G.b.Dik(i, k) * a[0][G.id(k, j, ex, ey)];
        amy_y += G.b.Dik(j, k) * a[1][G.id(i, k, ex, ey)];
        aE_x += G.b.Dik(i, k) * a[3][G.id(k, j, ex, ey)];
        aE_y += G.b.Dik(j, k) * a[3][G.id(i, k, ex, ey)];
      }
      amx_x *= invJx; aE_x *= invJx;
      amy_y *= invJy; aE_y *= invJy;
      const size_t n = G.id(i, j, ex, ey);
      const double ux = q[0][n] / q[2][n], uy = q[1][n] / q[2][n];
      b[n] = amx_x + amy_y + aE_x * ux + aE_y * uy;
    }
}

// compute_nonlocal_source!, adjoint_pde.jl:381-466 (d = 2):
//   W = grad(Pi div u) + div(Pi [Du]^T),  S_mu = -2 W / rho,
//   S_rho = [Pi R_tr + div(Pi grad(Sigma) / rho)] / rho + 2 (W . mu) / rho^2,  S_E = 0,
// with the velocity gradients taken of the nodal u = mu / rho.
inline void pde_nonlocal_source(const Grid2D& G, const double* Pi, const double* const q[4], const double* Sig,
                                double* const Sv[4]) {
  const int np = G.np;
  const size_t N = G.N;
  const double invJx = 1 / G.m.Jx, invJy = 1 / G.m.Jy;
  std::vector<double> ux(N), uy(N), Pdivu(N), Pxx(N), Pyx(N), Pxy(N), Pyy(N), Cx(N), Cy(N), Rtr(N);
  for (size_t n = 0; n < N; ++n) { ux[n] = q[0][n] / q[2][n]; uy[n] = q[1][n] / q[2][n]; }
  for (int ey = 0; ey < G.m.Ney; ++ey) for (int ex = 0; ex < G.m.Nex; ++ex)
    for (int j = 0; j < np; ++j) for (int i = 0; i < np; ++i) {
      double uxx = 0.0, uxy = 0.0, uyx = 0.0, uyy = 0.0, Sx = 0.0, Sy = 0.0;
      for (int k = 0; k < np; ++k) {
        const size_t kx = G.id(k, j, ex, ey), ky = G.id(i, k, ex, ey);
        uxx += G.b.Dik(i, k) * ux[kx]; uyx += G.b.Dik(i, k) * uy[kx];
        uxy += G.b.Dik(j, k) * ux[ky]; uyy += G.b.Dik(j, k) * uy[ky];
        Sx += G.b.Dik(i, k) * Sig[kx]; Sy += G.b.Dik(j, k) * Sig[ky];
      }
      uxx *= invJx; uyx *= invJx; Sx *= invJx;
      uxy *= invJy; uyy *= invJy; Sy *= invJy;
      const double divu = uxx + uyy;
      const size_t n = G.id(i, j, ex, ey);
      const double r = q[2][n], P = Pi[n];
      Pdivu[n] = P * divu;
      Pxx[n] = P * uxx; Pyx[n] = P * uyx;
      Pxy[n] = P * uxy; Pyy[n] = P * uyy;
      Cx[n] = P * Sx / r; Cy[n] = P * Sy / r;
      Rtr[n] = divu * divu + uxx * uxx + 2 * uxy * uyx + uyy * uyy;
    }
  for (int ey = 0; ey < G.m.Ney; ++ey) for (int ex = 0; ex < G.m.Nex; ++ex)
    for (int j = 0; j < np; ++j) for (int i = 0; i < np; ++i) {
      double dxPd = 0.0, dyPd = 0.0, dxPxx = 0.0, dyPyx = 0.0, dxPxy = 0.0, dyPyy = 0.0, dxCx = 0.0, dyCy = 0.0;
      for (int k = 0; k < np; ++k) {
        const size_t kx = G.id(k, j, ex, ey), ky = G.id(i, k, ex, ey);
        dxPd += G.b.Dik(i, k) * Pdivu[kx];
        dyPd += G.b.Dik(j, k) * Pdivu[ky];
        dxPxx += G.b.Dik(i, k) * Pxx[kx];
        dyPyx += G.b.Dik(j, k) * Pyx[ky];
        dxPxy += G.b.Dik(i, k) * Pxy[kx];
        dyPyy += G.b.Dik(j, k) * Pyy[ky];
        dxCx += G.b.Dik(i, k) * Cx[kx];
        dyCy += G.b.Dik(j, k) * Cy[ky];
      }
      dxPd *= invJx; dyPd *= invJy;
      dxPxx *= invJx; dyPyx *= invJy;
      dxPxy *= invJx; dyPyy *= invJy;
      dxCx *= invJx; dyCy *= invJy;
      const double Wx = dxPd + dxPxx + dyPyx;
      const double Wy = dyPd + dxPxy + dyPyy;
      const double divC = dxCx + dyCy;
      const size_t n = G.id(i, j, ex, ey);
      const double r = q[2][n], mx = q[0][n], my = q[1][n];
      Sv[0][n] = -2 * Wx / r;
      Sv[1][n] = -2 * Wy / r;
      Sv[2][n] = (Pi[n] * Rtr[n] + divC) / r + 2 * (Wx * mx + Wy * my) / (r * r);
      Sv[3][n] = 0.0;
    }
}

// compute_adjoint_rhs_conservative!, adjoint_pde.jl:481-516. Pi is the warm
// start, in-out. Unknown solver symbols skip the solve, as the reference's
// if/elseif chain does.
inline void pde_adjoint_rhs(const Grid2D& G, double g, double alpha, int n_iter, int solver, const double* const q[4],
                            const double* Sig, double* Pi, const double* const a[4], double* const da[4], Work2D<double>& W) {
  pde_hyperbolic_rhs_local(G, g, q, Sig, a, da);
  if (alpha > 0) {
    const int np = G.np;
    double* b = W.b.data();
    pde_elliptic_rhs(G, b, a, q);
    for (int ey = 0; ey < G.m.Ney; ++ey) for (int ex = 0; ex < G.m.Nex; ++ex)
      for (int j = 0; j < np; ++j) for (int i = 0; i < np; ++i)
        b[G.id(i, j, ex, ey)] *= alpha * G.b.w[i] * G.b.w[j] * G.m.Jx * G.m.Jy;
    sip_diagonal(G, W.M.data(), q[2], alpha);
    if (solver == SOLVER_PCG) pcg_fixed(G, Pi, b, W.M.data(), n_iter, q[2], alpha, W);
    else if (solver == SOLVER_JACOBI) jacobi_fixed(G, Pi, b, W.M.data(), n_iter, q[2], alpha, 2.0 / 3.0, W);
    else if (solver == SOLVER_CHEBYSHEV) chebyshev_fixed(G, Pi, b, W.M.data(), n_iter, q[2], alpha, W);
    std::vector<double> Sb[4];
    for (int v = 0; v < 4; ++v) Sb[v].resize(G.N);
    double* Sv[4] = {Sb[0].data(), Sb[1].data(), Sb[2].data(), Sb[3].data()};
    pde_nonlocal_source(G, Pi, q, Sig, Sv);
    for (int v = 0; v < 4; ++v) for (size_t n = 0; n < G.N; ++n) da[v][n] += Sv[v][n];
  }
}

// run_forward_store, forward.jl:111-158: snapshot k (k = 0..n_steps) holds
// (mux, muy, rho, E, Sigma) after step k; Sigma is solved once more after
// every step (and once at t = 0) and carries on as the next step's warm start.
// snaps: (n_steps + 1) * 5 * N doubles, snapshot-major. Returns n_steps.
inline int run_forward_store(const Grid2D& G, const double* const q0[4], double dt, double T_end, double g, double alpha,
                             int n_iter, int solver, std::vector<double>& snaps) {
  const size_t N = G.N;
  std::vector<double> qv[4], Sig(N, 0.0);
  for (int v = 0; v < 4; ++v) qv[v].assign(q0[v], q0[v] + N);
  double* q[4] = {qv[0].data(), qv[1].data(), qv[2].data(), qv[3].data()};
  const double* qc[4] = {q[0], q[1], q[2], q[3]};
  Work2D<double> W; W.alloc(N);
  if (solver != SOLVER_PCG && solver != SOLVER_JACOBI && solver != SOLVER_CHEBYSHEV && alpha > 0)
    throw std::invalid_argument("Unknown solver (use :pcg, :jacobi, or :chebyshev)");
  if (alpha > 0) solve_elliptic(G, Sig.data(), qc, alpha, n_iter, solver, W);
  double dtr;
  const int n_steps = rerounded_steps(dt, T_end, &dtr);
  snaps.assign((size_t)(n_steps + 1) * 5 * N, 0.0);
  auto push = [&](int k) {
    double* s = snaps.data() + (size_t)k * 5 * N;
    for (int v = 0; v < 4; ++v) std::copy(q[v], q[v] + N, s + v * N);
    std::copy(Sig.begin(), Sig.end(), s + 4 * N);
  };
  push(0);
  for (int s = 0; s < n_steps; ++s) {
    rk3_step(G, q, Sig.data(), g, alpha, dtr, n_iter, solver, W);
    if (alpha > 0) solve_elliptic(G, Sig.data(), qc, alpha, n_iter, solver, W);
    push(s + 1);
  }
  return n_steps;
}

// Terminal condition of run_adjoint_conservative (adjoint_pde.jl:542-584): the
// L2 gradient density of J at t = T. OBJ_WINDOW_RHO2 (nodal square window,
// a[rho] = 2 rho chi) extends the reference's list; other objectives raise.
inline void pde_terminal(const Grid2D& G, int obj, const double* const q[4], double g, const double* prm,
                         double* const a[4]) {
  const size_t N = G.N;
  const int np = G.np;
  const double pi = 3.14159265358979323846;
  for (int v = 0; v < 4; ++v) std::fill(a[v], a[v] + N, 0.0);
  if (obj == OBJ_KINETIC_ENERGY) {
    double KE = 0.0, Ms = 0.0;
    for (int ey = 0; ey < G.m.Ney; ++ey) for (int ex = 0; ex < G.m.Nex; ++ex)
      for (int j = 0; j < np; ++j) for (int i = 0; i < np; ++i) {
        const size_t n = G.id(i, j, ex, ey);
        const double wJ = G.b.w[i] * G.b.w[j] * G.m.Jx * G.m.Jy;
        KE += wJ * (q[0][n] * q[0][n] + q[1][n] * q[1][n]) / (2 * q[2][n]);
        Ms += wJ * q[2][n];
      }
    for (size_t n = 0; n < N; ++n) {
      const double ux = q[0][n] / q[2][n], uy = q[1][n] / q[2][n];
      a[0][n] = ux / Ms;
      a[1][n] = uy / Ms;
      a[2][n] = -(q[0][n] * q[0][n] + q[1][n] * q[1][n]) / (2 * (q[2][n] * q[2][n])) / Ms - KE / (Ms * Ms);
    }
    return;
  }
  for (int ey = 0; ey < G.m.Ney; ++ey) for (int ex = 0; ex < G.m.Nex; ++ex)
    for (int j = 0; j < np; ++j) for (int i = 0; i < np; ++i) {
      const size_t n = G.id(i, j, ex, ey);
      const double x = node_x(G.b, G.m, i, ex), y = node_y(G.b, G.m, j, ey);
      const double mx = q[0][n], my = q[1][n], r = q[2][n], E = q[3][n];
      switch (obj) {
        case OBJ_L2_DENSITY: a[2][n] = 2 * r; break;
        case OBJ_L2_PRESSURE: {
          const double P = (g - 1) * (E - (mx * mx + my * my) / (2 * r));
          const double ux = mx / r, uy = my / r;
          a[0][n] = -2 * (g - 1) * P * ux;
          a[1][n] = -2 * (g - 1) * P * uy;
          a[2][n] = (g - 1) * P * (ux * ux + uy * uy);
          a[3][n] = 2 * (g - 1) * P;
          break;
        }
        case OBJ_WEIGHTED_MOMENTUM: a[0][n] = std::sin(2 * pi * x / G.m.Lx) * std::sin(2 * pi * y / G.m.Ly); break;
        case OBJ_WINDOWED_KE: {
          const double w = std::exp(-((x - KE_XC) * (x - KE_XC) + (y - KE_YC) * (y - KE_YC)) / (KE_SIG * KE_SIG));
          const double ux = mx / r, uy = my / r;
          a[0][n] = w * ux;
          a[1][n] = w * uy;
          a[2][n] = -w * (ux * ux + uy * uy) / 2;
          break;
        }
        case OBJ_WINDOW_RHO2: a[2][n] = 2 * r * window_indicator(x, y, prm); break;
        default: throw std::invalid_argument("Unknown objective");
      }
    }
}

// run_adjoint_conservative, adjoint_pde.jl:527-611: backward SSP-RK3 over the
// stored snapshots, step n using snapshot n (the state after forward step n)
// for all three stages, dt = min(dt, T), Pi warm-started from zero and carried
// across stages and steps. a_out: the adjoint at t = 0.
inline void run_adjoint_conservative(const Grid2D& G, const double* snaps, int n_steps, double dt, double T_end,
                                     double g, double alpha, int n_iter, int objective, int solver, const double* prm,
                                     double* const a_out[4]) {
  const size_t N = G.N;
  const double* qT[4];
  for (int v = 0; v < 4; ++v) qT[v] = snaps + (size_t)n_steps * 5 * N + v * N;
  std::vector<double> av[4], a1v[4], a2v[4], dav[4], Pi(N, 0.0);
  for (int v = 0; v < 4; ++v) { av[v].resize(N); a1v[v].resize(N); a2v[v].resize(N); dav[v].resize(N); }
  double* a[4] = {av[0].data(), av[1].data(), av[2].data(), av[3].data()};
  double* a1[4] = {a1v[0].data(), a1v[1].data(), a1v[2].data(), a1v[3].data()};
  double* a2[4] = {a2v[0].data(), a2v[1].data(), a2v[2].data(), a2v[3].data()};
  double* da[4] = {dav[0].data(), dav[1].data(), dav[2].data(), dav[3].data()};
  pde_terminal(G, objective, qT, g, prm, a);
  Work2D<double> W; W.alloc(N);
  const double h = std::min(dt, T_end);
  for (int n = n_steps; n >= 1; --n) {
    const double* s = snaps + (size_t)n * 5 * N;
    const double* q[4] = {s, s + N, s + 2 * N, s + 3 * N};
    const double* Sig = s + 4 * N;
    const double* ac[4] = {a[0], a[1], a[2], a[3]};
    pde_adjoint_rhs(G, g, alpha, n_iter, solver, q, Sig, Pi.data(), ac, da, W);
    for (int v = 0; v < 4; ++v) for (size_t k = 0; k < N; ++k) a1[v][k] = a[v][k] + h * da[v][k];
    const double* a1c[4] = {a1[0], a1[1], a1[2], a1[3]};
    pde_adjoint_rhs(G, g, alpha, n_iter, solver, q, Sig, Pi.data(), a1c, da, W);
    for (int v = 0; v < 4; ++v) for (size_t k = 0; k < N; ++k)
      a2[v][k] = 3.0 / 4 * a[v][k] + 1.0 / 4 * a1[v][k] + 1.0 / 4 * h * da[v][k];
    const double* a2c[4] = {a2[0], a2[1], a2[2], a2[3]};
    pde_adjoint_rhs(G, g, alpha, n_iter, solver, q, Sig, Pi.data(), a2c, da, W);
    for (int v = 0; v < 4; ++v) for (size_t k = 0; k < N; ++k)
      a[v][k] = 1.0 / 3 * a[v][k] + 2.0 / 3 * a2[v][k] + 2.0 / 3 * h * da[v][k];
  }
  for (int v = 0; v < 4; ++v) std::copy(a[v], a[v] + N, a_out[v]);
}

}  // namespace igr
