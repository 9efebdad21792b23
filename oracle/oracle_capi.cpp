// ORACLE — test infrastructure only (see igr_common.hpp for the parity status).
// extern "C" entry points over the CPU restatement, loaded with ctypes by the
// tests and by the CPU-baseline leg of bench.py. Arrays use the reference's
// Julia column-major layout. Every function returns 0 on success, 1 on a bad
// argument (unknown solver/objective), 2 on any other exception.
#include <cstring>
#include <exception>
#include <string>

#include "igr1d.hpp"
#include "igr2d_adjoint.hpp"
#include "igr2d_pde_adjoint.hpp"
#include "igr1d_pde_adjoint.hpp"
#include "igr_ic.hpp"
#include "opcount.hpp"

using namespace igr;

namespace {
thread_local std::string g_err;
Grid2D make_grid(int p, const double* xi, const double* w, const double* Dcol, int Nex, int Ney, double Lx, double Ly) {
  Basis b = (xi && w && Dcol) ? basis_from_arrays(p, xi, w, Dcol) : make_basis(p);
  return Grid2D(b, make_mesh2d(Nex, Ney, Lx, Ly));
}
template <class F> int guard(F&& f) {
  try { f(); return 0; }
  catch (const std::invalid_argument& e) { g_err = e.what(); return 1; }
  catch (const std::exception& e) { g_err = e.what(); return 2; }
}
}  // namespace

#define GRID2D_ARGS int p, const double *xi, const double *w, const double *Dcol, int Nex, int Ney, double Lx, double Ly
#define GRID2D make_grid(p, xi, w, Dcol, Nex, Ney, Lx, Ly)

extern "C" {

const char* orc_last_error() { return g_err.c_str(); }

// Inner-product summation order of the solvers: 0 sequential (default), 1 reversed, 2 pairwise.
int orc_set_dot_order(int order) {
  if (order < 0 || order > 2) return 1;
  dot_order() = order;
  return 0;
}

// Algorithmic FP64 operations per node of the restated 2D arithmetic (opcount.hpp), on
// a smooth state of the given grid: out[2k] forward and out[2k+1] reverse-mode
// counts of family k = 0 stage setup (compute_igr_rhs! + compute_sip_diagonal),
// 1 one apply_sip!, 2 one iteration of the solver (its marginal cost), 3 the
// solver's fixed part (n_iter = 1 minus one iteration), 4 the hyperbolic RHS
// plus the RK stage combination (per stage), 5 one SSP-RK3 step with its
// three solves of n_iter iterations, 6 objective window rho^2 (J at T).
int orc2d_opcount(GRID2D_ARGS, int solver, int n_iter, double* out) {
  return guard([&] {
    if (solver < 0 || solver > 2) throw std::invalid_argument("Unknown solver");
    if (n_iter < 2) throw std::invalid_argument("n_iter must be >= 2");
    Grid2D G = GRID2D;
    const size_t N = G.N;
    std::vector<Ops> qv[4], S(N), b(N), M(N), x(N), y(N);
    for (int v = 0; v < 4; ++v) qv[v].resize(N);
    for (int ey = 0; ey < G.m.Ney; ++ey) for (int ex = 0; ex < G.m.Nex; ++ex)
      for (int j = 0; j < G.np; ++j) for (int i = 0; i < G.np; ++i) {
        const size_t n = G.id(i, j, ex, ey);
        const double X = node_x(G.b, G.m, i, ex), Y = node_y(G.b, G.m, j, ey);
        const double r = 1.0 + 0.2 * std::sin(6.283185307179586 * X) * std::cos(6.283185307179586 * Y);
        const double u = 0.1 * std::sin(6.283185307179586 * Y), w = 0.1 * std::cos(6.283185307179586 * X);
        qv[0][n] = r * u; qv[1][n] = r * w; qv[2][n] = r; qv[3][n] = 2.5 + 0.5 * r * (u * u + w * w);
        S[n] = 1e-3 * std::sin(6.283185307179586 * (X + Y)); x[n] = S[n].v;
      }
    const Ops g(1.4), alpha(3.0 / ((double)G.m.Nex * G.m.Nex));
    Work2D<Ops> W; W.alloc(N);
    auto measure = [&](auto&& f) {
      op_tally() = OpTally();
      f();
      const OpTally t = op_tally();
      return std::pair<double, double>((double)t.fwd / N, (double)t.rev / N);
    };
    auto solve = [&](int n) {
      std::vector<Ops> xx = x;
      if (solver == SOLVER_PCG) pcg_fixed(G, xx.data(), b.data(), M.data(), n, qv[2].data(), alpha, W);
      else if (solver == SOLVER_JACOBI) jacobi_fixed(G, xx.data(), b.data(), M.data(), n, qv[2].data(), alpha, 2.0 / 3.0, W);
      else chebyshev_fixed(G, xx.data(), b.data(), M.data(), n, qv[2].data(), alpha, W);
    };
    const auto setup = measure([&] {
      igr_rhs(G, b.data(), qv[0].data(), qv[1].data(), qv[2].data(), alpha);
      sip_diagonal(G, M.data(), qv[2].data(), alpha);
    });
    const auto apply = measure([&] { apply_sip(G, y.data(), x.data(), qv[2].data(), alpha); });
    const auto s1 = measure([&] { solve(1); });
    const auto s2 = measure([&] { solve(2); });
    std::vector<Ops> q0[4] = {qv[0], qv[1], qv[2], qv[3]};
    Ops* qs[4] = {q0[0].data(), q0[1].data(), q0[2].data(), q0[3].data()};
    std::vector<Ops> Sig = S;
    const auto step = measure([&] { rk3_step(G, qs, Sig.data(), g, alpha, 1e-4, n_iter, solver, W); });
    const Ops* qc[4] = {qv[0].data(), qv[1].data(), qv[2].data(), qv[3].data()};
    const double prm[4] = {0.2, 0.2, 0.5, 0.0};
    const auto obj = measure([&] { (void)objective2d(G, OBJ_WINDOW_RHO2, qc, g, prm); });
    const double it_f = s2.first - s1.first, it_r = s2.second - s1.second;
    const double sol_f = s1.first + (n_iter - 1) * it_f, sol_r = s1.second + (n_iter - 1) * it_r;
    const double vals[14] = {setup.first, setup.second, apply.first, apply.second, it_f, it_r, s1.first - it_f,
                             s1.second - it_r, (step.first - 3 * (setup.first + sol_f)) / 3,
                             (step.second - 3 * (setup.second + sol_r)) / 3, step.first, step.second, obj.first,
                             obj.second};
    for (int k = 0; k < 14; ++k) out[k] = vals[k];
  });
}

int orc_basis(int p, double* xi, double* w, double* Dcol) {
  return guard([&] {
    Basis b = make_basis(p);
    for (int i = 0; i < b.np; ++i) { xi[i] = b.xi[i]; w[i] = b.w[i]; }
    for (int i = 0; i < b.np; ++i) for (int k = 0; k < b.np; ++k) Dcol[i + (size_t)k * b.np] = b.Dik(i, k);
  });
}

int orc2d_hyperbolic_rhs(GRID2D_ARGS, double gamma, const double* mx, const double* my, const double* rho, const double* E,
                         const double* Sig, double* dmx, double* dmy, double* drho, double* dE) {
  return guard([&] {
    Grid2D G = GRID2D; const double* q[4] = {mx, my, rho, E}; double* dq[4] = {dmx, dmy, drho, dE};
    std::vector<double> F[8]; hyperbolic_rhs(G, gamma, q, Sig, dq, F);
  });
}

int orc2d_apply_sip(GRID2D_ARGS, double alpha, const double* x, const double* rho, double* y) {
  return guard([&] { Grid2D G = GRID2D; apply_sip(G, y, x, rho, alpha); });
}

int orc2d_igr_rhs(GRID2D_ARGS, double alpha, const double* mx, const double* my, const double* rho, double* b) {
  return guard([&] { Grid2D G = GRID2D; igr_rhs(G, b, mx, my, rho, alpha); });
}

int orc2d_sip_diagonal(GRID2D_ARGS, double alpha, const double* rho, double* M) {
  return guard([&] { Grid2D G = GRID2D; sip_diagonal(G, M, rho, alpha); });
}

int orc2d_solve_elliptic(GRID2D_ARGS, double alpha, int n_iter, int solver, const double* mx, const double* my,
                         const double* rho, const double* E, double* Sig) {
  return guard([&] {
    Grid2D G = GRID2D; const double* q[4] = {mx, my, rho, E};
    Work2D<double> W; W.alloc(G.N); solve_elliptic(G, Sig, q, alpha, n_iter, solver, W);
  });
}

// cg_solve! (tol exit) or cg_fixed! (fixed=1) on A x = b with A = SIP(rho, alpha).
int orc2d_cg(GRID2D_ARGS, double alpha, const double* rho, const double* b, double* x, double tol, int maxiter, int fixed, int* iters) {
  return guard([&] {
    Grid2D G = GRID2D; Work2D<double> W; W.alloc(G.N);
    *iters = cg_solve(G, x, b, rho, alpha, tol, maxiter, fixed != 0, W);
  });
}

int orc2d_igr_euler_rhs(GRID2D_ARGS, double gamma, double alpha, int n_iter, int solver, const double* mx, const double* my,
                        const double* rho, const double* E, double* Sig, double* dmx, double* dmy, double* drho, double* dE) {
  return guard([&] {
    Grid2D G = GRID2D; const double* q[4] = {mx, my, rho, E};
    Work2D<double> W; W.alloc(G.N); igr_euler_rhs(G, q, Sig, gamma, alpha, n_iter, solver, W);
    double* out[4] = {dmx, dmy, drho, dE};
    for (int v = 0; v < 4; ++v) std::memcpy(out[v], W.dq[v].data(), G.N * sizeof(double));
  });
}

int orc2d_run_forward(GRID2D_ARGS, double gamma, double alpha, double dt, double T_end, int n_iter, int solver,
                      double* mx, double* my, double* rho, double* E, double* Sig) {
  return guard([&] {
    if (solver < 0 || solver > 2) throw std::invalid_argument("Unknown solver");
    Grid2D G = GRID2D; double* q[4] = {mx, my, rho, E}; run_forward(G, q, Sig, dt, T_end, gamma, alpha, n_iter, solver);
  });
}

// Fixed-step forward (no dt re-rounding, Sigma from zero): the objective loop
// of enzyme_adjoint.jl. State in-out; Sig out (Sigma after the last stage); J out.
int orc2d_objective_run(GRID2D_ARGS, double gamma, double alpha, int n_steps, double dt, int n_iter, int solver, int obj,
                        const double* prm, double* mx, double* my, double* rho, double* E, double* J) {
  return guard([&] {
    if (solver < 0 || solver > 2) throw std::invalid_argument("Unknown solver");
    if (obj < 0 || obj > 5) throw std::invalid_argument("Unknown objective");
    Grid2D G = GRID2D; double* q[4] = {mx, my, rho, E};
    *J = objective_run(G, obj, q, n_steps, dt, gamma, alpha, n_iter, solver, prm);
  });
}

int orc2d_adjoint(GRID2D_ARGS, double gamma, double alpha, int n_steps, double dt, int n_iter, int solver, int obj,
                  const double* prm, const double* mx, const double* my, const double* rho, const double* E, double* J,
                  double* dmx, double* dmy, double* drho, double* dE, double* dgamma, double* dalpha) {
  return guard([&] {
    if (solver < 0 || solver > 2) throw std::invalid_argument("Unknown solver");
    if (obj < 0 || obj > 5) throw std::invalid_argument("Unknown objective");
    Grid2D G = GRID2D; const double* q0[4] = {mx, my, rho, E}; double* dq[4] = {dmx, dmy, drho, dE};
    *J = adjoint_ic(G, obj, prm, q0, n_steps, dt, gamma, alpha, n_iter, solver, dq, dgamma, dalpha);
  });
}

// Batched adjoint on the host: B instances sharing one mesh, each with its own
// state, gamma and alpha; OpenMP over instances (instance-major arrays).
int orc2d_adjoint_batch(GRID2D_ARGS, int B, const double* gammas, const double* alphas, int n_steps, double dt, int n_iter,
                        int solver, int obj, const double* prm, const double* q0, double* J, double* dq0, double* dgamma,
                        double* dalpha, int n_threads) {
  return guard([&] {
    if (solver < 0 || solver > 2) throw std::invalid_argument("Unknown solver");
    Grid2D G = GRID2D; const size_t N = G.N;
    std::string err;
#pragma omp parallel for schedule(dynamic, 1) num_threads(n_threads > 0 ? n_threads : 1)
    for (int b = 0; b < B; ++b) {
      try {
        const double* qi[4]; double* di[4];
        for (int v = 0; v < 4; ++v) { qi[v] = q0 + ((size_t)b * 4 + v) * N; di[v] = dq0 + ((size_t)b * 4 + v) * N; }
        J[b] = adjoint_ic(G, obj, prm, qi, n_steps, dt, gammas[b], alphas[b], n_iter, solver, di, dgamma + b, dalpha + b);
      } catch (const std::exception& e) {
#pragma omp critical
        err = e.what();
      }
    }
    if (!err.empty()) throw std::runtime_error(err);
  });
}

// Forward-mode directional derivative of the objective loop: seeds v (4 fields),
// vg (gamma) and va (alpha); returns J and dJ = <grad, (v, vg, va)>.
int orc2d_objective_dual(GRID2D_ARGS, double gamma, double alpha, int n_steps, double dt, int n_iter, int solver, int obj,
                         const double* prm, const double* mx, const double* my, const double* rho, const double* E,
                         const double* vmx, const double* vmy, const double* vrho, const double* vE, double vg, double va,
                         double* J, double* dJ) {
  return guard([&] {
    typedef Dual<1> D1;
    Grid2D G = GRID2D; const size_t N = G.N;
    std::vector<D1> q[4];
    const double* src[4] = {mx, my, rho, E}; const double* dir[4] = {vmx, vmy, vrho, vE};
    for (int v = 0; v < 4; ++v) { q[v].resize(N); for (size_t k = 0; k < N; ++k) { q[v][k].v = src[v][k]; q[v][k].d[0] = dir[v][k]; } }
    D1 g(gamma); g.d[0] = vg; D1 a(alpha); a.d[0] = va;
    D1* qp[4] = {q[0].data(), q[1].data(), q[2].data(), q[3].data()};
    D1 r = objective_run(G, obj, qp, n_steps, dt, g, a, n_iter, solver, prm);
    *J = r.v; *dJ = r.d[0];
  });
}

int orc2d_run_sensitivity(GRID2D_ARGS, double gamma, double alpha, double dt, double T_end, int n_iter, int solver, double s_gamma,
                          double* mx, double* my, double* rho, double* E, double* Sig, double* zx, double* zy, double* sr,
                          double* et, double* vs) {
  return guard([&] {
    if (solver < 0 || solver > 2) throw std::invalid_argument("Unknown solver");
    Grid2D G = GRID2D; double* q[4] = {mx, my, rho, E}; double* s[4] = {zx, zy, sr, et};
    run_sensitivity(G, q, s, Sig, vs, dt, T_end, gamma, alpha, n_iter, solver, s_gamma);
  });
}

// run_forward_store (forward.jl:111-158): snaps = (n_steps + 1) * 5 * N
// doubles, n_steps = ceil(T / dt) (the caller sizes the buffer).
int orc2d_run_forward_store(GRID2D_ARGS, double gamma, double alpha, double dt, double T_end, int n_iter, int solver,
                            const double* mx, const double* my, const double* rho, const double* E, double* snaps,
                            long long snaps_len, int* n_steps) {
  return guard([&] {
    if (solver < 0 || solver > 2) throw std::invalid_argument("Unknown solver");
    Grid2D G = GRID2D; const double* q0[4] = {mx, my, rho, E};
    std::vector<double> s;
    *n_steps = run_forward_store(G, q0, dt, T_end, gamma, alpha, n_iter, solver, s);
    if ((long long)s.size() != snaps_len) throw std::invalid_argument("snapshot buffer has the wrong size");
    std::memcpy(snaps, s.data(), s.size() * sizeof(double));
  });
}

// run_adjoint_conservative (adjoint_pde.jl:527-611) over caller-held snapshots.
int orc2d_run_adjoint_conservative(GRID2D_ARGS, double gamma, double alpha, int n_steps, double dt, double T_end,
                                   int n_iter, int obj, int solver, const double* prm, const double* snaps,
                                   double* amx, double* amy, double* arho, double* aE) {
  return guard([&] {
    if (solver < 0 || solver > 2) throw std::invalid_argument("Unknown solver");
    if (obj < 0 || obj > 5) throw std::invalid_argument("Unknown objective");
    Grid2D G = GRID2D; double* a[4] = {amx, amy, arho, aE};
    run_adjoint_conservative(G, snaps, n_steps, dt, T_end, gamma, alpha, n_iter, obj, solver, prm, a);
  });
}

// compute_adjoint_rhs_conservative! (adjoint_pde.jl:481-516): Pi in-out.
int orc2d_adjoint_rhs_conservative(GRID2D_ARGS, double gamma, double alpha, int n_iter, int solver, const double* mx,
                                   const double* my, const double* rho, const double* E, const double* Sig, double* Pi,
                                   const double* amx, const double* amy, const double* arho, const double* aE,
                                   double* dmx, double* dmy, double* drho, double* dE) {
  return guard([&] {
    Grid2D G = GRID2D; const double* q[4] = {mx, my, rho, E}; const double* a[4] = {amx, amy, arho, aE};
    double* da[4] = {dmx, dmy, drho, dE};
    Work2D<double> W; W.alloc(G.N);
    pde_adjoint_rhs(G, gamma, alpha, n_iter, solver, q, Sig, Pi, a, da, W);
  });
}

// Duality of the local adjoint operator (alpha = 0, Sigma frozen): lhs =
// <a, L dq>_M with L dq the exact directional derivative of the discrete
// hyperbolic RHS (forward-mode duals), rhs = <L_dag a, dq>_M with L_dag =
// compute_adjoint_hyperbolic_rhs_local!; M = nodal mass w_i w_j Jx Jy. Equal
// up to the discretisation error for smooth fields.
int orc2d_pde_duality(GRID2D_ARGS, double gamma, const double* q_in, const double* Sig, const double* a_in,
                      const double* dq_in, double* lhs, double* rhs) {
  return guard([&] {
    typedef Dual<1> D1;
    Grid2D G = GRID2D; const size_t N = G.N;
    std::vector<D1> qd[4], Sd(N), kd[4];
    for (int v = 0; v < 4; ++v) {
      qd[v].resize(N); kd[v].resize(N);
      for (size_t k = 0; k < N; ++k) { qd[v][k].v = q_in[v * N + k]; qd[v][k].d[0] = dq_in[v * N + k]; }
    }
    for (size_t k = 0; k < N; ++k) Sd[k] = D1(Sig[k]);
    const D1* qc[4] = {qd[0].data(), qd[1].data(), qd[2].data(), qd[3].data()};
    D1* kc[4] = {kd[0].data(), kd[1].data(), kd[2].data(), kd[3].data()};
    std::vector<D1> F[8];
    hyperbolic_rhs(G, D1(gamma), qc, Sd.data(), kc, F);
    const double* q[4] = {q_in, q_in + N, q_in + 2 * N, q_in + 3 * N};
    const double* a[4] = {a_in, a_in + N, a_in + 2 * N, a_in + 3 * N};
    std::vector<double> dav(4 * N);
    double* da[4] = {dav.data(), dav.data() + N, dav.data() + 2 * N, dav.data() + 3 * N};
    pde_hyperbolic_rhs_local(G, gamma, q, Sig, a, da);
    double l = 0.0, r = 0.0;
    const int np = G.np;
    for (int ey = 0; ey < G.m.Ney; ++ey) for (int ex = 0; ex < G.m.Nex; ++ex)
      for (int j = 0; j < np; ++j) for (int i = 0; i < np; ++i) {
        const size_t n = G.id(i, j, ex, ey);
        const double m = G.b.w[i] * G.b.w[j] * G.m.Jx * G.m.Jy;
        for (int v = 0; v < 4; ++v) { l += m * a[v][n] * kd[v][n].d[0]; r += m * da[v][n] * dq_in[v * N + n]; }
      }
    *lhs = l; *rhs = r;
  });
}

// ----------------------------------- 1D -----------------------------------
#define GRID1D_ARGS int p, const double *xi, const double *w, const double *Dcol, int Ne, double L
static Grid1D make_grid1(int p, const double* xi, const double* w, const double* Dcol, int Ne, double L) {
  Basis b = (xi && w && Dcol) ? basis_from_arrays(p, xi, w, Dcol) : make_basis(p);
  return Grid1D(b, make_mesh1d(Ne, L));
}
#define GRID1D make_grid1(p, xi, w, Dcol, Ne, L)

int orc1d_hyperbolic_rhs(GRID1D_ARGS, double gamma, const double* mu, const double* rho, const double* E, const double* Sig,
                         double* dmu, double* drho, double* dE) {
  return guard([&] {
    Grid1D G = GRID1D; const double* q[3] = {mu, rho, E}; double* dq[3] = {dmu, drho, dE};
    hyperbolic_rhs1d(G, gamma, q, Sig, dq);
  });
}

int orc1d_apply_sip(GRID1D_ARGS, double alpha, const double* x, const double* rho, double* y) {
  return guard([&] { Grid1D G = GRID1D; apply_sip1d(G, y, x, rho, alpha); });
}

int orc1d_igr_rhs(GRID1D_ARGS, double alpha, const double* mu, const double* rho, double* b) {
  return guard([&] { Grid1D G = GRID1D; igr_rhs1d(G, b, mu, rho, alpha); });
}

int orc1d_sip_diagonal(GRID1D_ARGS, double alpha, const double* rho, double* M) {
  return guard([&] { Grid1D G = GRID1D; sip_diagonal1d(G, M, rho, alpha); });
}

int orc1d_solve_elliptic(GRID1D_ARGS, double alpha, int n_iter, int solver, const double* mu, const double* rho,
                         const double* E, double* Sig) {
  return guard([&] {
    Grid1D G = GRID1D; const double* q[3] = {mu, rho, E};
    Work2D<double> W; W.alloc(G.N); solve_elliptic1d(G, Sig, q, alpha, n_iter, solver, W);
  });
}

int orc1d_igr_euler_rhs(GRID1D_ARGS, double gamma, double alpha, int n_iter, int solver, const double* mu,
                        const double* rho, const double* E, double* Sig, double* dmu, double* drho, double* dE) {
  return guard([&] {
    Grid1D G = GRID1D; const double* q[3] = {mu, rho, E};
    Work2D<double> W; W.alloc(G.N); igr_euler_rhs1d(G, q, Sig, gamma, alpha, n_iter, solver, W);
    double* out[3] = {dmu, drho, dE};
    for (int v = 0; v < 3; ++v) std::memcpy(out[v], W.dq[v].data(), G.N * sizeof(double));
  });
}

// cg_solve! (tol exit) or cg_fixed! (fixed=1) on A x = b with A = SIP(rho, alpha), IGR_adjoints_1d/elliptic.jl:163-292.
int orc1d_cg(GRID1D_ARGS, double alpha, const double* rho, const double* b, double* x, double tol, int maxiter, int fixed,
             int* iters) {
  return guard([&] {
    Grid1D G = GRID1D; Work2D<double> W; W.alloc(G.N);
    *iters = cg_solve(G, x, b, rho, alpha, tol, maxiter, fixed != 0, W);
  });
}

int orc1d_run_forward(GRID1D_ARGS, double gamma, double alpha, double dt, double T_end, int n_iter, int solver,
                      double* mu, double* rho, double* E, double* Sig) {
  return guard([&] {
    if (solver < 0 || solver > 2) throw std::invalid_argument("Unknown solver");
    Grid1D G = GRID1D; double* q[3] = {mu, rho, E}; run_forward1d(G, q, Sig, dt, T_end, gamma, alpha, n_iter, solver);
  });
}

int orc1d_objective_run(GRID1D_ARGS, double gamma, double alpha, int n_steps, double dt, int n_iter, int solver, int obj,
                        const double* prm, double* mu, double* rho, double* E, double* J) {
  return guard([&] {
    if (solver < 0 || solver > 2) throw std::invalid_argument("Unknown solver");
    Grid1D G = GRID1D; double* q[3] = {mu, rho, E};
    *J = objective_run1d(G, obj, q, n_steps, dt, gamma, alpha, n_iter, solver, prm);
  });
}

int orc1d_objective_dual(GRID1D_ARGS, double gamma, double alpha, int n_steps, double dt, int n_iter, int solver, int obj,
                         const double* prm, const double* mu, const double* rho, const double* E, const double* vmu,
                         const double* vrho, const double* vE, double vg, double va, double* J, double* dJ) {
  return guard([&] {
    typedef Dual<1> D1;
    Grid1D G = GRID1D; const size_t N = G.N;
    std::vector<D1> q[3];
    const double* src[3] = {mu, rho, E}; const double* dir[3] = {vmu, vrho, vE};
    for (int v = 0; v < 3; ++v) { q[v].resize(N); for (size_t k = 0; k < N; ++k) { q[v][k].v = src[v][k]; q[v][k].d[0] = dir[v][k]; } }
    D1 g(gamma); g.d[0] = vg; D1 a(alpha); a.d[0] = va;
    D1* qp[3] = {q[0].data(), q[1].data(), q[2].data()};
    D1 r = objective_run1d(G, obj, qp, n_steps, dt, g, a, n_iter, solver, prm);
    *J = r.v; *dJ = r.d[0];
  });
}

int orc1d_adjoint(GRID1D_ARGS, double gamma, double alpha, int n_steps, double dt, int n_iter, int solver, int obj,
                  const double* prm, const double* mu, const double* rho, const double* E, double* J, double* dmu,
                  double* drho, double* dE, double* dgamma, double* dalpha) {
  return guard([&] {
    if (solver < 0 || solver > 2) throw std::invalid_argument("Unknown solver");
    Grid1D G = GRID1D; const double* q0[3] = {mu, rho, E}; double* dq[3] = {dmu, drho, dE};
    *J = adjoint_ic1d(G, obj, prm, q0, n_steps, dt, gamma, alpha, n_iter, solver, dq, dgamma, dalpha);
  });
}

int orc1d_run_sensitivity(GRID1D_ARGS, double gamma, double alpha, double dt, double T_end, int n_iter, int solver, int form,
                          double s_gamma, double* mu, double* rho, double* E, double* Sig, double* smu, double* srho,
                          double* sE, double* sSig) {
  return guard([&] {
    if (solver < 0 || solver > 2) throw std::invalid_argument("Unknown solver");
    if (form != 1 && form != 2) throw std::invalid_argument("Unknown elliptic_rhs (use :form1 or :form2)");
    Grid1D G = GRID1D; double* q[3] = {mu, rho, E}; double* s[3] = {smu, srho, sE};
    run_sensitivity1d(G, q, s, Sig, sSig, dt, T_end, gamma, alpha, n_iter, solver, form, s_gamma);
  });
}

// run_forward_store (IGR_adjoints_1d/forward.jl:137-186): snaps = (n_steps + 1) * 4 * N doubles.
int orc1d_run_forward_store(GRID1D_ARGS, double gamma, double alpha, double dt, double T_end, int n_iter, int solver,
                            const double* mu, const double* rho, const double* E, double* snaps, long long snaps_len,
                            int* n_steps) {
  return guard([&] {
    if (solver < 0 || solver > 2) throw std::invalid_argument("Unknown solver");
    Grid1D G = GRID1D; const double* q0[3] = {mu, rho, E};
    std::vector<double> s;
    *n_steps = run_forward_store1d(G, q0, dt, T_end, gamma, alpha, n_iter, solver, s);
    if ((long long)s.size() != snaps_len) throw std::invalid_argument("snapshot buffer has the wrong size");
    std::memcpy(snaps, s.data(), s.size() * sizeof(double));
  });
}

// run_adjoint_conservative (IGR_adjoints_1d/adjoint_pde.jl:474-551).
int orc1d_run_adjoint_conservative(GRID1D_ARGS, double gamma, double alpha, int n_steps, double dt, double T_end,
                                   int n_iter, int obj, int solver, const double* prm, const double* snaps,
                                   double* amu, double* arho, double* aE) {
  return guard([&] {
    if (solver < 0 || solver > 2) throw std::invalid_argument("Unknown solver");
    Grid1D G = GRID1D; double* a[3] = {amu, arho, aE};
    run_adjoint_conservative1d(G, snaps, n_steps, dt, T_end, gamma, alpha, n_iter, obj, solver, prm, a);
  });
}

// compute_adjoint_rhs_conservative! (IGR_adjoints_1d/adjoint_pde.jl:410-456): Pi in-out.
int orc1d_adjoint_rhs_conservative(GRID1D_ARGS, double gamma, double alpha, int n_iter, int solver, const double* mu,
                                   const double* rho, const double* E, const double* Sig, double* Pi, const double* amu,
                                   const double* arho, const double* aE, double* dmu, double* drho, double* dE) {
  return guard([&] {
    Grid1D G = GRID1D; const double* q[3] = {mu, rho, E}; const double* a[3] = {amu, arho, aE};
    double* da[3] = {dmu, drho, dE};
    Work2D<double> W; W.alloc(G.N);
    pde1_adjoint_rhs(G, gamma, alpha, n_iter, solver, q, Sig, Pi, a, da, W);
  });
}

// 1D duality of the local adjoint operator (alpha = 0, Sigma frozen), as orc2d_pde_duality.
int orc1d_pde_duality(GRID1D_ARGS, double gamma, const double* q_in, const double* Sig, const double* a_in,
                      const double* dq_in, double* lhs, double* rhs) {
  return guard([&] {
    typedef Dual<1> D1;
    Grid1D G = GRID1D; const size_t N = G.N;
    std::vector<D1> qd[3], Sd(N), kd[3];
    for (int v = 0; v < 3; ++v) {
      qd[v].resize(N); kd[v].resize(N);
      for (size_t k = 0; k < N; ++k) { qd[v][k].v = q_in[v * N + k]; qd[v][k].d[0] = dq_in[v * N + k]; }
    }
    for (size_t k = 0; k < N; ++k) Sd[k] = D1(Sig[k]);
    const D1* qc[3] = {qd[0].data(), qd[1].data(), qd[2].data()};
    D1* kc[3] = {kd[0].data(), kd[1].data(), kd[2].data()};
    hyperbolic_rhs1d(G, D1(gamma), qc, Sd.data(), kc);
    const double* q[3] = {q_in, q_in + N, q_in + 2 * N};
    const double* a[3] = {a_in, a_in + N, a_in + 2 * N};
    std::vector<double> dav(3 * N);
    double* da[3] = {dav.data(), dav.data() + N, dav.data() + 2 * N};
    pde1_hyperbolic_rhs_local(G, gamma, q, Sig, a, da);
    double l = 0.0, r = 0.0;
    for (int e = 0; e < G.m.Ne; ++e)
      for (int i = 0; i < G.np; ++i) {
        const size_t n = G.id(i, e);
        const double m = G.b.w[i] * G.m.J;
        for (int v = 0; v < 3; ++v) { l += m * a[v][n] * kd[v][n].d[0]; r += m * da[v][n] * dq_in[v * N + n]; }
      }
    *lhs = l; *rhs = r;
  });
}

// IC builders (IGR_adjoints_2d/initial_conditions.jl:15-232; 1d :94-204) and l2_error.
int orc2d_build_ic(GRID2D_ARGS, int type, double gamma, double A, const double* prm, double* mx, double* my, double* rho,
                   double* E) {
  return guard([&] { Grid2D G = GRID2D; double* q[4] = {mx, my, rho, E}; build_ic2d(G, type, gamma, A, prm, q); });
}
int orc1d_build_ic(GRID1D_ARGS, int type, double gamma, double A, double* mu, double* rho, double* E) {
  return guard([&] { Grid1D G = GRID1D; double* q[3] = {mu, rho, E}; build_ic1d(G, type, gamma, A, q); });
}
int orc2d_l2_error(GRID2D_ARGS, const double* u, const double* r, double* out) {
  return guard([&] { Grid2D G = GRID2D; *out = l2_error2d(G, u, r); });
}

}  // extern "C"
