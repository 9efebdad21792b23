"""ctypes bindings for the CPU oracle (oracle/liboracle.so).

Test infrastructure only: the oracle is the parity checker for the CUDA path
and the CPU baseline, never part of the product. Arrays use the reference's
Julia column-major layout, flattened: 2D fields have N = np*np*N_ex*N_ey
entries with idx = i + np*(j + np*(ex + N_ex*ey)); 1D fields N = np*N_e.
"""
import ctypes as C
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
LIB_PATH = os.path.join(ORACLE_DIR, "liboracle.so")

SOLVERS = {"pcg": 0, "jacobi": 1, "chebyshev": 2}
OBJECTIVES_2D = {"l2_density": 0, "l2_pressure": 1, "kinetic_energy": 2, "windowed_kinetic_energy": 3,
                 "weighted_momentum": 4, "window_rho2": 5}
OBJECTIVES_1D = {"l2_density": 0, "l2_pressure": 1, "kinetic_energy": 2, "weighted_momentum": 4, "interval_rho": 6}

_lib = None
_D = C.POINTER(C.c_double)


def build():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = C.CDLL(LIB_PATH)
        _lib.orc_last_error.restype = C.c_char_p
    return _lib


def _p(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_D)


def _check(rc):
    if rc != 0:
        msg = lib().orc_last_error().decode()
        raise (ValueError if rc == 1 else RuntimeError)(msg)


OPCOUNT_FAMILIES = ("setup", "apply", "iteration", "solver_init", "hyperbolic_rk", "step", "objective")


def opcount_2d(G, solver, n_iter):
    """Algorithmic FP64 operations per node of the restated arithmetic
    (oracle/opcount.hpp): {family: (forward, reverse)}."""
    out = np.zeros(14)
    _check(lib().orc2d_opcount(*G.args(), C.c_int(SOLVERS.get(solver, -1)), C.c_int(n_iter), _p(out)))
    return {k: (out[2 * i], out[2 * i + 1]) for i, k in enumerate(OPCOUNT_FAMILIES)}


def set_dot_order(order):
    """Summation order of the oracle's solver inner products: 0 sequential (the
    default), 1 reversed, 2 pairwise (to measure a result's sensitivity to that
    order)."""
    _check(lib().orc_set_dot_order(C.c_int(order)))


def basis(p):
    n = p + 1
    xi = np.zeros(n)
    w = np.zeros(n)
    D = np.zeros(n * n)
    _check(lib().orc_basis(C.c_int(p), _p(xi), _p(w), _p(D)))
    return xi, w, D.reshape(n, n, order="F")


class Grid2D:
    """Basis + periodic Cartesian mesh, as IGR_adjoints_2d/mesh.jl:108-125."""

    def __init__(self, p, Nex, Ney, Lx=1.0, Ly=1.0):
        self.p, self.np, self.Nex, self.Ney, self.Lx, self.Ly = p, p + 1, Nex, Ney, float(Lx), float(Ly)
        self.xi, self.w, self.D = basis(p)
        self.Dcol = np.ascontiguousarray(self.D.reshape(-1, order="F"))
        self.N = self.np * self.np * Nex * Ney
        self.dx, self.dy = self.Lx / Nex, self.Ly / Ney
        self.Jx, self.Jy = self.dx / 2.0, self.dy / 2.0

    def args(self):
        return (C.c_int(self.p), _p(self.xi), _p(self.w), _p(self.Dcol), C.c_int(self.Nex), C.c_int(self.Ney),
                C.c_double(self.Lx), C.c_double(self.Ly))

    def coords(self):
        """Node coordinates (x, y), flat, Julia order."""
        i = np.arange(self.np)
        x = (np.arange(self.Nex)[None, :, None, None] * self.dx + self.Jx * (1.0 + self.xi[None, None, None, :]))
        y = (np.arange(self.Ney)[:, None, None, None] * self.dy + self.Jy * (1.0 + self.xi[None, None, :, None]))
        shape = (self.Ney, self.Nex, self.np, self.np)
        del i
        return np.broadcast_to(x, shape).reshape(-1).copy(), np.broadcast_to(y, shape).reshape(-1).copy()

    def zeros(self):
        return np.zeros(self.N)


class Grid1D:
    def __init__(self, p, Ne, L=1.0):
        self.p, self.np, self.Ne, self.L = p, p + 1, Ne, float(L)
        self.xi, self.w, self.D = basis(p)
        self.Dcol = np.ascontiguousarray(self.D.reshape(-1, order="F"))
        self.N = self.np * Ne
        self.dx = self.L / Ne
        self.J = self.dx / 2.0

    def args(self):
        return (C.c_int(self.p), _p(self.xi), _p(self.w), _p(self.Dcol), C.c_int(self.Ne), C.c_double(self.L))

    def coords(self):
        return (np.arange(self.Ne)[:, None] * self.dx + self.J * (1.0 + self.xi[None, :])).reshape(-1).copy()


def _f(x):
    return np.ascontiguousarray(x, dtype=np.float64)


# ------------------------------- 2D -------------------------------
def hyperbolic_rhs_2d(G, gamma, q, Sig):
    q = [_f(a) for a in q]
    out = [G.zeros() for _ in range(4)]
    _check(lib().orc2d_hyperbolic_rhs(*G.args(), C.c_double(gamma), *[_p(a) for a in q], _p(_f(Sig)),
                                      *[_p(a) for a in out]))
    return out


def apply_sip_2d(G, alpha, x, rho):
    y = G.zeros()
    _check(lib().orc2d_apply_sip(*G.args(), C.c_double(alpha), _p(_f(x)), _p(_f(rho)), _p(y)))
    return y


def igr_rhs_2d(G, alpha, mx, my, rho):
    b = G.zeros()
    _check(lib().orc2d_igr_rhs(*G.args(), C.c_double(alpha), _p(_f(mx)), _p(_f(my)), _p(_f(rho)), _p(b)))
    return b


def sip_diagonal_2d(G, alpha, rho):
    M = G.zeros()
    _check(lib().orc2d_sip_diagonal(*G.args(), C.c_double(alpha), _p(_f(rho)), _p(M)))
    return M


def solve_elliptic_2d(G, alpha, n_iter, solver, q, Sig0):
    Sig = _f(Sig0).copy()
    _check(lib().orc2d_solve_elliptic(*G.args(), C.c_double(alpha), C.c_int(n_iter), C.c_int(SOLVERS.get(solver, -1)),
                                      *[_p(_f(a)) for a in q], _p(Sig)))
    return Sig


def cg_2d(G, alpha, rho, b, x0, tol=1e-12, maxiter=5000, fixed=False):
    x = _f(x0).copy()
    it = C.c_int(0)
    _check(lib().orc2d_cg(*G.args(), C.c_double(alpha), _p(_f(rho)), _p(_f(b)), _p(x), C.c_double(tol),
                          C.c_int(maxiter), C.c_int(int(fixed)), C.byref(it)))
    return x, it.value


def igr_euler_rhs_2d(G, gamma, alpha, n_iter, solver, q, Sig0):
    Sig = _f(Sig0).copy()
    out = [G.zeros() for _ in range(4)]
    _check(lib().orc2d_igr_euler_rhs(*G.args(), C.c_double(gamma), C.c_double(alpha), C.c_int(n_iter),
                                     C.c_int(SOLVERS.get(solver, -1)), *[_p(_f(a)) for a in q], _p(Sig),
                                     *[_p(a) for a in out]))
    return out, Sig


def run_forward_2d(G, gamma, alpha, dt, T, n_iter, solver, q0):
    q = [_f(a).copy() for a in q0]
    Sig = G.zeros()
    _check(lib().orc2d_run_forward(*G.args(), C.c_double(gamma), C.c_double(alpha), C.c_double(dt), C.c_double(T),
                                   C.c_int(n_iter), C.c_int(SOLVERS.get(solver, -1)), *[_p(a) for a in q], _p(Sig)))
    return q, Sig


def _prm(prm):
    return _f(np.zeros(4) if prm is None else np.asarray(prm, dtype=np.float64))


def objective_run_2d(G, gamma, alpha, n_steps, dt, n_iter, solver, objective, q0, prm=None):
    q = [_f(a).copy() for a in q0]
    J = C.c_double(0.0)
    pr = _prm(prm)
    _check(lib().orc2d_objective_run(*G.args(), C.c_double(gamma), C.c_double(alpha), C.c_int(n_steps), C.c_double(dt),
                                     C.c_int(n_iter), C.c_int(SOLVERS.get(solver, -1)),
                                     C.c_int(OBJECTIVES_2D.get(objective, -1)), _p(pr), *[_p(a) for a in q], C.byref(J)))
    return J.value, q


def adjoint_2d(G, gamma, alpha, n_steps, dt, n_iter, solver, objective, q0, prm=None):
    out = [G.zeros() for _ in range(4)]
    J, dg, da = C.c_double(0.0), C.c_double(0.0), C.c_double(0.0)
    pr = _prm(prm)
    _check(lib().orc2d_adjoint(*G.args(), C.c_double(gamma), C.c_double(alpha), C.c_int(n_steps), C.c_double(dt),
                               C.c_int(n_iter), C.c_int(SOLVERS.get(solver, -1)),
                               C.c_int(OBJECTIVES_2D.get(objective, -1)), _p(pr), *[_p(_f(a)) for a in q0],
                               C.byref(J), *[_p(a) for a in out], C.byref(dg), C.byref(da)))
    return J.value, out, dg.value, da.value


def adjoint_batch_2d(G, gammas, alphas, n_steps, dt, n_iter, solver, objective, q0, prm=None, n_threads=1):
    """q0: (B, 4, N) array. Returns J (B,), dq0 (B, 4, N), dgamma (B,), dalpha (B,)."""
    q0 = _f(q0)
    B = q0.shape[0]
    J, dg, da = np.zeros(B), np.zeros(B), np.zeros(B)
    dq = np.zeros_like(q0)
    pr = _prm(prm)
    _check(lib().orc2d_adjoint_batch(*G.args(), C.c_int(B), _p(_f(gammas)), _p(_f(alphas)), C.c_int(n_steps),
                                     C.c_double(dt), C.c_int(n_iter), C.c_int(SOLVERS.get(solver, -1)),
                                     C.c_int(OBJECTIVES_2D.get(objective, -1)), _p(pr), _p(q0), _p(J), _p(dq), _p(dg),
                                     _p(da), C.c_int(n_threads)))
    return J, dq, dg, da


def objective_dual_2d(G, gamma, alpha, n_steps, dt, n_iter, solver, objective, q0, v, vg=0.0, va=0.0, prm=None):
    J, dJ = C.c_double(0.0), C.c_double(0.0)
    pr = _prm(prm)
    _check(lib().orc2d_objective_dual(*G.args(), C.c_double(gamma), C.c_double(alpha), C.c_int(n_steps),
                                      C.c_double(dt), C.c_int(n_iter), C.c_int(SOLVERS.get(solver, -1)),
                                      C.c_int(OBJECTIVES_2D.get(objective, -1)), _p(pr), *[_p(_f(a)) for a in q0],
                                      *[_p(_f(a)) for a in v], C.c_double(vg), C.c_double(va), C.byref(J), C.byref(dJ)))
    return J.value, dJ.value


def run_sensitivity_2d(G, gamma, alpha, dt, T, n_iter, solver, q0, s0, s_gamma=0.0):
    q = [_f(a).copy() for a in q0]
    s = [_f(a).copy() for a in s0]
    Sig, vs = G.zeros(), G.zeros()
    _check(lib().orc2d_run_sensitivity(*G.args(), C.c_double(gamma), C.c_double(alpha), C.c_double(dt), C.c_double(T),
                                       C.c_int(n_iter), C.c_int(SOLVERS.get(solver, -1)), C.c_double(s_gamma),
                                       *[_p(a) for a in q], _p(Sig), *[_p(a) for a in s], _p(vs)))
    return q, Sig, s, vs


def forward_store_steps(dt, T):
    """n_steps of run_forward_store (forward.jl:131): ceil(T / dt)."""
    return int(np.ceil(T / dt))


def run_forward_store_2d(G, gamma, alpha, dt, T, n_iter, solver, q0):
    """Snapshots (n_steps + 1, 5, N): (mux, muy, rho, E, Sigma) after each step."""
    n = forward_store_steps(dt, T)
    snaps = np.zeros((n + 1) * 5 * G.N)
    ns = C.c_int(0)
    _check(lib().orc2d_run_forward_store(*G.args(), C.c_double(gamma), C.c_double(alpha), C.c_double(dt), C.c_double(T),
                                         C.c_int(n_iter), C.c_int(SOLVERS.get(solver, -1)), *[_p(_f(a)) for a in q0],
                                         _p(snaps), C.c_longlong(snaps.size), C.byref(ns)))
    return snaps.reshape(n + 1, 5, G.N), ns.value


def run_adjoint_conservative_2d(G, snaps, n_steps, dt, T, gamma, alpha, n_iter, objective, solver, prm=None):
    out = [G.zeros() for _ in range(4)]
    _check(lib().orc2d_run_adjoint_conservative(*G.args(), C.c_double(gamma), C.c_double(alpha), C.c_int(n_steps),
                                                C.c_double(dt), C.c_double(T), C.c_int(n_iter),
                                                C.c_int(OBJECTIVES_2D.get(objective, -1)),
                                                C.c_int(SOLVERS.get(solver, -1)), _p(_prm(prm)),
                                                _p(_f(np.asarray(snaps).reshape(-1))), *[_p(a) for a in out]))
    return out


def adjoint_rhs_conservative_2d(G, gamma, alpha, n_iter, solver, q, Sig, Pi0, a):
    Pi = _f(Pi0).copy()
    out = [G.zeros() for _ in range(4)]
    _check(lib().orc2d_adjoint_rhs_conservative(*G.args(), C.c_double(gamma), C.c_double(alpha), C.c_int(n_iter),
                                                C.c_int(SOLVERS.get(solver, -1)), *[_p(_f(x)) for x in q],
                                                _p(_f(Sig)), _p(Pi), *[_p(_f(x)) for x in a], *[_p(x) for x in out]))
    return out, Pi


def pde_duality_2d(G, gamma, q, Sig, a, dq):
    """(<a, L dq>_M, <L_dag a, dq>_M) for the local adjoint operator (alpha = 0)."""
    l, r = C.c_double(0.0), C.c_double(0.0)
    _check(lib().orc2d_pde_duality(*G.args(), C.c_double(gamma), _p(_f(np.concatenate(q))), _p(_f(Sig)),
                                   _p(_f(np.concatenate(a))), _p(_f(np.concatenate(dq))), C.byref(l), C.byref(r)))
    return l.value, r.value


# ------------------------------- 1D -------------------------------
def hyperbolic_rhs_1d(G, gamma, q, Sig):
    out = [np.zeros(G.N) for _ in range(3)]
    _check(lib().orc1d_hyperbolic_rhs(*G.args(), C.c_double(gamma), *[_p(_f(a)) for a in q], _p(_f(Sig)),
                                      *[_p(a) for a in out]))
    return out


def apply_sip_1d(G, alpha, x, rho):
    y = np.zeros(G.N)
    _check(lib().orc1d_apply_sip(*G.args(), C.c_double(alpha), _p(_f(x)), _p(_f(rho)), _p(y)))
    return y


def igr_rhs_1d(G, alpha, mu, rho):
    b = np.zeros(G.N)
    _check(lib().orc1d_igr_rhs(*G.args(), C.c_double(alpha), _p(_f(mu)), _p(_f(rho)), _p(b)))
    return b


def sip_diagonal_1d(G, alpha, rho):
    M = np.zeros(G.N)
    _check(lib().orc1d_sip_diagonal(*G.args(), C.c_double(alpha), _p(_f(rho)), _p(M)))
    return M


def solve_elliptic_1d(G, alpha, n_iter, solver, q, Sig0):
    Sig = _f(Sig0).copy()
    _check(lib().orc1d_solve_elliptic(*G.args(), C.c_double(alpha), C.c_int(n_iter), C.c_int(SOLVERS.get(solver, -1)),
                                      *[_p(_f(a)) for a in q], _p(Sig)))
    return Sig


def igr_euler_rhs_1d(G, gamma, alpha, n_iter, solver, q, Sig0):
    Sig = _f(Sig0).copy()
    out = [np.zeros(G.N) for _ in range(3)]
    _check(lib().orc1d_igr_euler_rhs(*G.args(), C.c_double(gamma), C.c_double(alpha), C.c_int(n_iter),
                                     C.c_int(SOLVERS.get(solver, -1)), *[_p(_f(a)) for a in q], _p(Sig),
                                     *[_p(a) for a in out]))
    return out, Sig


def cg_1d(G, alpha, rho, b, x0, tol=1e-13, maxiter=1000, fixed=False):
    x = _f(x0).copy()
    it = C.c_int(0)
    _check(lib().orc1d_cg(*G.args(), C.c_double(alpha), _p(_f(rho)), _p(_f(b)), _p(x), C.c_double(tol),
                          C.c_int(maxiter), C.c_int(int(fixed)), C.byref(it)))
    return x, it.value


def run_forward_1d(G, gamma, alpha, dt, T, n_iter, solver, q0):
    q = [_f(a).copy() for a in q0]
    Sig = np.zeros(G.N)
    _check(lib().orc1d_run_forward(*G.args(), C.c_double(gamma), C.c_double(alpha), C.c_double(dt), C.c_double(T),
                                   C.c_int(n_iter), C.c_int(SOLVERS.get(solver, -1)), *[_p(a) for a in q], _p(Sig)))
    return q, Sig


def objective_run_1d(G, gamma, alpha, n_steps, dt, n_iter, solver, objective, q0, prm=None):
    q = [_f(a).copy() for a in q0]
    J = C.c_double(0.0)
    _check(lib().orc1d_objective_run(*G.args(), C.c_double(gamma), C.c_double(alpha), C.c_int(n_steps), C.c_double(dt),
                                     C.c_int(n_iter), C.c_int(SOLVERS.get(solver, -1)),
                                     C.c_int(OBJECTIVES_1D.get(objective, -1)), _p(_prm(prm)), *[_p(a) for a in q],
                                     C.byref(J)))
    return J.value, q


def objective_dual_1d(G, gamma, alpha, n_steps, dt, n_iter, solver, objective, q0, v, vg=0.0, va=0.0, prm=None):
    J, dJ = C.c_double(0.0), C.c_double(0.0)
    _check(lib().orc1d_objective_dual(*G.args(), C.c_double(gamma), C.c_double(alpha), C.c_int(n_steps),
                                      C.c_double(dt), C.c_int(n_iter), C.c_int(SOLVERS.get(solver, -1)),
                                      C.c_int(OBJECTIVES_1D.get(objective, -1)), _p(_prm(prm)),
                                      *[_p(_f(a)) for a in q0], *[_p(_f(a)) for a in v], C.c_double(vg),
                                      C.c_double(va), C.byref(J), C.byref(dJ)))
    return J.value, dJ.value


def adjoint_1d(G, gamma, alpha, n_steps, dt, n_iter, solver, objective, q0, prm=None):
    out = [np.zeros(G.N) for _ in range(3)]
    J, dg, da = C.c_double(0.0), C.c_double(0.0), C.c_double(0.0)
    _check(lib().orc1d_adjoint(*G.args(), C.c_double(gamma), C.c_double(alpha), C.c_int(n_steps), C.c_double(dt),
                               C.c_int(n_iter), C.c_int(SOLVERS.get(solver, -1)),
                               C.c_int(OBJECTIVES_1D.get(objective, -1)), _p(_prm(prm)), *[_p(_f(a)) for a in q0],
                               C.byref(J), *[_p(a) for a in out], C.byref(dg), C.byref(da)))
    return J.value, out, dg.value, da.value


def run_sensitivity_1d(G, gamma, alpha, dt, T, n_iter, solver, q0, s0, form=2, s_gamma=0.0):
    q = [_f(a).copy() for a in q0]
    s = [_f(a).copy() for a in s0]
    Sig, sSig = np.zeros(G.N), np.zeros(G.N)
    _check(lib().orc1d_run_sensitivity(*G.args(), C.c_double(gamma), C.c_double(alpha), C.c_double(dt), C.c_double(T),
                                       C.c_int(n_iter), C.c_int(SOLVERS.get(solver, -1)), C.c_int(form),
                                       C.c_double(s_gamma), *[_p(a) for a in q], _p(Sig), *[_p(a) for a in s],
                                       _p(sSig)))
    return q, Sig, s, sSig


def run_forward_store_1d(G, gamma, alpha, dt, T, n_iter, solver, q0):
    """Snapshots (n_steps + 1, 4, N): (mu, rho, E, Sigma) after each step."""
    n = forward_store_steps(dt, T)
    snaps = np.zeros((n + 1) * 4 * G.N)
    ns = C.c_int(0)
    _check(lib().orc1d_run_forward_store(*G.args(), C.c_double(gamma), C.c_double(alpha), C.c_double(dt), C.c_double(T),
                                         C.c_int(n_iter), C.c_int(SOLVERS.get(solver, -1)), *[_p(_f(a)) for a in q0],
                                         _p(snaps), C.c_longlong(snaps.size), C.byref(ns)))
    return snaps.reshape(n + 1, 4, G.N), ns.value


def run_adjoint_conservative_1d(G, snaps, n_steps, dt, T, gamma, alpha, n_iter, objective, solver, prm=None):
    out = [np.zeros(G.N) for _ in range(3)]
    _check(lib().orc1d_run_adjoint_conservative(*G.args(), C.c_double(gamma), C.c_double(alpha), C.c_int(n_steps),
                                                C.c_double(dt), C.c_double(T), C.c_int(n_iter),
                                                C.c_int(OBJECTIVES_1D.get(objective, -1)),
                                                C.c_int(SOLVERS.get(solver, -1)), _p(_prm(prm)),
                                                _p(_f(np.asarray(snaps).reshape(-1))), *[_p(a) for a in out]))
    return out


def adjoint_rhs_conservative_1d(G, gamma, alpha, n_iter, solver, q, Sig, Pi0, a):
    Pi = _f(Pi0).copy()
    out = [np.zeros(G.N) for _ in range(3)]
    _check(lib().orc1d_adjoint_rhs_conservative(*G.args(), C.c_double(gamma), C.c_double(alpha), C.c_int(n_iter),
                                                C.c_int(SOLVERS.get(solver, -1)), *[_p(_f(x)) for x in q],
                                                _p(_f(Sig)), _p(Pi), *[_p(_f(x)) for x in a], *[_p(x) for x in out]))
    return out, Pi


def pde_duality_1d(G, gamma, q, Sig, a, dq):
    l, r = C.c_double(0.0), C.c_double(0.0)
    _check(lib().orc1d_pde_duality(*G.args(), C.c_double(gamma), _p(_f(np.concatenate(q))), _p(_f(Sig)),
                                   _p(_f(np.concatenate(a))), _p(_f(np.concatenate(dq))), C.byref(l), C.byref(r)))
    return l.value, r.value


IC2D = {"constant": 0, "isentropic_vortex": 1, "taylor_green": 2, "sedov_blast": 3, "oseen_pair_blast": 4,
        "multi_blast": 5}
IC1D = {"acoustic_pulse": 0, "entropy_wave": 1, "density_pulse": 2, "pressure_pulse": 3, "velocity_pulse": 4}


def build_ic_2d(G, ic, gamma, A, prm):
    out = [G.zeros() for _ in range(4)]
    prm = np.zeros(15) + np.pad(np.asarray(prm, dtype=np.float64), (0, max(0, 15 - len(prm))))[:15]
    _check(lib().orc2d_build_ic(*G.args(), C.c_int(IC2D[ic]), C.c_double(gamma), C.c_double(A), _p(_f(prm)),
                                *[_p(a) for a in out]))
    return out


def build_ic_1d(G, ic, gamma, A):
    out = [np.zeros(G.N) for _ in range(3)]
    _check(lib().orc1d_build_ic(*G.args(), C.c_int(IC1D[ic]), C.c_double(gamma), C.c_double(A), *[_p(a) for a in out]))
    return out


def l2_error_2d(G, u, r):
    v = C.c_double(0.0)
    _check(lib().orc2d_l2_error(*G.args(), _p(_f(u)), _p(_f(r)), C.byref(v)))
    return v.value
