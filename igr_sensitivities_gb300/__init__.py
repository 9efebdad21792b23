"""GB300 engine for the IGR-regularised Euler forward map and its derivatives.

Host-side mirror of the reference's Julia module API (IGRAdjoints2D /
IGRAdjoints1D of f-t-s/IGR_sensitivities) over the C ABI in
include/igr_gb300.h. Function names, argument order and meaning follow the
reference; Julia's mutating `f!` functions are spelled `f_` here.

Arrays are numpy float64 arrays in the reference's layout: 2D fields have
shape (n_p, n_p, N_ex, N_ey) and 1D fields (n_p, N_e), indexed [i, j, ex, ey]
with the memory order of Julia (column-major, `order="F"`). All arithmetic
runs in the CUDA library; there is no CPU fallback, and importing a function
raises if the library is missing.
"""
import ctypes as C
import os

import numpy as np

from ._lib import Context, check, default_context, lib

__all__ = [
    "DGBasis", "CartesianMesh2D", "PeriodicMesh1D", "Context", "default_context",
    "run_forward", "run_forward_", "run_sensitivity", "sensitivity_batch", "enzyme_adjoint_ic", "adjoint_batch_meshes",
    "adjoint_batch", "adjoint_plan", "objective_value",
    "apply_sip_", "compute_hyperbolic_rhs_", "solve_elliptic_", "compute_igr_euler_rhs_", "compute_igr_rhs_",
    "compute_sip_diagonal", "SIPOperator", "sip_operator", "cg_solve_", "cg_fixed_", "SOLVERS", "OBJECTIVES",
    "Snapshots", "run_forward_store", "run_adjoint_conservative", "compute_adjoint_rhs_conservative_",
    "adjoint_conservative_ic", "adjoint_conservative_batch",
    "init_constant_state", "init_isentropic_vortex", "build_taylor_green_ic_", "build_sedov_blast_ic_",
    "build_oseen_pair_blast_ic_", "IC_BUILDERS", "ic_dA_weights", "l2_error", "build_ic_batch", "IC_TYPES",
    "forward_batch",
]

SOLVERS = {"pcg": 0, "jacobi": 1, "chebyshev": 2}
OBJECTIVES = {"l2_density": 0, "l2_pressure": 1, "kinetic_energy": 2, "windowed_kinetic_energy": 3,
              "weighted_momentum": 4, "window_rho2": 5, "interval_rho": 6}

_D = C.POINTER(C.c_double)


def _lgl(p):
    """LGL nodes and weights: closed forms for p <= 4 (the values
    FastGaussQuadrature.gausslobatto returns up to rounding), Newton on
    (1 - x^2) P_p'(x) above."""
    if p == 1:
        return np.array([-1.0, 1.0]), np.array([1.0, 1.0])
    if p == 2:
        return np.array([-1.0, 0.0, 1.0]), np.array([1 / 3, 4 / 3, 1 / 3])
    if p == 3:
        a = np.sqrt(1.0 / 5.0)
        return np.array([-1.0, -a, a, 1.0]), np.array([1 / 6, 5 / 6, 5 / 6, 1 / 6])
    if p == 4:
        a = np.sqrt(3.0 / 7.0)
        return np.array([-1.0, -a, 0.0, a, 1.0]), np.array([1 / 10, 49 / 90, 32 / 45, 49 / 90, 1 / 10])
    n = p + 1
    x = -np.cos(np.pi * np.arange(n) / p)
    for _ in range(100):
        P0, P1 = np.ones_like(x), x.copy()
        for k in range(2, p + 1):
            P0, P1 = P1, ((2 * k - 1) * x * P1 - (k - 1) * P0) / k
        dx = (x * P1 - P0) / (n * P1)
        x = x - dx
        if np.max(np.abs(dx)) < 1e-16:
            break
    P0, P1 = np.ones_like(x), x.copy()
    for k in range(2, p + 1):
        P0, P1 = P1, ((2 * k - 1) * x * P1 - (k - 1) * P0) / k
    return x, 2.0 / (p * n * P1 * P1)


class DGBasis:
    """DG basis of degree p: LGL nodes `xi`, weights `w`, differentiation
    matrix `D` (IGR_adjoints_2d/basis.jl:7-68)."""

    def __init__(self, p, xi=None, w=None, D=None):
        self.p = int(p)
        if xi is None:
            xi, w = _lgl(self.p)
        self.xi = np.ascontiguousarray(xi, dtype=np.float64)
        self.w = np.ascontiguousarray(w, dtype=np.float64)
        if D is None:
            n = self.p + 1
            lam = np.ones(n)  # barycentric weights, basis.jl:19-30
            for j in range(n):
                for i in range(n):
                    if i != j:
                        lam[j] *= self.xi[j] - self.xi[i]
                lam[j] = 1.0 / lam[j]
            D = np.zeros((n, n))  # basis.jl:38-49
            for j in range(n):
                for i in range(n):
                    if i == j:
                        continue
                    D[i, j] = (lam[j] / lam[i]) / (self.xi[i] - self.xi[j])
                    D[i, i] -= D[i, j]
        self.D = np.asarray(D, dtype=np.float64)
        self._Dcol = np.ascontiguousarray(self.D.reshape(-1, order="F"))

    @property
    def n_p(self):
        return self.p + 1


class CartesianMesh2D:
    """Uniform doubly-periodic mesh (IGR_adjoints_2d/mesh.jl:89-125)."""

    def __init__(self, N_ex, N_ey, Lx, Ly, basis):
        self.N_ex, self.N_ey, self.Lx, self.Ly = int(N_ex), int(N_ey), float(Lx), float(Ly)
        self.basis = basis  # node coordinates depend on it; the IC builders take (mesh, gamma) as the reference does
        self.dx, self.dy = self.Lx / self.N_ex, self.Ly / self.N_ey
        self.Jx, self.Jy = self.dx / 2.0, self.dy / 2.0
        n = basis.n_p
        ex = np.arange(self.N_ex)[None, None, :, None]
        ey = np.arange(self.N_ey)[None, None, None, :]
        self.x = np.asfortranarray(np.broadcast_to((ex * self.dx) + self.Jx * (1.0 + basis.xi[:, None, None, None]),
                                                   (n, n, self.N_ex, self.N_ey)))
        self.y = np.asfortranarray(np.broadcast_to((ey * self.dy) + self.Jy * (1.0 + basis.xi[None, :, None, None]),
                                                   (n, n, self.N_ex, self.N_ey)))

    def shape(self, basis):
        return (basis.n_p, basis.n_p, self.N_ex, self.N_ey)


class PeriodicMesh1D:
    """Uniform periodic 1D mesh (IGR_adjoints_1d/mesh.jl:7-33)."""

    def __init__(self, N_e, L, basis):
        self.N_e, self.L = int(N_e), float(L)
        self.basis = basis
        self.dx = self.L / self.N_e
        self.J = self.dx / 2.0
        e = np.arange(self.N_e)[None, :]
        self.x = np.asfortranarray((e * self.dx) + self.J * (1.0 + basis.xi[:, None]))


class _Disc2D(C.Structure):
    _fields_ = [("p", C.c_int), ("n_ex", C.c_int), ("n_ey", C.c_int), ("lx", C.c_double), ("ly", C.c_double),
                ("xi", _D), ("w", _D), ("D", _D)]


def _disc2d(basis, mesh):
    d = _Disc2D(basis.p, mesh.N_ex, mesh.N_ey, mesh.Lx, mesh.Ly, basis.xi.ctypes.data_as(_D),
                basis.w.ctypes.data_as(_D), basis._Dcol.ctypes.data_as(_D))
    d._keep = (basis,)
    return d


def _flat(a, n):
    f = np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1, order="F"))
    if f.size != n:
        raise ValueError("array has %d entries, expected %d" % (f.size, n))
    return f


def _ptr(a):
    return a.ctypes.data_as(_D)


def _solver(solver):
    if isinstance(solver, str):
        solver = solver.lstrip(":")
        if solver not in SOLVERS:
            raise ValueError("Unknown solver: %s (use :pcg, :jacobi, or :chebyshev)" % solver)
        return SOLVERS[solver]
    return int(solver)


def _objective(obj):
    if isinstance(obj, str):
        obj = obj.lstrip(":")
        if obj not in OBJECTIVES:
            raise ValueError("Unknown objective: %s" % obj)
        return OBJECTIVES[obj]
    return int(obj)


def _prm(obj_params):
    return np.ascontiguousarray(np.zeros(4) if obj_params is None else np.asarray(obj_params, dtype=np.float64))


def run_forward_(mux, muy, rho, E, Sigma, dt, T, basis, mesh, gamma, alpha, n_iter=10, solver="pcg", ctx=None):
    """run_forward! (IGR_adjoints_2d/forward.jl:41-75): state arrays updated in place to time T."""
    _solver(solver)  # validate before touching the device
    ctx = ctx or default_context()
    shape = mesh.shape(basis)
    n = int(np.prod(shape))
    q = [_flat(a, n) for a in (mux, muy, rho, E)]
    S = np.zeros(n)
    check(ctx, lib().igr2d_run_forward(ctx.handle, C.byref(_disc2d(basis, mesh)), C.c_double(gamma), C.c_double(alpha),
                                       C.c_double(dt), C.c_double(T), C.c_int(n_iter), C.c_int(_solver(solver)),
                                       *[_ptr(a) for a in q], _ptr(S)))
    for dst, src in zip((mux, muy, rho, E, Sigma), q + [S]):
        dst[...] = src.reshape(shape, order="F")


def run_forward(mux0, muy0, rho0, E0, dt, T, basis, mesh, gamma, alpha, n_iter=10, solver="pcg", ctx=None):
    """run_forward (IGR_adjoints_2d/forward.jl:84-99): returns (mux, muy, rho, E, Sigma) at time T."""
    shape = mesh.shape(basis)
    out = [np.array(np.asarray(a, dtype=np.float64).reshape(shape, order="F"), order="F") for a in (mux0, muy0, rho0, E0)]
    S = np.zeros(shape, order="F")
    run_forward_(*out, S, dt, T, basis, mesh, gamma, alpha, n_iter, solver, ctx)
    return (*out, S)


def run_sensitivity(mux0, muy0, rho0, E0, zetax0, zetay0, sigma0, eta0, dt, T, basis, mesh, gamma, alpha, n_iter=10,
                    solver="pcg", s_gamma=0.0, ctx=None):
    """run_sensitivity (IGR_adjoints_2d/sensitivity.jl:353-413).

    Advances the state and its tangent (zeta_x, zeta_y, sigma, eta) together
    to time T; returns (mux, muy, rho, E, Sigma, zetax, zetay, sigma, eta,
    varsigma). s_gamma adds the direct dP/dgamma tangent source (0 in the
    reference's 2D package).
    """
    _solver(solver)  # validate before touching the device
    ctx = ctx or default_context()
    shape = mesh.shape(basis)
    n = int(np.prod(shape))
    q = [_flat(a, n).copy() for a in (mux0, muy0, rho0, E0)]
    s = [_flat(a, n).copy() for a in (zetax0, zetay0, sigma0, eta0)]
    S, V = np.zeros(n), np.zeros(n)
    check(ctx, lib().igr2d_run_sensitivity(ctx.handle, C.byref(_disc2d(basis, mesh)), C.c_double(gamma),
                                           C.c_double(alpha), C.c_double(dt), C.c_double(T), C.c_int(n_iter),
                                           C.c_int(_solver(solver)), C.c_double(s_gamma), *[_ptr(a) for a in q], _ptr(S),
                                           *[_ptr(a) for a in s], _ptr(V)))
    r = lambda a: np.asfortranarray(a.reshape(shape, order="F"))
    return tuple(r(a) for a in q) + (r(S),) + tuple(r(a) for a in s) + (r(V),)


def adjoint_batch_meshes(states, basis, meshes, gammas, alphas, dts, n_steps, n_iter=10, solver="pcg",
                         objective="l2_density", obj_params=None, ctx=None):
    """Batched enzyme_adjoint_ic over instances with their own meshes.

    states: list of (mux0, muy0, rho0, E0) per instance (any array shape with
    the instance's node count, Julia order). Returns (J, [(dmux0, dmuy0,
    drho0, dE0)], dgamma, dalpha).
    """
    _solver(solver)
    _objective(objective)
    ctx = ctx or default_context()
    B = len(states)
    n = [int(np.prod(m.shape(basis))) for m in meshes]
    q = np.concatenate([np.concatenate([_flat(a, n[i]) for a in states[i]]) for i in range(B)])
    dq = np.zeros_like(q)
    i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
    f64 = lambda a: np.ascontiguousarray(np.broadcast_to(np.asarray(a, dtype=np.float64), (B,)))
    nex, ney = i32([m.N_ex for m in meshes]), i32([m.N_ey for m in meshes])
    lx, ly = f64([m.Lx for m in meshes]), f64([m.Ly for m in meshes])
    gs, als, dtv = f64(gammas), f64(alphas), f64(dts)
    J, dg, da = np.zeros(B), np.zeros(B), np.zeros(B)
    IP = C.POINTER(C.c_int)
    check(ctx, lib().igr2d_adjoint_batch_meshes(ctx.handle, C.c_int(basis.p), _ptr(basis.xi), _ptr(basis.w),
                                                _ptr(basis._Dcol), C.c_int(B), nex.ctypes.data_as(IP),
                                                ney.ctypes.data_as(IP), _ptr(lx), _ptr(ly), _ptr(gs), _ptr(als), _ptr(dtv),
                                                C.c_int(n_steps), C.c_int(n_iter), C.c_int(_solver(solver)),
                                                C.c_int(_objective(objective)), _ptr(_prm(obj_params)), _ptr(q), _ptr(J),
                                                _ptr(dq), _ptr(dg), _ptr(da)))
    out, o = [], 0
    for i in range(B):
        out.append(tuple(dq[o + v * n[i]:o + (v + 1) * n[i]] for v in range(4)))
        o += 4 * n[i]
    return J, out, dg, da


def sensitivity_batch(q0, s0, gammas, alphas, dts, n_steps, basis, mesh, n_iter=10, solver="pcg", s_gamma=0.0, ctx=None):
    """Batched run_sensitivity for n_steps fixed steps (per-instance gamma, alpha, dt).

    q0, s0: (n_inst, 4, N) float64 (variables mux, muy, rho, E and their
    tangents, Julia node order). Returns (q, Sigma, s, varsigma) with q, s of
    shape (n_inst, 4, N) and Sigma, varsigma of shape (n_inst, N).
    """
    _solver(solver)  # validate before touching the device
    ctx = ctx or default_context()
    q = np.array(q0, dtype=np.float64, order="C", copy=True)
    s = np.array(s0, dtype=np.float64, order="C", copy=True)
    B, _, n = q.shape
    f64 = lambda a: np.ascontiguousarray(np.broadcast_to(np.asarray(a, dtype=np.float64), (B,)))
    gs, als, dtv = f64(gammas), f64(alphas), f64(dts)
    S, V = np.zeros((B, n)), np.zeros((B, n))
    check(ctx, lib().igr2d_sensitivity_batch(ctx.handle, C.byref(_disc2d(basis, mesh)), C.c_int(B), _ptr(gs), _ptr(als),
                                             _ptr(dtv), C.c_int(n_steps), C.c_int(n_iter), C.c_int(_solver(solver)),
                                             C.c_double(s_gamma), _ptr(q), _ptr(s), _ptr(S), _ptr(V)))
    return q, S, s, V


def enzyme_adjoint_ic(mux0, muy0, rho0, E0, n_steps, dt, basis, mesh, gamma, alpha, n_iter=10, solver="pcg",
                      objective="l2_density", obj_params=None, with_params=False, ctx=None):
    """enzyme_adjoint_ic (IGR_adjoints_2d/enzyme_adjoint.jl:270-296).

    Returns (J, dmux0, dmuy0, drho0, dE0), the objective and its gradient with
    respect to the initial conservative state after `n_steps` SSP-RK3 steps of
    size `dt`, computed by the hand-written discrete adjoint on the GPU. With
    with_params=True, (dJ/dgamma, dJ/dalpha) are appended.
    """
    _solver(solver)  # validate before touching the device
    _objective(objective)
    ctx = ctx or default_context()
    shape = mesh.shape(basis)
    n = int(np.prod(shape))
    q = [_flat(a, n) for a in (mux0, muy0, rho0, E0)]
    dq = [np.zeros(n) for _ in range(4)]
    J, dg, da = C.c_double(0), C.c_double(0), C.c_double(0)
    prm = _prm(obj_params)
    check(ctx, lib().igr2d_adjoint_ic(ctx.handle, C.byref(_disc2d(basis, mesh)), C.c_double(gamma), C.c_double(alpha),
                                      C.c_int(n_steps), C.c_double(dt), C.c_int(max(n_iter, 1)), C.c_int(_solver(solver)),
                                      C.c_int(_objective(objective)), _ptr(prm), *[_ptr(a) for a in q], C.byref(J),
                                      *[_ptr(a) for a in dq], C.byref(dg), C.byref(da)))
    out = (J.value,) + tuple(a.reshape(shape, order="F") for a in dq)
    return out + (dg.value, da.value) if with_params else out


def adjoint_batch(q0, gammas, alphas, dts, n_steps, basis, mesh, n_iter=10, solver="pcg", objective="l2_density",
                  obj_params=None, ctx=None, device_arrays=False):
    """Batched enzyme_adjoint_ic over instances sharing one mesh.

    q0: (n_inst, 4, N) float64, variables (mux, muy, rho, E) in the Julia node
    order. Returns (J[n_inst], dq0 (n_inst, 4, N), dgamma[n_inst], dalpha[n_inst]).
    With device_arrays=True, q0 is a torch CUDA tensor and dq0 is returned as one.
    """
    _solver(solver)  # validate before touching the device
    _objective(objective)
    ctx = ctx or default_context()
    gammas = np.ascontiguousarray(gammas, dtype=np.float64)
    alphas = np.ascontiguousarray(alphas, dtype=np.float64)
    dts = np.ascontiguousarray(dts, dtype=np.float64)
    B = gammas.size
    J, dg, da = np.zeros(B), np.zeros(B), np.zeros(B)
    prm = _prm(obj_params)
    d = _disc2d(basis, mesh)
    if device_arrays:
        import torch
        dq = torch.empty_like(q0)
        check(ctx, lib().igr2d_adjoint_batch_dev(ctx.handle, C.byref(d), C.c_int(B), _ptr(gammas), _ptr(alphas), _ptr(dts),
                                                 C.c_int(n_steps), C.c_int(n_iter), C.c_int(_solver(solver)),
                                                 C.c_int(_objective(objective)), _ptr(prm),
                                                 C.cast(C.c_void_p(q0.data_ptr()), _D), _ptr(J),
                                                 C.cast(C.c_void_p(dq.data_ptr()), _D), _ptr(dg), _ptr(da)))
        return J, dq, dg, da
    q0 = np.ascontiguousarray(q0, dtype=np.float64)
    dq = np.zeros_like(q0)
    check(ctx, lib().igr2d_adjoint_batch(ctx.handle, C.byref(d), C.c_int(B), _ptr(gammas), _ptr(alphas), _ptr(dts),
                                         C.c_int(n_steps), C.c_int(n_iter), C.c_int(_solver(solver)),
                                         C.c_int(_objective(objective)), _ptr(prm), _ptr(q0), _ptr(J), _ptr(dq), _ptr(dg),
                                         _ptr(da)))
    return J, dq, dg, da


def adjoint_plan(n_inst, n_steps, basis, mesh, alpha, n_iter=10, solver="pcg", ctx=None):
    """The memory plan adjoint_batch would use, without running it:
    {"instances_per_group", "tape_steps", "snapshots", "step_evaluations"} (the
    revolve checkpoint schedule of one group; step_evaluations == n_steps means
    the whole tape fits and nothing is recomputed)."""
    ctx = ctx or default_context()
    g, w, s, e = C.c_int(0), C.c_int(0), C.c_int(0), C.c_longlong(0)
    check(ctx, lib().igr2d_adjoint_plan(ctx.handle, C.byref(_disc2d(basis, mesh)), C.c_int(n_inst), C.c_int(n_steps),
                                        C.c_int(n_iter), C.c_int(_solver(solver)), C.c_double(alpha), C.byref(g),
                                        C.byref(w), C.byref(s), C.byref(e)))
    return {"instances_per_group": g.value, "tape_steps": w.value, "snapshots": s.value, "step_evaluations": e.value}


def objective_value(mux0, muy0, rho0, E0, n_steps, dt, basis, mesh, gamma, alpha, n_iter=10, solver="pcg",
                    objective="l2_density", obj_params=None, ctx=None):
    """The primal objective of enzyme_adjoint_ic (the inlined RK3 loop of
    IGR_adjoints_2d/enzyme_adjoint.jl:56-71 and its objective tail, :72-81)."""
    _solver(solver)  # validate before touching the device
    _objective(objective)
    ctx = ctx or default_context()
    shape = mesh.shape(basis)
    n = int(np.prod(shape))
    q = [_flat(a, n).copy() for a in (mux0, muy0, rho0, E0)]
    J = C.c_double(0)
    check(ctx, lib().igr2d_objective(ctx.handle, C.byref(_disc2d(basis, mesh)), C.c_double(gamma), C.c_double(alpha),
                                     C.c_int(n_steps), C.c_double(dt), C.c_int(max(n_iter, 1)), C.c_int(_solver(solver)),
                                     C.c_int(_objective(objective)), _ptr(_prm(obj_params)), *[_ptr(a) for a in q],
                                     C.byref(J)))
    return J.value


def apply_sip_(y, x, rho, basis, mesh, alpha, ctx=None):
    """apply_sip! (IGR_adjoints_2d/elliptic.jl:30-145): y = A x."""
    ctx = ctx or default_context()
    shape = mesh.shape(basis)
    n = int(np.prod(shape))
    out = np.zeros(n)
    check(ctx, lib().igr2d_apply_sip(ctx.handle, C.byref(_disc2d(basis, mesh)), C.c_double(alpha), _ptr(_flat(x, n)),
                                     _ptr(_flat(rho, n)), _ptr(out)))
    y[...] = out.reshape(shape, order="F")


def compute_hyperbolic_rhs_(dmux, dmuy, drho, dE, mux, muy, rho, E, Sigma, basis, mesh, gamma, ctx=None):
    """compute_hyperbolic_rhs! (IGR_adjoints_2d/hyperbolic.jl:27-119)."""
    ctx = ctx or default_context()
    shape = mesh.shape(basis)
    n = int(np.prod(shape))
    q = [_flat(a, n) for a in (mux, muy, rho, E, Sigma)]
    out = [np.zeros(n) for _ in range(4)]
    check(ctx, lib().igr2d_hyperbolic_rhs(ctx.handle, C.byref(_disc2d(basis, mesh)), C.c_double(gamma),
                                          *[_ptr(a) for a in q], *[_ptr(a) for a in out]))
    for dst, src in zip((dmux, dmuy, drho, dE), out):
        dst[...] = src.reshape(shape, order="F")


def solve_elliptic_(Sigma, mux, muy, rho, E, basis, mesh, alpha, n_iter=10, solver="pcg", ctx=None):
    """solve_elliptic! (IGR_adjoints_2d/elliptic.jl:413-427); Sigma is the warm start and the result."""
    _solver(solver)  # validate before touching the device
    ctx = ctx or default_context()
    shape = mesh.shape(basis)
    n = int(np.prod(shape))
    q = [_flat(a, n) for a in (mux, muy, rho, E)]
    S = _flat(Sigma, n).copy()
    check(ctx, lib().igr2d_solve_elliptic(ctx.handle, C.byref(_disc2d(basis, mesh)), C.c_double(alpha), C.c_int(n_iter),
                                          C.c_int(_solver(solver)), *[_ptr(a) for a in q], _ptr(S)))
    Sigma[...] = S.reshape(shape, order="F")


def compute_igr_euler_rhs_(dmux, dmuy, drho, dE, mux, muy, rho, E, Sigma, basis, mesh, gamma, alpha, n_iter=10,
                           solver="pcg", ctx=None):
    """compute_igr_euler_rhs! (IGR_adjoints_2d/forward.jl:15-31): the Sigma solve
    (Sigma is the warm start and the result) when alpha > 0, else Sigma = 0;
    then the hyperbolic DG RHS at (q, Sigma) into (dmux, dmuy, drho, dE)."""
    _solver(solver)  # validate before touching the device
    ctx = ctx or default_context()
    shape = mesh.shape(basis)
    n = int(np.prod(shape))
    q = [_flat(a, n) for a in (mux, muy, rho, E)]
    S = _flat(Sigma, n).copy()
    out = [np.zeros(n) for _ in range(4)]
    check(ctx, lib().igr2d_igr_euler_rhs(ctx.handle, C.byref(_disc2d(basis, mesh)), C.c_double(gamma),
                                         C.c_double(alpha), C.c_int(n_iter), C.c_int(_solver(solver)),
                                         *[_ptr(a) for a in q], _ptr(S), *[_ptr(a) for a in out]))
    for dst, src in zip((dmux, dmuy, drho, dE), out):
        dst[...] = src.reshape(shape, order="F")
    Sigma[...] = S.reshape(shape, order="F")


def compute_igr_rhs_(b, mux, muy, rho, E, basis, mesh, alpha, ctx=None):
    """compute_igr_rhs! (IGR_adjoints_2d/elliptic.jl:159-197): the IGR source b."""
    ctx = ctx or default_context()
    shape = mesh.shape(basis)
    n = int(np.prod(shape))
    q = [_flat(a, n) for a in (mux, muy, rho, E)]
    out = np.zeros(n)
    check(ctx, lib().igr2d_igr_rhs(ctx.handle, C.byref(_disc2d(basis, mesh)), C.c_double(alpha),
                                   *[_ptr(a) for a in q], _ptr(out)))
    b[...] = out.reshape(shape, order="F")


def compute_sip_diagonal(rho, basis, mesh, alpha, ctx=None):
    """compute_sip_diagonal (IGR_adjoints_2d/elliptic.jl:205-264): diag(A) as a new array."""
    ctx = ctx or default_context()
    shape = mesh.shape(basis)
    n = int(np.prod(shape))
    out = np.zeros(n)
    check(ctx, lib().igr2d_sip_diagonal(ctx.handle, C.byref(_disc2d(basis, mesh)), C.c_double(alpha),
                                        _ptr(_flat(rho, n)), _ptr(out)))
    return np.asfortranarray(out.reshape(shape, order="F"))


class SIPOperator:
    """The operator the reference's tests hand to cg_solve! / cg_fixed!:
    `apply_A!(y, x) = apply_sip!(y, x, rho, basis, mesh, alpha)`
    (IGR_adjoints_2d/tests/run_euler_test.jl:64). Calling it applies A once
    (apply_sip_); cg_solve_ / cg_fixed_ recognise it and run the whole CG
    iteration on the GPU. `dim` is 2 (CartesianMesh2D) or 1 (PeriodicMesh1D)."""

    def __init__(self, rho, basis, mesh, alpha, ctx=None):
        self.rho, self.basis, self.mesh, self.alpha, self.ctx = rho, basis, mesh, float(alpha), ctx
        self.dim = 1 if hasattr(mesh, "N_e") else 2

    def __call__(self, y, x):
        if self.dim == 2:
            apply_sip_(y, x, self.rho, self.basis, self.mesh, self.alpha, self.ctx)
        else:
            from . import igr1d
            igr1d.apply_sip_(y, x, self.rho, self.basis, self.mesh, self.alpha, self.ctx)


def sip_operator(rho, basis, mesh, alpha, ctx=None):
    """apply_A! for cg_solve_ / cg_fixed_: y <- A(rho, alpha) x (2D or 1D mesh)."""
    return SIPOperator(rho, basis, mesh, alpha, ctx)


def _cg(x, apply_A, b, tol, maxiter, fixed):
    if not isinstance(apply_A, SIPOperator):
        raise TypeError("the GPU CG applies the SIP operator: pass apply_A = sip_operator(rho, basis, mesh, alpha)")
    op = apply_A
    ctx = op.ctx or default_context()
    n = x.size
    xf = _flat(x, n).copy()
    rho, bb = _flat(op.rho, n), _flat(b, n)
    it = C.c_int(0)
    if op.dim == 2:
        d = C.byref(_disc2d(op.basis, op.mesh))
        if fixed:
            check(ctx, lib().igr2d_cg_fixed(ctx.handle, d, C.c_double(op.alpha), _ptr(rho), _ptr(bb), _ptr(xf),
                                            C.c_int(maxiter)))
        else:
            check(ctx, lib().igr2d_cg_solve(ctx.handle, d, C.c_double(op.alpha), _ptr(rho), _ptr(bb), _ptr(xf),
                                            C.c_double(tol), C.c_int(maxiter), C.byref(it)))
    else:
        from .igr1d import _disc1d
        d = C.byref(_disc1d(op.basis, op.mesh))
        if fixed:
            check(ctx, lib().igr1d_cg_fixed(ctx.handle, d, C.c_double(op.alpha), _ptr(rho), _ptr(bb), _ptr(xf),
                                            C.c_int(maxiter)))
        else:
            check(ctx, lib().igr1d_cg_solve(ctx.handle, d, C.c_double(op.alpha), _ptr(rho), _ptr(bb), _ptr(xf),
                                            C.c_double(tol), C.c_int(maxiter), C.byref(it)))
    x[...] = xf.reshape(x.shape, order="F")
    return int(maxiter) if fixed else it.value


def cg_solve_(x, apply_A, b, tol, maxiter):
    """cg_solve! (IGR_adjoints_2d/elliptic.jl:278-297; 1D :163-199): CG with the
    exit sqrt(r.r) < tol tested before each iteration; x is the initial guess
    and the solution. Returns the reference's iteration count."""
    return _cg(x, apply_A, b, float(tol), int(maxiter), False)


def cg_fixed_(x, apply_A, b, n_iter):
    """cg_fixed! (IGR_adjoints_2d/elliptic.jl:304-320; 1D :265-292): n_iter CG
    iterations with the 1e-30 guards. Returns n_iter."""
    return _cg(x, apply_A, b, 0.0, int(n_iter), True)


# ---------------------------------------------------------------------------
# Continuous adjoint (IGR_adjoints_2d/adjoint_pde.jl, forward.jl:111-158)
# ---------------------------------------------------------------------------
class Snapshots:
    """The snapshot list run_forward_store returns (forward.jl:111-158):
    snapshots[k] is the tuple (mux, muy, rho, E, Sigma) after step k (k = 0:
    the initial state), each an (n_p, n_p, N_ex, N_ey) view in Julia order;
    len() = n_steps + 1 and negative indices count from the end, as
    snapshots[end] does in Julia. `data` is the flat (n_steps + 1, 5, N)
    buffer the C ABI reads and writes."""

    def __init__(self, data, shape):
        self.data = data
        self.shape = tuple(shape)

    def __len__(self):
        return self.data.shape[0]

    def __getitem__(self, k):
        return tuple(self.data[k, v].reshape(self.shape, order="F") for v in range(5))

    @classmethod
    def from_list(cls, snaps, shape):
        n = int(np.prod(shape))
        data = np.stack([np.stack([_flat(a, n) for a in snap]) for snap in snaps])
        return cls(np.ascontiguousarray(data), shape)


def run_forward_store(mux0, muy0, rho0, E0, dt, T, basis, mesh, gamma, alpha, n_iter=10, solver="pcg", ctx=None):
    """run_forward_store (IGR_adjoints_2d/forward.jl:111-158): returns
    (snapshots, n_steps) with snapshots[0] at t = 0 and snapshots[-1] at T."""
    _solver(solver)  # validate before touching the device
    ctx = ctx or default_context()
    shape = mesh.shape(basis)
    n = int(np.prod(shape))
    if not (dt > 0 and T > 0):
        raise ValueError("dt and T must be positive")
    steps = int(np.ceil(T / dt))
    data = np.zeros((steps + 1, 5, n))
    ns = C.c_int(0)
    q = [_flat(a, n) for a in (mux0, muy0, rho0, E0)]
    check(ctx, lib().igr2d_run_forward_store(ctx.handle, C.byref(_disc2d(basis, mesh)), C.c_double(gamma),
                                             C.c_double(alpha), C.c_double(dt), C.c_double(T), C.c_int(n_iter),
                                             C.c_int(_solver(solver)), *[_ptr(a) for a in q], _ptr(data),
                                             C.c_longlong(data.size), C.byref(ns)))
    return Snapshots(data, shape), ns.value


def run_adjoint_conservative(snapshots, n_steps, dt, T, basis, mesh, gamma, alpha, n_iter=10, objective="l2_density",
                             solver="pcg", obj_params=None, ctx=None):
    """run_adjoint_conservative (IGR_adjoints_2d/adjoint_pde.jl:527-611):
    the adjoint (a_mux, a_muy, a_rho, a_E) at t = 0, integrated backward over
    the snapshots of run_forward_store (a Snapshots or a list of 5-tuples)."""
    _solver(solver)  # validate before touching the device
    _objective(objective)
    ctx = ctx or default_context()
    shape = mesh.shape(basis)
    n = int(np.prod(shape))
    if not isinstance(snapshots, Snapshots):
        snapshots = Snapshots.from_list(snapshots, shape)
    data = np.ascontiguousarray(snapshots.data, dtype=np.float64)
    out = [np.zeros(n) for _ in range(4)]
    check(ctx, lib().igr2d_run_adjoint_conservative(ctx.handle, C.byref(_disc2d(basis, mesh)), _ptr(data),
                                                    C.c_longlong(data.size), C.c_int(n_steps), C.c_double(dt),
                                                    C.c_double(T), C.c_double(gamma), C.c_double(alpha),
                                                    C.c_int(n_iter), C.c_int(_objective(objective)),
                                                    C.c_int(_solver(solver)), _ptr(_prm(obj_params)),
                                                    *[_ptr(a) for a in out]))
    return tuple(np.asfortranarray(a.reshape(shape, order="F")) for a in out)


def compute_adjoint_rhs_conservative_(damux, damuy, darho, daE, amux, amuy, arho, aE, mux, muy, rho, E, Sigma, Pi,
                                      basis, mesh, gamma, alpha, n_iter=10, solver="pcg", ctx=None):
    """compute_adjoint_rhs_conservative! (IGR_adjoints_2d/adjoint_pde.jl:481-516):
    the adjoint operator applied to a at the state (q, Sigma); Pi is the warm
    start of the Pi solve and holds its result on return (alpha > 0)."""
    _solver(solver)  # validate before touching the device
    ctx = ctx or default_context()
    shape = mesh.shape(basis)
    n = int(np.prod(shape))
    q = [_flat(x, n) for x in (mux, muy, rho, E, Sigma)]
    a = [_flat(x, n) for x in (amux, amuy, arho, aE)]
    P = _flat(Pi, n).copy()
    out = [np.zeros(n) for _ in range(4)]
    check(ctx, lib().igr2d_adjoint_rhs_conservative(ctx.handle, C.byref(_disc2d(basis, mesh)), C.c_double(gamma),
                                                    C.c_double(alpha), C.c_int(n_iter), C.c_int(_solver(solver)),
                                                    *[_ptr(x) for x in q], _ptr(P), *[_ptr(x) for x in a],
                                                    *[_ptr(x) for x in out]))
    for dst, src in zip((damux, damuy, darho, daE), out):
        dst[...] = src.reshape(shape, order="F")
    Pi[...] = P.reshape(shape, order="F")


def adjoint_conservative_ic(mux0, muy0, rho0, E0, dt, T, basis, mesh, gamma, alpha, n_iter=10, solver="pcg",
                            objective="l2_density", obj_params=None, ctx=None):
    """run_forward_store followed by run_adjoint_conservative (as
    IGR_adjoints_2d/tests/run_adjoint_test.jl:59-62 pairs them) with the
    snapshots kept on the GPU; returns (a_mux, a_muy, a_rho, a_E) at t = 0."""
    _solver(solver)  # validate before touching the device
    _objective(objective)
    ctx = ctx or default_context()
    shape = mesh.shape(basis)
    n = int(np.prod(shape))
    q = [_flat(x, n) for x in (mux0, muy0, rho0, E0)]
    out = [np.zeros(n) for _ in range(4)]
    check(ctx, lib().igr2d_adjoint_conservative_ic(ctx.handle, C.byref(_disc2d(basis, mesh)), C.c_double(gamma),
                                                   C.c_double(alpha), C.c_double(dt), C.c_double(T), C.c_int(n_iter),
                                                   C.c_int(_solver(solver)), C.c_int(_objective(objective)),
                                                   _ptr(_prm(obj_params)), *[_ptr(x) for x in q],
                                                   *[_ptr(x) for x in out]))
    return tuple(np.asfortranarray(a.reshape(shape, order="F")) for a in out)


def adjoint_conservative_batch(q0, gammas, alphas, dts, T, basis, mesh, n_iter=10, solver="pcg",
                               objective="l2_density", obj_params=None, ctx=None):
    """Batched adjoint_conservative_ic over instances on one mesh: q0 is
    (n_inst, 4, N) in the Julia node order; returns the adjoints at t = 0 in
    the same layout. ceil(T / dts[i]) must agree across instances."""
    _solver(solver)  # validate before touching the device
    _objective(objective)
    ctx = ctx or default_context()
    gammas = np.ascontiguousarray(gammas, dtype=np.float64)
    alphas = np.ascontiguousarray(alphas, dtype=np.float64)
    dts = np.ascontiguousarray(dts, dtype=np.float64)
    q0 = np.ascontiguousarray(q0, dtype=np.float64)
    a0 = np.zeros_like(q0)
    check(ctx, lib().igr2d_adjoint_conservative_batch(ctx.handle, C.byref(_disc2d(basis, mesh)), C.c_int(gammas.size),
                                                      _ptr(gammas), _ptr(alphas), _ptr(dts), C.c_double(T),
                                                      C.c_int(n_iter), C.c_int(_solver(solver)),
                                                      C.c_int(_objective(objective)), _ptr(_prm(obj_params)), _ptr(q0),
                                                      _ptr(a0)))
    return a0


# ---------------------------------------------------------------------------
# Initial conditions (IGR_adjoints_2d/initial_conditions.jl), built on the GPU
# ---------------------------------------------------------------------------
IC_TYPES = {"constant": 0, "isentropic_vortex": 1, "taylor_green": 2, "sedov_blast": 3, "oseen_pair_blast": 4,
            "multi_blast": 5}


def build_ic_batch(ic_type, basis, mesh, gammas, amps, params=None, device_array=False, ctx=None):
    """Initial states of a batch on one mesh, built on the GPU: (n_inst, 4, N)
    in the Julia node order (numpy, or a torch CUDA tensor with
    device_array=True, the input adjoint_batch(device_arrays=True) takes).
    params: the builder's keyword arguments in the order of include/igr_gb300.h
    (None: the reference's defaults)."""
    key = ic_type.lstrip(":") if isinstance(ic_type, str) else ic_type
    if isinstance(key, str):
        if key not in IC_TYPES:
            raise ValueError("Unknown IC type: %s" % ic_type)
        key = IC_TYPES[key]
    ctx = ctx or default_context()
    gammas = np.ascontiguousarray(np.atleast_1d(np.asarray(gammas, dtype=np.float64)))
    B = gammas.size
    amps = np.ascontiguousarray(np.broadcast_to(np.asarray(amps, dtype=np.float64), (B,)))
    prm = None if params is None else np.ascontiguousarray(np.asarray(params, dtype=np.float64))
    pp = None if prm is None else _ptr(prm)
    n = mesh.x.size
    d = _disc2d(basis, mesh)
    if device_array:
        import torch
        q = torch.empty((B, 4, n), dtype=torch.float64, device="cuda")
        check(ctx, lib().igr2d_build_ic_dev(ctx.handle, C.byref(d), C.c_int(key), C.c_int(B), _ptr(gammas), _ptr(amps),
                                            pp, C.cast(C.c_void_p(q.data_ptr()), _D)))
        return q
    q = np.zeros((B, 4, n))
    check(ctx, lib().igr2d_build_ic(ctx.handle, C.byref(d), C.c_int(key), C.c_int(B), _ptr(gammas), _ptr(amps), pp,
                                    _ptr(q)))
    return q


def _build_one(ic_type, mesh, gamma, A, params, ctx):
    q = build_ic_batch(ic_type, mesh.basis, mesh, [gamma], [A], params, ctx=ctx)[0]
    shape = mesh.shape(mesh.basis)
    return tuple(np.asfortranarray(q[v].reshape(shape, order="F")) for v in range(4))


def init_constant_state(mesh, gamma, rho0=1.0, ux0=1.0, uy0=1.0, p0=1.0, ctx=None):
    """init_constant_state (initial_conditions.jl:15-22): (mux, muy, rho, E)."""
    return _build_one("constant", mesh, gamma, 0.0, [rho0, ux0, uy0, p0], ctx)


def init_isentropic_vortex(mesh, gamma, beta=5.0, ux0=1.0, uy0=1.0, ctx=None):
    """init_isentropic_vortex (initial_conditions.jl:39-67): (mux, muy, rho, E)."""
    return _build_one("isentropic_vortex", mesh, gamma, 0.0, [beta, ux0, uy0], ctx)


def _fill(dst, src):
    for a, b in zip(dst, src):
        a[...] = b


def build_taylor_green_ic_(mux0, muy0, rho0, E0, A, mesh, gamma, ctx=None):
    """build_taylor_green_ic! (initial_conditions.jl:105-121), in place."""
    _fill((mux0, muy0, rho0, E0), _build_one("taylor_green", mesh, gamma, A, None, ctx))


def build_sedov_blast_ic_(mux0, muy0, rho0, E0, A, mesh, gamma, p_bg=1.0, sigma=0.1, ctx=None):
    """build_sedov_blast_ic! (initial_conditions.jl:136-150), in place."""
    _fill((mux0, muy0, rho0, E0), _build_one("sedov_blast", mesh, gamma, A, [p_bg, sigma], ctx))


def build_oseen_pair_blast_ic_(mux0, muy0, rho0, E0, A, mesh, gamma, a_core=0.05, M_star=0.5,
                               vort_centers=((0.45, 0.60, +1), (0.45, 0.40, -1)), blast_xc=0.25, blast_yc=0.50,
                               sigma=0.09, ctx=None):
    """build_oseen_pair_blast_ic! (initial_conditions.jl:175-231), in place
    (two vortices, as the reference's pair)."""
    if len(vort_centers) != 2:
        raise ValueError("vort_centers must hold two (xc, yc, sign) triples")
    prm = [a_core, M_star, blast_xc, blast_yc, sigma] + [float(v) for c in vort_centers for v in c]
    _fill((mux0, muy0, rho0, E0), _build_one("oseen_pair_blast", mesh, gamma, A, prm, ctx))


# IC_BUILDERS and ic_dA_weights of initial_conditions.jl:240-258
IC_BUILDERS = {
    "taylor_green": (build_taylor_green_ic_, "ux=A sin cos, uy=-A cos sin, rho=1, p=1"),
    "sedov_blast": (build_sedov_blast_ic_, "rho=1, u=0, p=p_bg+A exp(-r^2/sigma^2)"),
}


def ic_dA_weights(ic_type):
    """(w_rho, w_ux, w_uy, w_p): which primitive variables carry d/dA."""
    key = ic_type.lstrip(":")
    if key == "taylor_green":
        return (0.0, 1.0, 1.0, 0.0)
    if key == "sedov_blast":
        return (0.0, 0.0, 0.0, 1.0)
    raise ValueError("Unknown IC type: %s" % ic_type)


def l2_error(u, u_ref, basis, mesh, ctx=None):
    """l2_error (initial_conditions.jl:74-87): the LGL-quadrature L2 norm of u - u_ref."""
    ctx = ctx or default_context()
    n = mesh.x.size
    v = C.c_double(0.0)
    check(ctx, lib().igr2d_l2_error(ctx.handle, C.byref(_disc2d(basis, mesh)), _ptr(_flat(u, n)), _ptr(_flat(u_ref, n)),
                                    C.byref(v)))
    return v.value


def forward_batch(q0, gammas, alphas, dts, n_steps, basis, mesh, n_iter=10, solver="pcg", final_solve=True, ctx=None):
    """run_forward! for a batch on one mesh (fixed n_steps; pass dt = T / n_steps
    for run_forward semantics). q0: (n_inst, 4, N). Returns (q (n_inst, 4, N),
    Sigma (n_inst, N))."""
    _solver(solver)  # validate before touching the device
    ctx = ctx or default_context()
    gammas = np.ascontiguousarray(gammas, dtype=np.float64)
    B = gammas.size
    f64 = lambda a: np.ascontiguousarray(np.broadcast_to(np.asarray(a, dtype=np.float64), (B,)))
    als, dtv = f64(alphas), f64(dts)
    q = np.array(q0, dtype=np.float64, order="C", copy=True)
    S = np.zeros((B, q.shape[2]))
    check(ctx, lib().igr2d_forward_batch(ctx.handle, C.byref(_disc2d(basis, mesh)), C.c_int(B), _ptr(gammas), _ptr(als),
                                         _ptr(dtv), C.c_int(n_steps), C.c_int(n_iter), C.c_int(_solver(solver)),
                                         C.c_int(1 if final_solve else 0), _ptr(q), _ptr(S)))
    return q, S
