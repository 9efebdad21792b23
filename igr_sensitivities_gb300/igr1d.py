"""1D half of the host mirror: the reference's IGRAdjoints1D module API
(f-t-s/IGR_sensitivities, IGR_adjoints_1d) over the C ABI.

Arrays are numpy float64 arrays shaped (n_p, N_e) in Julia column-major node
order (`order="F"`); the state ordering is (mu, rho, E)
(IGR_adjoints_1d/euler.jl:23). All arithmetic runs in the CUDA library.
"""
import ctypes as C

import numpy as np

from . import DGBasis, PeriodicMesh1D, _flat, _ptr, _solver
from ._lib import check, default_context, lib

__all__ = ["DGBasis", "PeriodicMesh1D", "run_forward", "run_forward_", "forward_batch", "run_sensitivity",
           "enzyme_adjoint_ic", "enzyme_dJ_dA", "adjoint_batch", "IC_BUILDERS", "ic_dA_weights",
           "Snapshots1D", "run_forward_store", "run_adjoint_conservative", "compute_adjoint_rhs_conservative_",
           "adjoint_conservative_batch", "build_ic_batch", "IC_TYPES", "apply_sip_", "compute_igr_rhs_",
           "compute_sip_diagonal", "solve_elliptic_", "compute_hyperbolic_rhs_", "compute_igr_euler_rhs_"]


class _Disc1D(C.Structure):
    _fields_ = [("p", C.c_int), ("n_e", C.c_int), ("L", C.c_double), ("xi", C.POINTER(C.c_double)),
                ("w", C.POINTER(C.c_double)), ("D", C.POINTER(C.c_double))]


def _disc1d(basis, mesh):
    D = C.POINTER(C.c_double)
    d = _Disc1D(basis.p, mesh.N_e, mesh.L, basis.xi.ctypes.data_as(D), basis.w.ctypes.data_as(D),
                basis._Dcol.ctypes.data_as(D))
    d._keep = (basis,)
    return d


def _shape(basis, mesh):
    return (basis.n_p, mesh.N_e)


def run_forward_(mu, rho, E, Sigma, dt, T, basis, mesh, gamma, alpha, n_iter=10, solver="pcg", ctx=None):
    """run_forward! (IGR_adjoints_1d/forward.jl:50-87): state updated in place to time T."""
    _solver(solver)  # validate before touching the device
    ctx = ctx or default_context()
    shape = _shape(basis, mesh)
    n = int(np.prod(shape))
    q = [_flat(a, n).copy() for a in (mu, rho, E)]
    S = np.zeros(n)
    check(ctx, lib().igr1d_run_forward(ctx.handle, C.byref(_disc1d(basis, mesh)), C.c_double(gamma), C.c_double(alpha),
                                       C.c_double(dt), C.c_double(T), C.c_int(n_iter), C.c_int(_solver(solver)),
                                       *[_ptr(a) for a in q], _ptr(S)))
    for dst, src in zip((mu, rho, E, Sigma), q + [S]):
        dst[...] = src.reshape(shape, order="F")


def run_forward(mu0, rho0, E0, dt, T, basis, mesh, gamma, alpha, n_iter=10, solver="pcg", ctx=None):
    """run_forward (IGR_adjoints_1d/forward.jl:97-102): returns (mu, rho, E, Sigma) at time T."""
    shape = _shape(basis, mesh)
    out = [np.array(np.asarray(a, dtype=np.float64).reshape(shape, order="F"), order="F") for a in (mu0, rho0, E0)]
    S = np.zeros(shape, order="F")
    run_forward_(*out, S, dt, T, basis, mesh, gamma, alpha, n_iter, solver, ctx)
    return (*out, S)


def forward_batch(states, basis, n_e, L, gammas, alphas, dts, n_steps, n_iter=10, solver="pcg", final_solve=True,
                  ctx=None):
    """Batched fixed-step 1D forward, one CTA per instance in one launch.

    states: list of (mu, rho, E) per instance (flat Julia order, N_i = n_p n_e[i]
    each). Returns the list of final (mu, rho, E, Sigma).
    """
    _solver(solver)  # validate before touching the device
    ctx = ctx or default_context()
    n_e = np.ascontiguousarray(n_e, dtype=np.int32)
    B = n_e.size
    sizes = basis.n_p * n_e
    q = np.concatenate([np.concatenate([_flat(x, int(sizes[i])) for x in states[i]]) for i in range(B)])
    sig = np.zeros(int(sizes.sum()))
    f64 = lambda a: np.ascontiguousarray(np.broadcast_to(np.asarray(a, dtype=np.float64), (B,)))
    i32 = lambda a: np.ascontiguousarray(np.broadcast_to(np.asarray(a, dtype=np.int32), (B,)))
    Ls, gs, als, dtv, ns = f64(L), f64(gammas), f64(alphas), f64(dts), i32(n_steps)
    IP = C.POINTER(C.c_int)
    check(ctx, lib().igr1d_forward_batch(ctx.handle, C.c_int(basis.p), _ptr(basis.xi), _ptr(basis.w), _ptr(basis._Dcol),
                                         C.c_int(B), n_e.ctypes.data_as(IP), _ptr(Ls), _ptr(gs), _ptr(als), _ptr(dtv),
                                         ns.ctypes.data_as(IP), C.c_int(n_iter), C.c_int(_solver(solver)),
                                         C.c_int(1 if final_solve else 0), _ptr(q), _ptr(sig)))
    out, o3, o1 = [], 0, 0
    for i in range(B):
        n = int(sizes[i])
        out.append((q[o3:o3 + n], q[o3 + n:o3 + 2 * n], q[o3 + 2 * n:o3 + 3 * n], sig[o1:o1 + n]))
        o3 += 3 * n
        o1 += n
    return out


# ----------------------------------------------------------------------------- operator-level calls
def apply_sip_(y, x, rho, basis, mesh, alpha, ctx=None):
    """apply_sip! (IGR_adjoints_1d/elliptic.jl:32-116): y = A(rho, alpha) x."""
    ctx = ctx or default_context()
    shape = _shape(basis, mesh)
    n = int(np.prod(shape))
    out = np.zeros(n)
    check(ctx, lib().igr1d_apply_sip(ctx.handle, C.byref(_disc1d(basis, mesh)), C.c_double(alpha), _ptr(_flat(x, n)),
                                     _ptr(_flat(rho, n)), _ptr(out)))
    y[...] = out.reshape(shape, order="F")


def compute_igr_rhs_(b, mu, rho, E, basis, mesh, alpha, ctx=None):
    """compute_igr_rhs! (IGR_adjoints_1d/elliptic.jl:126-154): b = w_i J 2 alpha (d_x u)^2."""
    ctx = ctx or default_context()
    shape = _shape(basis, mesh)
    n = int(np.prod(shape))
    out = np.zeros(n)
    check(ctx, lib().igr1d_igr_rhs(ctx.handle, C.byref(_disc1d(basis, mesh)), C.c_double(alpha),
                                   *[_ptr(_flat(a, n)) for a in (mu, rho, E)], _ptr(out)))
    b[...] = out.reshape(shape, order="F")


def compute_sip_diagonal(rho, basis, mesh, alpha, ctx=None):
    """compute_sip_diagonal (IGR_adjoints_1d/elliptic.jl:206-253): diag(A) as a new array."""
    ctx = ctx or default_context()
    shape = _shape(basis, mesh)
    n = int(np.prod(shape))
    out = np.zeros(n)
    check(ctx, lib().igr1d_sip_diagonal(ctx.handle, C.byref(_disc1d(basis, mesh)), C.c_double(alpha),
                                        _ptr(_flat(rho, n)), _ptr(out)))
    return np.asfortranarray(out.reshape(shape, order="F"))


def solve_elliptic_(Sigma, mu, rho, E, basis, mesh, alpha, n_iter=10, solver="pcg", ctx=None):
    """solve_elliptic! (IGR_adjoints_1d/elliptic.jl:446-467); Sigma is the warm start and the result."""
    _solver(solver)  # validate before touching the device
    ctx = ctx or default_context()
    shape = _shape(basis, mesh)
    n = int(np.prod(shape))
    S = _flat(Sigma, n).copy()
    check(ctx, lib().igr1d_solve_elliptic(ctx.handle, C.byref(_disc1d(basis, mesh)), C.c_double(alpha), C.c_int(n_iter),
                                          C.c_int(_solver(solver)), *[_ptr(_flat(a, n)) for a in (mu, rho, E)],
                                          _ptr(S)))
    Sigma[...] = S.reshape(shape, order="F")


def compute_hyperbolic_rhs_(dmu, drho, dE, mu, rho, E, Sigma, basis, mesh, gamma, ctx=None):
    """compute_hyperbolic_rhs! (IGR_adjoints_1d/hyperbolic.jl:23-83)."""
    ctx = ctx or default_context()
    shape = _shape(basis, mesh)
    n = int(np.prod(shape))
    out = [np.zeros(n) for _ in range(3)]
    check(ctx, lib().igr1d_hyperbolic_rhs(ctx.handle, C.byref(_disc1d(basis, mesh)), C.c_double(gamma),
                                          *[_ptr(_flat(a, n)) for a in (mu, rho, E, Sigma)], *[_ptr(a) for a in out]))
    for dst, src in zip((dmu, drho, dE), out):
        dst[...] = src.reshape(shape, order="F")


def compute_igr_euler_rhs_(dmu, drho, dE, mu, rho, E, Sigma, basis, mesh, gamma, alpha, n_iter=10, solver="pcg",
                           ctx=None):
    """compute_igr_euler_rhs! (IGR_adjoints_1d/forward.jl:17-33): the Sigma solve
    (warm start in Sigma, result out) when alpha > 0, else Sigma = 0; then the
    hyperbolic RHS at (q, Sigma)."""
    _solver(solver)  # validate before touching the device
    ctx = ctx or default_context()
    shape = _shape(basis, mesh)
    n = int(np.prod(shape))
    S = _flat(Sigma, n).copy()
    out = [np.zeros(n) for _ in range(3)]
    check(ctx, lib().igr1d_igr_euler_rhs(ctx.handle, C.byref(_disc1d(basis, mesh)), C.c_double(gamma),
                                         C.c_double(alpha), C.c_int(n_iter), C.c_int(_solver(solver)),
                                         *[_ptr(_flat(a, n)) for a in (mu, rho, E)], _ptr(S), *[_ptr(a) for a in out]))
    for dst, src in zip((dmu, drho, dE), out):
        dst[...] = src.reshape(shape, order="F")
    Sigma[...] = S.reshape(shape, order="F")


# ----------------------------------------------------------------------------- initial conditions
def _ic(rho_fn, u_fn, p_fn):
    def build(mu0, rho0, E0, A, mesh_x, L, gamma):
        s = np.sin(2 * np.pi * np.asarray(mesh_x) / L)
        rho, u, p = rho_fn(A, s), u_fn(A, s), p_fn(A, s)
        rho0[...] = rho
        mu0[...] = rho * u
        E0[...] = p / (gamma - 1) + 0.5 * rho * u ** 2
    return build


_one = lambda A, s: np.ones_like(s)
_zero = lambda A, s: np.zeros_like(s)
_pert = lambda A, s: 1 + A * s
# IC_BUILDERS of IGR_adjoints_1d/initial_conditions.jl:218-224 (builders :94-204)
IC_BUILDERS = {
    "acoustic_pulse": (_ic(_pert, lambda A, s: A * s, _pert), "rho=1+A sin, u=A sin, p=1+A sin"),
    "entropy_wave": (_ic(_pert, _one, _one), "rho=1+A sin, u=1, p=1"),
    "density_pulse": (_ic(_pert, _zero, _one), "rho=1+A sin, u=0, p=1"),
    "pressure_pulse": (_ic(_one, _zero, _pert), "rho=1, u=0, p=1+A sin"),
    "velocity_pulse": (_ic(_one, lambda A, s: A * s, _one), "rho=1, u=A sin, p=1"),
}


def ic_dA_weights(ic_type):
    """ic_dA_weights (initial_conditions.jl:232-246)."""
    w = {"acoustic_pulse": (1.0, 1.0, 1.0), "entropy_wave": (1.0, 0.0, 0.0), "density_pulse": (1.0, 0.0, 0.0),
         "pressure_pulse": (0.0, 0.0, 1.0), "velocity_pulse": (0.0, 1.0, 0.0)}
    key = ic_type.lstrip(":")
    if key not in w:
        raise ValueError("Unknown IC type: %s" % ic_type)
    return w[key]


# ----------------------------------------------------------------------------- tangent
def run_sensitivity(mu0, rho0, E0, smu0, srho0, sE0, dt, T, basis, mesh, gamma, alpha, n_iter=10, elliptic_rhs="form2",
                    solver="pcg", s_gamma=0.0, ctx=None):
    """run_sensitivity (IGR_adjoints_1d/sensitivity.jl:475-515): returns
    (mu, rho, E, Sigma, smu, srho, sE, sSigma) at time T."""
    _solver(solver)  # validate before touching the device
    form = {"form1": 1, "form2": 2}.get(str(elliptic_rhs).lstrip(":"))
    if form is None:
        raise ValueError("Unknown elliptic_rhs: %s (use :form1 or :form2)" % elliptic_rhs)
    ctx = ctx or default_context()
    shape = _shape(basis, mesh)
    n = int(np.prod(shape))
    q = [_flat(a, n).copy() for a in (mu0, rho0, E0)]
    s = [_flat(a, n).copy() for a in (smu0, srho0, sE0)]
    S, V = np.zeros(n), np.zeros(n)
    check(ctx, lib().igr1d_run_sensitivity(ctx.handle, C.byref(_disc1d(basis, mesh)), C.c_double(gamma),
                                           C.c_double(alpha), C.c_double(dt), C.c_double(T), C.c_int(n_iter),
                                           C.c_int(_solver(solver)), C.c_int(form), C.c_double(s_gamma),
                                           *[_ptr(a) for a in q], _ptr(S), *[_ptr(a) for a in s], _ptr(V)))
    r = lambda a: np.asfortranarray(a.reshape(shape, order="F"))
    return tuple(r(a) for a in q) + (r(S),) + tuple(r(a) for a in s) + (r(V),)


# ----------------------------------------------------------------------------- adjoint
_OBJ1 = {"l2_density": 0, "l2_pressure": 1, "kinetic_energy": 2, "weighted_momentum": 4, "interval_rho": 6}


def adjoint_batch(states, basis, n_e, L, gammas, alphas, dts, n_steps, n_iter=10, solver="pcg", objective="l2_density",
                  obj_params=None, ctx=None):
    """Batched discrete adjoint in conservative variables, one CTA per instance.

    states: list of (mu0, rho0, E0) (flat Julia order). Returns
    (J[n], [(dmu0, drho0, dE0)], dgamma[n], dalpha[n]).
    """
    _solver(solver)  # validate before touching the device
    obj = objective.lstrip(":") if isinstance(objective, str) else objective
    if isinstance(obj, str):
        if obj not in _OBJ1:
            raise ValueError("Unknown objective: %s" % objective)
        obj = _OBJ1[obj]
    ctx = ctx or default_context()
    n_e = np.ascontiguousarray(n_e, dtype=np.int32)
    B = n_e.size
    sizes = basis.n_p * n_e
    q = np.concatenate([np.concatenate([_flat(x, int(sizes[i])) for x in states[i]]) for i in range(B)])
    dq = np.zeros_like(q)
    f64 = lambda a: np.ascontiguousarray(np.broadcast_to(np.asarray(a, dtype=np.float64), (B,)))
    i32 = lambda a: np.ascontiguousarray(np.broadcast_to(np.asarray(a, dtype=np.int32), (B,)))
    Ls, gs, als, dtv, ns = f64(L), f64(gammas), f64(alphas), f64(dts), i32(n_steps)
    J, dg, da = np.zeros(B), np.zeros(B), np.zeros(B)
    prm = np.zeros(4) if obj_params is None else np.ascontiguousarray(np.resize(np.asarray(obj_params, np.float64), 4))
    IP = C.POINTER(C.c_int)
    check(ctx, lib().igr1d_adjoint_batch(ctx.handle, C.c_int(basis.p), _ptr(basis.xi), _ptr(basis.w), _ptr(basis._Dcol),
                                         C.c_int(B), n_e.ctypes.data_as(IP), _ptr(Ls), _ptr(gs), _ptr(als), _ptr(dtv),
                                         ns.ctypes.data_as(IP), C.c_int(n_iter), C.c_int(_solver(solver)), C.c_int(obj),
                                         _ptr(prm), _ptr(q), _ptr(J), _ptr(dq), _ptr(dg), _ptr(da)))
    out, o3 = [], 0
    for i in range(B):
        n = int(sizes[i])
        out.append((dq[o3:o3 + n], dq[o3 + n:o3 + 2 * n], dq[o3 + 2 * n:o3 + 3 * n]))
        o3 += 3 * n
    return J, out, dg, da


def enzyme_adjoint_ic(A, p, N_e, L, gamma, alpha, CFL, T, n_iter=10, ic_type="acoustic_pulse", solver="pcg",
                      objective="l2_density", ctx=None):
    """enzyme_adjoint_ic (IGR_adjoints_1d/enzyme_adjoint.jl:267-314).

    Builds the initial condition of family `ic_type` with amplitude A, runs
    n_steps = ceil(T / dt) steps of dt = T / n_steps (dt from the CFL rule
    CFL dx / ((2p+1) 2.5)), and returns (J, adj_rho, adj_u, adj_p): the
    gradient of J with respect to the primitive initial state.
    """
    obj = objective.lstrip(":")
    if obj not in ("l2_density", "l2_pressure"):
        raise ValueError("Unknown objective: %s (use :l2_density or :l2_pressure)" % objective)
    key = ic_type.lstrip(":")
    if key not in IC_BUILDERS:
        raise ValueError("Unknown IC type: %s" % ic_type)
    basis = DGBasis(p)
    mesh = PeriodicMesh1D(N_e, L, basis)
    dt = CFL * mesh.dx / ((2 * p + 1) * 2.5)
    n_steps = int(np.ceil(T / dt))
    dt = T / n_steps
    shape = (basis.n_p, N_e)
    mu0, rho0, E0 = np.zeros(shape, order="F"), np.zeros(shape, order="F"), np.zeros(shape, order="F")
    IC_BUILDERS[key][0](mu0, rho0, E0, A, mesh.x, L, gamma)
    J, dq, _, _ = adjoint_batch([(mu0, rho0, E0)], basis, [N_e], L, gamma, alpha, dt, n_steps, n_iter=max(n_iter, 1),
                                solver=solver, objective=obj, ctx=ctx)
    dmu, drho, dE = (a.reshape(shape, order="F") for a in dq[0])
    u0 = mu0 / rho0
    adj_rho = drho + u0 * dmu + (u0 ** 2 / 2) * dE
    adj_u = rho0 * dmu + rho0 * u0 * dE
    adj_p = dE / (gamma - 1)
    return J[0], adj_rho, adj_u, adj_p


def enzyme_dJ_dA(A0, p, N_e, L, gamma, alpha, CFL, T, n_iter=10, ic_type="acoustic_pulse", solver="pcg", ctx=None):
    """enzyme_dJ_dA (IGR_adjoints_1d/enzyme_adjoint.jl:232-248): (J, dJ/dA)."""
    J, ar, au, ap = enzyme_adjoint_ic(A0, p, N_e, L, gamma, alpha, CFL, T, n_iter=n_iter, ic_type=ic_type, solver=solver,
                                      ctx=ctx)
    basis = DGBasis(p)
    mesh = PeriodicMesh1D(N_e, L, basis)
    wr, wu, wp = ic_dA_weights(ic_type)
    s = np.sin(2 * np.pi * mesh.x / L)
    return J, float(np.sum((wr * ar + wu * au + wp * ap) * s))


# ---------------------------------------------------------------------------
# Continuous adjoint (IGR_adjoints_1d/adjoint_pde.jl, forward.jl:137-186)
# ---------------------------------------------------------------------------
def _obj1(objective):
    obj = objective.lstrip(":") if isinstance(objective, str) else objective
    if isinstance(obj, str):
        if obj not in _OBJ1:
            raise ValueError("Unknown objective: %s (use :l2_density, :l2_pressure, or :kinetic_energy)" % objective)
        obj = _OBJ1[obj]
    return obj


class Snapshots1D:
    """The snapshot list of run_forward_store (forward.jl:137-186):
    snapshots[k] = (mu, rho, E, Sigma) after step k, each (n_p, N_e) in Julia
    order; `data` is the flat (n_steps + 1, 4, N) buffer of the C ABI."""

    def __init__(self, data, shape):
        self.data = data
        self.shape = tuple(shape)

    def __len__(self):
        return self.data.shape[0]

    def __getitem__(self, k):
        return tuple(self.data[k, v].reshape(self.shape, order="F") for v in range(4))

    @classmethod
    def from_list(cls, snaps, shape):
        n = int(np.prod(shape))
        return cls(np.ascontiguousarray(np.stack([np.stack([_flat(a, n) for a in s]) for s in snaps])), shape)


def run_forward_store(mu0, rho0, E0, dt, T, basis, mesh, gamma, alpha, n_iter=10, solver="pcg", ctx=None):
    """run_forward_store (IGR_adjoints_1d/forward.jl:137-186): (snapshots, n_steps)."""
    _solver(solver)  # validate before touching the device
    ctx = ctx or default_context()
    shape = _shape(basis, mesh)
    n = int(np.prod(shape))
    if not (dt > 0 and T > 0):
        raise ValueError("dt and T must be positive")
    steps = int(np.ceil(T / dt))
    data = np.zeros((steps + 1, 4, n))
    ns = C.c_int(0)
    q = [_flat(a, n) for a in (mu0, rho0, E0)]
    check(ctx, lib().igr1d_run_forward_store(ctx.handle, C.byref(_disc1d(basis, mesh)), C.c_double(gamma),
                                             C.c_double(alpha), C.c_double(dt), C.c_double(T), C.c_int(n_iter),
                                             C.c_int(_solver(solver)), *[_ptr(a) for a in q], _ptr(data),
                                             C.c_longlong(data.size), C.byref(ns)))
    return Snapshots1D(data, shape), ns.value


def run_adjoint_conservative(snapshots, n_steps, dt, T, basis, mesh, gamma, alpha, n_iter=10, objective="l2_density",
                             solver="pcg", obj_params=None, ctx=None):
    """run_adjoint_conservative (IGR_adjoints_1d/adjoint_pde.jl:474-551):
    (a_mu, a_rho, a_E) at t = 0 from the snapshots of run_forward_store."""
    _solver(solver)  # validate before touching the device
    obj = _obj1(objective)
    ctx = ctx or default_context()
    shape = _shape(basis, mesh)
    n = int(np.prod(shape))
    if not isinstance(snapshots, Snapshots1D):
        snapshots = Snapshots1D.from_list(snapshots, shape)
    data = np.ascontiguousarray(snapshots.data, dtype=np.float64)
    prm = np.zeros(4) if obj_params is None else np.ascontiguousarray(np.resize(np.asarray(obj_params, np.float64), 4))
    out = [np.zeros(n) for _ in range(3)]
    check(ctx, lib().igr1d_run_adjoint_conservative(ctx.handle, C.byref(_disc1d(basis, mesh)), _ptr(data),
                                                    C.c_longlong(data.size), C.c_int(n_steps), C.c_double(dt),
                                                    C.c_double(T), C.c_double(gamma), C.c_double(alpha),
                                                    C.c_int(n_iter), C.c_int(obj), C.c_int(_solver(solver)), _ptr(prm),
                                                    *[_ptr(a) for a in out]))
    return tuple(np.asfortranarray(a.reshape(shape, order="F")) for a in out)


def compute_adjoint_rhs_conservative_(damu, darho, daE, amu, arho, aE, mu, rho, E, Sigma, Pi, basis, mesh, gamma, alpha,
                                      n_iter=10, solver="pcg", ctx=None):
    """compute_adjoint_rhs_conservative! (IGR_adjoints_1d/adjoint_pde.jl:410-456):
    in place; Pi is the warm start and returns the new Pi (alpha > 0)."""
    _solver(solver)  # validate before touching the device
    ctx = ctx or default_context()
    shape = _shape(basis, mesh)
    n = int(np.prod(shape))
    q = [_flat(x, n) for x in (mu, rho, E, Sigma)]
    a = [_flat(x, n) for x in (amu, arho, aE)]
    P = _flat(Pi, n).copy()
    out = [np.zeros(n) for _ in range(3)]
    check(ctx, lib().igr1d_adjoint_rhs_conservative(ctx.handle, C.byref(_disc1d(basis, mesh)), C.c_double(gamma),
                                                    C.c_double(alpha), C.c_int(n_iter), C.c_int(_solver(solver)),
                                                    *[_ptr(x) for x in q], _ptr(P), *[_ptr(x) for x in a],
                                                    *[_ptr(x) for x in out]))
    for dst, src in zip((damu, darho, daE), out):
        dst[...] = src.reshape(shape, order="F")
    Pi[...] = P.reshape(shape, order="F")


def adjoint_conservative_batch(states, basis, n_e, L, gammas, alphas, dts, T, n_iter=10, solver="pcg",
                               objective="l2_density", obj_params=None, ctx=None):
    """run_forward_store + run_adjoint_conservative for a batch of 1D instances
    in one launch (snapshots on the device). states: list of (mu0, rho0, E0);
    dts and T per instance (scalars broadcast). Returns [(a_mu, a_rho, a_E)]."""
    _solver(solver)  # validate before touching the device
    obj = _obj1(objective)
    ctx = ctx or default_context()
    n_e = np.ascontiguousarray(n_e, dtype=np.int32)
    B = n_e.size
    sizes = basis.n_p * n_e
    q = np.concatenate([np.concatenate([_flat(x, int(sizes[i])) for x in states[i]]) for i in range(B)])
    a0 = np.zeros_like(q)
    f64 = lambda a: np.ascontiguousarray(np.broadcast_to(np.asarray(a, dtype=np.float64), (B,)))
    Ls, gs, als, dtv, Ts = f64(L), f64(gammas), f64(alphas), f64(dts), f64(T)
    prm = np.zeros(4) if obj_params is None else np.ascontiguousarray(np.resize(np.asarray(obj_params, np.float64), 4))
    check(ctx, lib().igr1d_adjoint_conservative_batch(ctx.handle, C.c_int(basis.p), _ptr(basis.xi), _ptr(basis.w),
                                                      _ptr(basis._Dcol), C.c_int(B),
                                                      n_e.ctypes.data_as(C.POINTER(C.c_int)), _ptr(Ls), _ptr(gs),
                                                      _ptr(als), _ptr(dtv), _ptr(Ts), C.c_int(n_iter),
                                                      C.c_int(_solver(solver)), C.c_int(obj), _ptr(prm), _ptr(q),
                                                      _ptr(a0)))
    out, o3 = [], 0
    for i in range(B):
        n = int(sizes[i])
        out.append((a0[o3:o3 + n], a0[o3 + n:o3 + 2 * n], a0[o3 + 2 * n:o3 + 3 * n]))
        o3 += 3 * n
    return out


IC_TYPES = {"acoustic_pulse": 0, "entropy_wave": 1, "density_pulse": 2, "pressure_pulse": 3, "velocity_pulse": 4}


def build_ic_batch(ic_type, basis, n_e, L, gammas, amps, ctx=None):
    """The IC_BUILDERS of IGR_adjoints_1d/initial_conditions.jl:94-224 for a
    batch of instances (own n_e, L, gamma, amplitude A), built on the GPU.
    Returns [(mu0, rho0, E0)] (flat, Julia order), the input adjoint_batch and
    adjoint_conservative_batch take."""
    key = ic_type.lstrip(":") if isinstance(ic_type, str) else ic_type
    if isinstance(key, str):
        if key not in IC_TYPES:
            raise ValueError("Unknown IC type: %s" % ic_type)
        key = IC_TYPES[key]
    ctx = ctx or default_context()
    n_e = np.ascontiguousarray(np.atleast_1d(n_e), dtype=np.int32)
    B = n_e.size
    f64 = lambda a: np.ascontiguousarray(np.broadcast_to(np.asarray(a, dtype=np.float64), (B,)))
    Ls, gs, As = f64(L), f64(gammas), f64(amps)
    sizes = basis.n_p * n_e
    q = np.zeros(3 * int(sizes.sum()))
    check(ctx, lib().igr1d_build_ic(ctx.handle, C.c_int(basis.p), _ptr(basis.xi), _ptr(basis.w), _ptr(basis._Dcol),
                                    C.c_int(B), n_e.ctypes.data_as(C.POINTER(C.c_int)), _ptr(Ls), C.c_int(key), _ptr(gs),
                                    _ptr(As), _ptr(q)))
    out, o3 = [], 0
    for i in range(B):
        n = int(sizes[i])
        out.append((q[o3:o3 + n], q[o3 + n:o3 + 2 * n], q[o3 + 2 * n:o3 + 3 * n]))
        o3 += 3 * n
    return out
