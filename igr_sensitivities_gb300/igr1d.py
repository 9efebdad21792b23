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

__all__ = ["DGBasis", "PeriodicMesh1D", "run_forward", "run_forward_", "forward_batch"]


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
