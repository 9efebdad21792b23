"""Batched drivers of the reference's optimise-then-discretise (OtD) refinement
studies (IGR_adjoints_2d/paper_scripts/generate_otd_refinement_sedov_data.jl,
generate_otd_refinement_oseen_data.jl): at each mesh resolution, the
directional derivative dJ/dA of an initial-condition amplitude two ways,

  adjoint  <a, dq0/dA>_M   (continuous PDE adjoint at t = 0, M the nodal mass)
  FD       (J(A + eps) - J(A - eps)) / (2 eps)   (central difference of run_forward)

and their relative difference, the OtD gap. The arithmetic runs on the GPU: the
three initial states (A, A + eps, A - eps) are built in one launch, the store +
adjoint runs with device-resident snapshots, both FD forwards advance as one
batch and the objectives are evaluated by the engine; the host forms the
inner product <a, dq0/dA>_M and the difference quotient from the returned
arrays.
"""
import numpy as np

from . import (CartesianMesh2D, DGBasis, adjoint_conservative_batch, build_ic_batch, default_context, forward_batch,
               objective_value)
from .workloads import max_wavespeed_2d


def objective_at(q, objective, basis, mesh, gamma, obj_params=None, ctx=None):
    """J of a state q (4, N) by the engine's nodal quadrature on the GPU (the
    objective tails of IGR_adjoints_2d/enzyme_adjoint.jl:72-229, and
    window_rho2): igr2d_objective with zero steps."""
    shape = mesh.x.shape
    st = [np.asarray(a).reshape(shape, order="F") for a in q]
    return objective_value(*st, 0, 0.0, basis, mesh, gamma, 0.0, n_iter=1, solver="pcg", objective=objective,
                           obj_params=obj_params, ctx=ctx)


def otd_gap(ic_type, A, N_e, p=4, L=1.0, gamma=1.4, T=0.10, CFL=0.4, alpha=3.0 * (1.0 / 20) ** 2, n_iter=60,
            solver="pcg", objective="kinetic_energy", eps=5e-4, params=None, obj_params=None, ctx=None):
    """One resolution of the refinement study: returns (h, gap, adjoint, fd)."""
    ctx = ctx or default_context()
    basis = DGBasis(p)
    mesh = CartesianMesh2D(N_e, N_e, L, L, basis)
    q3 = build_ic_batch(ic_type, basis, mesh, [gamma] * 3, [A, A + eps, A - eps], params=params, ctx=ctx)
    # CFL step from the base state, re-rounded to T (the scripts' `timestep`)
    dt = CFL * min(mesh.dx, mesh.dy) / ((2 * p + 1) * max_wavespeed_2d(*q3[0], gamma))
    dt = T / int(np.ceil(T / dt))
    n_fwd = int(np.ceil(T / dt))  # what run_forward / run_forward_store re-derive from (dt, T)
    a = adjoint_conservative_batch(q3[:1], [gamma], [alpha], [dt], T, basis, mesh, n_iter=n_iter, solver=solver,
                                   objective=objective, obj_params=obj_params, ctx=ctx)[0]
    m = np.tile(np.outer(basis.w, basis.w).reshape(-1, order="F"), N_e * N_e) * mesh.Jx * mesh.Jy
    dq = (q3[1] - q3[2]) / (2 * eps)  # dq0/dA (exact for the builders' affine or quadratic dependence on A)
    adj = float(np.sum(m * np.sum(a * dq, axis=0)))
    qT, _ = forward_batch(q3[1:], [gamma] * 2, [alpha] * 2, [T / n_fwd] * 2, n_fwd, basis, mesh, n_iter=n_iter,
                          solver=solver, final_solve=False, ctx=ctx)
    fd = (objective_at(qT[0], objective, basis, mesh, gamma, obj_params, ctx) -
          objective_at(qT[1], objective, basis, mesh, gamma, obj_params, ctx)) / (2 * eps)
    return L / N_e, abs(adj - fd) / max(abs(fd), 1e-30), adj, fd


def otd_refinement(ic_type, A, N_e_list, csv_path=None, **kw):
    """The refinement sweep: one otd_gap row per resolution, plus the observed
    rates r = log(gap_i-1 / gap_i) / log(h_i-1 / h_i). Writes the scripts' CSV
    (h,gap,adjoint,fd) when csv_path is given."""
    rows = [otd_gap(ic_type, A, n, **kw) for n in N_e_list]
    rates = [float(np.log(rows[i - 1][1] / rows[i][1]) / np.log(rows[i - 1][0] / rows[i][0]))
             for i in range(1, len(rows))]
    if csv_path:
        with open(csv_path, "w") as f:
            f.write("h,gap,adjoint,fd\n")
            for h, g, a, d in rows:
                f.write("%.10e,%.10e,%.10e,%.10e\n" % (h, g, a, d))
    return rows, rates


# The two studies' settings (the scripts' headers).
SEDOV_THREE_BLASTS = dict(ic_type="multi_blast", A=6.0, p=4, T=0.10, CFL=0.4, alpha=3.0 * (1.0 / 20) ** 2, n_iter=60,
                          solver="pcg", objective="kinetic_energy", eps=5e-4,
                          params=[1.0, 0.09, 3, 0.30, 0.34, 6.0, 0.70, 0.40, 5.0, 0.52, 0.74, 5.5, 0, 0, 0])
SEDOV_N_E = [12, 16, 22, 30]
OSEEN_PAIR_BLAST = dict(ic_type="oseen_pair_blast", A=12.0, p=4, T=0.10, CFL=0.4, alpha=3.0 * (1.0 / 20) ** 2,
                        n_iter=60, solver="pcg", objective="windowed_kinetic_energy", eps=1e-3,
                        params=[0.05, 0.5, 0.25, 0.50, 0.09, 0.45, 0.60, 1.0, 0.45, 0.40, -1.0])
OSEEN_N_E = [16, 22, 30, 40, 54, 72]
