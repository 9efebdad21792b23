"""GPU parity tests of the 2D continuous adjoint (run_forward_store,
IGR_adjoints_2d/forward.jl:111-158; run_adjoint_conservative and
compute_adjoint_rhs_conservative!, IGR_adjoints_2d/adjoint_pde.jl:481-611)
against the CPU oracle, through the C ABI.

Tolerance: field-wise relative L2 <= 1e-11 against the oracle (IEEE FP64,
different association and FMA contraction). Paths that run the same kernels
in the same order (fused vs two calls, checkpointed vs resident snapshots,
batched vs single) are compared bitwise. The reference's own check of this
path (IGR_adjoints_2d/tests/run_adjoint_test.jl:72: PDE adjoint within 0.2
of the discrete gradient divided by the nodal mass) runs on GPU results."""
import numpy as np
import pytest

from igr_sensitivities_gb300 import workloads as W

pytestmark = pytest.mark.gpu

RTOL = 1e-11


def rel(a, b):
    a = np.asarray(a).reshape(-1, order="F")
    b = np.asarray(b).reshape(-1, order="F")
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def flat(a):
    return np.ascontiguousarray(np.asarray(a).reshape(-1, order="F"))


def tg_case(igr, oracle, p, ne, g=1.4, A=0.4, cfl=0.4, T=0.06):
    """The reference test's setup (run_adjoint_test.jl:15-44): Taylor-Green,
    dt = CFL min(dx, dy) / ((2p+1) max wave speed), re-rounded to T."""
    basis = igr.DGBasis(p)
    mesh = igr.CartesianMesh2D(ne, ne, 1.0, 1.0, basis)
    G = oracle.Grid2D(p, ne, ne)
    q0 = W.taylor_green_ic(mesh, g, A)
    dt = W.cfl_dt_2d(mesh, p, q0, g, cfl)
    n = int(np.ceil(T / dt))
    return basis, mesh, G, q0, T / n, T, n


def pulse_case(igr, oracle, p, ne, seed, g=1.4):
    basis = igr.DGBasis(p)
    mesh = igr.CartesianMesh2D(ne, ne, 1.0, 1.0, basis)
    G = oracle.Grid2D(p, ne, ne)
    q0 = W.seeded_pulses_2d(mesh, g, W.seed_for(2, seed), width=0.12)
    rng = np.random.default_rng(seed)
    q0 = tuple(np.asfortranarray(a + 0.02 * rng.standard_normal(a.shape) * (v < 2)) for v, a in enumerate(q0))
    dt = W.cfl_dt_2d(mesh, p, q0, g, 0.1)
    return basis, mesh, G, q0, dt


@pytest.mark.parametrize("p,ne,alpha,solver,n_iter", [
    (3, 6, 0.0, "pcg", 1), (3, 6, 0.05, "pcg", 8), (3, 5, 0.05, "chebyshev", 5), (3, 6, 0.05, "jacobi", 4),
    (2, 6, 0.03, "pcg", 6), (4, 4, 0.05, "chebyshev", 5), (1, 8, 0.05, "pcg", 6),
])
def test_adjoint_rhs_matches_oracle(igr, oracle, p, ne, alpha, solver, n_iter):
    g = 1.4
    basis, mesh, G, q0, _ = pulse_case(igr, oracle, p, ne, 3 + p)
    rng = np.random.default_rng(11 + p)
    Sig = np.asfortranarray(0.05 * rng.standard_normal(mesh.x.shape))
    a = [np.asfortranarray(rng.standard_normal(mesh.x.shape)) for _ in range(4)]
    Pi = np.asfortranarray(0.01 * rng.standard_normal(mesh.x.shape))
    da = [np.zeros(mesh.x.shape, order="F") for _ in range(4)]
    Pg = Pi.copy(order="F")
    igr.compute_adjoint_rhs_conservative_(*da, *a, *q0, Sig, Pg, basis, mesh, g, alpha, n_iter=n_iter, solver=solver)
    ref, Pr = oracle.adjoint_rhs_conservative_2d(G, g, alpha, n_iter, solver, [flat(x) for x in q0], flat(Sig),
                                                 flat(Pi), [flat(x) for x in a])
    for x, y in zip(da, ref):
        assert rel(x, y) <= RTOL
    assert rel(Pg, Pr) <= RTOL


@pytest.mark.parametrize("alpha,solver,n_iter", [(0.0, "pcg", 1), (0.05, "pcg", 8), (0.05, "chebyshev", 5),
                                                 (0.05, "jacobi", 4)])
def test_run_forward_store_matches_oracle(igr, oracle, alpha, solver, n_iter):
    g = 1.4
    basis, mesh, G, q0, dt = pulse_case(igr, oracle, 3, 6, 7)
    T = 9.5 * dt
    snaps, n = igr.run_forward_store(*q0, dt, T, basis, mesh, g, alpha, n_iter=n_iter, solver=solver)
    ref, nr = oracle.run_forward_store_2d(G, g, alpha, dt, T, n_iter, solver, [flat(x) for x in q0])
    assert n == nr == 10 and len(snaps) == n + 1
    for k in range(n + 1):
        for v in range(5):
            if v == 4 and alpha == 0:
                assert np.all(snaps.data[k, v] == 0)
            else:
                assert rel(snaps.data[k, v], ref[k, v]) <= RTOL, (k, v)


@pytest.mark.parametrize("objective,alpha,solver,n_iter", [
    ("l2_density", 0.0, "chebyshev", 1), ("l2_density", 1.5e-3, "chebyshev", 30),
    ("weighted_momentum", 1.5e-3, "pcg", 10), ("kinetic_energy", 1.5e-3, "jacobi", 6),
    ("l2_pressure", 1.5e-3, "chebyshev", 10), ("windowed_kinetic_energy", 0.0, "pcg", 1),
    ("window_rho2", 1.5e-3, "pcg", 10),
])
def test_run_adjoint_conservative_matches_oracle(igr, oracle, objective, alpha, solver, n_iter):
    g = 1.4
    basis, mesh, G, q0, dt, T, n = tg_case(igr, oracle, 3, 6)
    prm = (0.3, 0.25, 0.35)
    snaps, ns = igr.run_forward_store(*q0, dt, T, basis, mesh, g, alpha, n_iter=n_iter, solver=solver)
    a = igr.run_adjoint_conservative(snaps, ns, dt, T, basis, mesh, g, alpha, n_iter=n_iter, objective=objective,
                                     solver=solver, obj_params=prm)
    ref_s, _ = oracle.run_forward_store_2d(G, g, alpha, dt, T, n_iter, solver, [flat(x) for x in q0])
    ref = oracle.run_adjoint_conservative_2d(G, ref_s, ns, dt, T, g, alpha, n_iter, objective, solver, prm)
    for x, y in zip(a, ref):
        if np.linalg.norm(y) == 0:
            assert np.all(x == 0)
        else:
            assert rel(x, y) <= RTOL, objective
    # fed the oracle's snapshots, the GPU adjoint agrees as well
    a2 = igr.run_adjoint_conservative(igr.Snapshots(ref_s, mesh.shape(basis)), ns, dt, T, basis, mesh, g, alpha,
                                      n_iter=n_iter, objective=objective, solver=solver, obj_params=prm)
    for x, y in zip(a2, ref):
        assert rel(x, y) <= RTOL or np.linalg.norm(y) == 0


def test_fused_equals_two_calls_and_checkpointing_is_exact(igr, oracle):
    """adjoint_conservative_ic (device-resident snapshots) == run_forward_store
    + run_adjoint_conservative bitwise; with a memory budget that forces
    sqrt(n)-step segments (forward recomputed from checkpoints) and per-step
    snapshot transfers in the host-array calls, still bitwise."""
    g, alpha, nit = 1.4, 1.5e-3, 8
    basis, mesh, G, q0, dt, T, n = tg_case(igr, oracle, 3, 8)
    ref = igr.adjoint_conservative_ic(*q0, dt, T, basis, mesh, g, alpha, n_iter=nit, solver="pcg")
    ctx = igr.default_context()
    assert ctx.last_adjoint_plan()["segments"] == 1
    snaps, ns = igr.run_forward_store(*q0, dt, T, basis, mesh, g, alpha, n_iter=nit, solver="pcg")
    two = igr.run_adjoint_conservative(snaps, ns, dt, T, basis, mesh, g, alpha, n_iter=nit, solver="pcg")
    for x, y in zip(two, ref):
        assert np.array_equal(x, y)
    N = mesh.x.size
    ctx.set_tape_budget(8 * 5 * N * 12)  # room for 12 snapshots of n = 14 + 1
    try:
        seg = igr.adjoint_conservative_ic(*q0, dt, T, basis, mesh, g, alpha, n_iter=nit, solver="pcg")
        plan = ctx.last_adjoint_plan()
        K, nseg = plan["steps_per_segment"], plan["segments"]
        assert nseg > 1 and K * nseg >= n
        snaps2, _ = igr.run_forward_store(*q0, dt, T, basis, mesh, g, alpha, n_iter=nit, solver="pcg")
        two2 = igr.run_adjoint_conservative(snaps2, ns, dt, T, basis, mesh, g, alpha, n_iter=nit, solver="pcg")
    finally:
        ctx.set_tape_budget(0)
    assert np.array_equal(snaps2.data, snaps.data)
    for x, y, z in zip(seg, two2, ref):
        assert np.array_equal(x, z) and np.array_equal(y, z)


def test_batch_equals_single_calls(igr, oracle):
    """Instances on one mesh with their own gamma, alpha, dt (same step count)
    advance together bitwise as they do alone; the kinetic-energy objective
    exercises the per-instance sums of the terminal condition."""
    p, ne, nit, T = 3, 6, 6, 0.03
    basis = igr.DGBasis(p)
    mesh = igr.CartesianMesh2D(ne, ne, 1.0, 1.0, basis)
    gam = [1.4, 1.3, 1.6]
    als = [1.5e-3, 2e-3, 1e-3]
    q0 = np.stack([np.stack([flat(x) for x in W.taylor_green_ic(mesh, g, 0.3 + 0.1 * b)]) for b, g in enumerate(gam)])
    dts = [T / 7, T / 7 * 1.01, T / 7 * 1.05]  # ceil(T / dt) = 7 for all three
    for obj in ("kinetic_energy", "l2_density"):
        a0 = igr.adjoint_conservative_batch(q0, gam, als, dts, T, basis, mesh, n_iter=nit, solver="pcg", objective=obj)
        shape = mesh.shape(basis)
        for b in range(3):
            one = igr.adjoint_conservative_ic(*[q0[b, v].reshape(shape, order="F") for v in range(4)], dts[b], T, basis,
                                              mesh, gam[b], als[b], n_iter=nit, solver="pcg", objective=obj)
            for v in range(4):
                assert np.array_equal(a0[b, v], flat(one[v]))
    with pytest.raises(igr._lib.IGRError):
        igr.adjoint_conservative_batch(q0, gam, als, [T / 7, T / 9, T / 7], T, basis, mesh, n_iter=nit)


@pytest.mark.parametrize("objective", ["l2_density", "weighted_momentum", "kinetic_energy"])
@pytest.mark.parametrize("alpha", [0.0, 1.5e-3])
def test_pde_adjoint_within_otd_gap_of_discrete_gradient(igr, oracle, objective, alpha):
    """IGR_adjoints_2d/tests/run_adjoint_test.jl:15-78 on GPU results: p = 3,
    N_e = 8, T = 0.06, Taylor-Green A = 0.4, CFL 0.4, Chebyshev, n_iter = 100
    (alpha > 0) or 1; the discrete gradient (enzyme_adjoint_ic) divided by the
    nodal mass against the PDE adjoint, combined relative L2 < 0.2."""
    g = 1.4
    basis, mesh, G, q0, dt, T, n = tg_case(igr, oracle, 3, 8)
    nit = 100 if alpha > 0 else 1
    J, *dq = igr.enzyme_adjoint_ic(*q0, n, dt, basis, mesh, g, alpha, n_iter=nit, solver="chebyshev",
                                   objective=objective)
    m = np.outer(basis.w, basis.w)[:, :, None, None] * mesh.Jx * mesh.Jy
    enz = np.concatenate([flat(d / m) for d in dq])
    pde = igr.adjoint_conservative_ic(*q0, dt, T, basis, mesh, g, alpha, n_iter=nit, solver="chebyshev",
                                      objective=objective)
    gap = rel(np.concatenate([flat(x) for x in pde]), enz)
    assert gap < 0.2
    snaps, _ = oracle.run_forward_store_2d(G, g, alpha, dt, T, nit, "chebyshev", [flat(x) for x in q0])
    ref = oracle.run_adjoint_conservative_2d(G, snaps, n, dt, T, g, alpha, nit, objective, "chebyshev")
    assert rel(np.concatenate([flat(x) for x in pde]), np.concatenate(ref)) <= RTOL
