"""GPU parity tests of the 1D continuous adjoint (run_forward_store,
IGR_adjoints_1d/forward.jl:137-186; run_adjoint_conservative and
compute_adjoint_rhs_conservative!, IGR_adjoints_1d/adjoint_pde.jl:410-551)
against the CPU oracle, through the C ABI.

Tolerance: field-wise relative L2 <= 1e-11 against the oracle. Paths that run
the same arithmetic (fused vs two calls, checkpointed vs resident snapshots,
batch vs single instance) are compared bitwise. The reference's own check
(IGR_adjoints_1d/tests/run_adjoint_conservative_test.jl: dJ/dA from the
adjoint vs central differences, 1e-2 at alpha = 0, 5e-2 at alpha > 0) runs on
GPU results."""
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


def case(igr, oracle, p, ne, seed, g=1.4):
    basis = igr.DGBasis(p)
    mesh = igr.PeriodicMesh1D(ne, 1.0, basis)
    G = oracle.Grid1D(p, ne)
    q0 = W.seeded_pulses_1d(mesh, g, W.seed_for(1, seed), n_pulses=2, width=0.08)
    dt = W.cfl_dt_1d(mesh, p, q0, g, 0.1)
    return basis, mesh, G, q0, dt


@pytest.mark.parametrize("p,ne,alpha,solver,n_iter", [
    (3, 12, 0.0, "pcg", 1), (3, 12, 0.01, "pcg", 10), (3, 10, 0.01, "chebyshev", 5), (3, 12, 0.01, "jacobi", 6),
    (2, 16, 0.005, "pcg", 8), (4, 8, 0.01, "pcg", 8), (1, 20, 0.01, "chebyshev", 5),
])
def test_adjoint_rhs_matches_oracle(igr, oracle, p, ne, alpha, solver, n_iter):
    from igr_sensitivities_gb300 import igr1d
    g = 1.4
    basis, mesh, G, q0, _ = case(igr, oracle, p, ne, 3 + p)
    rng = np.random.default_rng(5 + p)
    shp = mesh.x.shape
    Sig = np.asfortranarray(0.05 * rng.standard_normal(shp))
    a = [np.asfortranarray(rng.standard_normal(shp)) for _ in range(3)]
    Pi = np.asfortranarray(0.01 * rng.standard_normal(shp))
    da = [np.zeros(shp, order="F") for _ in range(3)]
    Pg = Pi.copy(order="F")
    igr1d.compute_adjoint_rhs_conservative_(*da, *a, *q0, Sig, Pg, basis, mesh, g, alpha, n_iter=n_iter, solver=solver)
    ref, Pr = oracle.adjoint_rhs_conservative_1d(G, g, alpha, n_iter, solver, [flat(x) for x in q0], flat(Sig), flat(Pi),
                                                 [flat(x) for x in a])
    for x, y in zip(da, ref):
        assert rel(x, y) <= RTOL
    if alpha > 0:
        assert rel(Pg, Pr) <= RTOL


@pytest.mark.parametrize("objective,alpha,solver,n_iter", [
    ("l2_density", 0.0, "pcg", 1), ("l2_density", 0.01, "pcg", 10), ("l2_pressure", 0.01, "chebyshev", 5),
    ("kinetic_energy", 0.01, "jacobi", 6), ("weighted_momentum", 0.005, "pcg", 8), ("interval_rho", 0.01, "pcg", 8),
])
def test_store_and_adjoint_match_oracle(igr, oracle, objective, alpha, solver, n_iter):
    from igr_sensitivities_gb300 import igr1d
    g = 1.4
    basis, mesh, G, q0, dt = case(igr, oracle, 3, 16, 11)
    T = 14.5 * dt
    prm = (0.3, 0.6)
    snaps, n = igr1d.run_forward_store(*q0, dt, T, basis, mesh, g, alpha, n_iter=n_iter, solver=solver)
    ref_s, nr = oracle.run_forward_store_1d(G, g, alpha, dt, T, n_iter, solver, [flat(x) for x in q0])
    assert n == nr == 15 and len(snaps) == n + 1
    for k in range(n + 1):
        for v in range(4):
            if v == 3 and alpha == 0:
                assert np.all(snaps.data[k, v] == 0)
            else:
                assert rel(snaps.data[k, v], ref_s[k, v]) <= RTOL, (k, v)
    a = igr1d.run_adjoint_conservative(snaps, n, dt, T, basis, mesh, g, alpha, n_iter=n_iter, objective=objective,
                                       solver=solver, obj_params=prm)
    ref = oracle.run_adjoint_conservative_1d(G, ref_s, n, dt, T, g, alpha, n_iter, objective, solver, prm)
    for x, y in zip(a, ref):
        assert rel(x, y) <= RTOL, objective
    # the fused batch call (snapshots kept on the device) is bitwise the two-call result
    out = igr1d.adjoint_conservative_batch([tuple(flat(x) for x in q0)], basis, [16], 1.0, g, alpha, dt, T,
                                           n_iter=n_iter, solver=solver, objective=objective, obj_params=prm)
    for x, y in zip(out[0], a):
        assert np.array_equal(x, flat(y))


def test_batch_uneven_equals_single_and_checkpointing_is_exact(igr, oracle):
    from igr_sensitivities_gb300 import igr1d
    basis = igr.DGBasis(3)
    nes = [12, 32, 20]
    gs = [1.4, 1.3, 1.6]
    als = [0.01, 0.0, 0.02]
    states, dts, Ts = [], [], []
    for i, ne in enumerate(nes):
        mesh = igr.PeriodicMesh1D(ne, 1.0, basis)
        q = W.seeded_pulses_1d(mesh, gs[i], W.seed_for(1, 20 + i), n_pulses=2, width=0.08)
        states.append(tuple(flat(x) for x in q))
        dt = W.cfl_dt_1d(mesh, 3, q, gs[i], 0.1)
        dts.append(dt)
        Ts.append((9 + 3 * i) * dt * 0.97)
    out = igr1d.adjoint_conservative_batch(states, basis, nes, 1.0, gs, als, dts, Ts, n_iter=8, solver="pcg")
    for i, ne in enumerate(nes):
        one = igr1d.adjoint_conservative_batch([states[i]], basis, [ne], 1.0, gs[i], als[i], dts[i], Ts[i], n_iter=8,
                                               solver="pcg")
        for x, y in zip(out[i], one[0]):
            assert np.array_equal(x, y)
    ctx = igr.default_context()
    N = sum(4 * ne for ne in nes)
    ctx.set_tape_budget(8 * N * 100)  # 100 fields per node: too small for every snapshot, room for sqrt(n)-step segments
    try:
        seg = igr1d.adjoint_conservative_batch(states, basis, nes, 1.0, gs, als, dts, Ts, n_iter=8, solver="pcg")
        assert ctx.last_adjoint_plan()["steps_per_segment"] < 15
    finally:
        ctx.set_tape_budget(0)
    for i in range(3):
        for x, y in zip(seg[i], out[i]):
            assert np.array_equal(x, y)


@pytest.mark.parametrize("ic,alpha,n_iter,tol", [
    ("acoustic_pulse", 0.0, 10, 1e-2), ("pressure_pulse", 0.0, 10, 1e-2), ("velocity_pulse", 0.0, 10, 1e-2),
    ("acoustic_pulse", 0.01, 200, 5e-2), ("acoustic_pulse", 0.05, 200, 5e-2),
])
def test_dJ_dA_vs_fd(igr, oracle, ic, alpha, n_iter, tol):
    """run_adjoint_conservative_test.jl:19-137 on GPU results: p = 2, N_e = 16,
    CFL 0.3 (dt = CFL dx / ((2p+1) 2.5)), T = 0.05, A0 = 0.2."""
    from igr_sensitivities_gb300 import igr1d
    g, L, p, Ne, T, A0 = 1.4, 1.0, 2, 16, 0.05, 0.2
    basis = igr.DGBasis(p)
    mesh = igr.PeriodicMesh1D(Ne, L, basis)
    dt = 0.3 * mesh.dx / ((2 * p + 1) * 2.5)
    dt = T / int(np.ceil(T / dt))
    build = igr1d.IC_BUILDERS[ic][0]

    def ic_of(A):
        q = [np.zeros(mesh.x.shape, order="F") for _ in range(3)]
        build(*q, A, mesh.x, L, g)
        return q

    q0 = ic_of(A0)
    snaps, n = igr1d.run_forward_store(*q0, dt, T, basis, mesh, g, alpha, n_iter=n_iter)
    am, ar, aE = igr1d.run_adjoint_conservative(snaps, n, dt, T, basis, mesh, g, alpha, n_iter=n_iter)
    wr, wu, wp = igr1d.ic_dA_weights(ic)
    s = np.sin(2 * np.pi * mesh.x / L)
    rho, u = q0[1], q0[0] / q0[1]
    drho, du, dp = wr * s, wu * s, wp * s
    dmu = rho * du + u * drho
    dE = dp / (g - 1) + 0.5 * (drho * u ** 2 + 2 * rho * u * du)
    wJ = basis.w[:, None] * mesh.J
    dJ = float(np.sum(wJ * (am * dmu + ar * drho + aE * dE)))

    def J_of(A):
        out = igr1d.run_forward(*ic_of(A), dt, T, basis, mesh, g, alpha, n_iter=n_iter)
        return float(np.sum(wJ * out[1] ** 2))

    fd = (J_of(A0 + 1e-6) - J_of(A0 - 1e-6)) / 2e-6
    assert abs(dJ - fd) / abs(fd) < tol
