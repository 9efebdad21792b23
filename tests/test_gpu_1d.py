"""GPU parity tests of the 1D engine (one CTA per instance) against the CPU
oracle, through the C ABI. Tolerance for the forward state: relative L2 1e-11."""
import numpy as np
import pytest

from igr_sensitivities_gb300 import workloads as W

pytestmark = pytest.mark.gpu

RTOL_FWD = 1e-11


def rel(a, b):
    a = np.asarray(a).reshape(-1, order="F")
    b = np.asarray(b).reshape(-1, order="F")
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def flat(a):
    return np.ascontiguousarray(np.asarray(a).reshape(-1, order="F"))


@pytest.fixture(scope="module")
def igr1d(igr):
    from igr_sensitivities_gb300 import igr1d as m
    return m


def setup1(igr, oracle, p, ne, L=1.0):
    basis = igr.DGBasis(p)
    mesh = igr.PeriodicMesh1D(ne, L, basis)
    return basis, mesh, oracle.Grid1D(p, ne, L)


@pytest.mark.parametrize("p,ne,solver,n_iter,alpha_scale", [
    (3, 32, "jacobi", 50, 3.0), (3, 32, "pcg", 20, 3.0), (3, 40, "chebyshev", 5, 3.0), (3, 24, "pcg", 5, 0.0),
    (1, 30, "pcg", 10, 3.0), (2, 20, "jacobi", 8, 3.0), (4, 16, "pcg", 12, 3.0), (3, 1, "jacobi", 3, 3.0),
    (3, 300, "pcg", 15, 3.0),
])
def test_run_forward_1d_matches_oracle(igr, igr1d, oracle, p, ne, solver, n_iter, alpha_scale):
    """Forward parity. The one-element mesh runs Jacobi: CG on its 4-node
    system converges within the 3 iterations, after which the recurrence is
    driven by rounding (the oracle itself moves by 5e-3 under a 1e-15 change
    of the initial state), so that case has no implementation-independent
    answer under PCG."""
    g = 1.4
    basis, mesh, G = setup1(igr, oracle, p, ne)
    if ne >= 8:
        q0 = W.seeded_pulses_1d(mesh, g, W.seed_for(1, p * 100 + ne), width=0.1)
    else:  # a pulse resolved by a handful of nodes blows up (in the oracle too): use a weak, wide one
        q0 = W.pulse_ic_1d(mesh, g, [0.05], [0.5], 0.3)
    dt = W.cfl_dt_1d(mesh, p, q0, g, 0.1)
    alpha = alpha_scale * mesh.dx ** 2
    T = 20 * dt * 0.999
    out = igr1d.run_forward(*q0, dt, T, basis, mesh, g, alpha, n_iter=n_iter, solver=solver)
    ref, Sr = oracle.run_forward_1d(G, g, alpha, dt, T, n_iter, solver, [flat(a) for a in q0])
    for a, b in zip(out[:3], ref):
        assert rel(a, b) <= RTOL_FWD
    if alpha > 0:
        assert rel(out[3], Sr) <= RTOL_FWD
    else:
        assert np.all(out[3] == 0)


def test_forward_batch_matches_single(igr, igr1d, oracle):
    """Instances of different sizes, gammas, alphas, dts and step counts in one
    launch give bitwise the single-instance results."""
    import math
    basis = igr.DGBasis(3)
    nes, gs, nst = [48, 16, 96, 16], [1.4, 1.3, 1.6, 1.5], [7, 11, 5, 9]
    states, Ts, dts, dtr, als = [], [], [], [], []
    for i, ne in enumerate(nes):
        mesh = igr.PeriodicMesh1D(ne, 1.0, basis)
        q0 = W.seeded_pulses_1d(mesh, gs[i], W.seed_for(4, i), width=0.08)
        states.append(tuple(flat(a) for a in q0))
        dt = W.cfl_dt_1d(mesh, 3, q0, gs[i], 0.1)
        T = nst[i] * dt * 0.999
        assert math.ceil(T / dt) == nst[i]
        dts.append(dt); Ts.append(T); dtr.append(T / nst[i])  # run_forward!'s re-rounding
        als.append(3.0 * mesh.dx ** 2)
    out = igr1d.forward_batch(states, basis, nes, 1.0, gs, als, dtr, nst, n_iter=9, solver="pcg")
    for i, ne in enumerate(nes):
        mesh = igr.PeriodicMesh1D(ne, 1.0, basis)
        one = igr1d.run_forward(*[a.reshape(4, ne, order="F") for a in states[i]], dts[i], Ts[i], basis, mesh, gs[i],
                                als[i], n_iter=9, solver="pcg")
        for a, b in zip(out[i], one):
            assert np.array_equal(a, flat(b))
        G = oracle.Grid1D(3, ne)
        ref, Sr = oracle.run_forward_1d(G, gs[i], als[i], dts[i], Ts[i], 9, "pcg", list(states[i]))
        for a, b in zip(out[i][:3], ref):
            assert rel(a, b) <= RTOL_FWD
        assert rel(out[i][3], Sr) <= RTOL_FWD


RTOL_GRAD = 1e-9


def grad_rel(dq, dqr):
    num = np.sqrt(sum(np.sum((np.asarray(a).ravel() - np.asarray(b).ravel()) ** 2) for a, b in zip(dq, dqr)))
    den = np.sqrt(sum(np.sum(np.asarray(b) ** 2) for b in dqr))
    return num / den


@pytest.mark.parametrize("p,ne,solver,n_iter,objective,alpha_scale", [
    (3, 24, "pcg", 6, "l2_density", 3.0), (3, 24, "jacobi", 5, "l2_pressure", 3.0),
    (3, 24, "chebyshev", 5, "kinetic_energy", 3.0), (3, 20, "pcg", 7, "weighted_momentum", 3.0),
    (3, 20, "pcg", 6, "interval_rho", 3.0), (3, 20, "chebyshev", 4, "l2_density", 0.0), (2, 18, "pcg", 6, "l2_pressure", 3.0),
    (4, 12, "jacobi", 4, "l2_density", 3.0), (1, 30, "chebyshev", 3, "l2_density", 3.0),
])
def test_adjoint_1d_matches_oracle(igr, igr1d, oracle, p, ne, solver, n_iter, objective, alpha_scale):
    g = 1.4
    basis, mesh, G = setup1(igr, oracle, p, ne)
    q0 = W.seeded_pulses_1d(mesh, g, W.seed_for(4, p * 10 + ne), width=0.1)
    dt = W.cfl_dt_1d(mesh, p, q0, g, 0.1)
    alpha = alpha_scale * mesh.dx ** 2
    prm = (0.3, 0.6) if objective == "interval_rho" else None
    J, dq, dg, da = igr1d.adjoint_batch([tuple(flat(a) for a in q0)], basis, [ne], 1.0, g, alpha, dt, 9, n_iter=n_iter,
                                        solver=solver, objective=objective, obj_params=prm)
    Jr, dqr, dgr, dar = oracle.adjoint_1d(G, g, alpha, 9, dt, n_iter, solver, objective, [flat(a) for a in q0], prm)
    assert abs(J[0] - Jr) <= 1e-12 * abs(Jr)
    assert grad_rel(dq[0], dqr) <= RTOL_GRAD
    assert abs(dg[0] - dgr) <= RTOL_GRAD * max(abs(dgr), 1e-300)
    if alpha > 0:
        assert abs(da[0] - dar) <= RTOL_GRAD * abs(dar)
    else:
        assert da[0] == 0.0


def test_adjoint_1d_segments_equal_full(igr, igr1d, oracle):
    """A memory budget below the full step history switches to sqrt(n)-step
    segments (one more forward re-run); the gradient stays bitwise equal."""
    from igr_sensitivities_gb300 import Context
    g = 1.4
    basis, mesh, G = setup1(igr, oracle, 3, 16)
    q0 = tuple(flat(a) for a in W.seeded_pulses_1d(mesh, g, W.seed_for(4, 77), width=0.1))
    dt = W.cfl_dt_1d(mesh, 3, [a.reshape(4, 16, order="F") for a in q0], g, 0.1)
    alpha = 3.0 * mesh.dx ** 2
    ctx = Context(0)
    full = igr1d.adjoint_batch([q0], basis, [16], 1.0, g, alpha, dt, 9, n_iter=5, solver="pcg", ctx=ctx)
    assert ctx.last_adjoint_plan()["steps_per_segment"] == 9
    ctx.set_tape_budget(200 * 64 * 8)  # full history needs 173 fields of 64 nodes, sqrt segments 157
    seg = igr1d.adjoint_batch([q0], basis, [16], 1.0, g, alpha, dt, 9, n_iter=5, solver="pcg", ctx=ctx)
    assert ctx.last_adjoint_plan()["steps_per_segment"] == 3
    assert full[0][0] == seg[0][0] and full[2][0] == seg[2][0] and full[3][0] == seg[3][0]
    for a, b in zip(full[1][0], seg[1][0]):
        assert np.array_equal(a, b)


def test_adjoint_1d_uneven_batch_equals_single(igr, igr1d, oracle):
    basis = igr.DGBasis(3)
    nes, gs, nst = [40, 8, 24], [1.4, 1.25, 1.7], [6, 9, 4]
    states, dts, als = [], [], []
    for i, ne in enumerate(nes):
        mesh = igr.PeriodicMesh1D(ne, 1.0, basis)
        q0 = W.seeded_pulses_1d(mesh, gs[i], W.seed_for(4, 200 + i), width=0.12)
        states.append(tuple(flat(a) for a in q0))
        dts.append(W.cfl_dt_1d(mesh, 3, q0, gs[i], 0.1))
        als.append(3.0 * mesh.dx ** 2)
    J, dq, dg, da = igr1d.adjoint_batch(states, basis, nes, 1.0, gs, als, dts, nst, n_iter=6, solver="pcg",
                                        objective="interval_rho", obj_params=(0.25, 0.55))
    for i, ne in enumerate(nes):
        J1, dq1, dg1, da1 = igr1d.adjoint_batch([states[i]], basis, [ne], 1.0, gs[i], als[i], dts[i], nst[i], n_iter=6,
                                                solver="pcg", objective="interval_rho", obj_params=(0.25, 0.55))
        assert J[i] == J1[0] and dg[i] == dg1[0] and da[i] == da1[0]
        for a, b in zip(dq[i], dq1[0]):
            assert np.array_equal(a, b)


def test_enzyme_adjoint_ic_1d_primitive_transform(igr, igr1d, oracle):
    """enzyme_adjoint_ic's IC builder, step rule and conservative-to-primitive
    transform. Its sine initial states put element faces on symmetry points of
    the solution, where the LLF max() and the penalty max() tie to rounding
    level: there the discrete map has no unique derivative (the oracle's own
    gradient moves by 6e-5 under a 1e-15 change of the state), so the
    conservative gradient is compared with the GPU batch call on the same
    inputs (bitwise) and J with the oracle; gradient parity is tested on the
    pulse states above."""
    p, ne, L, g, A, CFL, T = 3, 16, 1.0, 1.4, 0.05, 0.5, 0.02
    alpha = 3.0 * (L / ne) ** 2
    J, ar, au, ap = igr1d.enzyme_adjoint_ic(A, p, ne, L, g, alpha, CFL, T, n_iter=5, ic_type="acoustic_pulse", solver="pcg")
    basis = igr.DGBasis(p)
    mesh = igr.PeriodicMesh1D(ne, L, basis)
    mu0, rho0, E0 = (np.zeros((p + 1, ne), order="F") for _ in range(3))
    igr1d.IC_BUILDERS["acoustic_pulse"][0](mu0, rho0, E0, A, mesh.x, L, g)
    dt = CFL * mesh.dx / ((2 * p + 1) * 2.5)  # IGR_adjoints_1d/enzyme_adjoint.jl:272-275
    n = int(np.ceil(T / dt))
    Jb, dq, _, _ = igr1d.adjoint_batch([tuple(flat(a) for a in (mu0, rho0, E0))], basis, [ne], L, g, alpha, T / n, n,
                                       n_iter=5, solver="pcg")
    dmu, drho, dE = dq[0]
    u0 = flat(mu0) / flat(rho0)
    assert J == Jb[0]
    assert np.array_equal(flat(ar), drho + u0 * dmu + (u0 ** 2 / 2) * dE)
    assert np.array_equal(flat(au), flat(rho0) * dmu + flat(rho0) * u0 * dE)
    assert np.array_equal(flat(ap), dE / (g - 1))
    G = oracle.Grid1D(p, ne, L)
    Jr, _ = oracle.objective_run_1d(G, g, alpha, n, T / n, 5, "pcg", "l2_density", [flat(a) for a in (mu0, rho0, E0)])
    assert abs(J - Jr) <= 1e-12 * abs(Jr)
    with pytest.raises(ValueError):
        igr1d.enzyme_adjoint_ic(A, p, ne, L, g, alpha, CFL, T, objective="kinetic_energy")


@pytest.mark.parametrize("p,ne,solver,n_iter,form,s_gamma,alpha_scale", [
    (3, 24, "pcg", 8, 2, 0.0, 3.0), (3, 24, "pcg", 8, 1, 0.0, 3.0), (3, 20, "jacobi", 6, 2, 0.5, 3.0),
    (3, 20, "chebyshev", 5, 1, 0.0, 3.0), (2, 16, "pcg", 6, 2, 0.0, 0.0), (4, 12, "pcg", 6, 1, 1.0, 3.0),
])
def test_run_sensitivity_1d_matches_oracle(igr, igr1d, oracle, p, ne, solver, n_iter, form, s_gamma, alpha_scale):
    g = 1.4
    basis, mesh, G = setup1(igr, oracle, p, ne)
    q0 = W.seeded_pulses_1d(mesh, g, W.seed_for(6, p * 10 + ne), width=0.1)
    rng = np.random.default_rng(ne)
    s0 = [np.asfortranarray(0.1 * rng.standard_normal(mesh.x.shape)) for _ in range(3)]
    dt = W.cfl_dt_1d(mesh, p, q0, g, 0.1)
    alpha = alpha_scale * mesh.dx ** 2
    T = 7.4 * dt  # a partial last step: the while-loop stepping of ssp_rk3_coupled
    out = igr1d.run_sensitivity(*q0, *s0, dt, T, basis, mesh, g, alpha, n_iter=n_iter, elliptic_rhs="form%d" % form,
                                solver=solver, s_gamma=s_gamma)
    qr, Sr, sr, vr = oracle.run_sensitivity_1d(G, g, alpha, dt, T, n_iter, solver, [flat(a) for a in q0],
                                               [flat(a) for a in s0], form=form, s_gamma=s_gamma)
    for a, b in zip(out[:3], qr):
        assert rel(a, b) <= RTOL_FWD
    for a, b in zip(out[4:7], sr):
        assert rel(a, b) <= RTOL_FWD
    if alpha > 0:
        assert rel(out[3], Sr) <= RTOL_FWD and rel(out[7], vr) <= RTOL_FWD


@pytest.mark.parametrize("solver", ["pcg", "chebyshev"])
def test_cluster_size_does_not_change_results(igr, igr1d, oracle, solver):
    """One instance spread over a cluster of 2..16 CTAs gives bitwise the
    results of one CTA (forward, tangent and adjoint): every reduction runs
    over per-element partials in one fixed order."""
    from igr_sensitivities_gb300 import Context
    g = 1.4
    basis, mesh, G = setup1(igr, oracle, 3, 64)
    q0 = W.seeded_pulses_1d(mesh, g, W.seed_for(1, 900), width=0.08)
    dt = W.cfl_dt_1d(mesh, 3, q0, g, 0.1)
    alpha = 3.0 * mesh.dx ** 2
    rng = np.random.default_rng(3)
    s0 = [np.asfortranarray(0.1 * rng.standard_normal(mesh.x.shape)) for _ in range(3)]
    ctx = Context(0)
    out = {}
    for cs in (1, 2, 16):
        ctx.set_cluster_size_1d(cs)
        f = igr1d.run_forward(*q0, dt, 6 * dt, basis, mesh, g, alpha, n_iter=7, solver=solver, ctx=ctx)
        assert ctx.last_cluster_size_1d() == cs
        t = igr1d.run_sensitivity(*q0, *s0, dt, 5.5 * dt, basis, mesh, g, alpha, n_iter=7, solver=solver, ctx=ctx)
        a = igr1d.adjoint_batch([tuple(flat(x) for x in q0)], basis, [64], 1.0, g, alpha, dt, 5, n_iter=7, solver=solver,
                                objective="l2_pressure", ctx=ctx)
        out[cs] = (f, t, a)
    ctx.set_cluster_size_1d(0)
    igr1d.run_forward(*q0, dt, 6 * dt, basis, mesh, g, alpha, n_iter=7, solver=solver, ctx=ctx)
    assert ctx.last_cluster_size_1d() == 1  # automatic choice below 256 elements: one CTA
    for cs in (2, 16):
        for x, y in zip(out[1][0] + out[1][1], out[cs][0] + out[cs][1]):
            assert np.array_equal(x, y)
        a1, ac = out[1][2], out[cs][2]
        assert a1[0][0] == ac[0][0] and a1[2][0] == ac[2][0] and a1[3][0] == ac[3][0]
        for x, y in zip(a1[1][0], ac[1][0]):
            assert np.array_equal(x, y)
    ref, _ = oracle.run_forward_1d(G, g, alpha, dt, 6 * dt, 7, solver, [flat(x) for x in q0])
    for x, y in zip(out[16][0][:3], ref):
        assert rel(x, y) <= RTOL_FWD


@pytest.mark.parametrize("solver", ["jacobi", "pcg"])
def test_node_and_element_apply_agree_bitwise(igr, igr1d, oracle, solver):
    """CTAs with at most 32 elements (P3) apply the operator one lane per
    node, larger ones one thread per element; the forms give the same bits.
    N_e = 96 on one or two CTAs runs the element form, on four the node form."""
    from igr_sensitivities_gb300 import Context
    g = 1.4
    basis, mesh, G = setup1(igr, oracle, 3, 96)
    q0 = W.seeded_pulses_1d(mesh, g, W.seed_for(1, 901), width=0.08)
    dt = W.cfl_dt_1d(mesh, 3, q0, g, 0.1)
    alpha = 3.0 * mesh.dx ** 2
    ctx = Context(0)
    out = {}
    for cs in (1, 2, 4):
        ctx.set_cluster_size_1d(cs)
        out[cs] = igr1d.run_forward(*q0, dt, 5 * dt, basis, mesh, g, alpha, n_iter=9, solver=solver, ctx=ctx)
    for cs in (2, 4):
        for x, y in zip(out[1], out[cs]):
            assert np.array_equal(x, y)
    ref, _ = oracle.run_forward_1d(G, g, alpha, dt, 5 * dt, 9, solver, [flat(x) for x in q0])
    for x, y in zip(out[4][:3], ref):
        assert rel(x, y) <= RTOL_FWD


@pytest.mark.parametrize("ne,cs", [(16, 16), (3, 2), (2, 2), (5, 4)])
@pytest.mark.parametrize("solver", ["jacobi", "chebyshev"])
def test_local_solve_edge_splits(igr, igr1d, oracle, ne, cs, solver):
    """Small instances keep the Jacobi / Chebyshev iterate in shared memory and
    read the halo from the neighbouring CTAs: one element per CTA, uneven
    splits and two CTAs that are each other's left and right neighbour give
    bitwise the one-CTA results, and match the oracle."""
    from igr_sensitivities_gb300 import Context
    g = 1.4
    basis, mesh, G = setup1(igr, oracle, 3, ne)
    q0 = W.seeded_pulses_1d(mesh, g, W.seed_for(1, 910 + ne), width=0.2)
    dt = W.cfl_dt_1d(mesh, 3, q0, g, 0.1)
    alpha = 3.0 * mesh.dx ** 2
    ctx = Context(0)
    out = {}
    for c in (1, cs):
        ctx.set_cluster_size_1d(c)
        out[c] = igr1d.run_forward(*q0, dt, 4 * dt, basis, mesh, g, alpha, n_iter=6, solver=solver, ctx=ctx)
    for x, y in zip(out[1], out[cs]):
        assert np.array_equal(x, y)
    ref, _ = oracle.run_forward_1d(G, g, alpha, dt, 4 * dt, 6, solver, [flat(x) for x in q0])
    for x, y in zip(out[cs][:3], ref):
        assert rel(x, y) <= RTOL_FWD
