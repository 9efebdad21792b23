"""GPU parity tests of the 2D engine against the CPU oracle (through the C ABI).

Tolerances (field-wise relative L2, ||a-b||/||b||, as the reference's own
tests measure error, IGR_adjoints_2d/tests/run_sensitivity_test.jl:169):
  operators (one application)           1e-13
  forward state after many steps        1e-11
  gradients (discrete adjoint)          1e-9
"""
import numpy as np
import pytest

from igr_sensitivities_gb300 import workloads as W

pytestmark = pytest.mark.gpu

RTOL_OP, RTOL_FWD, RTOL_GRAD = 1e-13, 1e-11, 1e-9


def rel(a, b):
    a = np.asarray(a).reshape(-1, order="F")
    b = np.asarray(b).reshape(-1, order="F")
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def flat(a):
    return np.ascontiguousarray(np.asarray(a).reshape(-1, order="F"))


def setup(igr, oracle, p, nex, ney, lx=1.0, ly=1.0):
    basis = igr.DGBasis(p)
    mesh = igr.CartesianMesh2D(nex, ney, lx, ly, basis)
    G = oracle.Grid2D(p, nex, ney, lx, ly)
    return basis, mesh, G


def random_state(mesh, seed, gamma=1.4):
    rng = np.random.default_rng(seed)
    shape = mesh.x.shape
    rho = 1.0 + 0.3 * rng.random(shape)
    mux = 0.2 * rng.standard_normal(shape)
    muy = 0.2 * rng.standard_normal(shape)
    p = 1.0 + 0.5 * rng.random(shape)
    E = p / (gamma - 1) + 0.5 * (mux ** 2 + muy ** 2) / rho
    return [np.asfortranarray(a) for a in (mux, muy, rho, E)]


@pytest.mark.parametrize("p,nex,ney", [(3, 7, 5), (3, 8, 8), (1, 5, 6), (2, 4, 3), (4, 6, 5), (3, 1, 3)])
def test_apply_sip_matches_oracle(igr, oracle, p, nex, ney):
    basis, mesh, G = setup(igr, oracle, p, nex, ney, 1.0, 1.3)
    rng = np.random.default_rng(p * 100 + nex)
    x = rng.standard_normal(mesh.x.shape)
    rho = 0.5 + 1.5 * rng.random(mesh.x.shape)
    alpha = 3e-3
    y = np.zeros(mesh.x.shape, order="F")
    igr.apply_sip_(y, x, rho, basis, mesh, alpha)
    yr = oracle.apply_sip_2d(G, alpha, flat(x), flat(rho))
    assert rel(y, yr) <= RTOL_OP


def test_apply_sip_symmetric(igr, oracle):
    basis, mesh, G = setup(igr, oracle, 3, 6, 4)
    rng = np.random.default_rng(7)
    x, z = rng.standard_normal((2,) + mesh.x.shape)
    rho = 0.5 + rng.random(mesh.x.shape)
    Ax = np.zeros(mesh.x.shape, order="F")
    Az = np.zeros(mesh.x.shape, order="F")
    igr.apply_sip_(Ax, x, rho, basis, mesh, 1e-2)
    igr.apply_sip_(Az, z, rho, basis, mesh, 1e-2)
    a, b = np.sum(z * Ax), np.sum(x * Az)
    assert abs(a - b) <= 1e-13 * max(abs(a), abs(b))


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_hyperbolic_rhs_matches_oracle(igr, oracle, p):
    basis, mesh, G = setup(igr, oracle, p, 6, 5, 1.0, 1.3)
    q = random_state(mesh, p)
    S = 0.01 * np.random.default_rng(3).standard_normal(mesh.x.shape)
    out = [np.zeros(mesh.x.shape, order="F") for _ in range(4)]
    igr.compute_hyperbolic_rhs_(*out, *q, S, basis, mesh, 1.4)
    ref = oracle.hyperbolic_rhs_2d(G, 1.4, [flat(a) for a in q], flat(S))
    for a, b in zip(out, ref):
        assert rel(a, b) <= RTOL_OP


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_freestream_preservation(igr, oracle, p):
    # IGR_adjoints_2d/tests/run_euler_test.jl:15-33: max|dq| < 1e-11 for a constant state
    basis, mesh, G = setup(igr, oracle, p, 6, 5, 1.0, 1.3)
    g = 1.4
    sh = mesh.x.shape
    mux, muy, rho = np.full(sh, 1.0), np.full(sh, -0.7), np.ones(sh)
    E = np.full(sh, 1.0 / (g - 1) + 0.5 * (1.0 + 0.49))
    out = [np.zeros(sh, order="F") for _ in range(4)]
    igr.compute_hyperbolic_rhs_(*out, mux, muy, rho, E, np.zeros(sh), basis, mesh, g)
    assert max(np.max(np.abs(a)) for a in out) < 1e-11


@pytest.mark.parametrize("solver", ["chebyshev", "jacobi", "pcg"])
def test_solve_elliptic_matches_oracle(igr, oracle, solver):
    basis, mesh, G = setup(igr, oracle, 3, 8, 6)
    q = random_state(mesh, 11)
    S0 = 0.01 * np.random.default_rng(4).standard_normal(mesh.x.shape)
    S = np.array(S0, order="F")
    igr.solve_elliptic_(S, *q, basis, mesh, 5e-3, n_iter=7, solver=solver)
    Sr = oracle.solve_elliptic_2d(G, 5e-3, 7, solver, [flat(a) for a in q], flat(S0))
    assert rel(S, Sr) <= 1e-12


@pytest.mark.parametrize("solver,alpha,n_iter", [("chebyshev", 3.0 * (1 / 8) ** 2, 5), ("jacobi", 3.0 * (1 / 8) ** 2, 6),
                                                 ("chebyshev", 0.0, 5), ("pcg", 3.0 * (1 / 8) ** 2, 12),
                                                 ("pcg", 3.0 * (1 / 8) ** 2, 1)])
def test_run_forward_matches_oracle(igr, oracle, solver, alpha, n_iter):
    g = 1.4
    basis, mesh, G = setup(igr, oracle, 3, 8, 8)
    q0 = W.seeded_pulses_2d(mesh, g, W.seed_for(2, 0), width=0.1)
    dt = W.cfl_dt_2d(mesh, 3, q0, g, 0.1)
    T = 25 * dt * 0.999
    out = igr.run_forward(*q0, dt, T, basis, mesh, g, alpha, n_iter=n_iter, solver=solver)
    ref, Sr = oracle.run_forward_2d(G, g, alpha, dt, T, n_iter, solver, [flat(a) for a in q0])
    for a, b in zip(out[:4], ref):
        assert rel(a, b) <= RTOL_FWD
    if alpha > 0:
        assert rel(out[4], Sr) <= RTOL_FWD


@pytest.mark.parametrize("solver,objective", [("chebyshev", "window_rho2"), ("jacobi", "l2_density"),
                                              ("chebyshev", "kinetic_energy"), ("chebyshev", "l2_pressure"),
                                              ("jacobi", "weighted_momentum"), ("chebyshev", "windowed_kinetic_energy"),
                                              ("pcg", "window_rho2"), ("pcg", "l2_pressure"), ("pcg", "kinetic_energy")])
def test_adjoint_matches_oracle(igr, oracle, solver, objective):
    g = 1.4
    basis, mesh, G = setup(igr, oracle, 3, 6, 5)
    alpha = 3.0 * (1 / 6) ** 2
    q0 = W.seeded_pulses_2d(mesh, g, W.seed_for(3, 1), width=0.12)
    dt = W.cfl_dt_2d(mesh, 3, q0, g, 0.1)
    prm = (0.2, 0.3, 0.4)
    res = igr.enzyme_adjoint_ic(*q0, 6, dt, basis, mesh, g, alpha, n_iter=5, solver=solver, objective=objective,
                                obj_params=prm, with_params=True)
    J, dq, dgam, dalp = res[0], res[1:5], res[5], res[6]
    Jr, dqr, dgr, dar = oracle.adjoint_2d(G, g, alpha, 6, dt, 5, solver, objective, [flat(a) for a in q0], prm)
    assert abs(J - Jr) <= 1e-12 * abs(Jr)
    num = np.sqrt(sum(np.sum((flat(a) - b) ** 2) for a, b in zip(dq, dqr)))
    den = np.sqrt(sum(np.sum(b ** 2) for b in dqr))
    assert num <= RTOL_GRAD * den
    assert abs(dgam - dgr) <= RTOL_GRAD * max(abs(dgr), 1e-300)
    assert abs(dalp - dar) <= RTOL_GRAD * max(abs(dar), 1e-300)


@pytest.mark.parametrize("p,ic,alpha,nex", [(2, "tgp", 0.0, 4), (3, "tgp", 0.0, 4), (3, "pulse", 0.0, 6), (2, "pulse", 0.02, 6),
                                             (3, "tg", 0.02, 4), (3, "pulse", 0.02, 4), (1, "pulse", 0.02, 5),
                                             (4, "pulse", 0.01, 5)])
def test_adjoint_degrees_and_ics(igr, oracle, p, ic, alpha, nex):
    """Gradients for p = 1..4, alpha = 0 and > 0, several initial states.

    The Taylor-Green state is mirror-symmetric: face pairs on its symmetry
    lines keep exactly tied LLF wave speeds with nonzero jumps, where
    max(.,.) is not differentiable and a 1-ulp rounding difference between two
    implementations flips which side receives the derivative. Parity is tested
    on a perturbed copy ("tgp"), off the kink.
    """
    g = 1.4
    basis, mesh, G = setup(igr, oracle, p, nex, nex)
    if ic in ("tg", "tgp"):
        q0 = list(W.taylor_green_ic(mesh, g, 0.4))
        if ic == "tgp":
            rng = np.random.default_rng(p)
            q0[0] = q0[0] + 1e-3 * rng.standard_normal(q0[0].shape)
            q0[1] = q0[1] + 1e-3 * rng.standard_normal(q0[1].shape)
    else:
        q0 = W.seeded_pulses_2d(mesh, g, W.seed_for(7, p), width=0.15)
    dt = 0.4 * W.cfl_dt_2d(mesh, p, q0, g, 0.1)
    n_iter = 3 if alpha > 0 else 1
    res = igr.enzyme_adjoint_ic(*q0, 8, dt, basis, mesh, g, alpha, n_iter=n_iter, solver="chebyshev",
                                objective="l2_density", with_params=True)
    Jr, dqr, dgr, dar = oracle.adjoint_2d(G, g, alpha, 8, dt, n_iter, "chebyshev", "l2_density", [flat(a) for a in q0])
    assert abs(res[0] - Jr) <= 1e-12 * abs(Jr)
    num = np.sqrt(sum(np.sum((flat(a) - b) ** 2) for a, b in zip(res[1:5], dqr)))
    den = np.sqrt(sum(np.sum(b ** 2) for b in dqr))
    assert num <= RTOL_GRAD * den, [rel(a, b) for a, b in zip(res[1:5], dqr)]
    assert abs(res[5] - dgr) <= RTOL_GRAD * abs(dgr)


@pytest.mark.parametrize("solver", ["chebyshev", "pcg"])
def test_checkpointed_adjoint_equals_full_tape(igr, oracle, solver):
    """A tape budget of a few steps forces checkpointing + recompute (a revolve
    schedule over super-steps of several taped steps); the gradient must be
    bitwise the one of the full tape."""
    g = 1.4
    basis, mesh, _ = setup(igr, oracle, 3, 5, 4)
    alpha = 3.0 * (1 / 5) ** 2
    q0 = W.seeded_pulses_2d(mesh, g, W.seed_for(3, 2), width=0.12)
    dt = W.cfl_dt_2d(mesh, 3, q0, g, 0.1)
    ctx = igr.Context(0)
    full = igr.enzyme_adjoint_ic(*q0, 11, dt, basis, mesh, g, alpha, n_iter=5, solver=solver, objective="l2_density",
                                 with_params=True, ctx=ctx)
    n = mesh.x.size
    # fields of one taped stage (upper bound for either solver at n_iter = 5)
    step_bytes = 3 * (16 + 1 + 6 + 2 * 5 + 1) * n * 8
    ctx.set_tape_budget(3 * step_bytes + 10 * 6 * n * 8)
    seg = igr.enzyme_adjoint_ic(*q0, 11, dt, basis, mesh, g, alpha, n_iter=5, solver=solver, objective="l2_density",
                                with_params=True, ctx=ctx)
    plan = ctx.last_adjoint_plan()
    assert plan["segments"] > 1
    assert full[0] == seg[0]
    for a, b in zip(full[1:5], seg[1:5]):
        assert np.array_equal(a, b)
    assert full[5] == seg[5] and full[6] == seg[6]


def revolve_evaluations(n, slots):
    """Fewest forward evaluations of a binomial (revolve) reversal of n steps
    with `slots` checkpoint slots beyond the first state (taped runs counted)."""
    cost = {}
    for k in range(1, n + 1):
        for s in range(0, k):
            if k == 1:
                cost[(k, s)] = 1
            elif s == 0:
                cost[(k, s)] = k * (k + 1) // 2
            else:
                cost[(k, s)] = min(m + cost[(k - m, min(s - 1, k - m - 1))] + cost[(m, min(s, m - 1))]
                                   for m in range(1, k))
    return cost[(n, min(slots, n - 1))]


@pytest.mark.parametrize("solver,slots", [("chebyshev", 2), ("pcg", 1), ("chebyshev", 0)])
def test_revolve_adjoint_equals_full_tape(igr, oracle, solver, slots):
    """Binomial checkpointing: room for one taped step and 1 + slots stored
    states; 13 steps are reversed with recomputation from the stored states,
    bitwise equal to the full tape, with the optimal revolve evaluation count."""
    g, nst = 1.4, 13
    basis, mesh, _ = setup(igr, oracle, 3, 4, 5)
    alpha = 3.0 * (1 / 5) ** 2
    q0 = W.seeded_pulses_2d(mesh, g, W.seed_for(3, 5), width=0.12)
    dt = W.cfl_dt_2d(mesh, 3, q0, g, 0.1)
    ctx = igr.Context(0)
    full = igr.enzyme_adjoint_ic(*q0, nst, dt, basis, mesh, g, alpha, n_iter=5, solver=solver, objective="l2_density",
                                 with_params=True, ctx=ctx)
    assert ctx.last_checkpoint_schedule() == {"tape_steps": nst, "snapshots": 0, "step_evaluations": nst}
    n = mesh.x.size
    F = 16 + (1 + 6 + 2 * 5 + 1 if solver == "pcg" else 2 * 5)  # fields of one taped stage at n_iter = 5
    ctx.set_tape_budget(3 * F * n * 8 + (1 + slots) * 6 * n * 8)
    rev = igr.enzyme_adjoint_ic(*q0, nst, dt, basis, mesh, g, alpha, n_iter=5, solver=solver, objective="l2_density",
                                with_params=True, ctx=ctx)
    sched = ctx.last_checkpoint_schedule()
    assert sched["tape_steps"] == 1 and sched["snapshots"] == slots
    assert sched["step_evaluations"] == revolve_evaluations(nst, slots) > nst
    plan = igr.adjoint_plan(1, nst, basis, mesh, alpha, n_iter=5, solver=solver, ctx=ctx)  # the same, without running
    assert plan == {"instances_per_group": 1, "tape_steps": 1, "snapshots": slots,
                    "step_evaluations": sched["step_evaluations"]}
    assert full[0] == rev[0]
    for a, b in zip(full[1:5], rev[1:5]):
        assert np.array_equal(a, b)
    assert full[5] == rev[5] and full[6] == rev[6]


@pytest.mark.parametrize("solver", ["chebyshev", "pcg"])
def test_batched_adjoint_matches_single(igr, oracle, solver):
    g0 = 1.4
    basis, mesh, G = setup(igr, oracle, 3, 4, 4)
    B = 3
    qs, gammas, alphas, dts = [], [], [], []
    for b in range(B):
        gam = 1.3 + 0.1 * b
        q0 = W.seeded_pulses_2d(mesh, gam, W.seed_for(5, b), width=0.12)
        qs.append(np.stack([flat(a) for a in q0]))
        gammas.append(gam)
        alphas.append(3.0 * (1 / 4) ** 2 * (1 + 0.2 * b))
        dts.append(W.cfl_dt_2d(mesh, 3, q0, gam, 0.1))
    q0 = np.stack(qs)
    prm = (0.1, 0.2, 0.5)
    J, dq, dg, da = igr.adjoint_batch(q0, gammas, alphas, dts, 5, basis, mesh, n_iter=5, solver=solver,
                                      objective="window_rho2", obj_params=prm)
    for b in range(B):
        Jr, dqr, dgr, dar = oracle.adjoint_2d(G, gammas[b], alphas[b], 5, dts[b], 5, solver, "window_rho2", list(q0[b]),
                                              prm)
        # batching does not change any reduction order: bitwise equal to the single-instance call
        one = igr.enzyme_adjoint_ic(*[np.asfortranarray(q0[b, v].reshape(mesh.x.shape, order="F")) for v in range(4)], 5,
                                    dts[b], basis, mesh, gammas[b], alphas[b], n_iter=5, solver=solver,
                                    objective="window_rho2", obj_params=prm, with_params=True)
        assert one[0] == J[b] and one[5] == dg[b] and one[6] == da[b]
        for v in range(4):
            assert np.array_equal(flat(one[1 + v]), dq[b, v])
        assert abs(J[b] - Jr) <= 1e-12 * abs(Jr)
        num = np.sqrt(sum(np.sum((dq[b, v] - dqr[v]) ** 2) for v in range(4)))
        den = np.sqrt(sum(np.sum(dqr[v] ** 2) for v in range(4)))
        assert num <= RTOL_GRAD * den
        assert abs(dg[b] - dgr) <= RTOL_GRAD * abs(dgr)
        assert abs(da[b] - dar) <= RTOL_GRAD * abs(dar)
    del g0


def test_bad_solver_and_objective_raise(igr, oracle):
    basis, mesh, _ = setup(igr, oracle, 3, 2, 2)
    q0 = W.taylor_green_ic(mesh, 1.4, 0.1)
    with pytest.raises(ValueError):
        igr.run_forward(*q0, 0.01, 0.02, basis, mesh, 1.4, 0.01, n_iter=2, solver="gmres")
    with pytest.raises(ValueError):
        igr.enzyme_adjoint_ic(*q0, 2, 0.01, basis, mesh, 1.4, 0.01, objective="entropy")
    with pytest.raises(Exception) as ei:
        igr.run_forward(*q0, 0.01, 0.02, basis, mesh, 1.4, 0.01, n_iter=2, solver=7)
    assert "IGR_EINVAL" in str(ei.value)


def test_nonfinite_state_is_reported(igr, oracle):
    basis, mesh, _ = setup(igr, oracle, 3, 4, 4)
    q0 = list(W.taylor_green_ic(mesh, 1.4, 0.1))
    q0[2] = q0[2].copy()
    q0[2][1, 1, 2, 2] = np.nan
    with pytest.raises(Exception) as ei:
        igr.run_forward(*q0, 0.01, 0.03, basis, mesh, 1.4, 0.01, n_iter=2, solver="chebyshev")
    assert "IGR_ENONFINITE" in str(ei.value)


def test_adjoint_batch_of_uneven_meshes_equals_single_calls(igr, oracle):
    """Instances with different meshes, gammas, alphas and dts in one batch
    (one launch per kernel over all their tiles) give bitwise the
    single-instance gradients; one of them is checked against the oracle."""
    basis = igr.DGBasis(3)
    meshes = [igr.CartesianMesh2D(6, 4, 1.0, 0.8, basis), igr.CartesianMesh2D(3, 5, 0.6, 1.0, basis),
              igr.CartesianMesh2D(8, 8, 1.0, 1.0, basis)]
    gams, states, dts, als = [1.4, 1.3, 1.6], [], [], []
    for i, m in enumerate(meshes):
        q = W.seeded_pulses_2d(m, gams[i], W.seed_for(3, 40 + i), width=0.12)
        states.append(tuple(flat(a) for a in q))
        dts.append(W.cfl_dt_2d(m, 3, q, gams[i], 0.1))
        als.append(3.0 * min(m.dx, m.dy) ** 2)
    prm = (0.1, 0.1, 0.5)
    J, dq, dg, da = igr.adjoint_batch_meshes(states, basis, meshes, gams, als, dts, 5, n_iter=6, solver="pcg",
                                             objective="window_rho2", obj_params=prm)
    for i, m in enumerate(meshes):
        one = igr.enzyme_adjoint_ic(*[a.reshape(m.shape(basis), order="F") for a in states[i]], 5, dts[i], basis, m,
                                    gams[i], als[i], n_iter=6, solver="pcg", objective="window_rho2", obj_params=prm,
                                    with_params=True)
        assert one[0] == J[i] and one[5] == dg[i] and one[6] == da[i]
        for v in range(4):
            assert np.array_equal(flat(one[1 + v]), dq[i][v])
    G = oracle.Grid2D(3, 3, 5, 0.6, 1.0)
    Jr, dqr, dgr, dar = oracle.adjoint_2d(G, gams[1], als[1], 5, dts[1], 6, "pcg", "window_rho2", list(states[1]), prm)
    assert abs(J[1] - Jr) <= 1e-12 * abs(Jr)
    num = np.sqrt(sum(np.sum((dq[1][v] - dqr[v]) ** 2) for v in range(4)))
    assert num <= RTOL_GRAD * np.sqrt(sum(np.sum(b ** 2) for b in dqr))


def test_pcg_sums_fused_and_separate_agree_bitwise(igr, oracle):
    """The PCG inner products are completed inside their kernels for small
    grids and by a separate launch for large ones; both give the same bits.
    A 64^2 instance alone (256 tiles: fused) and inside a batch with a
    256 x 260 instance (4416 tiles: separate) has bitwise equal gradients."""
    basis = igr.DGBasis(3)
    meshes = [igr.CartesianMesh2D(64, 64, 1.0, 1.0, basis), igr.CartesianMesh2D(256, 260, 1.0, 1.0, basis)]
    gams, states, dts, als = [1.4, 1.5], [], [], []
    for i, m in enumerate(meshes):
        q = W.seeded_pulses_2d(m, gams[i], W.seed_for(3, 60 + i), width=0.12)
        states.append(tuple(flat(a) for a in q))
        dts.append(W.cfl_dt_2d(m, 3, q, gams[i], 0.1))
        als.append(3.0 * min(m.dx, m.dy) ** 2)
    prm = (0.1, 0.1, 0.5)
    J, dq, dg, da = igr.adjoint_batch_meshes(states, basis, meshes, gams, als, dts, 2, n_iter=4, solver="pcg",
                                             objective="window_rho2", obj_params=prm)
    m = meshes[0]
    one = igr.enzyme_adjoint_ic(*[a.reshape(m.shape(basis), order="F") for a in states[0]], 2, dts[0], basis, m,
                                gams[0], als[0], n_iter=4, solver="pcg", objective="window_rho2", obj_params=prm,
                                with_params=True)
    assert one[0] == J[0] and one[5] == dg[0] and one[6] == da[0]
    for v in range(4):
        assert np.array_equal(flat(one[1 + v]), dq[0][v])


@pytest.mark.parametrize("solver", ["pcg", "chebyshev"])
def test_forward_graph_replay_equals_eager_launches(igr, oracle, solver):
    """From the second step on the forward replays each RK step as a CUDA
    graph; launching every kernel from the host gives bitwise the same state
    and Sigma, and the launch count is the same."""
    from igr_sensitivities_gb300._lib import default_context
    g = 1.4
    basis, mesh, _ = setup(igr, oracle, 3, 8, 8)
    q0 = W.seeded_pulses_2d(mesh, g, W.seed_for(2, 1), width=0.1)
    dt = W.cfl_dt_2d(mesh, 3, q0, g, 0.1)
    ctx = default_context()
    outs, counts = [], []
    try:
        for on in (False, True):
            ctx.set_graphs(on)
            outs.append(igr.run_forward(*q0, dt, 6 * dt * 0.999, basis, mesh, g, 3.0 * (1 / 8) ** 2, n_iter=7,
                                        solver=solver))
            counts.append(ctx.last_launch_count())
    finally:
        ctx.set_graphs(True)
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(flat(a), flat(b))
    assert counts[0] == counts[1] > 0


def test_tangent_graph_replay_equals_eager_launches(igr, oracle):
    """run_sensitivity replays steps of each parity as a CUDA graph from the
    third step on; eager launches give bitwise the same ten fields."""
    from igr_sensitivities_gb300._lib import default_context
    g = 1.4
    basis, mesh, _ = setup(igr, oracle, 3, 8, 8)
    q0 = W.seeded_pulses_2d(mesh, g, W.seed_for(2, 2), width=0.1)
    rng = np.random.default_rng(11)
    s0 = [np.asfortranarray(0.1 * rng.standard_normal(mesh.x.shape)) for _ in range(4)]
    dt = W.cfl_dt_2d(mesh, 3, q0, g, 0.1)
    ctx = default_context()
    outs = []
    try:
        for on in (False, True):
            ctx.set_graphs(on)
            outs.append(igr.run_sensitivity(*q0, *s0, dt, 7 * dt * 0.999, basis, mesh, g, 3.0 * (1 / 8) ** 2, n_iter=6,
                                            solver="pcg"))
    finally:
        ctx.set_graphs(True)
    assert len(outs[0]) == 10
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(flat(a), flat(b))


@pytest.mark.parametrize("p,nex,ney", [(1, 6, 5), (2, 5, 4), (4, 5, 3)])
def test_pcg_forward_and_adjoint_other_degrees(igr, oracle, p, nex, ney):
    """PCG (its pointwise kernels are compiled per degree) for p = 1, 2, 4 on
    ragged tile grids: forward state and gradient against the oracle."""
    g = 1.4
    basis, mesh, G = setup(igr, oracle, p, nex, ney)
    q0 = W.seeded_pulses_2d(mesh, g, W.seed_for(8, p), width=0.15)
    dt = 0.4 * W.cfl_dt_2d(mesh, p, q0, g, 0.1)
    alpha = 0.02
    out = igr.run_forward(*q0, dt, 4 * dt * 0.999, basis, mesh, g, alpha, n_iter=7, solver="pcg")
    ref, Sr = oracle.run_forward_2d(G, g, alpha, dt, 4 * dt * 0.999, 7, "pcg", [flat(a) for a in q0])
    for a, b in zip(out[:4], ref):
        assert rel(a, b) <= RTOL_FWD
    assert rel(out[4], Sr) <= RTOL_FWD
    res = igr.enzyme_adjoint_ic(*q0, 4, dt, basis, mesh, g, alpha, n_iter=7, solver="pcg", objective="l2_density",
                                with_params=True)
    Jr, dqr, dgr, dar = oracle.adjoint_2d(G, g, alpha, 4, dt, 7, "pcg", "l2_density", [flat(a) for a in q0])
    assert abs(res[0] - Jr) <= 1e-12 * abs(Jr)
    num = np.sqrt(sum(np.sum((flat(a) - b) ** 2) for a, b in zip(res[1:5], dqr)))
    den = np.sqrt(sum(np.sum(b ** 2) for b in dqr))
    assert num <= RTOL_GRAD * den
    assert abs(res[5] - dgr) <= RTOL_GRAD * abs(dgr)
    assert abs(res[6] - dar) <= RTOL_GRAD * abs(dar)


@pytest.mark.parametrize("case", ["forward", "forward_batch", "tangent", "solve", "forward_128", "forward_p1",
                                  "forward_p2", "forward_p4", "batch_published"])
def test_persistent_pcg_equals_two_kernel_form(igr, oracle, case):
    """The persistent PCG solve (one cooperative launch per solve, per-instance
    hand-offs of the inner products) gives bitwise the two-kernel result, also
    when the forward's RK steps replay as CUDA graphs. Counted hand-offs (up to
    256 tiles per instance) and published ones (forward_128: 1024 tiles;
    batch_published: two 72^2 instances of 324 tiles) at p = 1..4."""
    from igr_sensitivities_gb300 import Context
    g = 1.4
    p = {"forward_p1": 1, "forward_p2": 2, "forward_p4": 4}.get(case, 3)
    ne = {"forward_128": (128, 128), "forward_p1": (13, 9), "forward_p2": (10, 14), "forward_p4": (22, 22),
          "batch_published": (72, 72)}.get(case, (8, 6))
    basis, mesh, _ = setup(igr, oracle, p, *ne)
    alpha = 3.0 / (ne[0] * ne[1])
    q0 = W.seeded_pulses_2d(mesh, g, W.seed_for(2, 7), width=0.12 if ne[0] < 32 else 0.03)
    dt = W.cfl_dt_2d(mesh, p, q0, g, 0.1)

    def run(ctx):
        rng = np.random.default_rng(4)
        if case.startswith("forward") and case != "forward_batch":
            return igr.run_forward(*q0, dt, 3 * dt * 0.999, basis, mesh, g, alpha, n_iter=12, solver="pcg", ctx=ctx)
        if case in ("forward_batch", "batch_published"):
            nb = 3 if case == "forward_batch" else 2
            q = np.stack([np.stack([flat(a) for a in q0])] * nb)
            return igr.forward_batch(q, [1.3, 1.4, 1.5][:nb], [alpha, 0.5 * alpha, 2 * alpha][:nb], [dt] * nb, 3,
                                     basis, mesh, n_iter=10, solver="pcg", ctx=ctx)
        if case == "tangent":
            s0 = [rng.standard_normal(mesh.x.shape) * 1e-3 for _ in range(4)]
            return igr.run_sensitivity(*q0, *s0, dt, 3 * dt * 0.999, basis, mesh, g, alpha, n_iter=9, solver="pcg",
                                       ctx=ctx)
        S = np.zeros(mesh.x.shape, order="F")
        igr.solve_elliptic_(S, *q0, basis, mesh, alpha, n_iter=25, solver="pcg", ctx=ctx)
        return (S,)

    a_ctx, b_ctx = Context(0), Context(0)
    b_ctx.set_pcg_persistent(False)
    A, B = run(a_ctx), run(b_ctx)
    for x, y in zip(A, B):
        assert np.array_equal(np.asarray(x), np.asarray(y))


@pytest.mark.parametrize("ne,drop", [((8, 6), 0), ((8, 6), 3), ((72, 72), 0), ((72, 72), 201)])
def test_persistent_pcg_wait_times_out_and_context_recovers(igr, oracle, ne, drop):
    """A CTA of the persistent PCG solve that leaves early (the test hook drops
    one tile's CTA before its first p.Ap hand-off) makes the instance's other
    CTAs give up after their bounded wait: the call returns IGR_ETIMEOUT, and
    the same context then solves normally, bitwise as a fresh one. 8 x 6 runs
    the counted hand-off (4 tiles), 72^2 the published one (324 tiles); tile 0
    is the instance's writer CTA."""
    from igr_sensitivities_gb300 import Context
    from igr_sensitivities_gb300._lib import IGRError
    g = 1.4
    basis, mesh, _ = setup(igr, oracle, 3, *ne)
    alpha = 3.0 / (ne[0] * ne[1])
    q0 = W.seeded_pulses_2d(mesh, g, W.seed_for(2, 11), width=0.1)

    def solve(ctx):
        S = np.zeros(mesh.x.shape, order="F")
        igr.solve_elliptic_(S, *q0, basis, mesh, alpha, n_iter=20, solver="pcg", ctx=ctx)
        return S

    ctx = Context(0)
    ctx.test_pcg_drop_tile(drop)
    with pytest.raises(IGRError) as err:
        solve(ctx)
    assert err.value.code == 6
    assert np.array_equal(solve(ctx), solve(Context(0)))
