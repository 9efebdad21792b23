"""CPU tests of the oracle against the reference's own known-answer tests.

The reference ships no golden vectors (paper_data/ is empty); its tests are
scripts that check properties at run time. Each test here ports one of them,
citing the reference file it follows, at sizes that finish in seconds.
"""
import numpy as np
import pytest

from igr_sensitivities_gb300 import workloads as W


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


def test_basis_sum_weights_and_exact_derivative(oracle):
    # IGR_adjoints_1d/tests/run_euler_test.jl:15-41: sum(w) = 2, D exact to degree p
    for p in range(1, 6):
        xi, w, D = oracle.basis(p)
        assert abs(w.sum() - 2.0) < 1e-14
        for deg in range(p + 1):
            f, df = xi ** deg, deg * xi ** max(deg - 1, 0)
            assert np.max(np.abs(D @ f - df)) < 1e-12


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_freestream_2d(oracle, p):
    # IGR_adjoints_2d/tests/run_euler_test.jl:15-33
    G = oracle.Grid2D(p, 6, 5, 1.0, 1.3)
    g = 1.4
    N = G.N
    q = [np.full(N, 1.0), np.full(N, -0.7), np.ones(N), np.full(N, 1 / (g - 1) + 0.5 * (1 + 0.49))]
    d = oracle.hyperbolic_rhs_2d(G, g, q, np.zeros(N))
    assert max(np.abs(a).max() for a in d) < 1e-11


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_freestream_1d(oracle, p):
    # IGR_adjoints_1d/tests/run_euler_test.jl:46-72
    G = oracle.Grid1D(p, 8)
    g = 1.4
    q = [np.ones(G.N), np.ones(G.N), np.full(G.N, 1 / (g - 1) + 0.5)]
    d = oracle.hyperbolic_rhs_1d(G, g, q, np.zeros(G.N))
    assert max(np.abs(a).max() for a in d) < 1e-12


def test_sip_manufactured_solution_order(oracle):
    # IGR_adjoints_2d/tests/run_euler_test.jl:38-79 (orders printed there; asserted here as >= p + 0.5)
    alpha, p = 0.1, 2
    errs = []
    for ne in (4, 8):
        G = oracle.Grid2D(p, ne, ne)
        x, y = G.coords()
        ex = np.sin(2 * np.pi * x) * np.sin(2 * np.pi * y)
        k2 = 2 * (2 * np.pi) ** 2
        ww = np.tile(np.outer(G.w, G.w).reshape(-1), ne * ne) * G.Jx * G.Jy
        b = ww * (1 + alpha * k2) * ex
        sol, _ = oracle.cg_2d(G, alpha, np.ones(G.N), b, np.zeros(G.N), tol=1e-12, maxiter=5000)
        errs.append(np.sqrt(np.sum(ww * (sol - ex) ** 2)))
    order = np.log(errs[0] / errs[1]) / np.log(2)
    assert order > p + 0.5


def test_quasi1d_equals_1d(oracle):
    # IGR_adjoints_2d/tests/run_quasi1d_test.jl: forward (alpha = 0 and > 0) and tangent, |2D - 1D| < 1e-9
    g, L, p, Ne, A, T, CFL, Ney, Ly = 1.4, 1.0, 3, 12, 0.4, 0.08, 0.5, 4, 0.5
    G1, G2 = oracle.Grid1D(p, Ne, L), oracle.Grid2D(p, Ne, Ney, L, Ly)
    x1 = G1.coords()
    u = A * np.sin(2 * np.pi * x1 / L)
    q1 = [u.copy(), np.ones(G1.N), 1 / (g - 1) + 0.5 * u ** 2]
    x2, _ = G2.coords()
    u2 = A * np.sin(2 * np.pi * x2 / L)
    q2 = [u2.copy(), np.zeros(G2.N), np.ones(G2.N), 1 / (g - 1) + 0.5 * u2 ** 2]
    ws = np.max(np.abs(u) + np.sqrt(g * (g - 1) * (q1[2] - u ** 2 / 2)))
    dt = CFL * G1.dx / ((2 * p + 1) * ws)
    n = int(np.ceil(T / dt))
    dt = T / n
    alpha = 3.0 * (L / Ne) ** 2

    def dev(f2, f1):
        f2 = f2.reshape(Ney, Ne, p + 1, p + 1)
        return np.max(np.abs(f2 - f1.reshape(Ne, p + 1)[None, :, None, :])), np.max(np.abs(f2 - f2[0:1, :, 0:1, :]))

    for a, nit in ((0.0, 1), (alpha, 100)):
        r1, S1 = oracle.run_forward_1d(G1, g, a, dt, T, nit, "pcg", q1)
        r2, S2 = oracle.run_forward_2d(G2, g, a, dt, T, nit, "pcg", q2)
        for f2, f1 in ((r2[0], r1[0]), (r2[2], r1[1]), (r2[3], r1[2]), (S2, S1)):
            d, ynu = dev(f2, f1)
            assert d < 1e-9 and ynu < 1e-11
        assert np.abs(r2[1]).max() < 1e-11
    s1 = [np.sin(2 * np.pi * x1 / L), np.zeros(G1.N), A * np.sin(2 * np.pi * x1 / L) ** 2]
    s2 = [np.sin(2 * np.pi * x2 / L), np.zeros(G2.N), np.zeros(G2.N), A * np.sin(2 * np.pi * x2 / L) ** 2]
    _, _, ss1, _ = oracle.run_sensitivity_1d(G1, g, alpha, dt, T, 100, "pcg", q1, s1, form=2)
    _, _, ss2, _ = oracle.run_sensitivity_2d(G2, g, alpha, dt, T, 100, "pcg", q2, s2)
    for f2, f1 in ((ss2[0], ss1[0]), (ss2[2], ss1[1]), (ss2[3], ss1[2])):
        d, ynu = dev(f2, f1)
        assert d < 1e-9 and ynu < 1e-11


@pytest.mark.parametrize("solver", ["pcg", "jacobi", "chebyshev"])
@pytest.mark.parametrize("objective", ["l2_density", "l2_pressure", "kinetic_energy", "windowed_kinetic_energy",
                                       "weighted_momentum", "window_rho2"])
def test_reverse_equals_dual_2d(oracle, solver, objective):
    # Enzyme == ForwardDiff (IGR_adjoints_1d/tests/run_enzyme_test.jl:24-91, tolerance 1e-8): here the
    # hand-written reverse against forward-mode duals on 3 seeded directions, including gamma and alpha.
    G = oracle.Grid2D(2, 4, 3)
    g, alpha = 1.4, 2e-2
    x, y = G.coords()
    q0 = [0.3 * np.sin(2 * np.pi * x) * np.cos(2 * np.pi * y), -0.2 * np.cos(2 * np.pi * x), 1 + 0.2 * np.sin(2 * np.pi * y),
          2.5 + 0.3 * np.cos(2 * np.pi * (x + y))]
    prm = (0.2, 0.1, 0.5)
    J, dq, dg, da = oracle.adjoint_2d(G, g, alpha, 5, 0.004, 4, solver, objective, q0, prm)
    rng = np.random.default_rng(0)
    for _ in range(3):
        v = [rng.standard_normal(G.N) for _ in range(4)]
        vg, va = rng.standard_normal(2)
        J2, dJ = oracle.objective_dual_2d(G, g, alpha, 5, 0.004, 4, solver, objective, q0, v, vg, va, prm)
        rev = sum(np.dot(a, b) for a, b in zip(dq, v)) + dg * vg + da * va
        assert J == J2
        assert abs(rev - dJ) <= 1e-12 * max(abs(dJ), 1e-14)


@pytest.mark.parametrize("objective", ["l2_density", "l2_pressure", "kinetic_energy", "weighted_momentum", "interval_rho"])
def test_reverse_equals_dual_1d(oracle, objective):
    G = oracle.Grid1D(3, 8)
    g = 1.4
    x = G.coords()
    q0 = [0.1 * np.sin(2 * np.pi * x), 1 + 0.2 * np.sin(2 * np.pi * x), 1 / (g - 1) + 0.3 * np.cos(2 * np.pi * x)]
    J, dq, dg, da = oracle.adjoint_1d(G, g, 0.01, 10, 0.002, 7, "pcg", objective, q0, (0.3, 0.6))
    rng = np.random.default_rng(1)
    v = [rng.standard_normal(G.N) for _ in range(3)]
    _, dJ = oracle.objective_dual_1d(G, g, 0.01, 10, 0.002, 7, "pcg", objective, q0, v, 0.3, 0.7, (0.3, 0.6))
    rev = sum(np.dot(a, b) for a, b in zip(dq, v)) + dg * 0.3 + da * 0.7
    assert abs(rev - dJ) <= 1e-12 * abs(dJ)


def test_gradient_vs_central_fd_2d(oracle):
    # IGR_adjoints_2d/tests/run_enzyme_test.jl:14-99: FD at 6 seeded nodes, h = 1e-6, rel < 1e-3
    G = oracle.Grid2D(2, 4, 4)
    g, alpha = 1.4, 1.5e-3
    x, y = G.coords()
    A = 0.4
    ux, uy = A * np.sin(2 * np.pi * x) * np.cos(2 * np.pi * y), -A * np.cos(2 * np.pi * x) * np.sin(2 * np.pi * y)
    q0 = [ux, uy, np.ones(G.N), 1 / (g - 1) + 0.5 * (ux ** 2 + uy ** 2)]
    q0 = [a + 1e-3 * np.random.default_rng(5).standard_normal(G.N) for a in q0]
    dt, n, nit = 0.005, 16, 60
    J, dq, _, _ = oracle.adjoint_2d(G, g, alpha, n, dt, nit, "chebyshev", "l2_density", q0)
    rng = np.random.default_rng(42)
    idxs = rng.integers(0, G.N, 6)
    h = 1e-6
    errs, scale = [], max(np.abs(a).max() for a in dq)
    for f in range(4):
        for i in idxs:
            qp = [a.copy() for a in q0]
            qm = [a.copy() for a in q0]
            qp[f][i] += h
            qm[f][i] -= h
            Jp, _ = oracle.objective_run_2d(G, g, alpha, n, dt, nit, "chebyshev", "l2_density", qp)
            Jm, _ = oracle.objective_run_2d(G, g, alpha, n, dt, nit, "chebyshev", "l2_density", qm)
            errs.append(abs((Jp - Jm) / (2 * h) - dq[f][i]))
    assert max(errs) / scale < 1e-3


def test_tangent_vs_central_fd_2d(oracle):
    # IGR_adjoints_2d/tests/run_sensitivity_test.jl:27-90 (theta = Taylor-Green amplitude), combined rel-L2 < 5e-4
    G = oracle.Grid2D(3, 8, 8)
    g, A, alpha, T = 1.4, 0.4, 1.5e-3, 0.1
    x, y = G.coords()
    cx, cy = 2 * np.pi * x, 2 * np.pi * y

    def ic(a):
        ux, uy = a * np.sin(cx) * np.cos(cy), -a * np.cos(cx) * np.sin(cy)
        return [ux, uy, np.ones(G.N), 1 / (g - 1) + 0.5 * (ux ** 2 + uy ** 2)]

    s0 = [np.sin(cx) * np.cos(cy), -np.cos(cx) * np.sin(cy), np.zeros(G.N),
          A * (np.sin(cx) ** 2 * np.cos(cy) ** 2 + np.cos(cx) ** 2 * np.sin(cy) ** 2)]
    q = ic(A)
    P = (g - 1) * (q[3] - (q[0] ** 2 + q[1] ** 2) / 2)
    ws = np.max(np.maximum(np.abs(q[0]), np.abs(q[1])) + np.sqrt(g * P))
    dt = 0.4 * G.dx / ((2 * 3 + 1) * ws)
    _, _, s, _ = oracle.run_sensitivity_2d(G, g, alpha, dt, T, 100, "chebyshev", ic(A), s0)
    h = 1e-5
    qp, _ = oracle.run_forward_2d(G, g, alpha, dt, T, 100, "chebyshev", ic(A + h))
    qm, _ = oracle.run_forward_2d(G, g, alpha, dt, T, 100, "chebyshev", ic(A - h))
    fd = np.concatenate([(a - b) / (2 * h) for a, b in zip(qp, qm)])
    assert rel(np.concatenate(s), fd) < 5e-4


def test_forward_consistency_objective_loop(oracle):
    # IGR_adjoints_1d/tests/run_enzyme_test.jl:96-144: the inlined objective loop == run_forward (1e-14)
    G = oracle.Grid2D(3, 4, 4)
    g, alpha = 1.4, 0.01
    mesh_q = [np.zeros(G.N), np.zeros(G.N), np.ones(G.N), np.full(G.N, 2.5)]
    x, y = G.coords()
    mesh_q[3] = mesh_q[3] + np.exp(-((x - 0.5) ** 2 + (y - 0.5) ** 2) / 0.05)
    dt = 0.003
    n = 7
    J, qf = oracle.objective_run_2d(G, g, alpha, n, dt, 5, "pcg", "l2_density", mesh_q)
    ref, _ = oracle.run_forward_2d(G, g, alpha, dt, n * dt, 5, "pcg", mesh_q)
    for a, b in zip(qf, ref):
        assert rel(a, b) < 1e-14


def test_unknown_solver_raises(oracle):
    G = oracle.Grid2D(2, 2, 2)
    q = [np.zeros(G.N), np.zeros(G.N), np.ones(G.N), np.full(G.N, 2.5)]
    with pytest.raises(ValueError):
        oracle.run_forward_2d(G, 1.4, 0.01, 0.01, 0.02, 2, "gmres", q)


def test_splitmix_seeds_are_stable():
    r = W.SplitMix64(W.seed_for(3, 0))
    a = [r.next_u64() for _ in range(3)]
    r2 = W.SplitMix64(W.seed_for(3, 0))
    assert a == [r2.next_u64() for _ in range(3)]
    u = W.SplitMix64(1).uniform(1.0, 10.0)
    assert 1.0 <= u <= 10.0


# ---------------------------------------------------------------------------
# Continuous adjoint (run_forward_store + run_adjoint_conservative)
# ---------------------------------------------------------------------------
def _taylor_green(G, g, A):
    # build_taylor_green_ic!, IGR_adjoints_2d/initial_conditions.jl:105-121
    x, y = G.coords()
    cx, cy = 2 * np.pi * x / G.Lx, 2 * np.pi * y / G.Ly
    ux, uy = A * np.sin(cx) * np.cos(cy), -A * np.cos(cx) * np.sin(cy)
    return [ux, uy, np.ones(G.N), 1.0 / (g - 1) + 0.5 * (ux ** 2 + uy ** 2)]


def _pde_vs_discrete(oracle, objective, alpha, p=3, Ne=8, T=0.06):
    """IGR_adjoints_2d/tests/run_adjoint_test.jl:15-78: the discrete gradient
    divided by the nodal mass against the PDE adjoint at t = 0 (Taylor-Green,
    A = 0.4, CFL 0.4, Chebyshev, n_iter = 100 if alpha > 0 else 1)."""
    g = 1.4
    G = oracle.Grid2D(p, Ne, Ne)
    q0 = _taylor_green(G, g, 0.4)
    mws = W.max_wavespeed_2d(*q0, g)
    dt = 0.4 * min(G.dx, G.dy) / ((2 * p + 1) * mws)
    n = int(np.ceil(T / dt))
    dt = T / n
    nit = 100 if alpha > 0 else 1
    _, dq, _, _ = oracle.adjoint_2d(G, g, alpha, n, dt, nit, "chebyshev", objective, q0)
    m = np.tile(np.outer(G.w, G.w).reshape(-1, order="F"), Ne * Ne) * G.Jx * G.Jy
    enz = [d / m for d in dq]
    snaps, nf = oracle.run_forward_store_2d(G, g, alpha, dt, T, nit, "chebyshev", q0)
    assert nf == n and snaps.shape == (n + 1, 5, G.N)
    pde = oracle.run_adjoint_conservative_2d(G, snaps, nf, dt, T, g, alpha, nit, objective, "chebyshev")
    return rel(np.concatenate(pde), np.concatenate(enz))


@pytest.mark.parametrize("objective", ["l2_density", "weighted_momentum", "kinetic_energy"])
@pytest.mark.parametrize("alpha", [0.0, 1.5e-3])
def test_pde_adjoint_within_otd_gap_of_discrete(oracle, objective, alpha):
    # run_adjoint_test.jl:72 asserts combined < 0.2 (a sign or derivation error
    # gives O(1)); the restatement measures 5e-5 .. 2e-2 here, bounded at 0.05.
    e = _pde_vs_discrete(oracle, objective, alpha)
    assert e < 0.2
    assert e < 0.05


def test_pde_adjoint_otd_gap_does_not_grow(oracle):
    # run_adjoint_test.jl:90-97: l2_density, alpha = 1.5e-3, N_e 6 -> 12
    e_coarse = _pde_vs_discrete(oracle, "l2_density", 1.5e-3, Ne=6)
    e_fine = _pde_vs_discrete(oracle, "l2_density", 1.5e-3, Ne=12)
    assert e_fine < 2 * e_coarse


def test_pde_local_operator_is_the_dual_of_the_linearised_rhs(oracle):
    """<a, L dq>_M == <L_dag a, dq>_M for smooth periodic fields, L the exact
    (forward-mode dual) linearisation of the discrete hyperbolic RHS with Sigma
    frozen and L_dag compute_adjoint_hyperbolic_rhs_local!: it pins the adjoint
    flux (adjoint_pde.jl:41-80), the flipped LLF faces and the local source
    (:138-217) to the forward flux. The gap is the LLF jump term; it falls from
    1e-2 (4^2 elements) to round-off (16^2)."""
    g = 1.4
    gaps = []
    for Ne in (4, 8, 16):
        G = oracle.Grid2D(3, Ne, Ne)
        x, y = G.coords()

        def s(kx, ky, ph):
            return np.sin(2 * np.pi * (kx * x + ky * y) + ph)

        q = [0.3 * s(1, 0, 0.1) + 0.1 * s(0, 1, 0.7), 0.2 * s(0, 1, 0.3) - 0.1 * s(1, 1, 0.2), 1 + 0.2 * s(1, 1, 0.5),
             2.5 + 0.3 * s(1, 0, 0.9)]
        a = [s(1, 0, 0.4), s(0, 1, 1.3), s(1, 1, 2.0), s(1, -1, 0.6)]
        dq = [s(0, 1, 0.2), s(1, 0, 2.2), s(1, 1, 0.8), s(-1, 1, 1.7)]
        lhs, rhs = oracle.pde_duality_2d(G, g, q, 0.05 * s(1, 1, 1.1), a, dq)
        gaps.append(abs(lhs - rhs) / abs(lhs))
    assert gaps[0] > gaps[1] > gaps[2]
    assert gaps[2] < 1e-12


def test_pde_adjoint_unknown_objective_raises(oracle):
    G = oracle.Grid2D(2, 2, 2)
    q = [np.zeros(G.N), np.zeros(G.N), np.ones(G.N), np.full(G.N, 2.5)]
    snaps, n = oracle.run_forward_store_2d(G, 1.4, 0.0, 0.01, 0.02, 1, "pcg", q)
    with pytest.raises(ValueError):
        oracle.run_adjoint_conservative_2d(G, snaps, n, 0.01, 0.02, 1.4, 0.0, 1, "entropy", "pcg")


def _pde1_dJ_dA(oracle, ic, alpha, n_iter, T, p=2, Ne=16, CFL=0.3, A0=0.2):
    """IGR_adjoints_1d/tests/run_adjoint_conservative_test.jl:19-137: dJ/dA
    assembled from the conservative adjoint at t = 0 (J = sum w J rho^2, the
    IC family's dq0/dA) and central differences of J(A), h = 1e-6."""
    from igr_sensitivities_gb300 import igr1d
    g, L = 1.4, 1.0
    G = oracle.Grid1D(p, Ne, L)
    x = G.coords()
    dt = CFL * G.dx / ((2 * p + 1) * 2.5)
    n = int(np.ceil(T / dt))
    dt = T / n
    build = igr1d.IC_BUILDERS[ic][0]

    def ic_of(A):
        mu, rho, E = np.zeros(G.N), np.zeros(G.N), np.zeros(G.N)
        build(mu, rho, E, A, x, L, g)
        return [mu, rho, E]

    q0 = ic_of(A0)
    snaps, ns = oracle.run_forward_store_1d(G, g, alpha, dt, T, n_iter, "pcg", q0)
    assert ns == n and snaps.shape == (n + 1, 4, G.N)
    am, ar, aE = oracle.run_adjoint_conservative_1d(G, snaps, ns, dt, T, g, alpha, n_iter, "l2_density", "pcg")
    wr, wu, wp = igr1d.ic_dA_weights(ic)
    s = np.sin(2 * np.pi * x / L)
    rho, u = q0[1], q0[0] / q0[1]
    drho, du, dp = wr * s, wu * s, wp * s
    dmu = rho * du + u * drho
    dE = dp / (g - 1) + 0.5 * (drho * u ** 2 + 2 * rho * u * du)
    wJ = np.tile(G.w, Ne) * G.J
    dJ = float(np.sum(wJ * (am * dmu + ar * drho + aE * dE)))

    def J_of(A):
        q, _ = oracle.run_forward_1d(G, g, alpha, dt, T, n_iter, "pcg", ic_of(A))
        return float(np.sum(wJ * q[1] ** 2))

    fd = (J_of(A0 + 1e-6) - J_of(A0 - 1e-6)) / 2e-6
    return abs(dJ - fd) / max(abs(fd), 1e-15)


@pytest.mark.parametrize("ic", ["acoustic_pulse", "entropy_wave", "density_pulse", "pressure_pulse", "velocity_pulse"])
def test_pde1_adjoint_dJ_dA_vs_fd_ic_sweep(oracle, ic):
    # run_adjoint_conservative_test.jl:233-237 (Test 3): alpha = 0, n_iter = 10, tol 1e-2 (measured <= 2e-5)
    assert _pde1_dJ_dA(oracle, ic, 0.0, 10, 0.05) < 1e-2


@pytest.mark.parametrize("alpha", [0.0, 0.001, 0.01, 0.05])
def test_pde1_adjoint_dJ_dA_vs_fd_alpha_sweep(oracle, alpha):
    # Tests 1, 2 and 4 (:226-243): n_iter = 200, tol 5e-2 (measured <= 9e-5)
    assert _pde1_dJ_dA(oracle, "acoustic_pulse", alpha, 200, 0.05) < 5e-2


def test_pde1_adjoint_long_time(oracle):
    # Test 5 (:246-247): alpha = 0.01, T = 1.0, tol 0.10 (measured 0.073: the OtD gap grows with T)
    assert _pde1_dJ_dA(oracle, "acoustic_pulse", 0.01, 200, 1.0) < 0.10


def test_pde1_local_operator_is_the_dual_of_the_linearised_rhs(oracle):
    """1D form of the 2D duality test: the gap converges at ~6th order
    (3e-3 at 4 elements, 6e-10 at 64)."""
    g = 1.4
    gaps = []
    for Ne in (16, 32, 64):
        G = oracle.Grid1D(3, Ne)
        x = G.coords()

        def s(k, ph):
            return np.sin(2 * np.pi * k * x + ph)

        q = [0.3 * s(1, 0.1), 1 + 0.2 * s(1, 0.5), 2.5 + 0.3 * s(2, 0.9)]
        lhs, rhs = oracle.pde_duality_1d(G, g, q, 0.05 * s(1, 1.1), [s(1, 0.4), s(2, 1.3), s(1, 2.0)],
                                         [s(2, 0.2), s(1, 2.2), s(1, 0.8)])
        gaps.append(abs(lhs - rhs) / abs(lhs))
    assert gaps[0] > 30 * gaps[1] > 900 * gaps[2]
    assert gaps[2] < 1e-8


def _acoustic_1d(G, eps, g=1.4):
    x = G.coords()
    s = np.sin(2 * np.pi * x / G.L)
    rho, u, p = 1.0 + eps * s, eps * s, 1.0 + eps * s
    return [rho * u, rho, p / (g - 1) + 0.5 * rho * u ** 2], s


def test_dJ_dalpha_dual_vs_fd_1d(oracle):
    """IGR_adjoints_1d/tests/run_forwarddiff_test.jl:31-91: dJ/dalpha of
    J = int rho(T)^2 (p = 3, N_e = 8, CFL 0.3, T = 0.1, alpha = 0.01, PCG 100)
    by forward-mode duals against central differences (h = 1e-7), rel < 1e-5;
    the hand-written reverse's dJ/dalpha agrees with the dual."""
    g, alpha, T = 1.4, 0.01, 0.1
    G = oracle.Grid1D(3, 8)
    q0, _ = _acoustic_1d(G, 0.2)
    ws = np.max(np.abs(q0[0] / q0[1]) + np.sqrt(g * (g - 1) * (q0[2] - 0.5 * q0[0] ** 2 / q0[1]) / q0[1]))
    dt = 0.3 * G.dx / (7 * ws)
    n = int(np.ceil(T / dt))
    dtr = T / n  # run_forward's re-rounded step: the fixed-step loop with it is run_forward
    zero = [np.zeros(G.N)] * 3
    J, dJ = oracle.objective_dual_1d(G, g, alpha, n, dtr, 100, "pcg", "l2_density", q0, zero, va=1.0)

    def Jf(a):
        q, _ = oracle.run_forward_1d(G, g, a, dt, T, 100, "pcg", q0)
        return float(np.sum(np.tile(G.w, 8) * G.J * q[1] ** 2))

    assert abs(J - Jf(alpha)) <= 1e-13 * abs(J)
    h = 1e-7
    fd = (Jf(alpha + h) - Jf(alpha - h)) / (2 * h)
    assert abs(dJ - fd) / abs(fd) < 1e-5
    _, _, _, da = oracle.adjoint_1d(G, g, alpha, n, dtr, 100, "pcg", "l2_density", q0)
    assert abs(da - dJ) <= 1e-9 * abs(dJ)


@pytest.mark.parametrize("form", [1, 2])
def test_tangent_dJ_dA_vs_dual_1d(oracle, form):
    """run_sensitivity_test.jl:240-329 (Test 5): dJ/dA from the hand-coded
    tangent (form1 / form2 elliptic source) against forward-mode AD of the
    forward map, rel < 1e-2 (linearise-then-discretise vs the discrete map)."""
    g, alpha, T = 1.4, 0.01, 0.05
    G = oracle.Grid1D(3, 8)
    dt = 0.3 * G.dx / (7 * 2.5)
    q0, s = _acoustic_1d(G, 0.2)
    rho, u = q0[1], q0[0] / q0[1]
    s0 = [s * u + rho * s, s, s / (g - 1) + 0.5 * (s * u ** 2 + 2 * rho * u * s)]
    q, _, sv, _ = oracle.run_sensitivity_1d(G, g, alpha, dt, T, 100, "pcg", q0, s0, form=form)
    wJ = np.tile(G.w, 8) * G.J
    dJ_tan = float(np.sum(wJ * 2 * q[1] * sv[1]))
    n = int(np.ceil(T / dt))
    _, dJ_ad = oracle.objective_dual_1d(G, g, alpha, n, T / n, 100, "pcg", "l2_density", q0, s0)
    assert abs(dJ_tan - dJ_ad) / abs(dJ_ad) < 1e-2


def test_form1_vs_form2_1d(oracle):
    """run_sensitivity_test.jl:335-396 (Test 6): the two tangent elliptic
    sources share the primal exactly and agree on the tangent within 1e-2."""
    g, alpha, T = 1.4, 0.01, 0.05
    G = oracle.Grid1D(3, 8)
    dt = 0.3 * G.dx / (7 * 2.5)
    q0, s = _acoustic_1d(G, 0.2)
    rho, u = q0[1], q0[0] / q0[1]
    s0 = [s * u + rho * s, s, s / (g - 1) + 0.5 * (s * u ** 2 + 2 * rho * u * s)]
    q1, S1, t1, v1 = oracle.run_sensitivity_1d(G, g, alpha, dt, T, 100, "pcg", q0, s0, form=1)
    q2, S2, t2, v2 = oracle.run_sensitivity_1d(G, g, alpha, dt, T, 100, "pcg", q0, s0, form=2)
    assert rel(q1[1], q2[1]) < 1e-14
    for a, b in zip(t1 + [v1], t2 + [v2]):
        assert rel(a, b) < 1e-2


def test_solver_summation_order_moves_results_at_rounding_level(oracle):
    """The solver inner products' summation order (sequential, reversed,
    pairwise: the GPU sums in a fixed tree order) moves a short PCG forward by
    rounding only; the differences bound what the parity tests can demand."""
    g, p, ne = 1.4, 3, 6
    G = oracle.Grid2D(p, ne, ne)
    x, y = G.coords()
    rho = 1.0 + 0.2 * np.exp(-((x - 0.4) ** 2 + (y - 0.6) ** 2) / 0.02)
    q0 = [0.1 * np.sin(2 * np.pi * y), 0.1 * np.cos(2 * np.pi * x), rho, 1.0 / (g - 1) + 0.01 / rho]
    ref = oracle.run_forward_2d(G, g, 3.0 / ne ** 2, 2e-3, 6e-3, 20, "pcg", q0)
    try:
        for order in (1, 2):
            oracle.set_dot_order(order)
            q, S = oracle.run_forward_2d(G, g, 3.0 / ne ** 2, 2e-3, 6e-3, 20, "pcg", q0)
            assert max(rel(a, b) for a, b in zip(q, ref[0])) < 1e-13
            assert 0 < rel(S, ref[1]) < 1e-10
    finally:
        oracle.set_dot_order(0)
