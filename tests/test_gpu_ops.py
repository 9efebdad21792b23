"""Operator-level drop-in calls against the CPU oracle, through the C ABI:
compute_igr_euler_rhs!, compute_igr_rhs!, compute_sip_diagonal, cg_solve! and
cg_fixed! (2D and 1D) and the 1D apply_sip!, solve_elliptic! and
compute_hyperbolic_rhs!.

Tolerances (relative L2 per field): one operator application 1e-13; one
fixed-count solve, or an operator that contains one, 1e-12; a CG solve run to
its tolerance 1e-9 on the manufactured solution (a few iterations), and 1e3
times the tolerance on random systems that take hundreds of iterations. The
stopping iteration may differ by one when sqrt(r.r) crosses the tolerance
between the GPU's tree-ordered and the oracle's sequential inner products.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL_OP, RTOL_SOLVE, RTOL_CG = 1e-13, 1e-12, 1e-9


def rel(a, b):
    a = np.asarray(a).reshape(-1, order="F")
    b = np.asarray(b).reshape(-1, order="F")
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def flat(a):
    return np.ascontiguousarray(np.asarray(a).reshape(-1, order="F"))


def state2d(mesh, seed, gamma=1.4):
    rng = np.random.default_rng(seed)
    sh = mesh.x.shape
    rho = 1.0 + 0.3 * rng.random(sh)
    mux, muy = 0.2 * rng.standard_normal(sh), 0.2 * rng.standard_normal(sh)
    E = (1.0 + 0.5 * rng.random(sh)) / (gamma - 1) + 0.5 * (mux ** 2 + muy ** 2) / rho
    return [np.asfortranarray(a) for a in (mux, muy, rho, E)]


def state1d(mesh, seed, gamma=1.4):
    rng = np.random.default_rng(seed)
    sh = mesh.x.shape
    rho = 1.0 + 0.3 * rng.random(sh)
    mu = 0.2 * rng.standard_normal(sh)
    E = (1.0 + 0.5 * rng.random(sh)) / (gamma - 1) + 0.5 * mu ** 2 / rho
    return [np.asfortranarray(a) for a in (mu, rho, E)]


# ------------------------------------------------------------------------------------------ 2D
@pytest.mark.parametrize("p,solver,alpha", [(3, "pcg", 5e-3), (3, "chebyshev", 5e-3), (3, "jacobi", 5e-3),
                                            (1, "pcg", 1e-2), (2, "chebyshev", 1e-2), (4, "pcg", 4e-3),
                                            (3, "pcg", 0.0)])
def test_igr_euler_rhs_2d_matches_oracle(igr, oracle, p, solver, alpha):
    # compute_igr_euler_rhs! (IGR_adjoints_2d/forward.jl:22-31): warm-started solve, then the DG RHS
    basis = igr.DGBasis(p)
    mesh = igr.CartesianMesh2D(7, 5, 1.0, 1.3, basis)
    G = oracle.Grid2D(p, 7, 5, 1.0, 1.3)
    q = state2d(mesh, 10 + p)
    S0 = 0.01 * np.random.default_rng(5).standard_normal(mesh.x.shape)
    S = np.array(S0, order="F")
    out = [np.zeros(mesh.x.shape, order="F") for _ in range(4)]
    igr.compute_igr_euler_rhs_(*out, *q, S, basis, mesh, 1.4, alpha, n_iter=9, solver=solver)
    ref, Sr = oracle.igr_euler_rhs_2d(G, 1.4, alpha, 9, solver, [flat(a) for a in q], flat(S0))
    if alpha > 0:
        assert rel(S, Sr) <= RTOL_SOLVE
    else:
        assert np.all(S == 0.0)
    for a, b in zip(out, ref):
        assert rel(a, b) <= RTOL_SOLVE


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_igr_rhs_and_sip_diagonal_2d_match_oracle(igr, oracle, p):
    basis = igr.DGBasis(p)
    mesh = igr.CartesianMesh2D(6, 7, 1.2, 1.0, basis)
    G = oracle.Grid2D(p, 6, 7, 1.2, 1.0)
    q = state2d(mesh, 20 + p)
    b = np.zeros(mesh.x.shape, order="F")
    igr.compute_igr_rhs_(b, *q, basis, mesh, 7e-3)
    assert rel(b, oracle.igr_rhs_2d(G, 7e-3, flat(q[0]), flat(q[1]), flat(q[2]))) <= RTOL_OP
    M = igr.compute_sip_diagonal(q[2], basis, mesh, 7e-3)
    assert rel(M, oracle.sip_diagonal_2d(G, 7e-3, flat(q[2]))) <= RTOL_OP


def test_solve_elliptic_2d_with_alpha_zero_matches_oracle(igr, oracle):
    # solve_elliptic! has no alpha test (elliptic.jl:413-427): with alpha = 0 the
    # Jacobi sweep on the mass operator still runs (x -> x / 3 per iteration)
    basis = igr.DGBasis(3)
    mesh = igr.CartesianMesh2D(5, 4, 1.0, 1.0, basis)
    G = oracle.Grid2D(3, 5, 4)
    q = state2d(mesh, 3)
    S0 = np.random.default_rng(8).standard_normal(mesh.x.shape)
    S = np.array(S0, order="F")
    igr.solve_elliptic_(S, *q, basis, mesh, 0.0, n_iter=4, solver="jacobi")
    Sr = oracle.solve_elliptic_2d(G, 0.0, 4, "jacobi", [flat(a) for a in q], flat(S0))
    assert rel(S, Sr) <= RTOL_SOLVE and rel(S, S0) > 0.5


def test_cg_fixed_2d_matches_oracle(igr, oracle):
    basis = igr.DGBasis(3)
    mesh = igr.CartesianMesh2D(6, 6, 1.0, 1.0, basis)
    G = oracle.Grid2D(3, 6, 6)
    rng = np.random.default_rng(31)
    rho = 0.6 + rng.random(mesh.x.shape)
    b = rng.standard_normal(mesh.x.shape)
    x0 = 0.1 * rng.standard_normal(mesh.x.shape)
    x = np.array(x0, order="F")
    n = igr.cg_fixed_(x, igr.sip_operator(rho, basis, mesh, 2e-2), b, 15)
    xr, nr = oracle.cg_2d(G, 2e-2, flat(rho), flat(b), flat(x0), maxiter=15, fixed=True)
    assert n == nr == 15
    assert rel(x, xr) <= RTOL_SOLVE


@pytest.mark.parametrize("tol", [1e-6, 1e-10])
def test_cg_solve_2d_random_system_matches_oracle(igr, oracle, tol):
    # 130-190 iterations: several rounds of the chunked stopping test
    basis = igr.DGBasis(3)
    mesh = igr.CartesianMesh2D(8, 8, 1.0, 1.0, basis)
    G = oracle.Grid2D(3, 8, 8)
    rng = np.random.default_rng(5)
    rho = np.asfortranarray((0.6 + rng.random(G.N)).reshape(mesh.x.shape, order="F"))
    b = np.asfortranarray(rng.standard_normal(G.N).reshape(mesh.x.shape, order="F"))
    x = np.zeros(mesh.x.shape, order="F")
    it = igr.cg_solve_(x, igr.sip_operator(rho, basis, mesh, 2e-2), b, tol, 3000)
    xr, itr = oracle.cg_2d(G, 2e-2, flat(rho), flat(b), np.zeros(G.N), tol=tol, maxiter=3000)
    assert abs(it - itr) <= 1
    # after ~150 iterations the rounding of the two summation orders has moved the iterates; both stop at
    # residual norm < tol, so they agree to the accuracy that residual allows
    assert rel(x, xr) <= max(RTOL_CG, 1e3 * tol)


def test_cg_solve_rejects_other_operators(igr):
    basis = igr.DGBasis(2)
    mesh = igr.CartesianMesh2D(2, 2, 1.0, 1.0, basis)
    x = np.zeros(mesh.x.shape)
    with pytest.raises(TypeError):
        igr.cg_solve_(x, lambda y, v: None, x, 1e-12, 10)


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_cg_solve_2d_manufactured_solution(igr, oracle, p):
    # IGR_adjoints_2d/tests/run_euler_test.jl:38-79 on the CUDA operator: Sigma = sin(2 pi x) sin(2 pi y), rho = 1,
    # cg_solve!(Sigma, apply_A!, b, 1e-12, 5000) for N_e = 4, 8, 16, 32; the L2 error converges at order ~ p + 1
    alpha = 0.1
    errs = []
    for ne in (4, 8, 16, 32):
        basis = igr.DGBasis(p)
        mesh = igr.CartesianMesh2D(ne, ne, 1.0, 1.0, basis)
        G = oracle.Grid2D(p, ne, ne)
        ex = np.sin(2 * np.pi * mesh.x) * np.sin(2 * np.pi * mesh.y)
        k2 = 2 * (2 * np.pi) ** 2
        ww = np.outer(basis.w, basis.w)[:, :, None, None] * mesh.Jx * mesh.Jy
        b = np.asfortranarray(ww * (1 + alpha * k2) * ex)
        rho = np.ones(mesh.x.shape, order="F")
        S = np.zeros(mesh.x.shape, order="F")
        it = igr.cg_solve_(S, igr.sip_operator(rho, basis, mesh, alpha), b, 1e-12, 5000)
        Sr, itr = oracle.cg_2d(G, alpha, flat(rho), flat(b), np.zeros(G.N), tol=1e-12, maxiter=5000)
        assert abs(it - itr) <= 1 and it < 5000
        assert rel(S, Sr) <= RTOL_CG
        errs.append(igr.l2_error(S, ex, basis, mesh))
    orders = [np.log(errs[i - 1] / errs[i]) / np.log(2) for i in range(1, len(errs)) if errs[i] > 1e-13]
    assert orders and min(orders) > p + 0.5, (p, errs, orders)


# ------------------------------------------------------------------------------------------ 1D
@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_operators_1d_match_oracle(igr, oracle, p):
    from igr_sensitivities_gb300 import igr1d
    basis = igr.DGBasis(p)
    mesh = igr.PeriodicMesh1D(13, 1.3, basis)
    G = oracle.Grid1D(p, 13, 1.3)
    q = state1d(mesh, 40 + p)
    rng = np.random.default_rng(p)
    x = rng.standard_normal(mesh.x.shape)
    y = np.zeros(mesh.x.shape, order="F")
    igr1d.apply_sip_(y, x, q[1], basis, mesh, 6e-3)
    assert rel(y, oracle.apply_sip_1d(G, 6e-3, flat(x), flat(q[1]))) <= RTOL_OP
    b = np.zeros(mesh.x.shape, order="F")
    igr1d.compute_igr_rhs_(b, *q, basis, mesh, 6e-3)
    assert rel(b, oracle.igr_rhs_1d(G, 6e-3, flat(q[0]), flat(q[1]))) <= RTOL_OP
    M = igr1d.compute_sip_diagonal(q[1], basis, mesh, 6e-3)
    assert rel(M, oracle.sip_diagonal_1d(G, 6e-3, flat(q[1]))) <= RTOL_OP
    S = 0.01 * rng.standard_normal(mesh.x.shape)
    k = [np.zeros(mesh.x.shape, order="F") for _ in range(3)]
    igr1d.compute_hyperbolic_rhs_(*k, *q, S, basis, mesh, 1.4)
    for a, r in zip(k, oracle.hyperbolic_rhs_1d(G, 1.4, [flat(a) for a in q], flat(S))):
        assert rel(a, r) <= RTOL_OP


@pytest.mark.parametrize("solver,ne", [("pcg", 13), ("chebyshev", 13), ("jacobi", 13), ("chebyshev", 96),
                                       ("pcg", 300)])
def test_solve_elliptic_and_euler_rhs_1d_match_oracle(igr, oracle, solver, ne):
    # ne = 96: small enough to spread over a thread-block cluster (distributed shared memory solver)
    from igr_sensitivities_gb300 import igr1d
    basis = igr.DGBasis(3)
    mesh = igr.PeriodicMesh1D(ne, 1.0, basis)
    G = oracle.Grid1D(3, ne)
    q = state1d(mesh, ne)
    S0 = 0.01 * np.random.default_rng(9).standard_normal(mesh.x.shape)
    alpha = 3.0 * mesh.dx ** 2
    S = np.array(S0, order="F")
    igr1d.solve_elliptic_(S, *q, basis, mesh, alpha, n_iter=8, solver=solver)
    assert rel(S, oracle.solve_elliptic_1d(G, alpha, 8, solver, [flat(a) for a in q], flat(S0))) <= RTOL_SOLVE
    for a in (alpha, 0.0):
        S = np.array(S0, order="F")
        k = [np.zeros(mesh.x.shape, order="F") for _ in range(3)]
        igr1d.compute_igr_euler_rhs_(*k, *q, S, basis, mesh, 1.4, a, n_iter=8, solver=solver)
        ref, Sr = oracle.igr_euler_rhs_1d(G, 1.4, a, 8, solver, [flat(x) for x in q], flat(S0))
        assert rel(S, Sr) <= RTOL_SOLVE if a > 0 else np.all(S == 0.0)
        for x, r in zip(k, ref):
            assert rel(x, r) <= RTOL_SOLVE


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_cg_solve_1d_manufactured_solution(igr, oracle, p):
    # IGR_adjoints_1d/tests/run_euler_test.jl:127-170: Sigma = sin(2 pi x), rho = 1,
    # cg_solve!(Sigma, apply_A!, b, 1e-13, 1000) for N_e = 4, 8, 16, 32
    alpha = 0.1
    errs = []
    for ne in (4, 8, 16, 32):
        basis = igr.DGBasis(p)
        mesh = igr.PeriodicMesh1D(ne, 1.0, basis)
        G = oracle.Grid1D(p, ne)
        ex = np.sin(2 * np.pi * mesh.x)
        b = np.asfortranarray(basis.w[:, None] * mesh.J * (1 + 4 * np.pi ** 2 * alpha) * ex)
        rho = np.ones(mesh.x.shape, order="F")
        S = np.zeros(mesh.x.shape, order="F")
        it = igr.cg_solve_(S, igr.sip_operator(rho, basis, mesh, alpha), b, 1e-13, 1000)
        Sr, itr = oracle.cg_1d(G, alpha, flat(rho), flat(b), np.zeros(G.N), tol=1e-13, maxiter=1000)
        assert abs(it - itr) <= 1 and it < 1000
        assert rel(S, Sr) <= RTOL_CG
        w = basis.w[:, None] * mesh.J
        errs.append(np.sqrt(np.sum(w * (S - ex) ** 2)))
    orders = [np.log(errs[i - 1] / errs[i]) / np.log(2) for i in range(1, len(errs)) if errs[i] > 1e-14]
    assert orders and min(orders) > p + 0.5, (p, errs, orders)


def test_cg_solve_1d_random_system_matches_oracle(igr, oracle):
    basis = igr.DGBasis(3)
    mesh = igr.PeriodicMesh1D(64, 1.0, basis)
    G = oracle.Grid1D(3, 64)
    rng = np.random.default_rng(5)
    rho = np.asfortranarray((0.6 + rng.random(G.N)).reshape(mesh.x.shape, order="F"))
    b = np.asfortranarray(rng.standard_normal(G.N).reshape(mesh.x.shape, order="F"))
    x = np.zeros(mesh.x.shape, order="F")
    it = igr.cg_solve_(x, igr.sip_operator(rho, basis, mesh, 2e-2), b, 1e-8, 3000)
    xr, itr = oracle.cg_1d(G, 2e-2, flat(rho), flat(b), np.zeros(G.N), tol=1e-8, maxiter=3000)
    assert abs(it - itr) <= 1
    assert rel(x, xr) <= 1e-5  # both stop at residual norm < 1e-8 (see the 2D random-system test)


def test_cg_fixed_1d_matches_oracle(igr, oracle):
    basis = igr.DGBasis(3)
    mesh = igr.PeriodicMesh1D(20, 1.0, basis)
    G = oracle.Grid1D(3, 20)
    rng = np.random.default_rng(2)
    rho = 0.6 + rng.random(mesh.x.shape)
    b = rng.standard_normal(mesh.x.shape)
    x0 = 0.1 * rng.standard_normal(mesh.x.shape)
    x = np.array(x0, order="F")
    n = igr.cg_fixed_(x, igr.sip_operator(rho, basis, mesh, 1e-2), b, 12)
    xr, nr = oracle.cg_1d(G, 1e-2, flat(rho), flat(b), flat(x0), maxiter=12, fixed=True)
    assert n == nr == 12
    assert rel(x, xr) <= RTOL_SOLVE
