"""GPU parity tests of the 2D tangent (run_sensitivity, IGR_adjoints_2d/
sensitivity.jl:353-413) against the CPU oracle, through the C ABI.

Tolerance: field-wise relative L2 <= 1e-11 for the state, Sigma, the
tangent and varsigma (the forward-state bar; the reference's own tangent
test compares against finite differences at 5e-4,
IGR_adjoints_2d/tests/run_sensitivity_test.jl:169)."""
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


def case(igr, oracle, p, ne, seed):
    g = 1.4
    basis = igr.DGBasis(p)
    mesh = igr.CartesianMesh2D(ne, ne, 1.0, 1.0, basis)
    G = oracle.Grid2D(p, ne, ne, 1.0, 1.0)
    q0 = W.seeded_pulses_2d(mesh, g, W.seed_for(2, seed), width=0.12)
    rng = np.random.default_rng(seed)
    s0 = [np.asfortranarray(0.05 * rng.standard_normal(mesh.x.shape)) for _ in range(4)]
    s0[2] = np.asfortranarray(np.abs(s0[2]))
    dt = W.cfl_dt_2d(mesh, p, q0, g, 0.1)
    return g, basis, mesh, G, q0, s0, dt


@pytest.mark.parametrize("p,ne,solver,alpha_scale,n_iter,s_gamma", [
    (3, 6, "pcg", 3.0, 8, 0.0),
    (3, 6, "chebyshev", 3.0, 5, 0.0),
    (3, 5, "jacobi", 3.0, 4, 0.0),
    (2, 6, "pcg", 2.0, 6, 0.0),
    (3, 6, "pcg", 0.0, 3, 0.0),
    (3, 6, "chebyshev", 3.0, 5, 0.7),
    (4, 4, "pcg", 3.0, 5, 0.0),
    (1, 6, "chebyshev", 3.0, 5, 0.0),
])
def test_run_sensitivity_matches_oracle(igr, oracle, p, ne, solver, alpha_scale, n_iter, s_gamma):
    g, basis, mesh, G, q0, s0, dt = case(igr, oracle, p, ne, 3 + p)
    alpha = alpha_scale * (1.0 / ne) ** 2
    T = 12 * dt * 0.999
    out = igr.run_sensitivity(*q0, *s0, dt, T, basis, mesh, g, alpha, n_iter=n_iter, solver=solver, s_gamma=s_gamma)
    qr, Sr, sr, vr = oracle.run_sensitivity_2d(G, g, alpha, dt, T, n_iter, solver, [flat(a) for a in q0],
                                               [flat(a) for a in s0], s_gamma=s_gamma)
    for a, b in zip(out[:4], qr):
        assert rel(a, b) <= RTOL
    for a, b in zip(out[5:9], sr):
        assert rel(a, b) <= RTOL, [rel(x, y) for x, y in zip(out[5:9], sr)]
    if alpha > 0:
        assert rel(out[4], Sr) <= RTOL
        assert rel(out[9], vr) <= RTOL
    else:
        assert np.all(out[4] == 0) and np.all(out[9] == 0)


def test_tangent_is_homogeneous(igr, oracle):
    """The tangent system is linear in its initial direction and every solver
    iteration is scale-invariant, so doubling s0 doubles the tangent (exactly
    in floating point, away from the 1e-30 guards) at any size."""
    g, basis, mesh, G, q0, s0, dt = case(igr, oracle, 3, 16, 11)
    alpha = 3.0 * (1.0 / 16) ** 2
    T = 6 * dt * 0.999
    a = igr.run_sensitivity(*q0, *s0, dt, T, basis, mesh, g, alpha, n_iter=10, solver="pcg")
    b = igr.run_sensitivity(*q0, *[2.0 * x for x in s0], dt, T, basis, mesh, g, alpha, n_iter=10, solver="pcg")
    for x, y in zip(a[:5], b[:5]):
        assert np.array_equal(x, y)  # primal untouched by the tangent
    for x, y in zip(a[5:], b[5:]):
        assert rel(2.0 * x, y) <= 1e-14


def test_zero_direction_gives_zero_tangent(igr, oracle):
    g, basis, mesh, G, q0, s0, dt = case(igr, oracle, 3, 8, 5)
    z = [np.zeros_like(x) for x in s0]
    out = igr.run_sensitivity(*q0, *z, dt, 5 * dt, basis, mesh, g, 3.0 / 64, n_iter=6, solver="pcg")
    for x in out[5:]:
        assert np.all(x == 0)


def test_batched_tangent_matches_single_and_gamma_cross_check(igr, oracle):
    """The batched tangent equals the single-instance call bitwise; on the
    vortex-pair + pulse family, the tangent's dJ/dgamma (s0 = 0, s_gamma = 1)
    agrees with the adjoint's dJ/dgamma up to the frozen-wave-speed term
    (sensitivity.jl:81-84 omits d lambda), and the adjoint agrees with central
    finite differences."""
    p, ne, n, nit = 3, 10, 6, 8
    basis = igr.DGBasis(p)
    mesh = igr.CartesianMesh2D(ne, ne, 1.0, 1.0, basis)
    G = oracle.Grid2D(p, ne, ne)
    gam = [1.5, 1.35, 1.65]
    q0, dts = [], []
    for b, g in enumerate(gam):
        q = W.oseen_pair_pulse_2d(mesh, g, W.seed_for(5, b))
        q0.append(np.stack([flat(a) for a in q]))
        dts.append(W.cfl_dt_2d(mesh, p, q, g, 0.1))
    q0 = np.stack(q0)
    alpha = 3.0 / ne ** 2
    Ts = [n * dt * 0.999 for dt in dts]
    dtr = [T / n for T in Ts]  # run_sensitivity's re-rounded step
    s0 = np.zeros_like(q0)
    qb, Sb, sb, Vb = igr.sensitivity_batch(q0, s0, gam, alpha, dtr, n, basis, mesh, n_iter=nit, solver="pcg", s_gamma=1.0)
    prm = (0.3, 0.3, 0.4)
    x, y = flat(mesh.x), flat(mesh.y)
    c = np.tile(np.outer(basis.w, basis.w).reshape(-1, order="F"), ne * ne) * mesh.Jx * mesh.Jy
    chi = ((x >= prm[0]) & (x <= prm[0] + prm[2]) & (y >= prm[1]) & (y <= prm[1] + prm[2])).astype(float)
    shape = mesh.x.shape
    for b, g in enumerate(gam):
        one = igr.run_sensitivity(*[q0[b, v].reshape(shape, order="F") for v in range(4)],
                                  *[np.zeros(shape, order="F") for _ in range(4)], dts[b], Ts[b], basis, mesh, g, alpha,
                                  n_iter=nit, solver="pcg", s_gamma=1.0)
        for v in range(4):
            assert np.array_equal(qb[b, v], flat(one[v])) and np.array_equal(sb[b, v], flat(one[5 + v]))
        assert np.array_equal(Sb[b], flat(one[4])) and np.array_equal(Vb[b], flat(one[9]))
        qr, Sr, sr, vr = oracle.run_sensitivity_2d(G, g, alpha, dts[b], Ts[b], nit, "pcg", list(q0[b]),
                                                   [np.zeros(G.N)] * 4, s_gamma=1.0)
        for v in range(4):
            assert rel(sb[b, v], sr[v]) <= RTOL
        tangent = float(np.sum(c * 2.0 * qb[b, 2] * chi * sb[b, 2]))
        res = igr.enzyme_adjoint_ic(*[q0[b, v].reshape(shape, order="F") for v in range(4)], n, dtr[b], basis, mesh, g,
                                    alpha, n_iter=nit, solver="pcg", objective="window_rho2", obj_params=prm,
                                    with_params=True)
        adj = res[5]
        h = 1e-6
        Jp = igr.objective_value(*[q0[b, v].reshape(shape, order="F") for v in range(4)], n, dtr[b], basis, mesh, g + h,
                                 alpha, n_iter=nit, solver="pcg", objective="window_rho2", obj_params=prm)
        Jm = igr.objective_value(*[q0[b, v].reshape(shape, order="F") for v in range(4)], n, dtr[b], basis, mesh, g - h,
                                 alpha, n_iter=nit, solver="pcg", objective="window_rho2", obj_params=prm)
        fd = (Jp - Jm) / (2 * h)
        scale = max(abs(adj), 1e-4)  # dJ/dgamma passes near zero for some draws: compare on the problem's scale
        assert abs(adj - fd) <= 1e-5 * scale
        assert abs(tangent - adj) <= 2e-2 * scale
