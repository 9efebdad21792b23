"""GPU initial-condition builders (IGR_adjoints_2d/initial_conditions.jl,
IGR_adjoints_1d/initial_conditions.jl) and l2_error against the oracle's
restatement, through the C ABI. Tolerance 1e-13 relative per field (the GPU's
exp/sin/pow and FMA contraction differ from the host's by ulps); batches are
bitwise equal to single builds."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-13
OSEEN_DEFAULT = [0.05, 0.5, 0.25, 0.50, 0.09, 0.45, 0.60, 1.0, 0.45, 0.40, -1.0]


def rel(a, b):
    a = np.asarray(a).reshape(-1, order="F")
    b = np.asarray(b).reshape(-1, order="F")
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("ic,A,prm", [
    ("constant", 0.0, [1.0, 1.0, 1.0, 1.0]), ("constant", 0.0, [1.3, 0.2, -0.4, 2.0]),
    ("isentropic_vortex", 0.0, [5.0, 1.0, 1.0]), ("isentropic_vortex", 0.0, [2.0, 0.5, 0.0]),
    ("taylor_green", 0.4, [0.0]), ("sedov_blast", 6.0, [1.0, 0.1]), ("sedov_blast", 3.0, [0.5, 0.2]),
    ("oseen_pair_blast", 5.0, OSEEN_DEFAULT),
    ("oseen_pair_blast", 2.0, [0.04, 0.4, 0.3, 0.6, 0.1, 0.5, 0.55, 1.0, 0.5, 0.35, -1.0]),
])
@pytest.mark.parametrize("gamma", [1.4, 1.3])
def test_build_ic_2d_matches_oracle(igr, oracle, ic, A, prm, gamma):
    basis = igr.DGBasis(3)
    mesh = igr.CartesianMesh2D(10, 8, 1.0, 1.0, basis)
    G = oracle.Grid2D(3, 10, 8)
    q = igr.build_ic_batch(ic, basis, mesh, [gamma], [A], params=prm if ic != "taylor_green" else None)[0]
    ref = oracle.build_ic_2d(G, ic, gamma, A, prm + [0.0] * (11 - len(prm)))
    for v in range(4):
        if np.linalg.norm(ref[v]) == 0:
            assert np.all(q[v] == 0)
        else:
            assert rel(q[v], ref[v]) <= RTOL, (ic, v, rel(q[v], ref[v]))


def test_reference_named_builders_and_batch(igr, oracle):
    basis = igr.DGBasis(3)
    mesh = igr.CartesianMesh2D(8, 8, 1.0, 1.0, basis)
    G = oracle.Grid2D(3, 8, 8)
    shape = mesh.shape(basis)
    z = [np.zeros(shape, order="F") for _ in range(4)]
    igr.build_oseen_pair_blast_ic_(*z, 5.0, mesh, 1.4)
    ref = oracle.build_ic_2d(G, "oseen_pair_blast", 1.4, 5.0, OSEEN_DEFAULT)
    for a, b in zip(z, ref):
        assert rel(a, b) <= RTOL
    igr.IC_BUILDERS["sedov_blast"][0](*z, 4.0, mesh, 1.4)
    ref = oracle.build_ic_2d(G, "sedov_blast", 1.4, 4.0, [1.0, 0.1] + [0.0] * 9)
    for a, b in zip(z, ref):
        assert rel(a, b) <= RTOL
    tg = igr.init_isentropic_vortex(mesh, 1.4)
    ref = oracle.build_ic_2d(G, "isentropic_vortex", 1.4, 0.0, [5.0, 1.0, 1.0] + [0.0] * 8)
    for a, b in zip(tg, ref):
        assert rel(a, b) <= RTOL
    # a batch with per-instance gamma and amplitude == single builds, bitwise
    gs, As = [1.4, 1.3, 1.6], [5.0, 2.0, 7.5]
    qb = igr.build_ic_batch("oseen_pair_blast", basis, mesh, gs, As)
    for b in range(3):
        one = igr.build_ic_batch("oseen_pair_blast", basis, mesh, [gs[b]], [As[b]])[0]
        assert np.array_equal(qb[b], one)
    with pytest.raises(ValueError):
        igr.build_ic_batch("kelvin_helmholtz", basis, mesh, [1.4], [1.0])


def test_l2_error_matches_oracle(igr, oracle):
    basis = igr.DGBasis(3)
    mesh = igr.CartesianMesh2D(9, 7, 1.0, 2.0, basis)
    G = oracle.Grid2D(3, 9, 7, 1.0, 2.0)
    rng = np.random.default_rng(3)
    u, r = rng.standard_normal(G.N), rng.standard_normal(G.N)
    e = igr.l2_error(u.reshape(mesh.x.shape, order="F"), r.reshape(mesh.x.shape, order="F"), basis, mesh)
    assert abs(e - oracle.l2_error_2d(G, u, r)) <= 1e-14 * e


@pytest.mark.parametrize("ic", ["acoustic_pulse", "entropy_wave", "density_pulse", "pressure_pulse", "velocity_pulse"])
def test_build_ic_1d_matches_oracle_and_host_builders(igr, oracle, ic):
    from igr_sensitivities_gb300 import igr1d
    basis = igr.DGBasis(3)
    nes, gs, As = [8, 20, 13], [1.4, 1.3, 1.6], [0.2, 0.1, 0.3]
    out = igr1d.build_ic_batch(ic, basis, nes, 1.0, gs, As)
    for i, ne in enumerate(nes):
        G = oracle.Grid1D(3, ne)
        ref = oracle.build_ic_1d(G, ic, gs[i], As[i])
        for a, b in zip(out[i], ref):
            assert rel(a, b) <= RTOL or np.linalg.norm(b) == 0


def test_device_ic_feeds_the_device_batch_adjoint(igr):
    """build_ic_batch(device_array=True) -> adjoint_batch(device_arrays=True):
    the sweep never leaves the GPU, and equals the host-array call bitwise."""
    torch = pytest.importorskip("torch")
    basis = igr.DGBasis(3)
    mesh = igr.CartesianMesh2D(8, 8, 1.0, 1.0, basis)
    gs, As = [1.4, 1.4, 1.4], [2.0, 4.0, 6.0]
    qd = igr.build_ic_batch("sedov_blast", basis, mesh, gs, As, params=[1.0, 0.1], device_array=True)
    qh = igr.build_ic_batch("sedov_blast", basis, mesh, gs, As, params=[1.0, 0.1])
    assert np.array_equal(qd.cpu().numpy(), qh)
    dts, als = [1e-3] * 3, [3.0 / 400] * 3
    Jd, dqd, _, _ = igr.adjoint_batch(qd, gs, als, dts, 4, basis, mesh, n_iter=5, solver="chebyshev",
                                      objective="kinetic_energy", device_arrays=True)
    Jh, dqh, _, _ = igr.adjoint_batch(qh, gs, als, dts, 4, basis, mesh, n_iter=5, solver="chebyshev",
                                      objective="kinetic_energy")
    torch.cuda.synchronize()
    assert np.array_equal(Jd, Jh) and np.array_equal(dqd.cpu().numpy(), dqh)


def test_sedov_otd_gap_of_the_continuous_adjoint(igr):
    """The paper's OtD-gap measure (2d/paper_scripts/generate_otd_refinement_sedov_data.jl:
    adjoint directional derivative <a, dq0/dA>_M against a central difference of
    the forward map) on one Sedov blast: the continuous adjoint agrees with FD
    within the optimise-then-discretise gap."""
    g, p, ne, T = 1.4, 3, 10, 0.02
    basis = igr.DGBasis(p)
    mesh = igr.CartesianMesh2D(ne, ne, 1.0, 1.0, basis)
    alpha, nit, A0, sig = 3.0 * (1.0 / 20) ** 2, 60, 6.0, 0.1
    shape = mesh.shape(basis)
    q0 = [np.zeros(shape, order="F") for _ in range(4)]
    igr.build_sedov_blast_ic_(*q0, A0, mesh, g, sigma=sig)
    from igr_sensitivities_gb300 import workloads as W
    dt = W.cfl_dt_2d(mesh, p, q0, g, 0.4)
    dt = T / int(np.ceil(T / dt))  # the step both the store and the backward integration use
    a = igr.adjoint_conservative_ic(*q0, dt, T, basis, mesh, g, alpha, n_iter=nit, solver="pcg",
                                    objective="kinetic_energy")
    m = np.outer(basis.w, basis.w)[:, :, None, None] * mesh.Jx * mesh.Jy
    r2 = (mesh.x - 0.5) ** 2 + (mesh.y - 0.5) ** 2
    dE = np.exp(-r2 / sig ** 2) / (g - 1)
    adj = float(np.sum(m * a[3] * dE))

    def J(A):
        q = [np.zeros(shape, order="F") for _ in range(4)]
        igr.build_sedov_blast_ic_(*q, A, mesh, g, sigma=sig)
        mx, my, rho, E, _ = igr.run_forward(*q, dt, T, basis, mesh, g, alpha, n_iter=nit, solver="pcg")
        return float(np.sum(m * (mx ** 2 + my ** 2) / (2 * rho)) / np.sum(m * rho))

    eps = 5e-4
    fd = (J(A0 + eps) - J(A0 - eps)) / (2 * eps)
    assert abs(adj - fd) <= 0.1 * abs(fd), (adj, fd)
