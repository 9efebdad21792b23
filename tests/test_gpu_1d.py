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
    (1, 30, "pcg", 10, 3.0), (2, 20, "jacobi", 8, 3.0), (4, 16, "pcg", 12, 3.0), (3, 1, "pcg", 3, 3.0),
    (3, 300, "pcg", 15, 3.0),
])
def test_run_forward_1d_matches_oracle(igr, igr1d, oracle, p, ne, solver, n_iter, alpha_scale):
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
