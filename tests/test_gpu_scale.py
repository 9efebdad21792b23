"""GPU parity against the CPU oracle at the benchmark configurations' mesh
sizes, through the C ABI (the code paths the benchmarks run: 1024-tile
instances, several instance groups per batch, PCG inner products completed by
a separate launch above 4096 tiles, the 1D single-instance cluster path).

Each case runs the configuration's mesh, degree, solver and objective for a
step count the oracle finishes in seconds (OpenMP over instances):
  2D 64^2 P3 gradient, Chebyshev 5, window rho^2, 20 of 200 steps
  2D 128^2 P3 gradients, the benchmark's batch workload, 10 instances in two
      groups of 5 (5120 tiles per group), 3 of 200 steps
  2D 128^2 P3 gradients with PCG 10 in one group of 5 (5120 tiles: the
      separate-launch inner products), 2 steps
  2D 128^2 P3 forward, PCG 60, 3 of 500 steps (persistent solves, published hand-offs)
  2D 64^2 P3 and 22^2 P4 forwards, PCG 60, 3 steps (persistent solves, counted hand-offs)
  1D N_e = 256 P3 forward, Jacobi 50, the whole T = 0.1
Tolerances (relative L2): forward state and Sigma 1e-11 (Sigma of the PCG-60
forward: 3x the oracle's own change under a one-ulp input perturbation,
which is larger), gradients 1e-9,
J 1e-11, dJ/dgamma and dJ/dalpha 1e-9 (of the value, or of J / parameter
where the value is at the rounding level of J: a window away from the
pulses barely feels gamma or alpha within a few steps; a pressure objective
checks a large dJ/dgamma).
"""
import os
import sys

import numpy as np
import pytest

from igr_sensitivities_gb300 import workloads as W

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
RTOL_FWD, RTOL_GRAD, RTOL_J = 1e-11, 1e-9, 1e-11
THREADS = os.cpu_count() or 1


def rel(a, b):
    a, b = np.ravel(a), np.ravel(b)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def flat(a):
    return np.ascontiguousarray(np.asarray(a).reshape(-1, order="F"))


def batch_128(igr, B, first=0):
    sys.path.insert(0, ROOT)
    import bench
    basis, mesh, q0, gam, alp, dts, prm = bench.make_batch(igr, W, B, first=first)
    dt = float(dts[0])  # the oracle's batch call takes one step size
    return basis, mesh, q0, gam, alp, np.full(B, dt), prm


def check_params(J, dg, da, Jr, dgr, dar, gamma, alpha):
    # dJ/dgamma, dJ/dalpha: relative error 1e-9, or, where the window objective is insensitive to the parameter
    # over a few steps (the value sits at the rounding level of J's sum), 1e-9 on the scale of J / parameter
    for d, dr, par in ((dg, dgr, gamma), (da, dar, alpha)):
        d, dr, par, Jr_ = np.ravel(d), np.ravel(dr), np.ravel(par) * np.ones(np.size(dr)), np.ravel(Jr)
        for k in range(dr.size):
            assert abs(d[k] - dr[k]) <= RTOL_GRAD * max(abs(dr[k]), abs(Jr_[k]) / par[k]), (k, d[k], dr[k])


def check_gradients(out, ref, gam, alp):
    J, dq, dg, da = out
    Jr, dqr, dgr, dar = ref
    assert rel(J, Jr) <= RTOL_J
    for b in range(len(J)):
        assert rel(dq[b], dqr[b]) <= RTOL_GRAD, b
    check_params(J, dg, da, Jr, dgr, dar, gam, alp)


def test_adjoint_64_chebyshev_matches_oracle(igr, oracle):
    # the single-instance adjoint configuration: 64^2 P3, Chebyshev 5, window rho^2 (20 of its 200 steps)
    g, p, ne, nst = 1.4, 3, 64, 20
    basis = igr.DGBasis(p)
    mesh = igr.CartesianMesh2D(ne, ne, 1.0, 1.0, basis)
    q0 = W.seeded_pulses_2d(mesh, g, W.seed_for(3, 0), n_pulses=3, width=0.03)
    dt = W.cfl_dt_2d(mesh, p, q0, g, 0.1)
    alpha = 3.0 / ne ** 2
    prm = W.seeded_window(W.seed_for(3, 0))
    out = igr.enzyme_adjoint_ic(*q0, nst, dt, basis, mesh, g, alpha, n_iter=5, solver="chebyshev",
                                objective="window_rho2", obj_params=prm, with_params=True)
    G = oracle.Grid2D(p, ne, ne)
    Jr, dqr, dgr, dar = oracle.adjoint_2d(G, g, alpha, nst, dt, 5, "chebyshev", "window_rho2", [flat(a) for a in q0], prm)
    assert rel(out[0], Jr) <= RTOL_J
    assert rel(np.concatenate([flat(a) for a in out[1:5]]), np.concatenate(dqr)) <= RTOL_GRAD
    check_params(out[0], out[5], out[6], Jr, dgr, dar, g, alpha)


def test_adjoint_64_l2_pressure_gamma_gradient_matches_oracle(igr, oracle):
    # the same mesh and solver with J = integral of P^2, which depends on gamma directly: dJ/dgamma is large
    g, p, ne, nst = 1.4, 3, 64, 10
    basis = igr.DGBasis(p)
    mesh = igr.CartesianMesh2D(ne, ne, 1.0, 1.0, basis)
    q0 = W.seeded_pulses_2d(mesh, g, W.seed_for(3, 1), n_pulses=3, width=0.03)
    dt = W.cfl_dt_2d(mesh, p, q0, g, 0.1)
    alpha = 3.0 / ne ** 2
    out = igr.enzyme_adjoint_ic(*q0, nst, dt, basis, mesh, g, alpha, n_iter=5, solver="chebyshev",
                                objective="l2_pressure", with_params=True)
    G = oracle.Grid2D(p, ne, ne)
    Jr, dqr, dgr, dar = oracle.adjoint_2d(G, g, alpha, nst, dt, 5, "chebyshev", "l2_pressure", [flat(a) for a in q0])
    assert abs(dgr) * g > 0.1 * abs(Jr)
    assert rel(out[0], Jr) <= RTOL_J and rel(out[5], dgr) <= RTOL_GRAD
    assert rel(np.concatenate([flat(a) for a in out[1:5]]), np.concatenate(dqr)) <= RTOL_GRAD


def test_adjoint_batch_128_two_groups_matches_oracle(igr, oracle):
    # the benchmark's 128^2 batch (Chebyshev 5, window rho^2): a tape budget of five instances' full tapes splits
    # ten instances into two groups of five, as the 200-step workload splits 32 instances into four groups of eight
    B, nst = 10, 3
    basis, mesh, q0, gam, alp, dts, prm = batch_128(igr, B)
    N = mesh.x.size
    F = 16 + 2 * 5  # fields of one taped Chebyshev-5 stage
    ctx = igr.Context(0)
    ctx.set_tape_budget(5 * (3 * F * nst + 6) * N * 8 + 1024)
    out = igr.adjoint_batch(q0, gam, alp, dts, nst, basis, mesh, n_iter=5, solver="chebyshev", objective="window_rho2",
                            obj_params=prm, ctx=ctx)
    plan = ctx.last_adjoint_plan()
    assert plan["groups"] == 2 and plan["instances_per_group"] == 5 and plan["segments"] == 1
    G = oracle.Grid2D(3, 128, 128)
    ref = oracle.adjoint_batch_2d(G, gam, alp, nst, float(dts[0]), 5, "chebyshev", "window_rho2", q0, prm,
                                  n_threads=THREADS)
    check_gradients(out, ref, gam, alp)


def test_adjoint_batch_128_pcg_separate_sums_matches_oracle(igr, oracle):
    # five 128^2 instances in one group: 5120 tiles, above the 4096 up to which the PCG inner products complete
    # inside their kernels, so the forward and reverse sums run as separate launches
    B, nst = 5, 2
    basis, mesh, q0, gam, alp, dts, prm = batch_128(igr, B, first=40)
    ctx = igr.Context(0)
    out = igr.adjoint_batch(q0, gam, alp, dts, nst, basis, mesh, n_iter=10, solver="pcg", objective="window_rho2",
                            obj_params=prm, ctx=ctx)
    assert ctx.last_adjoint_plan()["groups"] == 1
    G = oracle.Grid2D(3, 128, 128)
    ref = oracle.adjoint_batch_2d(G, gam, alp, nst, float(dts[0]), 10, "pcg", "window_rho2", q0, prm,
                                  n_threads=THREADS)
    check_gradients(out, ref, gam, alp)


def test_forward_128_pcg60_matches_oracle(igr, oracle):
    # the 2D forward configuration: 128^2 P3, PCG 60 per stage (3 of its 500 steps), run_forward with re-rounding
    g, p, ne = 1.4, 3, 128
    basis = igr.DGBasis(p)
    mesh = igr.CartesianMesh2D(ne, ne, 1.0, 1.0, basis)
    q0 = W.seeded_pulses_2d(mesh, g, W.seed_for(2, 0), n_pulses=3, width=0.03)
    dt = W.cfl_dt_2d(mesh, p, q0, g, 0.1)
    alpha, T = 3.0 / ne ** 2, 3 * dt * 0.999
    out = igr.run_forward(*q0, dt, T, basis, mesh, g, alpha, n_iter=60, solver="pcg")
    G = oracle.Grid2D(p, ne, ne)
    f0 = [flat(a) for a in q0]
    qr, Sr = oracle.run_forward_2d(G, g, alpha, dt, T, 60, "pcg", f0)
    for a, b in zip(out[:4], qr):
        assert rel(flat(a), b) <= RTOL_FWD
    # Sigma of this state is sensitive to rounding: the oracle's own Sigma moves by ~4e-10 (relative L2) when
    # rho0 and E0 move by one ulp (state: ~5e-14), more than the GPU differs from it. Its bound is that spread.
    rng = np.random.default_rng(0)
    fp = [np.nextafter(a, a + rng.choice([-1.0, 1.0], size=a.size)) if v >= 2 else a for v, a in enumerate(f0)]
    _, Sp = oracle.run_forward_2d(G, g, alpha, dt, T, 60, "pcg", fp)
    spread = rel(Sp, Sr)
    assert rel(flat(out[4]), Sr) <= max(RTOL_FWD, 3.0 * spread), spread


@pytest.mark.parametrize("p,ne,nst", [(3, 64, 3), (4, 22, 3)])
def test_forward_pcg60_counted_handoff_matches_oracle(igr, oracle, p, ne, nst):
    # single instances whose PCG-60 solves run as persistent launches with counted hand-offs (256 P3 tiles at
    # 64^2; 66 P4 tiles at 22^2, the finest OtD resolution below 30), against the oracle
    g = 1.4
    basis = igr.DGBasis(p)
    mesh = igr.CartesianMesh2D(ne, ne, 1.0, 1.0, basis)
    q0 = W.seeded_pulses_2d(mesh, g, W.seed_for(2, 1), n_pulses=3, width=0.05)
    dt = W.cfl_dt_2d(mesh, p, q0, g, 0.1)
    alpha, T = 3.0 / ne ** 2, nst * dt * 0.999
    out = igr.run_forward(*q0, dt, T, basis, mesh, g, alpha, n_iter=60, solver="pcg")
    G = oracle.Grid2D(p, ne, ne)
    f0 = [flat(a) for a in q0]
    qr, Sr = oracle.run_forward_2d(G, g, alpha, dt, T, 60, "pcg", f0)
    for a, b in zip(out[:4], qr):
        assert rel(flat(a), b) <= RTOL_FWD
    # Sigma on the scale of the oracle's own change under a one-ulp input perturbation (as for 128^2)
    rng = np.random.default_rng(1)
    fp = [np.nextafter(a, a + rng.choice([-1.0, 1.0], size=a.size)) if v >= 2 else a for v, a in enumerate(f0)]
    _, Sp = oracle.run_forward_2d(G, g, alpha, dt, T, 60, "pcg", fp)
    assert rel(flat(out[4]), Sr) <= max(RTOL_FWD, 3.0 * rel(Sp, Sr))


def test_forward_1d_256_jacobi50_full_matches_oracle(igr, oracle):
    # the 1D forward configuration in full: N_e = 256 P3, two pulses (width 0.02), Jacobi 50, T = 0.1
    from igr_sensitivities_gb300 import igr1d
    g, p, ne, T = 1.4, 3, 256, 0.1
    basis = igr.DGBasis(p)
    mesh = igr.PeriodicMesh1D(ne, 1.0, basis)
    q0 = W.seeded_pulses_1d(mesh, g, W.seed_for(1, 0), n_pulses=2, width=0.02)
    dt = W.cfl_dt_1d(mesh, p, q0, g, 0.1)
    alpha = 3.0 * mesh.dx ** 2
    out = igr1d.run_forward(*q0, dt, T, basis, mesh, g, alpha, n_iter=50, solver="jacobi")
    G = oracle.Grid1D(p, ne)
    qr, Sr = oracle.run_forward_1d(G, g, alpha, dt, T, 50, "jacobi", [flat(a) for a in q0])
    assert int(np.ceil(T / dt)) > 4000
    for a, b in zip(out[:3], qr):
        assert rel(flat(a), b) <= RTOL_FWD
    assert rel(flat(out[3]), Sr) <= RTOL_FWD
