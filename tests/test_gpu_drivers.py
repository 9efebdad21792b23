"""The batched OtD refinement driver (IGR_adjoints_2d/paper_scripts/
generate_otd_refinement_{sedov,oseen}_data.jl) against the same pipeline run
on the oracle (IC builder, run_forward_store + run_adjoint_conservative,
central differences of run_forward), at sizes the oracle finishes in seconds."""
import numpy as np
import pytest

from igr_sensitivities_gb300 import drivers
from igr_sensitivities_gb300.workloads import max_wavespeed_2d

pytestmark = pytest.mark.gpu

PRM3 = [1.0, 0.09, 3, 0.30, 0.34, 6.0, 0.70, 0.40, 5.0, 0.52, 0.74, 5.5, 0, 0, 0]


def oracle_gap(igr, oracle, ic, A, Ne, p, T, alpha, nit, objective, eps, prm, g=1.4, CFL=0.4):
    G = oracle.Grid2D(p, Ne, Ne)
    qs = [oracle.build_ic_2d(G, ic, g, a, prm) for a in (A, A + eps, A - eps)]
    dt = CFL * min(G.dx, G.dy) / ((2 * p + 1) * max_wavespeed_2d(*qs[0], g))
    dt = T / int(np.ceil(T / dt))
    snaps, n = oracle.run_forward_store_2d(G, g, alpha, dt, T, nit, "pcg", qs[0])
    a = oracle.run_adjoint_conservative_2d(G, snaps, n, dt, T, g, alpha, nit, objective, "pcg")
    m = np.tile(np.outer(G.w, G.w).reshape(-1, order="F"), Ne * Ne) * G.Jx * G.Jy
    adj = float(sum(np.sum(m * a[v] * (qs[1][v] - qs[2][v]) / (2 * eps)) for v in range(4)))
    J = []
    for q in qs[1:]:
        qT, _ = oracle.run_forward_2d(G, g, alpha, dt, T, nit, "pcg", q)
        J.append(oracle.objective_run_2d(G, g, alpha, 0, dt, nit, "pcg", objective, qT)[0])  # J(q_T) on the CPU
    fd = (J[0] - J[1]) / (2 * eps)
    return adj, fd


@pytest.mark.parametrize("ic,A,prm,objective,eps", [
    ("multi_blast", 6.0, PRM3, "kinetic_energy", 5e-4),
    ("oseen_pair_blast", 12.0, [0.05, 0.5, 0.25, 0.50, 0.09, 0.45, 0.60, 1.0, 0.45, 0.40, -1.0],
     "windowed_kinetic_energy", 1e-3),
])
def test_otd_driver_matches_oracle_pipeline(igr, oracle, ic, A, prm, objective, eps):
    p, T, alpha, nit = 3, 0.01, 3.0 * (1.0 / 20) ** 2, 20
    rows, rates = drivers.otd_refinement(ic, A, [6, 8], p=p, T=T, alpha=alpha, n_iter=nit, solver="pcg",
                                         objective=objective, eps=eps, params=prm)
    assert len(rates) == 1
    for (h, gap, adj, fd), Ne in zip(rows, [6, 8]):
        ra, rf = oracle_gap(igr, oracle, ic, A, Ne, p, T, alpha, nit, objective, eps, prm)
        assert abs(adj - ra) <= 1e-9 * abs(ra), (adj, ra)
        assert abs(fd - rf) <= 1e-7 * abs(rf), (fd, rf)  # FD of nearly equal objectives: ~1e-16 J / (eps dJ)
        assert gap < 0.2 and abs(h - 1.0 / Ne) < 1e-15
