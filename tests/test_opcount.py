"""The algorithmic FP64 operation counts recorded for the benchmark's roofline:
the restated reference arithmetic (oracle) run with an operation-counting
scalar, forward and reverse (operation-by-operation adjoint rule), per node of
a 2D P3 mesh. The numbers are the ones bench.py's ALG_OPS_PER_NODE carries."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_p3_counts_match_the_recorded_constants(oracle):
    sys.path.insert(0, ROOT)
    import bench
    G = oracle.Grid2D(3, 12, 12)
    c = oracle.opcount_2d(G, "chebyshev", 5)
    assert c["setup"] == (131.0, 350.0)
    assert c["apply"] == (106.0, 249.0)
    assert c["iteration"] == (112.0, 264.0) and c["solver_init"] == (105.0, 247.0)
    assert c["hyperbolic_rk"] == (168.0, 406.5)
    assert c["step"] == (2892.0, 6970.5)
    assert bench.ALG_OPS_PER_NODE_STEP == c["step"][0] + c["step"][1]
    # per-launch figures of the six kernel families (Chebyshev 5: five operator launches per stage)
    fam = bench.ALG_OPS_PER_NODE
    assert fam[0] == c["setup"][0] and fam[5] == c["setup"][1]
    assert fam[2] == c["hyperbolic_rk"][0] and fam[3] == c["hyperbolic_rk"][1]
    assert fam[1] == pytest.approx((c["solver_init"][0] + 5 * c["iteration"][0]) / 5)
    assert fam[4] == pytest.approx((c["solver_init"][1] + 5 * c["iteration"][1]) / 5)


def test_counts_do_not_depend_on_the_mesh_size(oracle):
    a = oracle.opcount_2d(oracle.Grid2D(3, 8, 8), "pcg", 60)
    b = oracle.opcount_2d(oracle.Grid2D(3, 16, 16), "pcg", 60)
    for k in ("setup", "apply", "hyperbolic_rk"):
        assert a[k] == b[k]
    # the PCG scalars (alpha, beta) are per solve, not per node: a share that shrinks with the mesh
    assert a["iteration"][0] == pytest.approx(b["iteration"][0], rel=1e-4)
    assert a["step"][0] == pytest.approx(b["step"][0], rel=1e-4)
