"""The C-ABI library builds, loads and exports every entry point that
include/igr_gb300.h declares (no GPU calls), and the host API rejects bad
arguments before reaching the device."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "igr_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(igr\w+)\s*\(", src, flags=re.M)))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("igr2d_run_forward", "igr2d_adjoint_ic", "igr2d_adjoint_batch", "igr_ctx_create"):
        assert must in names


def test_library_exports_every_declared_symbol(igr):
    lib = ctypes.CDLL(os.path.join(os.path.dirname(igr.__file__), "libigr_gb300.so"))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_api_rejects_unknown_symbols(igr):
    basis = igr.DGBasis(3)
    mesh = igr.CartesianMesh2D(2, 2, 1.0, 1.0, basis)
    z = np.zeros(mesh.x.shape)
    with pytest.raises(ValueError):
        igr._solver("gmres")
    with pytest.raises(ValueError):
        igr._objective(":entropy")
    assert igr._solver(":chebyshev") == 2
    del z


def test_basis_matches_oracle(igr, oracle):
    for p in range(1, 5):
        b = igr.DGBasis(p)
        xi, w, D = oracle.basis(p)
        assert np.array_equal(b.xi, xi) and np.array_equal(b.w, w)
        assert np.max(np.abs(b.D - D)) == 0.0


def test_mesh_coordinates_match_reference_formula(igr):
    b = igr.DGBasis(3)
    m = igr.CartesianMesh2D(3, 2, 1.0, 0.5, b)
    # mesh.jl:116-122: x = (ex-1) dx + Jx (1 + xi_i), y = (ey-1) dy + Jy (1 + xi_j)
    assert m.x[2, 1, 1, 0] == 1 * m.dx + m.Jx * (1.0 + b.xi[2])
    assert m.y[0, 3, 2, 1] == 1 * m.dy + m.Jy * (1.0 + b.xi[3])
