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


def test_python_mirror_rejects_bad_symbols_before_any_device_call(igr):
    """Unknown solver / objective / elliptic_rhs / IC symbols raise with the
    reference's message before a context (or a GPU) is needed."""
    from igr_sensitivities_gb300 import igr1d
    basis = igr.DGBasis(3)
    m2 = igr.CartesianMesh2D(2, 2, 1.0, 1.0, basis)
    m1 = igr.PeriodicMesh1D(4, 1.0, basis)
    z2 = np.zeros(m2.x.shape)
    z1 = np.zeros(m1.x.shape)
    with pytest.raises(ValueError, match="Unknown solver"):
        igr.run_forward(z2, z2, z2, z2, 0.1, 0.2, basis, m2, 1.4, 0.1, solver="gmres")
    with pytest.raises(ValueError, match="Unknown objective"):
        igr.enzyme_adjoint_ic(z2, z2, z2, z2, 1, 0.1, basis, m2, 1.4, 0.1, objective="entropy")
    with pytest.raises(ValueError, match="Unknown elliptic_rhs"):
        igr1d.run_sensitivity(z1, z1, z1, z1, z1, z1, 0.1, 0.2, basis, m1, 1.4, 0.1, elliptic_rhs="form3")
    with pytest.raises(ValueError, match="Unknown solver"):
        igr1d.run_forward(z1, z1, z1, 0.1, 0.2, basis, m1, 1.4, 0.1, solver="cg")
    with pytest.raises(ValueError, match="Unknown objective"):
        igr1d.adjoint_batch([(z1, z1, z1)], basis, [4], 1.0, 1.4, 0.1, 0.1, 1, objective="entropy")
    with pytest.raises(ValueError, match="use :l2_density or :l2_pressure"):
        igr1d.enzyme_adjoint_ic(0.1, 3, 4, 1.0, 1.4, 0.1, 0.5, 0.1, objective="kinetic_energy")
    with pytest.raises(ValueError, match="Unknown IC type"):
        igr1d.enzyme_adjoint_ic(0.1, 3, 4, 1.0, 1.4, 0.1, 0.5, 0.1, ic_type="shock")
    snaps = [(z2, z2, z2, z2, z2)] * 2
    with pytest.raises(ValueError, match="Unknown objective"):
        igr.run_adjoint_conservative(snaps, 1, 0.1, 0.1, basis, m2, 1.4, 0.1, objective="entropy")
    with pytest.raises(ValueError, match="Unknown solver"):
        igr.run_forward_store(z2, z2, z2, z2, 0.1, 0.2, basis, m2, 1.4, 0.1, solver="gmres")
    with pytest.raises(ValueError, match="Unknown solver"):
        igr.adjoint_conservative_ic(z2, z2, z2, z2, 0.1, 0.2, basis, m2, 1.4, 0.1, solver="gmres")


def test_snapshots_index_like_the_reference_list(igr):
    """Snapshots mirrors the Vector of (mux, muy, rho, E, Sigma) tuples that
    run_forward_store returns (forward.jl:111-158): snapshots[k] unpacks into
    five (n_p, n_p, N_ex, N_ey) fields and snapshots[-1] is the state at T."""
    basis = igr.DGBasis(2)
    mesh = igr.CartesianMesh2D(3, 2, 1.0, 1.0, basis)
    shape = mesh.shape(basis)
    n = int(np.prod(shape))
    data = np.arange(3 * 5 * n, dtype=np.float64).reshape(3, 5, n)
    s = igr.Snapshots(data, shape)
    assert len(s) == 3
    mx, my, rho, E, Sig = s[-1]
    assert mx.shape == shape and np.array_equal(Sig.reshape(-1, order="F"), data[2, 4])
    again = igr.Snapshots.from_list([s[k] for k in range(3)], shape)
    assert np.array_equal(again.data, data)


def test_ic_builders_match_reference_formulas():
    """IC_BUILDERS (IGR_adjoints_1d/initial_conditions.jl:94-224): the primitive
    profiles and the conservative conversion."""
    from igr_sensitivities_gb300 import igr1d
    import igr_sensitivities_gb300 as igr
    basis = igr.DGBasis(3)
    mesh = igr.PeriodicMesh1D(5, 2.0, basis)
    s = np.sin(2 * np.pi * mesh.x / 2.0)
    A, g = 0.1, 1.4
    expect = {"acoustic_pulse": (1 + A * s, A * s, 1 + A * s), "entropy_wave": (1 + A * s, 1 + 0 * s, 1 + 0 * s),
              "density_pulse": (1 + A * s, 0 * s, 1 + 0 * s), "pressure_pulse": (1 + 0 * s, 0 * s, 1 + A * s),
              "velocity_pulse": (1 + 0 * s, A * s, 1 + 0 * s)}
    for name, (rho, u, p) in expect.items():
        mu0, rho0, E0 = np.zeros(mesh.x.shape), np.zeros(mesh.x.shape), np.zeros(mesh.x.shape)
        igr1d.IC_BUILDERS[name][0](mu0, rho0, E0, A, mesh.x, 2.0, g)
        assert np.allclose(rho0, rho, rtol=0, atol=1e-15)
        assert np.allclose(mu0, rho * u, rtol=0, atol=1e-15)
        assert np.allclose(E0, p / (g - 1) + 0.5 * rho * u ** 2, rtol=0, atol=1e-14)
    assert igr1d.ic_dA_weights(":pressure_pulse") == (0.0, 0.0, 1.0)
