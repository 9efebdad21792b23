"""igr2d_apply_sip_noalloc against the regular igr2d_apply_sip.

The no-allocation entry point serves callers whose device memory belongs to
another allocator (or that cannot take a synchronising cudaMalloc): it keeps
its scratch in a fixed device array shared by every call. This file is
collected last on purpose, and each test must pass both alone in a fresh
process and after the rest of the suite (which leaves other state behind).
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(igr, basis, mesh, alpha, x, rho):
    import torch
    lib = igr._lib.lib()
    d = igr._disc2d(basis, mesh)
    dev = torch.device("cuda", 0)
    xd = torch.from_numpy(np.asarray(x).reshape(-1, order="F").copy()).to(dev)
    rd = torch.from_numpy(np.asarray(rho).reshape(-1, order="F").copy()).to(dev)
    yd = torch.full_like(xd, float("nan"))
    torch.cuda.synchronize()
    D = C.POINTER(C.c_double)
    rc = lib.igr2d_apply_sip_noalloc(C.byref(d), C.c_double(alpha), C.cast(C.c_void_p(xd.data_ptr()), D),
                                     C.cast(C.c_void_p(rd.data_ptr()), D), C.cast(C.c_void_p(yd.data_ptr()), D), None)
    return rc, yd.cpu().numpy()


def test_apply_sip_noalloc_matches_regular_entry_point_twice(igr):
    basis = igr.DGBasis(3)
    mesh = igr.CartesianMesh2D(16, 12, 1.0, 1.3, basis)
    for call, alpha in enumerate((3e-3, 2e-2)):   # two calls in a row, different data
        rng = np.random.default_rng(100 + call)
        x = rng.standard_normal(mesh.x.shape)
        rho = 0.5 + 1.5 * rng.random(mesh.x.shape)
        rc, y = _call(igr, basis, mesh, alpha, x, rho)
        assert rc == 0
        ref = np.zeros(mesh.x.shape, order="F")
        igr.apply_sip_(ref, x, rho, basis, mesh, alpha)
        ref = ref.reshape(-1, order="F")
        assert np.all(np.isfinite(y))
        assert np.linalg.norm(y - ref) <= 1e-13 * np.linalg.norm(ref)


@pytest.mark.parametrize("p,nex,ney", [(1, 1, 16384), (1, 16384, 1), (4, 20, 16), (2, 3, 500)])
def test_apply_sip_noalloc_any_mesh_under_the_node_limit(igr, p, nex, ney):
    # the node count is the only limit: P1 one element wide (4,096 tiles, 65,536 nodes) and other degrees
    basis = igr.DGBasis(p)
    mesh = igr.CartesianMesh2D(nex, ney, 1.0, 1.0, basis)
    rng = np.random.default_rng(p + nex)
    x = rng.standard_normal(mesh.x.shape)
    rho = 0.5 + 1.5 * rng.random(mesh.x.shape)
    rc, y = _call(igr, basis, mesh, 4e-3, x, rho)
    assert rc == 0
    ref = np.zeros(mesh.x.shape, order="F")
    igr.apply_sip_(ref, x, rho, basis, mesh, 4e-3)
    ref = ref.reshape(-1, order="F")
    assert np.linalg.norm(y - ref) <= 1e-13 * np.linalg.norm(ref)


def test_apply_sip_noalloc_rejects_oversize(igr):
    basis = igr.DGBasis(3)
    mesh = igr.CartesianMesh2D(65, 64, 1.0, 1.0, basis)  # 66,560 nodes > 65,536
    x = np.zeros(mesh.x.shape)
    rc, _ = _call(igr, basis, mesh, 1e-3, x, np.ones(mesh.x.shape))
    assert rc == 1  # IGR_EINVAL


def test_apply_sip_noalloc_refuses_stream_capture(igr):
    # the call synchronises its stream, so on a capturing stream it must return IGR_EINVAL without touching it,
    # leaving the caller's capture valid
    import torch
    lib = igr._lib.lib()
    basis = igr.DGBasis(3)
    mesh = igr.CartesianMesh2D(8, 8, 1.0, 1.0, basis)
    d = igr._disc2d(basis, mesh)
    dev = torch.device("cuda", 0)
    xd = torch.ones(mesh.x.size, dtype=torch.float64, device=dev)
    rd = torch.ones_like(xd)
    yd = torch.zeros_like(xd)
    D = C.POINTER(C.c_double)
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.graph(g, stream=s):
        rc = lib.igr2d_apply_sip_noalloc(C.byref(d), C.c_double(1e-3), C.cast(C.c_void_p(xd.data_ptr()), D),
                                         C.cast(C.c_void_p(rd.data_ptr()), D), C.cast(C.c_void_p(yd.data_ptr()), D),
                                         C.c_void_p(s.cuda_stream))
        out = xd * 3.0
    assert rc == 1  # IGR_EINVAL
    g.replay()
    torch.cuda.synchronize()
    assert torch.all(out == 3.0) and torch.all(yd == 0.0)
