"""RWG set-up on the device (bemgpu_tree_create_body_device, bemgpu_tree_concat):
the RWG tables equal the host builder's (the reference's edge-creation order,
src/ShapeMesh.cpp:857-928), and the half-RWG frames (src/RWG.cpp:7-39) give
the host-built trees' impedance matrices and spectral power."""
import ctypes

import numpy as np
import pytest

from bem_gb300 import api, mesh, _lib
from tests.cases import row_scaled_err

pytestmark = pytest.mark.gpu

MESHES = {
    "cube4": lambda: mesh.cube(1.0, 4),
    "ico2": lambda: mesh.icosphere(1.0, 2, jitter=0.02, seed=12345),
    "slab": lambda: mesh.box(0.5, 10.0, 10.0, 2, 12, 12),
    "tip": lambda: mesh.cone_tip(0.5, 1.0, 0.1, n_around=14, n_side=6, n_cap=3, n_base=3),
}


@pytest.mark.parametrize("name", sorted(MESHES))
def test_device_trees_equal_host_trees(name):
    v, t = MESHES[name]()
    b2 = mesh.Body.from_mesh(v, t)
    v1, t1 = mesh.icosphere(1.0, 1, jitter=0.02, seed=3)
    b1 = mesh.Body.from_mesh(v1 + mesh.gap_translation(v1, v, 0.05), t1)
    d = api.FixedLorentz(*api.SIC_CONFIG)
    ctx = api.Context(0)
    host = api.parseShapes(b1, b2, d, d, ctx)
    dev = api.parseShapes(b1, b2, d, d, ctx, setup="device")
    for th, td in zip(host, dev):
        assert np.array_equal(th.rwg, td.rwg)
    g = api.GreensFunction(1.0, 1.0, 0.5, True)
    assert row_scaled_err(api.Zts(dev[0], dev[0], g), api.Zts(host[0], host[0], g)) < 1e-13
    gi = api.GreensFunction(d.eps(0.11), 1.0, 0.5)
    assert row_scaled_err(api.Zts(dev[2], dev[2], gi), api.Zts(host[2], host[2], gi)) < 1e-13
    Ph = api.CalcHeatTransfer(1e-6, 0.11, 300.0, 0.0, *host)
    Pd = api.CalcHeatTransfer(1e-6, 0.11, 300.0, 0.0, *dev)
    assert abs(Pd / Ph - 1) < 1e-12, (Pd, Ph)


def test_device_setup_rejects_an_open_body():
    v, t = mesh.cube(1.0, 2)
    ctx = api.Context(0)
    geom = api.Geometry(v, t, ctx)
    L = _lib.load()
    h = ctypes.c_void_p()
    assert L.bemgpu_tree_create_body_device(geom.handle, 0, t.shape[0] - 1, ctypes.byref(h)) == _lib.ERR_MESH
    assert b"not closed" in L.bemgpu_ctx_last_error(ctx.handle)
    assert L.bemgpu_tree_create_body_device(geom.handle, 0, t.shape[0] + 1, ctypes.byref(h)) == _lib.ERR_ARG
    assert L.bemgpu_tree_create_body_device(geom.handle, 0, t.shape[0], ctypes.byref(h)) == _lib.OK
    tree = api.RWGTree._adopt(geom, h)
    assert np.array_equal(tree.rwg, mesh.build_rwgs(t))
