"""bemgpu_zts_noalloc: the impedance fill for callers that cannot allocate
device memory while they run (graph capture, real-time loops, hosts whose
memory pool owns the device).  It fills the caller's buffer using a fixed
file-scope scratch array instead of allocating; its output must equal the
allocating bemgpu_zts's within the fill tolerance, on two calls in a row
(the scratch keeps the previous call's contents)."""
import ctypes

import numpy as np
import pytest

from bem_gb300 import api, mesh, _lib
from tests.cases import row_scaled_err

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _noalloc(ctx, t, s, g):
    import torch
    m, n = 2 * t.rwgs, 2 * s.rwgs
    out = torch.zeros((n, m), dtype=torch.complex128, device="cuda")  # column-major m x n
    torch.cuda.synchronize()
    rc = _lib.load().bemgpu_zts_noalloc(ctx.handle, t.handle, s.handle, ctypes.byref(g._g),
                                        ctypes.byref(api.Options()._c()), ctypes.c_void_p(out.data_ptr()), m, None)
    return rc, out.cpu().numpy().T


def test_noalloc_matches_allocating_fill_twice():
    pytest.importorskip("torch")
    v, t = mesh.cube(1.0, 3)
    b2 = mesh.Body.from_mesh(v, t)
    b1 = b2.translated(mesh.gap_translation(v, v, 0.1))
    d = api.FixedLorentz(*api.SIC_CONFIG)
    top, s, tt = api.parseShapes(b1, b2, d, d)
    ctx = top.geom.ctx
    g_ext = api.GreensFunction(1.0, 1.0, 0.5, True)
    g_int = api.GreensFunction(d.eps(0.1), 1.0, 0.5)
    ref_top = api.Zts(top, top, g_ext)
    ref_s = api.Zts(s, s, g_int)
    for _ in range(2):
        rc, Z = _noalloc(ctx, top, top, g_ext)
        assert rc == 0, api._lib.load().bemgpu_ctx_last_error(ctx.handle)
        assert row_scaled_err(Z, ref_top) < TOL
        rc, Zs = _noalloc(ctx, s, s, g_int)
        assert rc == 0
        assert row_scaled_err(Zs, ref_s) < TOL


def test_noalloc_rejects_sizes_beyond_its_scratch():
    pytest.importorskip("torch")
    v, t = mesh.cube(1.0, 4)
    b2 = mesh.Body.from_mesh(v, t)
    b1 = b2.translated(mesh.gap_translation(v, v, 0.1))
    d = api.FixedLorentz(*api.SIC_CONFIG)
    top, s, tt = api.parseShapes(b1, b2, d, d)   # 576 x 576 RWG pairs > 245760
    rc, _ = _noalloc(top.geom.ctx, top, top, api.GreensFunction(1.0, 1.0, 0.5, True))
    assert rc == _lib.ERR_ARG
    assert b"fixed scratch" in _lib.load().bemgpu_ctx_last_error(top.geom.ctx.handle)
