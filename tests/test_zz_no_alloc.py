"""bemgpu_zts_noalloc: the impedance fill for callers that must not allocate
device memory while they run (a solver loop with a latency budget that cannot
stall in cudaMalloc, a host application whose own memory pool has claimed the
GPU).  It fills the caller's buffer using a fixed file-scope scratch array
instead of allocating.  Checked here: its output equals the allocating
bemgpu_zts's within the fill tolerance on calls in a row (the scratch keeps the
previous call's contents), on the context's stream and on a caller's stream;
the free device memory and the context's workspace do not change across the
calls; sizes beyond the scratch are rejected."""
import ctypes

import numpy as np
import pytest

from bem_gb300 import api, mesh, _lib
from tests.cases import row_scaled_err

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _call(ctx, t, s, g, out, stream=None):
    m = 2 * t.rwgs
    return _lib.load().bemgpu_zts_noalloc(ctx.handle, t.handle, s.handle, ctypes.byref(g._g),
                                          ctypes.byref(api.Options()._c()), ctypes.c_void_p(out.data_ptr()), m,
                                          ctypes.c_void_p(stream) if stream else None)


def _out(t, s):
    import torch
    return torch.zeros((2 * s.rwgs, 2 * t.rwgs), dtype=torch.complex128, device="cuda")  # column-major


def test_noalloc_matches_allocating_fill_twice_without_allocating():
    torch = pytest.importorskip("torch")
    v, t = mesh.cube(1.0, 3)
    b2 = mesh.Body.from_mesh(v, t)
    b1 = b2.translated(mesh.gap_translation(v, v, 0.1))
    d = api.FixedLorentz(*api.SIC_CONFIG)
    top, s, tt = api.parseShapes(b1, b2, d, d)
    ctx = top.geom.ctx
    L = _lib.load()
    g_ext = api.GreensFunction(1.0, 1.0, 0.5, True)
    g_int = api.GreensFunction(d.eps(0.1), 1.0, 0.5)
    ref_top = api.Zts(top, top, g_ext)
    ref_s = api.Zts(s, s, g_int)
    out_top, out_s = _out(top, top), _out(s, s)
    side = torch.cuda.Stream()
    torch.cuda.synchronize()
    ws0 = L.bemgpu_ctx_workspace_bytes(ctx.handle)
    free = []
    for k in range(3):
        # the third round runs on a stream the caller created
        stream = side.cuda_stream if k == 2 else None
        out_top.zero_()
        out_s.zero_()
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
        rc = _call(ctx, top, top, g_ext, out_top, stream)
        assert rc == 0, L.bemgpu_ctx_last_error(ctx.handle)
        rc = _call(ctx, s, s, g_int, out_s, stream)
        assert rc == 0, L.bemgpu_ctx_last_error(ctx.handle)
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
        assert row_scaled_err(out_top.cpu().numpy().T, ref_top) < TOL
        assert row_scaled_err(out_s.cpu().numpy().T, ref_s) < TOL
        assert L.bemgpu_ctx_workspace_bytes(ctx.handle) == ws0
    # The first call on a device may load the module that holds the scratch
    # (lazy module loading); from then on no call changes the free memory.
    assert len(set(free[1:])) == 1, free


def test_noalloc_rejects_sizes_beyond_its_scratch():
    pytest.importorskip("torch")
    v, t = mesh.cube(1.0, 4)
    b2 = mesh.Body.from_mesh(v, t)
    b1 = b2.translated(mesh.gap_translation(v, v, 0.1))
    d = api.FixedLorentz(*api.SIC_CONFIG)
    top, s, tt = api.parseShapes(b1, b2, d, d)   # 576 x 576 RWG pairs > 245760
    out = _out(top, top)
    rc = _call(top.geom.ctx, top, top, api.GreensFunction(1.0, 1.0, 0.5, True), out)
    assert rc == _lib.ERR_ARG
    assert b"fixed scratch" in _lib.load().bemgpu_ctx_last_error(top.geom.ctx.handle)
