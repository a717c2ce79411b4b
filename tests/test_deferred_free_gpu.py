"""Destroying trees and geometries defers their device memory to a batch free
(bemgpu_tree_destroy, bemgpu_geom_destroy): the memory waits in a list that is
freed after one device synchronisation, so a serving loop that drops each
request's geometry does not drain the other lanes' work per request.
Checked: destroyed systems' memory is pending until bemgpu_ctx_trim frees it,
the list flushes itself once it holds 96 blocks, and solves on fresh
geometries give the same spectral power throughout, alone and through the
farm while other geometries are destroyed."""
import gc

import pytest

from bem_gb300 import api, mesh, _lib

pytestmark = pytest.mark.gpu


def _system(ctx, gap=0.05):
    v, t = mesh.icosphere(1.0, 2, jitter=0.02, seed=7)
    b2 = mesh.Body.from_mesh(v, t)
    b1 = b2.translated(mesh.gap_translation(v, v, gap))
    d = api.FixedLorentz(*api.SIC_CONFIG)
    return api.parseShapes(b1, b2, d, d, ctx)


def test_destroyed_systems_wait_for_a_batch_free():
    L = _lib.load()
    ctx = api.Context(0)
    L.bemgpu_ctx_trim(ctx.handle)
    assert L.bemgpu_pending_free_bytes() == 0
    P0 = None
    for k in range(4):
        top, s, t = _system(ctx)
        P = api.CalcHeatTransfer(1e-6, 0.1, 300.0, 0.0, top, s, t, precision=_lib.PREC_MIXED_LA)
        P0 = P if P0 is None else P0
        assert P == P0
        del top, s, t
        gc.collect()
        # three trees (triangle records) and their near-pair lists per system
        assert L.bemgpu_pending_free_bytes() > 0
    assert L.bemgpu_ctx_trim(ctx.handle) == _lib.OK
    assert L.bemgpu_pending_free_bytes() == 0


def test_the_list_flushes_itself_and_farm_results_stay_the_same():
    L = _lib.load()
    ctx = api.Context(0)
    L.bemgpu_ctx_trim(ctx.handle)
    farm = api.Farm(2, 0)
    Ps = []
    # 40 systems x (3 trees + 3 near-pair lists) = 240 blocks: the list flushes
    # at 96 blocks, so it never holds more than 96
    most = 0
    for k in range(40):
        sysk = _system(ctx)
        tk = farm.submit(1e-6, 0.1, 300.0, 0.0, *sysk, precision=_lib.PREC_MIXED_LA)
        del sysk
        Ps.append(farm.result(tk))
        gc.collect()
        most = max(most, L.bemgpu_pending_free_bytes())
    assert len(set(Ps)) == 1
    # ico2 system: 2 x 320 + 640 triangle records (~0.6 MB) plus near lists
    assert 0 < most < 96 * (1 << 20)
    del farm
    gc.collect()
    assert L.bemgpu_ctx_trim(ctx.handle) == _lib.OK
    assert L.bemgpu_pending_free_bytes() == 0
