"""The autotuner's cache and size classes (CPU), and on the GPU: the launch
shapes it chooses between leave every result bit for bit unchanged, and a
tuning run returns valid settings and caches them."""
import json

import pytest

from bem_gb300 import tuning


def test_size_classes_and_cache_roundtrip(tmp_path):
    assert tuning.size_class(1152) == "n2048" and tuning.size_class(7680) == "n8192"
    assert tuning.size_class(8192) == "n8192" and tuning.size_class(8193) == "n16384"
    path = str(tmp_path / "t.json")
    tuning.store("GB300|n8192", {"near_minb": 4, "far_rows": 2, "raster": 16}, path)
    tuning.store("GB300|n2048", {"near_minb": 2, "far_rows": 8, "raster": 4}, path)
    data = json.load(open(path))
    assert data["GB300|n8192"]["raster"] == 16 and data["GB300|n2048"]["far_rows"] == 8
    assert tuning.load_cache(str(tmp_path / "missing.json")) == {}
    assert set(tuning.DEFAULTS) == set(tuning.KNOBS)


@pytest.mark.gpu
def test_results_do_not_depend_on_the_launch_shapes(tmp_path):
    from bem_gb300 import api, mesh, _lib
    v, t = mesh.icosphere(1.0, 2, jitter=0.02, seed=12345)
    b2 = mesh.Body.from_mesh(v, t)
    b1 = b2.translated(mesh.gap_translation(v, v, 0.05))
    d = api.FixedLorentz(*api.SIC_CONFIG)
    ctx = api.Context(0)
    top, s, tt = api.parseShapes(b1, b2, d, d, ctx)
    g = api.GreensFunction(1.0, 1.0, 0.55, True)

    def run():
        return (api.CalcHeatTransfer(1e-6, 0.116, 300.0, 0.0, top, s, tt, precision=_lib.PREC_MIXED_LA),
                api.Zts(top, top, g, precision=_lib.PREC_MIXED_LA).tobytes())

    base = run()
    for name, (_, cands, _) in tuning.KNOBS.items():
        for v in cands:
            tuning.apply(ctx.handle, dict(tuning.DEFAULTS, **{name: v}))
            assert run() == base, (name, v)
    L = _lib.load()
    # knobs the tuner leaves at their measured defaults: the same results too
    for knob, vals in ((_lib.TUNE_NEAR_SYNC, (0, 1)), (_lib.TUNE_NEAR_GRID, (2, 16)),
                       (_lib.TUNE_PANEL_CTAS, (38, 0))):
        for v in vals:
            assert L.bemgpu_ctx_set_tuning(ctx.handle, knob, v) == _lib.OK
            assert run() == base, (knob, v)
    params, timings = tuning.tune(lambda: api.CalcHeatTransfer(1e-6, 0.116, 300.0, 0.0, top, s, tt,
                                                               precision=_lib.PREC_MIXED_LA), ctx.handle, reps=1)
    assert all(params[k] in tuning.KNOBS[k][1] for k in tuning.KNOBS)
    assert tuning.current(ctx.handle) == params
    assert all(ms > 0 for ms in timings["near_minb"].values())
    path = str(tmp_path / "cache.json")
    tuning.store(tuning.cache_key(2 * top.rwgs), params, path)
    p3, src = tuning.tuned(lambda: None, ctx.handle, 2 * top.rwgs, path=path)
    assert src == "cache" and p3 == params
    assert L.bemgpu_ctx_set_tuning(ctx.handle, _lib.TUNE_NEAR_MINB, 5) == _lib.ERR_ARG
    assert L.bemgpu_ctx_set_tuning(ctx.handle, _lib.TUNE_NEAR_SYNC, 2) == _lib.ERR_ARG
    assert L.bemgpu_ctx_set_tuning(ctx.handle, _lib.TUNE_NEAR_GRID, 0) == _lib.ERR_ARG
    assert L.bemgpu_ctx_set_tuning(ctx.handle, _lib.TUNE_PANEL_CTAS, -1) == _lib.ERR_ARG
    assert L.bemgpu_ctx_set_tuning(ctx.handle, _lib.TUNE_EX_WIDE, 3) == _lib.ERR_ARG
    assert L.bemgpu_ctx_set_tuning(ctx.handle, 99, 1) == _lib.ERR_ARG


@pytest.mark.gpu
@pytest.mark.parametrize("mesh_kind", ["ico2", "cube4"])
def test_paired_lu_panels_factor_as_well(mesh_kind):
    """BEMGPU_TUNE_LU_SUPER: the complex64 LU with its panels in pairs (one
    K = 256 trailing update per pair) against one panel at a time.  The
    refinement would hide a wrong factorization as slow convergence, so both
    must converge on the complex64 path in the same number of steps, to the
    same spectral power within the refinement's accuracy.  ico2 (N = 1920:
    15 panels, an unpaired last one) and cube4 (N = 1152: 9 panels)."""
    from bem_gb300 import api, mesh, _lib
    L = _lib.load()
    if mesh_kind == "ico2":
        v, t = mesh.icosphere(1.0, 2, jitter=0.02, seed=12345)
    else:
        v, t = mesh.cube(1.0, 4)
    b2 = mesh.Body.from_mesh(v, t)
    b1 = b2.translated(mesh.gap_translation(v, v, 0.05))
    d = api.FixedLorentz(*api.SIC_CONFIG)
    ctx = api.Context(0)
    top, s, tt = api.parseShapes(b1, b2, d, d, ctx)
    assert L.bemgpu_ctx_set_solver(ctx.handle, 1) == _lib.OK  # complex64 only: no escalation
    out = {}
    for sup in (0, 1):
        assert L.bemgpu_ctx_set_tuning(ctx.handle, _lib.TUNE_LU_SUPER, sup) == _lib.OK
        info = {}
        P = api.CalcHeatTransfer(1e-6, 0.1, 300.0, 0.0, top, s, tt, precision=_lib.PREC_MIXED_LA, info=info)
        out[sup] = (P, info["solver"], info["refine_iters"], info["err_est"])
    assert out[0][1] == out[1][1] == 1
    assert abs(out[0][2] - out[1][2]) <= 1, out
    assert abs(out[1][0] / out[0][0] - 1) < 1e-8, out
    assert out[1][3] < 1e-6, out
    assert L.bemgpu_ctx_set_tuning(ctx.handle, _lib.TUNE_LU_SUPER, 2) == _lib.ERR_ARG
