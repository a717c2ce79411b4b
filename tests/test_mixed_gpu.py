"""Mixed-precision paths against the plain FP64 GPU path and the reference's
golden outputs.

BEMGPU_PREC_MIXED_LA (FP64 fill, complex64 LU + refinement): spectral power
within 1e-6 relative of FP64.  BEMGPU_PREC_MIXED (FP32 far pairs as well):
the four triangle-pair terms of an RWG pair's scalar-potential entry cancel
like a dipole-dipole interaction, amplifying FP32 rounding by ~(R/h)^2, so this
mode is held to 1e-5 and its fill entries to 1e-6 of their row's scale."""
import numpy as np
import pytest

from bem_gb300 import api, mesh, _lib
from tests.cases import golden_geometry, row_scaled_err

pytestmark = pytest.mark.gpu
TOL_P = 1e-6


def _pair(level, gap, seed=12345):
    v, t = mesh.icosphere(1.0, level, jitter=0.02, seed=seed)
    b2 = mesh.Body.from_mesh(v, t)
    b1 = b2.translated(mesh.gap_translation(v, v, gap))
    d = api.FixedLorentz(*api.SIC_CONFIG)
    return api.parseShapes(b1, b2, d, d)


def test_double_float_fill_matches_fp64():
    """BEMGPU_PREC_MIXED_LA fills every quadrature node pair in double-float
    (FP32 pairs, ~48 bits) on the FP32 pipes: entries within 1e-11 of their
    row's scale of the FP64 fill, exterior (lossless) and interior (lossy)
    media, the two-body tree and a one-body tree; the reference's cube4
    golden matrix likewise."""
    top, s, t = _pair(2, 0.05)
    g = api.GreensFunction(1.0, 1.0, 0.55, True)
    assert row_scaled_err(api.Zts(top, top, g, precision=_lib.PREC_MIXED_LA), api.Zts(top, top, g)) < 1e-11
    gi = api.GreensFunction(api.FixedLorentz(*api.SIC_CONFIG).eps(0.1), 1.0, 0.5)
    assert row_scaled_err(api.Zts(s, s, gi, precision=_lib.PREC_MIXED_LA), api.Zts(s, s, gi)) < 1e-11


def test_mixed_fill_close_to_fp64():
    top, s, t = _pair(2, 0.05)
    g = api.GreensFunction(1.0, 1.0, 0.55, True)
    Z64 = api.Zts(top, top, g, precision=_lib.PREC_FP64)
    Zmx = api.Zts(top, top, g, precision=_lib.PREC_MIXED)
    err = row_scaled_err(Zmx, Z64)
    assert 0 < err < 1e-6, err
    gi = api.GreensFunction(api.FixedLorentz(*api.SIC_CONFIG).eps(0.1), 1.0, 0.5)
    assert row_scaled_err(api.Zts(s, s, gi, precision=_lib.PREC_MIXED), api.Zts(s, s, gi)) < 1e-6


@pytest.mark.parametrize("gap", [0.02, 0.1, 1.0])
def test_mixed_spectral_power_within_1e6_of_fp64(gap):
    top, s, t = _pair(2, gap)
    for eV in (0.085, 0.0983, 0.116, 0.125):
        info = {}
        Pm = api.CalcHeatTransfer(1e-6, eV, 300.0, 0.0, top, s, t, precision=_lib.PREC_MIXED_LA, info=info)
        P64 = api.CalcHeatTransfer(1e-6, eV, 300.0, 0.0, top, s, t, precision=_lib.PREC_FP64)
        rel = abs(Pm / P64 - 1)
        assert rel < TOL_P, (gap, eV, rel, info["err_est"], info["refine_iters"])
        assert info["refine_iters"] >= 1 and info["err_est"] >= 0.0
        Pf = api.CalcHeatTransfer(1e-6, eV, 300.0, 0.0, top, s, t, precision=_lib.PREC_MIXED, strict=False)
        assert abs(Pf / P64 - 1) < 1e-5


def test_mixed_hardest_workload_point():
    """Icospheres L3 (N = 7680) at 20 nm and 0.08 eV, the low-loss point where
    the refinement residual needs its finest near/far split."""
    top, s, t = _pair(3, 0.02)
    info = {}
    Pm = api.CalcHeatTransfer(1e-6, 0.08, 300.0, 0.0, top, s, t, precision=_lib.PREC_MIXED_LA, info=info)
    P64 = api.CalcHeatTransfer(1e-6, 0.08, 300.0, 0.0, top, s, t, precision=_lib.PREC_FP64)
    assert abs(Pm / P64 - 1) < TOL_P, (abs(Pm / P64 - 1), info["err_est"], info["refine_iters"])


def test_mixed_matches_reference_cube_workload(golden):
    rec = golden("cube4_gap100nm")
    b1, b2 = golden_geometry(rec)
    d = api.FixedLorentz(*[float(x) for x in rec["lorentz1"]])
    top, s, t = api.parseShapes(b1, b2, d, d)
    for f, Pref in list(zip(rec["freqs"], rec["P"]))[::3]:
        P = api.CalcHeatTransfer(rec["a"], float(f), rec["T1"], rec["T2"], top, s, t, precision=_lib.PREC_MIXED_LA)
        assert abs(P / Pref - 1) < TOL_P, (f, P, Pref)


@pytest.mark.parametrize("case", ["ico2_gap50nm", "ico3_gap20nm"])
def test_mixed_matches_reference_icospheres(golden, case):
    """The mixed path against the reference binary's own spectral power on
    the precision-form icospheres (L3, N = 7680, 20 nm) and on L2."""
    rec = golden(case)
    b1, b2 = golden_geometry(rec)
    d = api.FixedLorentz(*[float(x) for x in rec["lorentz1"]])
    top, s, t = api.parseShapes(b1, b2, d, d)
    for f, Pref in zip(rec["freqs"], rec["P"]):
        info = {}
        P = api.CalcHeatTransfer(rec["a"], float(f), rec["T1"], rec["T2"], top, s, t, precision=_lib.PREC_MIXED_LA,
                                 info=info)
        assert abs(P / Pref - 1) < TOL_P, (case, f, P, Pref, info["err_est"], info["solver"])


def test_mixed_same_result_twice():
    top, s, t = _pair(1, 0.1)
    a = api.CalcHeatTransfer(1e-6, 0.11, 300.0, 0.0, top, s, t, precision=_lib.PREC_MIXED_LA)
    b = api.CalcHeatTransfer(1e-6, 0.11, 300.0, 0.0, top, s, t, precision=_lib.PREC_MIXED_LA)
    assert a == b


def test_fp64_class_tensor_core_lu_matches_fp64_path():
    """The FP64-class factorization (LU and blocked solves whose updates are
    5-slice exact tensor-core products) gives the FP64 path's spectral power to
    the plain path's own bar, and the escalating default stays on complex64
    for a well-conditioned system."""
    v, t = mesh.icosphere(1.0, 2, jitter=0.02, seed=12345)
    b2 = mesh.Body.from_mesh(v, t)
    b1 = b2.translated(mesh.gap_translation(v, v, 0.05))
    d = api.FixedLorentz(*api.SIC_CONFIG)
    ctx = api.Context(0)
    top, s, tt = api.parseShapes(b1, b2, d, d, ctx)
    for eV in (0.09, 0.117):
        P64 = api.CalcHeatTransfer(1e-6, eV, 300.0, 0.0, top, s, tt, precision=_lib.PREC_FP64)
        ctx.set_solver(2)
        info = {}
        P2 = api.CalcHeatTransfer(1e-6, eV, 300.0, 0.0, top, s, tt, precision=_lib.PREC_MIXED_LA, info=info)
        assert info["solver"] == 2 and info["err_est"] < 1e-6
        assert abs(P2 / P64 - 1) < 1e-8, (eV, P2, P64)
        ctx.set_solver(0)
        info = {}
        P0 = api.CalcHeatTransfer(1e-6, eV, 300.0, 0.0, top, s, tt, precision=_lib.PREC_MIXED_LA, info=info)
        assert info["solver"] == 1 and abs(P0 / P64 - 1) < 1e-6


def test_escalation_to_fp64_class_lu():
    """Mode 0 escalates when the complex64 refinement's error estimate stays
    above the tolerance: with a tolerance no estimate can meet, every solve
    takes the FP64-class factorization and still meets the FP64 path."""
    v, t = mesh.icosphere(1.0, 2, jitter=0.02, seed=12345)
    b2 = mesh.Body.from_mesh(v, t)
    b1 = b2.translated(mesh.gap_translation(v, v, 0.1))
    d = api.FixedLorentz(*api.SIC_CONFIG)
    ctx = api.Context(0)
    top, s, tt = api.parseShapes(b1, b2, d, d, ctx)
    L = _lib.load()
    assert L.bemgpu_ctx_set_escalation_tol(ctx.handle, 0.0) == 0
    P64 = api.CalcHeatTransfer(1e-6, 0.1, 300.0, 0.0, top, s, tt, precision=_lib.PREC_FP64)
    info = {}
    P = api.CalcHeatTransfer(1e-6, 0.1, 300.0, 0.0, top, s, tt, precision=_lib.PREC_MIXED_LA, info=info)
    assert info["solver"] == 2 and info["err_est"] < 1e-6
    assert abs(P / P64 - 1) < 1e-8
    assert L.bemgpu_ctx_set_escalation_tol(ctx.handle, 1e-6) == 0
    info = {}
    api.CalcHeatTransfer(1e-6, 0.1, 300.0, 0.0, top, s, tt, precision=_lib.PREC_MIXED_LA, info=info)
    assert info["solver"] == 1


def test_fallback_to_the_fp64_path():
    """When the FP64-class refinement stays above the fallback tolerance, mode 0
    solves the same (double-float-filled) W on the plain FP64 path: forced here
    with both tolerances at 0, the result is the FP64 path's to the fill's
    accuracy, err_est is 0 and info reports solver 3."""
    v, t = mesh.icosphere(1.0, 1, jitter=0.02, seed=12345)
    b2 = mesh.Body.from_mesh(v, t)
    b1 = b2.translated(mesh.gap_translation(v, v, 0.05))
    d = api.FixedLorentz(*api.SIC_CONFIG)
    ctx = api.Context(0)
    top, s, tt = api.parseShapes(b1, b2, d, d, ctx)
    L = _lib.load()
    P64 = api.CalcHeatTransfer(1e-6, 0.11, 300.0, 0.0, top, s, tt, precision=_lib.PREC_FP64)
    assert L.bemgpu_ctx_set_escalation_tol(ctx.handle, 0.0) == 0
    assert L.bemgpu_ctx_set_fp64_fallback_tol(ctx.handle, 0.0) == 0
    info = {}
    P = api.CalcHeatTransfer(1e-6, 0.11, 300.0, 0.0, top, s, tt, precision=_lib.PREC_MIXED_LA, info=info)
    assert info["solver"] == 3 and info["err_est"] == 0.0
    assert abs(P / P64 - 1) < 1e-10, (P, P64)
    # the same request again gives the same bits (W is kept as filled)
    assert api.CalcHeatTransfer(1e-6, 0.11, 300.0, 0.0, top, s, tt, precision=_lib.PREC_MIXED_LA) == P
    assert L.bemgpu_ctx_set_fp64_fallback_tol(ctx.handle, -1.0) == _lib.ERR_ARG
    assert L.bemgpu_ctx_set_fp64_fallback_tol(ctx.handle, 1e-6) == 0
    assert L.bemgpu_ctx_set_escalation_tol(ctx.handle, 1e-6) == 0
    info = {}
    api.CalcHeatTransfer(1e-6, 0.11, 300.0, 0.0, top, s, tt, precision=_lib.PREC_MIXED_LA, info=info)
    assert info["solver"] == 1
