"""The mixed-precision path against the plain FP64 path on each synthetic
workload: the spectral power of every sampled solve within 1e-6 relative
(TOL_P), whatever factorization the solve ended on (complex64, the FP64-class
escalation, or the FP64 fallback).

Workloads (seeded; the same generators as bench.py):
  * the precision form: icospheres L3 (N = 7680), every gap of its grid at the
    resonance frequencies 0.0983 eV (omega_TO) and 0.116 eV;
  * tip over plate: requests of uneven N (4488-6600), some of which escalate
    to the FP64-class factorization;
  * the serving mix: one SiC and one alumina request;
  * a reduced thin-slab pair (10 x 10 x 0.5 um, N = 16128) at SiC's surface
    phonon resonance, where the complex64 refinement contracts slowly, once as
    it is solved and once with the escalation forced.
The spectral power is CalcHeatTransfer's result (src/HeatTransfer.cpp:8-59)."""
import numpy as np
import pytest

import bench
from bem_gb300 import api, mesh, _lib

pytestmark = pytest.mark.gpu
TOL_P = 1e-6


def _solve_both(ctx, b1, b2, cfg, eV, T1=300.0):
    d = api.FixedLorentz(*cfg)
    top, s, t = api.parseShapes(b1, b2, d, d, ctx)
    info = {}
    Pm = api.CalcHeatTransfer(1e-6, eV, T1, 0.0, top, s, t, precision=_lib.PREC_MIXED_LA, info=info)
    P64 = api.CalcHeatTransfer(1e-6, eV, T1, 0.0, top, s, t, precision=_lib.PREC_FP64)
    return Pm, P64, info


@pytest.fixture(scope="module")
def ctx():
    c = api.Context(0)
    yield c
    c.close()


def test_precision_form_every_gap(ctx):
    wl = bench.WORKLOADS["ico3"]
    v, t = mesh.icosphere(1.0, 3, jitter=0.02, seed=12345)
    b2 = mesh.Body.from_mesh(v, t)
    worst = 0.0
    for gap in wl["gaps"]:
        b1 = b2.translated(mesh.gap_translation(v, v, gap))
        for eV in (0.0983, 0.116):
            Pm, P64, info = _solve_both(ctx, b1, b2, bench.SIC, eV)
            rel = abs(Pm / P64 - 1)
            worst = max(worst, rel)
            assert rel < TOL_P, (gap, eV, rel, info["err_est"], info["solver"])
    print(f"ico3: worst relative error vs FP64 over 12 solves {worst:.2e}")


def test_tip_requests_including_escalations(ctx):
    reqs = bench.tip_requests(bench.WORKLOADS["tip"])
    solvers = []
    for i in (0, 1, 2, 3, 10, 13):
        b1, b2, eV = reqs[i]
        Pm, P64, info = _solve_both(ctx, b1, b2, bench.SIC, eV)
        solvers.append(info["solver"])
        assert abs(Pm / P64 - 1) < TOL_P, (i, abs(Pm / P64 - 1), info["err_est"], info["solver"])
    assert 2 in solvers, solvers  # at least one of them took the FP64-class factorization


def test_serving_mix_requests(ctx):
    wl = bench.WORKLOADS["mix"]
    reqs = bench.mix_requests(wl)
    freqs = bench.mix_freqs(wl)
    for i in (4, 13):  # SiC (N = 3624) and alumina (N = 4098)
        b1, b2, cfg, T1 = reqs[i]
        for eV in (float(freqs[8]), float(freqs[23])):
            Pm, P64, info = _solve_both(ctx, b1, b2, cfg, eV, T1)
            assert abs(Pm / P64 - 1) < TOL_P, (i, eV, abs(Pm / P64 - 1), info["err_est"])


def test_reduced_slab_at_resonance_and_its_escalation():
    v, t = mesh.box(0.5, 10.0, 10.0, 2, 24, 24)
    b2 = mesh.Body.from_mesh(v, t)
    b1 = b2.translated(mesh.gap_translation(v, v, 0.05))
    d = api.FixedLorentz(*bench.SIC)
    c = api.Context(0)
    try:
        top, s, tt = api.parseShapes(b1, b2, d, d, c)
        assert 2 * top.rwgs == 16128
        P64 = api.CalcHeatTransfer(1e-6, 0.117, 300.0, 0.0, top, s, tt, precision=_lib.PREC_FP64)
        info = {}
        Pm = api.CalcHeatTransfer(1e-6, 0.117, 300.0, 0.0, top, s, tt, precision=_lib.PREC_MIXED_LA, info=info)
        assert abs(Pm / P64 - 1) < TOL_P, (abs(Pm / P64 - 1), info)
        # escalation forced: the FP64-class factorization and its refinement
        assert _lib.load().bemgpu_ctx_set_escalation_tol(c.handle, 0.0) == 0
        info = {}
        Pe = api.CalcHeatTransfer(1e-6, 0.117, 300.0, 0.0, top, s, tt, precision=_lib.PREC_MIXED_LA, info=info)
        assert info["solver"] in (2, 3)
        assert abs(Pe / P64 - 1) < 1e-8, (abs(Pe / P64 - 1), info)
    finally:
        c.close()
