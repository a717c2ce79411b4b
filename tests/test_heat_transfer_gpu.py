"""GPU per-frequency solve (bemgpu_heat_transfer through the C ABI) against
the reference's CalcHeatTransfer output (golden fixtures) and the oracle.
Bar on the plain FP64 path: spectral power within 1e-8 relative."""
import numpy as np
import pytest

from bem_gb300 import api, mesh
from oracle import oracle
from tests.cases import golden_geometry, lorentz_eps

pytestmark = pytest.mark.gpu
TOL = 1e-8


def _system(rec):
    b1, b2 = golden_geometry(rec)
    d1 = api.FixedLorentz(*[float(x) for x in rec["lorentz1"]])
    d2 = api.FixedLorentz(*[float(x) for x in rec["lorentz2"]])
    return b1, b2, api.parseShapes(b1, b2, d1, d2)


@pytest.mark.parametrize("case", ["cube1_gap100nm", "cube4_gap100nm", "ico1_gap20nm", "cube2_alumina_gap50nm",
                                  "ico2_gap50nm", "ico3_gap20nm"])
def test_spectral_power_matches_reference(golden, case):
    rec = golden(case)
    _, _, (top, s, t) = _system(rec)
    for f, Pref in zip(rec["freqs"], rec["P"]):
        P = api.CalcHeatTransfer(rec["a"], float(f), rec["T1"], rec["T2"], top, s, t)
        assert abs(P / Pref - 1) < TOL, (case, f, P, Pref)


def test_spectral_power_matches_oracle_icosphere2():
    v, t = mesh.icosphere(1.0, 2, jitter=0.02, seed=12345)
    b2 = mesh.Body.from_mesh(v, t)
    b1 = b2.translated(mesh.gap_translation(v, v, 0.1))
    d = api.FixedLorentz(*api.SIC_CONFIG)
    top, s, tt = api.parseShapes(b1, b2, d, d)
    xyz, tris, rwg, ns = mesh.two_body(b1, b2)
    for eV in (0.09, 0.116):
        info = {}
        P = api.CalcHeatTransfer(1e-6, eV, 300.0, 0.0, top, s, tt, info=info)
        e = d.eps(eV)
        Po = oracle.calc_heat_transfer(1e-6, eV, 300.0, 0.0, xyz, tris, rwg, ns, e, e)
        assert abs(P / Po - 1) < TOL, (eV, P, Po)
        assert info["pairs_near"] > 0 and info["ms_fill"] > 0


def test_permuted_rwg_order_matches_oracle():
    """The RWG order fixes each triangle's quadrature frame (the first half-RWG's
    free vertex, src/Impedance.cpp:283,156) and the 91/105-point rules are not
    rotation-symmetric, so a permuted order changes P at the quadrature-error
    level (~1e-4) in the reference as well; parity holds order by order."""
    v, t = mesh.cube(1.0, 2)
    b2 = mesh.Body.from_mesh(v, t)
    b1 = b2.translated(mesh.gap_translation(v, v, 0.1))
    d = api.FixedLorentz(*api.SIC_CONFIG)
    P0 = api.CalcHeatTransfer(1e-6, 0.1, 300.0, 0.0, *api.parseShapes(b1, b2, d, d))
    rng = np.random.default_rng(0)
    b1p = mesh.Body(b1.verts, b1.tris, b1.rwg[rng.permutation(b1.nrwg)])
    b2p = mesh.Body(b2.verts, b2.tris, b2.rwg[rng.permutation(b2.nrwg)])
    P1 = api.CalcHeatTransfer(1e-6, 0.1, 300.0, 0.0, *api.parseShapes(b1p, b2p, d, d))
    xyz, tris, rwg, ns = mesh.two_body(b1p, b2p)
    e = d.eps(0.1)
    Po = oracle.calc_heat_transfer(1e-6, 0.1, 300.0, 0.0, xyz, tris, rwg, ns, e, e)
    assert abs(P1 / Po - 1) < TOL
    assert abs(P1 / P0 - 1) < 1e-2


def test_size_mismatch_is_rejected():
    v, t = mesh.cube(1.0, 1)
    b2 = mesh.Body.from_mesh(v, t)
    b1 = b2.translated([2.0, 0, 0])
    d = api.FixedLorentz(*api.SIC_CONFIG)
    top, s, tt = api.parseShapes(b1, b2, d, d)
    with pytest.raises(Exception) as e:
        api.CalcHeatTransfer(1e-6, 0.1, 300.0, 0.0, s, s, tt)
    assert "ARG" in str(e.value)


def test_bounded_wait_timeout_leaves_the_context_usable():
    """Failure detection without a GPU fault: a wait on a flag that nothing
    sets gives up after its budget and reports BEMGPU_ERR_TIMEOUT through the
    same error flag the tensor-core pipelines and grid barriers use; the next
    solve on the same context runs normally."""
    from bem_gb300 import _lib
    ctx = api.Context(0)
    L = _lib.load()
    assert L.bemgpu_ctx_wait_selftest(ctx.handle, 1000) == _lib.ERR_TIMEOUT
    assert "ran out" in L.bemgpu_ctx_last_error(ctx.handle).decode()
    v, t = mesh.cube(1.0, 2)
    b2 = mesh.Body.from_mesh(v, t)
    b1 = b2.translated(mesh.gap_translation(v, v, 0.1))
    d = api.FixedLorentz(*api.SIC_CONFIG)
    top, s, tt = api.parseShapes(b1, b2, d, d, ctx)
    ref = api.CalcHeatTransfer(1e-6, 0.1, 300.0, 0.0, *api.parseShapes(b1, b2, d, d))
    for prec in (_lib.PREC_FP64, _lib.PREC_MIXED_LA):
        P = api.CalcHeatTransfer(1e-6, 0.1, 300.0, 0.0, top, s, tt, precision=prec)
        assert abs(P / ref - 1) < (1e-12 if prec == _lib.PREC_FP64 else 1e-6)
    assert L.bemgpu_ctx_wait_selftest(ctx.handle, 10) == _lib.ERR_TIMEOUT
