"""The oracle restatement (oracle/bem_oracle.c + oracle/oracle.py) against
golden fixtures produced by the reference's own C++ (tests/golden/make_golden.py).
CPU only."""
import numpy as np
import pytest

from oracle import oracle
from tests.cases import golden_geometry, lorentz_eps, row_scaled_err
from bem_gb300 import mesh


def _fills(rec, eV):
    b1, b2 = golden_geometry(rec)
    xyz, tris, rwg, ns = mesh.two_body(b1, b2)
    om = oracle.dimensionless_omega(rec["a"], eV)
    e1 = lorentz_eps(rec["lorentz1"], eV)
    e2 = lorentz_eps(rec["lorentz2"], eV)
    Z = oracle.zts(xyz, tris, rwg, rwg, 1 + 0j, 1 + 0j, om)
    G1 = oracle.zts(xyz, tris, rwg[:ns], rwg[:ns], e1, 1 + 0j, om)
    G2 = oracle.zts(xyz, tris, rwg[ns:], rwg[ns:], e2, 1 + 0j, om)
    return Z, G1, G2


def test_cube1_matrices_match_reference(golden):
    rec = golden("cube1_gap100nm")
    Z, G1, G2 = _fills(rec, float(rec["z_eV"]))
    assert row_scaled_err(Z, rec["Zext"]) < 1e-12
    assert row_scaled_err(G1, rec["G1"]) < 1e-12
    assert row_scaled_err(G2, rec["G2"]) < 1e-12


@pytest.mark.parametrize("case", ["cube4_gap100nm", "ico1_gap20nm", "ico2_gap50nm"])
def test_sampled_matrices_match_reference(golden, case):
    rec = golden(case)
    Z, G1, G2 = _fills(rec, float(rec["z_eV"]))
    for key, M in (("Zext", Z), ("G1", G1), ("G2", G2)):
        idx = rec[key + "_idx"]
        rowabs = rec[key + "_rowabs"]
        got = M[idx[:, 0], idx[:, 1]]
        err = np.abs(got - rec[key + "_val"]) / (rowabs[idx[:, 0]] / M.shape[1])
        assert err.max() < 1e-10, (key, err.max())
        assert np.allclose(np.abs(M).sum(1), rowabs, rtol=1e-12, atol=0)


@pytest.mark.parametrize("case,stride", [("cube1_gap100nm", 1), ("cube4_gap100nm", 4), ("ico1_gap20nm", 1),
                                         ("cube2_alumina_gap50nm", 1), ("ico2_gap50nm", 1)])
def test_spectral_power_matches_reference(golden, case, stride):
    rec = golden(case)
    b1, b2 = golden_geometry(rec)
    xyz, tris, rwg, ns = mesh.two_body(b1, b2)
    for f, Pref in list(zip(rec["freqs"], rec["P"]))[::stride]:
        e1 = lorentz_eps(rec["lorentz1"], f)
        e2 = lorentz_eps(rec["lorentz2"], f)
        P = oracle.calc_heat_transfer(rec["a"], f, rec["T1"], rec["T2"], xyz, tris, rwg, ns, e1, e2)
        assert abs(P / Pref - 1) < 1e-10, (case, f, P, Pref)


def test_far_rule_selection(golden):
    """Rule choice of LKTriangle (src/Impedance.cpp:327-360).  With the default
    thresholds 12 > 8 > 4 > 2 a pair that fails d*12 > emax^2 fails every later
    test too, so only Gauss6 and Gauss36 are reachable; the facing faces of the
    cube pair at 100 nm take Gauss36."""
    rec = golden("cube4_gap100nm")
    b1, b2 = golden_geometry(rec)
    xyz, tris, rwg, ns = mesh.two_body(b1, b2)
    _, counts = oracle.zts(xyz, tris, rwg, rwg, 1 + 0j, 1 + 0j, 0.5, counts=True)
    assert counts["same"] == b1.nt + b2.nt
    assert counts["neighbour"] > 0 and counts["g6"] > 0 and counts["g36"] > 0
    assert counts["g10"] == counts["g15"] == counts["g21"] == 0
    # with thresholds in increasing order every rule is reachable
    _, c2 = oracle.zts(xyz, tris, rwg, rwg, 1 + 0j, 1 + 0j, 0.5, far=(2.0, 4.0, 8.0, 12.0), counts=True)
    assert min(c2["g6"], c2["g10"], c2["g15"], c2["g36"]) > 0, c2   # the grid has no 21-point distance


def test_green_constants():
    c = oracle.green_constants(16.4 + 0.14j, 1 + 0j, 0.5 + 0j)
    ksq = 16.4 + 0.14j
    ksq = ksq * 0.25
    assert abs(c["ksquared"] - ksq) < 1e-15
    assert abs(c["k"] - np.sqrt(ksq)) < 1e-15
    assert abs(c["k2"] + 0.5 * ksq) < 1e-15
    assert abs(c["Zeps"] - 1 / (1j * 0.5 * (16.4 + 0.14j))) < 1e-14


def test_theta_quirk_dimensionless_omega():
    """Theta is evaluated with the dimensionless omega (src/HeatTransfer.cpp:11,58):
    x = hbar*omega/(kb*T) ~ 1e-14, so exp(x) - 1 is a small multiple of one ulp
    of 1.0 and Theta carries a rounding artefact of about 1 % that parity must
    reproduce (same libm exp, no expm1)."""
    import math
    om = oracle.dimensionless_omega(1e-6, 0.1)
    assert 0.5 < om < 0.51
    th = oracle.theta(om, 300.0)
    x = oracle.HBAR * om / (oracle.KB * 300.0)
    assert th == oracle.HBAR * om / (math.exp(x) - 1)
    ulps = (math.exp(x) - 1) / 2.0 ** -52
    assert ulps == round(ulps)                              # quantized
    assert abs(th / (oracle.KB * 300.0) - 1) < 0.02         # ~kT, up to the quantization
    assert oracle.theta(om, 0.0) == 0.0
