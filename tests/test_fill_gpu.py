"""GPU impedance fill (bemgpu_zts through the C ABI) against the reference's
matrices (golden fixtures) and the oracle.  Bar: every entry within 1e-10
of its row's scale (row-scaled error; near-zero entries have no meaningful
relative error)."""
import numpy as np
import pytest

from bem_gb300 import api, mesh
from oracle import oracle
from tests.cases import golden_geometry, lorentz_eps, row_scaled_err

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _trees(rec):
    b1, b2 = golden_geometry(rec)
    d1 = api.FixedLorentz(*[float(x) for x in rec["lorentz1"]])
    d2 = api.FixedLorentz(*[float(x) for x in rec["lorentz2"]])
    top, s, t = api.parseShapes(b1, b2, d1, d2)
    return b1, b2, top, s, t


def test_cube1_fill_matches_reference_matrices(golden):
    rec = golden("cube1_gap100nm")
    _, _, top, s, t = _trees(rec)
    eV = float(rec["z_eV"])
    om = api.dimensionless_omega(rec["a"], eV)
    Z = api.Zts(top, top, api.GreensFunction(1.0, 1.0, om, True))
    G1 = api.Zts(s, s, api.GreensFunction(lorentz_eps(rec["lorentz1"], eV), 1.0, om))
    G2 = api.Zts(t, t, api.GreensFunction(lorentz_eps(rec["lorentz2"], eV), 1.0, om))
    assert row_scaled_err(Z, rec["Zext"]) < TOL
    assert row_scaled_err(G1, rec["G1"]) < TOL
    assert row_scaled_err(G2, rec["G2"]) < TOL


@pytest.mark.parametrize("case", ["cube4_gap100nm", "ico1_gap20nm"])
def test_fill_matches_reference_samples(golden, case):
    rec = golden(case)
    _, _, top, s, t = _trees(rec)
    eV = float(rec["z_eV"])
    om = api.dimensionless_omega(rec["a"], eV)
    mats = {"Zext": api.Zts(top, top, api.GreensFunction(1.0, 1.0, om, True)),
            "G1": api.Zts(s, s, api.GreensFunction(lorentz_eps(rec["lorentz1"], eV), 1.0, om)),
            "G2": api.Zts(t, t, api.GreensFunction(lorentz_eps(rec["lorentz2"], eV), 1.0, om))}
    for key, M in mats.items():
        idx = rec[key + "_idx"]
        rowmax_proxy = rec[key + "_rowabs"][idx[:, 0]] / M.shape[1]
        err = np.abs(M[idx[:, 0], idx[:, 1]] - rec[key + "_val"]) / rowmax_proxy
        assert err.max() < TOL, (key, err.max())
        assert np.allclose(np.abs(M).sum(1), rec[key + "_rowabs"], rtol=1e-11, atol=0)


@pytest.mark.parametrize("case", ["cube4_gap100nm", "ico1_gap20nm", "cube2_alumina_gap50nm", "ico2_gap50nm",
                                  "ico3_gap20nm"])
def test_fill_matches_oracle_entrywise(golden, case):
    rec = golden(case)
    b1, b2, top, s, t = _trees(rec)
    xyz, tris, rwg, ns = mesh.two_body(b1, b2)
    eV = float(rec["freqs"][-1])
    om = api.dimensionless_omega(rec["a"], eV)
    e1 = lorentz_eps(rec["lorentz1"], eV)
    Z = api.Zts(top, top, api.GreensFunction(1.0, 1.0, om, True))
    assert row_scaled_err(Z, oracle.zts(xyz, tris, rwg, rwg, 1 + 0j, 1 + 0j, om)) < TOL
    G1 = api.Zts(s, s, api.GreensFunction(e1, 1.0, om))
    assert row_scaled_err(G1, oracle.zts(xyz, tris, rwg[:ns], rwg[:ns], e1, 1 + 0j, om)) < TOL


def test_fill_is_deterministic():
    v, t = mesh.icosphere(1.0, 2, jitter=0.02, seed=3)
    b2 = mesh.Body.from_mesh(v, t)
    b1 = b2.translated(mesh.gap_translation(v, v, 0.05))
    d = api.FixedLorentz(*api.SIC_CONFIG)
    top, s, tt = api.parseShapes(b1, b2, d, d)
    g = api.GreensFunction(1.0, 1.0, 0.5, True)
    Z1 = api.Zts(top, top, g)
    Z2 = api.Zts(top, top, g)
    Z3 = api.Zts(top, top, g)
    assert np.array_equal(Z1, Z2) and np.array_equal(Z2, Z3)


def test_rectangular_block_of_two_trees():
    """Zts(t, s) with different row and column trees (s-rows x t-columns block
    of the two-body matrix)."""
    v, t = mesh.cube(1.0, 2)
    b2 = mesh.Body.from_mesh(v, t)
    b1 = b2.translated(mesh.gap_translation(v, v, 0.1))
    d = api.FixedLorentz(*api.SIC_CONFIG)
    top, s, tt = api.parseShapes(b1, b2, d, d)
    g = api.GreensFunction(1.0, 1.0, 0.45, True)
    full = api.Zts(top, top, g)
    blk = api.Zts(s, tt, g)
    ns2 = 2 * s.rwgs
    assert row_scaled_err(blk, full[:ns2, ns2:]) < 1e-13


def test_invalid_mesh_is_rejected():
    v, t = mesh.cube(1.0, 1)
    geom = api.Geometry(v, t)
    bad = np.array([[0, 0, 0, 1]], dtype=np.int32)  # pos == neg
    with pytest.raises(Exception) as e:
        api.RWGTree(geom, bad)
    assert "MESH" in str(e.value)


def test_handles_can_be_released_in_any_order():
    """A caller's garbage collector may finalize the context, the geometry and
    the trees in any order (e.g. objects in a reference cycle)."""
    import ctypes
    from bem_gb300 import _lib
    L = _lib.load()
    v, t = mesh.cube(1.0, 1)
    b = mesh.Body.from_mesh(v, t)
    for order in ("ctx-geom-tree", "geom-tree-ctx", "tree-ctx-geom"):
        ctx, geom, tree = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        assert L.bemgpu_ctx_create(0, ctypes.byref(ctx)) == 0
        xyz = np.ascontiguousarray(b.verts)
        tri = np.ascontiguousarray(b.tris, dtype=np.int32)
        rwg = np.ascontiguousarray(b.rwg, dtype=np.int32)
        assert L.bemgpu_geom_create(ctx, xyz.ctypes.data, b.nv, tri.ctypes.data, b.nt, ctypes.byref(geom)) == 0
        assert L.bemgpu_tree_create(geom, rwg.ctypes.data, b.nrwg, ctypes.byref(tree)) == 0
        rel = {"ctx": lambda: L.bemgpu_ctx_destroy(ctx), "geom": lambda: L.bemgpu_geom_destroy(geom),
               "tree": lambda: L.bemgpu_tree_destroy(tree)}
        for name in order.split("-"):
            assert rel[name]() == 0
