"""Mesh generators and the RWG builder (host set-up).  CPU only."""
import numpy as np
import pytest

from bem_gb300 import mesh


def _check_closed(v, t):
    b = mesh.Body.from_mesh(v, t)
    assert b.nrwg * 2 == 3 * b.nt                   # closed surface: E = 3T/2
    assert b.nv - b.nrwg + b.nt == 2                # genus 0
    for pos, neg, e1, e2 in b.rwg:
        assert pos != neg
        for tr in (pos, neg):
            assert e1 in t[tr] and e2 in t[tr]
    # outward orientation: signed volume positive
    a, bb, c = v[t[:, 0]], v[t[:, 1]], v[t[:, 2]]
    vol = np.einsum("ij,ij->i", a, np.cross(bb, c)).sum() / 6
    assert vol > 0
    return b


@pytest.mark.parametrize("nsub", [1, 2, 4])
def test_cube(nsub):
    v, t = mesh.cube(1.0, nsub)
    b = _check_closed(v, t)
    assert b.nt == 12 * nsub * nsub
    assert np.allclose(v.min(0), -0.5) and np.allclose(v.max(0), 0.5)


def test_cube4_is_the_plain_workload():
    v, t = mesh.cube(1.0, 4)
    b = mesh.Body.from_mesh(v, t)
    assert (b.nt, b.nrwg) == (192, 288)             # N = 2 * 2 * 288 = 1152 unknowns for two cubes


@pytest.mark.parametrize("level", [1, 2, 3])
def test_icosphere(level):
    v, t = mesh.icosphere(1.0, level, jitter=0.02, seed=12345)
    b = _check_closed(v, t)
    assert b.nt == 20 * 4 ** level
    r = np.linalg.norm(v, axis=1)
    assert abs(r.mean() - 1) < 0.02


def test_icosphere_jitter_is_seeded():
    v1, _ = mesh.icosphere(1.0, 2, jitter=0.02, seed=12345)
    v2, _ = mesh.icosphere(1.0, 2, jitter=0.02, seed=12345)
    v3, _ = mesh.icosphere(1.0, 2, jitter=0.02, seed=1)
    assert np.array_equal(v1, v2) and not np.array_equal(v1, v3)


def test_gap_translation():
    v, t = mesh.cube(1.0, 2)
    d = mesh.gap_translation(v, v, 0.1)
    assert abs((v + d)[:, 0].min() - v[:, 0].max() - 0.1) < 1e-12


def test_two_body_offsets():
    v, t = mesh.cube(1.0, 1)
    b2 = mesh.Body.from_mesh(v, t)
    b1 = b2.translated([2.0, 0, 0])
    xyz, tris, rwg, ns = mesh.two_body(b1, b2)
    assert ns == b1.nrwg and rwg.shape[0] == 2 * ns
    assert (rwg[ns:, 0] >= b1.nt).all() and (rwg[ns:, 2] >= b1.nv).all()
    assert xyz.shape[0] == 2 * b1.nv


def test_non_manifold_rejected():
    v, t = mesh.cube(1.0, 1)
    with pytest.raises(ValueError):
        mesh.build_rwgs(t[:-1])


def _reference_edges(v1, t1, v2, t2):
    """Each body's edges in the order the reference's ShapeMesh created them
    (src/ShapeMesh.cpp:857-928), from the reference's own code via the oracle
    harness: rows (first triangle, second triangle, p1, p2), local ids."""
    import os
    import subprocess
    import tempfile
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    harness = os.path.join(root, "oracle", "_ref", "ref_harness")
    if not os.path.exists(harness):
        pytest.skip("the reference harness is built only where the reference checkout is present")
    with tempfile.TemporaryDirectory() as td:
        m1, m2, out = (os.path.join(td, x) for x in ("m1.txt", "m2.txt", "edges.txt"))
        mesh.write_mesh_txt(m1, v1, t1)
        mesh.write_mesh_txt(m2, v2, t2)
        subprocess.run([harness, "--mesh1", m1, "--mesh2", m2, "--gap", "5,0,0", "--lorentz1", "6.7,0.0983,0.12,0.00059",
                        "--lorentz2", "6.7,0.0983,0.12,0.00059", "--edges", out], check=True, capture_output=True)
        e = np.loadtxt(out, dtype=np.int64).reshape(-1, 5)
    return [e[e[:, 0] == b][:, 1:] for b in (0, 1)]


@pytest.mark.parametrize("make", [lambda: mesh.cube(1.0, 4), lambda: mesh.icosphere(1.0, 2, jitter=0.02, seed=12345),
                                  lambda: mesh.box(0.5, 10.0, 10.0, 2, 12, 12),
                                  lambda: mesh.cone_tip(0.5, 1.0, 0.1, n_around=14, n_side=6, n_cap=3, n_base=3)])
def test_rwg_tables_follow_the_reference_edge_creation_order(make):
    """bemgpu_mesh_rwgs (the C-ABI host builder) and mesh.build_rwgs give each
    body's RWGs in exactly the reference's ShapeMesh edge order: same rows,
    same positive / negative triangles, same edge vertex order."""
    v, t = make()
    v2, t2 = mesh.icosphere(1.0, 1)
    ref, _ = _reference_edges(v, t, v2, t2)
    native = mesh.build_rwgs_native(t, v.shape[0])
    assert np.array_equal(native, ref)
    assert np.array_equal(mesh.build_rwgs(t), ref)
