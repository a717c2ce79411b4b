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
