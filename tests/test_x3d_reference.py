"""The X3D reader (bem_gb300.x3d) against the reference's own parser on the
reference's example files: ShapeParserHandler (src/ShapeParser.cpp:83-153,
with its Transform stack, src/util/Transform.cpp, and the FaceIndex /
Vector3 string parsers) built by oracle/Makefile.ref over a small stand-in for
Xerces-C (oracle/shim/), run by the oracle harness (--x3d).  Every vertex
after the transforms, every face and the Dielectric must agree.  CPU only;
skipped where the reference checkout (its examples) or the harness is absent."""
import glob
import os
import subprocess

import numpy as np
import pytest

from bem_gb300 import x3d

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")


def _examples():
    import __graft_entry__ as g
    d = os.path.join(os.path.dirname(g.REFERENCE_SRC), "examples")
    return sorted(glob.glob(os.path.join(d, "*.x3d")))


def _reference_parse(path, tmp_path):
    out = str(tmp_path / "shape.txt")
    subprocess.run([HARNESS, "--x3d", path, "--shape-out", out], check=True, capture_output=True)
    lines = open(out).read().splitlines()
    nv, nt = map(int, lines[0].split())
    V = np.array([[float(x) for x in ln.split()] for ln in lines[1:1 + nv]]).reshape(-1, 3)
    F = np.array([[int(x) for x in ln.split()] for ln in lines[1 + nv:1 + nv + nt]]).reshape(-1, 4)
    last = lines[1 + nv + nt].split()
    eps = complex(float(last[1]), float(last[2])) if last[0] == "eps" else None
    return V, F, eps


@pytest.mark.skipif(not os.path.exists(HARNESS), reason="the reference harness is not built here")
def test_reader_matches_the_reference_parser_on_its_examples(tmp_path):
    files = _examples()
    if not files:
        pytest.skip("the reference's example files are not here")
    sin_table = (np.array([0.05, 0.2]), np.array([2.0, 2.0]), np.array([0.1, 0.1]))
    for path in files:
        V, F, eps = _reference_parse(path, tmp_path)
        sh = x3d.read_x3d(path, table=sin_table)
        mv = np.array(sh.coord, dtype=np.float64).reshape(-1, 3)
        mf = np.array(sh.faces, dtype=np.int64).reshape(-1, 3)
        name = os.path.basename(path)
        assert (F[:, 3] == -1).all(), name             # every example face is a triangle
        assert np.array_equal(mf, F[:, :3]), name
        assert mv.shape == V.shape, name
        scale = max(1.0, float(np.abs(V).max()))
        assert float(np.abs(mv - V).max()) <= 4 * np.finfo(float).eps * scale, name
        assert (sh.dielectric is None) == (eps is None), name
        if eps is not None and "SiN" not in open(path).read():
            assert abs(sh.dielectric.eps(0.1) / eps - 1) < 1e-14, name
