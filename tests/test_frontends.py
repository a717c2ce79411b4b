"""Host-side callers of the path: the dielectric registry
(src/util/Dielectrics.cpp:15-63 and the models it returns), the X3D reader
(src/ShapeParser.cpp:83-153, Transform src/util/Transform.cpp:43-72), and the
transfer / transfer-mpi job front ends (src/transfer.cpp, src/transfer-mpi.cpp).
No GPU: the sweep's solves are covered by tests/test_farm_gpu.py and the GPU
test at the end of this file."""
import math
import os

import numpy as np
import pytest

from bem_gb300 import api, dielectrics, mesh, transfer, x3d

EV, HBAR = 1.60217646e-19, 1.05457148e-34


def test_models_follow_their_formulas():
    w = 0.1 * EV / HBAR
    al = dielectrics.Al().eps(0.1)
    w0, g0 = 1.50690679e14, 3.76734192e13
    assert al == pytest.approx(2.2281 + 1.30601 * w0 ** 2 / (w0 ** 2 - w ** 2 - 2j * w * g0), rel=1e-15)
    au = dielectrics.Au().eps(0.1)
    assert au == pytest.approx(1.0 - 1.366592804e16 ** 2 / (w * (w + 1j * 4.08407045e13)), rel=1e-15)
    assert dielectrics.SiliconDoped(0.0).eps(0.1) == 11.7
    n = dielectrics.SiliconDoped(-1e25).eps(0.1)
    p = dielectrics.SiliconDoped(1e25).eps(0.1)
    assert n.real < 11.7 and n.imag > 0 and p.real < 11.7 and p.imag > 0
    for d in (dielectrics.Al(), dielectrics.Au(), dielectrics.Vacuum()):
        assert d.mu(0.1) == 1.0
    # SiC at 300 K is the fixed-Lorentz form with its room-temperature constants
    sic = api.SiC()
    sic.setTemperature(300.0)
    assert abs(sic.eps(0.1)) > 0 and sic.eps(0.1).imag > 0


def test_tabulated_interpolates_and_extends():
    t = dielectrics.Tabulated([0.1, 0.2, 0.4], [1.0, 2.0, 4.0], [0.0, 0.5, 0.5])
    assert t.eps(0.15) == pytest.approx(complex(1.5, 0.25) ** 2)
    assert t.eps(0.3) == pytest.approx(complex(3.0, 0.5) ** 2)
    assert t.eps(0.5) == pytest.approx(complex(5.0, 0.5) ** 2)   # last segment extended
    assert t.eps(0.05) == pytest.approx(complex(0.5, -0.25) ** 2)
    with pytest.raises(ValueError):
        dielectrics.Tabulated([0.2, 0.1], [1, 1], [0, 0])


def test_registry_caches_and_falls_back_to_constant():
    a = dielectrics.getDielectric("Au")
    assert a is dielectrics.getDielectric("Au")
    c = dielectrics.getDielectric("Glass", {"eps": dielectrics.parse_param("(2.25,0.01)")})
    assert c.eps(0.1) == complex(2.25, 0.01) and c.mu(0.1) == 1.0
    assert dielectrics.getDielectric("Nothing").eps(0.3) == 1.0
    with pytest.raises(ValueError):
        dielectrics.getDielectric("SiN")
    s = dielectrics.getDielectric("SiN", table=([0.1, 0.2], [2.0, 2.0], [0.0, 0.0]))
    assert s.eps(0.15) == pytest.approx(4.0)
    assert dielectrics.parse_param("3") == 3 and dielectrics.parse_param("2.5") == 2.5
    assert dielectrics.parse_param("1+2i") == 1 + 2j and dielectrics.parse_param("SiC") == "SiC"


X3D = """<?xml version="1.0" encoding="UTF-8"?>
<X3D version="3.0"><Scene>
<Transform translation="1 2 3" scale="2 2 2" rotation="0 0 1 1.5707963267948966">
 <Shape><Dielectric material="Glass" eps="(4,0.5)"/>
 <IndexedFaceSet coordIndex="0 1 2 -1, 0 2 3 -1, 0 3 1 -1, 1 3 2 -1">
  <Coordinate point="0 0 0, 1 0 0, 0 1 0, 0 0 1"/>
 </IndexedFaceSet></Shape>
</Transform></Scene></X3D>
"""


def test_x3d_reader_applies_transform_and_material(tmp_path):
    p = tmp_path / "tet.x3d"
    p.write_text(X3D)
    sh = x3d.read_x3d(str(p))
    assert sh.faces == [(0, 1, 2), (0, 2, 3), (0, 3, 1), (1, 3, 2)]
    P = np.array(sh.coord)
    # scale 2, the reference's rotation (by -phi about z: (x, y) -> (y, -x)), then the translation
    expect = np.array([[0, 0, 0], [0, -2, 0], [2, 0, 0], [0, 0, 2]], float) + [1, 2, 3]
    assert np.abs(P - expect).max() < 1e-12
    assert sh.dielectric.eps(0.1) == complex(4, 0.5)
    b, d = x3d.body_from_x3d(str(p))
    assert b.nt == 4 and b.nrwg == 6 and d is sh.dielectric


def test_x3d_round_trip_of_a_generated_mesh(tmp_path):
    v, t = mesh.icosphere(1.0, 1, jitter=0.02, seed=1)
    pts = ", ".join(" ".join(f"{c:.17g}" for c in row) for row in v)
    idx = ", ".join(f"{a} {b} {c} -1" for a, b, c in t)
    p = tmp_path / "ico.x3d"
    p.write_text(f'<X3D><Scene><Shape><IndexedFaceSet coordIndex="{idx}"><Coordinate point="{pts}"/>'
                 f'</IndexedFaceSet></Shape></Scene></X3D>')
    b, d = x3d.body_from_x3d(str(p))
    assert d is None
    assert np.array_equal(b.verts, v) and np.array_equal(b.tris, t)
    assert np.array_equal(b.rwg, mesh.Body.from_mesh(v, t).rwg)


def test_job_files_and_grid(tmp_path):
    (tmp_path / "gaps.txt").write_text("0.1 0 0\n0.2 0 0\n")
    (tmp_path / "temps.txt").write_text("300 0\n400 0\n")
    (tmp_path / "freqs.txt").write_text("0.09 0.1\n0.11\nend\n0.5\n")
    assert transfer.push_file_values(str(tmp_path / "gaps.txt"), 3) == [(0.1, 0, 0), (0.2, 0, 0)]
    assert transfer.push_file_values(str(tmp_path / "temps.txt"), 2) == [(300, 0), (400, 0)]
    assert transfer.push_file_values(str(tmp_path / "freqs.txt"), 1) == [0.09, 0.1, 0.11]
    g = transfer.job_grid([1e-6], [(0.1, 0, 0), (0.2, 0, 0)], [0.09, 0.1], [(300, 0), (400, 0)])
    assert len(g) == 8
    assert g[0] == (1e-6, (0.1, 0, 0), 0.09, (300, 0)) and g[1][2] == 0.1 and g[2][1] == (0.2, 0, 0)
    assert g[4][3] == (400, 0)


@pytest.mark.gpu
def test_sweep_writes_and_resumes(tmp_path):
    v, t = mesh.cube(1.0, 2)
    body = mesh.Body.from_mesh(v, t)
    d = api.FixedLorentz(*api.SIC_CONFIG)
    gaps = [(1.1, 0.0, 0.0), (1.2, 0.0, 0.0)]
    freqs = [0.09, 0.11]
    out = str(tmp_path / "output")
    n = transfer.run_sweep(body, body, d, d, [1e-6], gaps, freqs, [(300.0, 0.0)], out, lanes=2,
                           precision=0)
    assert n == 4
    lines = open(out).read().splitlines()
    assert len(lines) == 4
    for ln, (a, g, f, T) in zip(lines, transfer.job_grid([1e-6], gaps, freqs, [(300.0, 0.0)])):
        c = ln.split()
        P = api.CalcHeatTransfer(a, f, 300.0, 0.0, *api.parseShapes(body.translated(g), body, d, d))
        assert float(c[1]) == g[0] and float(c[4]) == f
        assert float(c[5]) == pytest.approx(P, rel=1e-13)
    assert transfer.run_sweep(body, body, d, d, [1e-6], gaps, freqs, [(300.0, 0.0)], out, lanes=2) == 0
    open(out, "w").write("\n".join(lines[:3]) + "\n")
    assert transfer.run_sweep(body, body, d, d, [1e-6], gaps, freqs, [(300.0, 0.0)], out, lanes=2,
                              precision=0) == 1
    assert open(out).read().splitlines()[3] == lines[3]
    assert not math.isnan(float(lines[0].split()[5]))
    assert os.path.getsize(out) > 0
