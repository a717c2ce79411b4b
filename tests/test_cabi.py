"""The C-ABI library: builds, loads, exports every symbol include/bemgpu.h
declares, and its host-only helpers agree with the oracle.  CPU only (no
compute call needs a GPU here)."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from bem_gb300 import build, _lib
    build.build()
    return _lib.load()


def _declared():
    src = open(os.path.join(ROOT, "include", "bemgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(bemgpu_[a-z0-9_]+)\s*\(", src)))


def test_header_matches_binding_list():
    from bem_gb300 import _lib
    assert _declared() == sorted(_lib.EXPORTED)


def test_every_declared_symbol_is_exported(lib):
    for name in _declared():
        assert hasattr(lib, name), name


def test_version(lib):
    assert b"sm_103a" in lib.bemgpu_version()


def test_green_init_matches_oracle(lib):
    from bem_gb300 import _lib
    from oracle import oracle
    g = _lib.Green()
    eps, mu, om = 16.4 + 0.14j, 1 + 0j, 0.5068
    rc = lib.bemgpu_green_init((ctypes.c_double * 2)(eps.real, eps.imag), (ctypes.c_double * 2)(1.0, 0.0),
                               (ctypes.c_double * 2)(om, 0.0), 0, ctypes.byref(g))
    assert rc == 0
    ref = oracle.green_constants(eps, mu, om + 0j)
    for k in ("ksquared", "k", "ik", "k2", "Zeps", "Zmu"):
        v = getattr(g, k)
        assert abs(complex(v[0], v[1]) - ref[k]) <= 1e-15 * abs(ref[k]), k


def test_theta_and_omega_match_oracle(lib):
    from oracle import oracle
    for a, eV in ((1e-6, 0.08), (1e-6, 0.13), (2e-7, 0.1)):
        om = lib.bemgpu_dimensionless_omega(a, eV)
        assert om == pytest.approx(oracle.dimensionless_omega(a, eV), rel=1e-15)
        for T in (0.0, 300.0, 600.0):
            assert lib.bemgpu_theta(om, T) == pytest.approx(oracle.theta(om, T), rel=1e-14, abs=0)


def test_options_default(lib):
    from bem_gb300 import _lib
    o = _lib.Options()
    lib.bemgpu_options_default(ctypes.byref(o))
    assert (o.farThresh6, o.farThresh10, o.farThresh15, o.farThresh21) == (12.0, 8.0, 4.0, 2.0)


def test_null_arguments_are_rejected(lib):
    assert lib.bemgpu_ctx_create(0, None) == -1
    assert lib.bemgpu_zts(None, None, None, None, None, 0, None, 0, None) == -1
    assert lib.bemgpu_tree_size(None) == -1


def test_api_mirror_frequency_sweep(tmp_path):
    from bem_gb300 import api
    p = tmp_path / "freqs.txt"
    p.write_text("0.06\n0.08\n0.1\n")
    assert api.FrequencySweep(str(p)).f == [0.06, 0.08, 0.1]
    assert api.FrequencySweep(str(tmp_path / "missing.txt")).f == []


def test_sic_temperature_model():
    from bem_gb300 import api
    s = api.SiC()
    e300 = s.eps(0.1)
    s.setTemperature(600.0)
    assert s.eps(0.1) != e300
    f = api.FixedLorentz(*api.SIC_CONFIG)
    from oracle import oracle
    assert f.eps(0.1) == pytest.approx(oracle.lorentz_eps(0.1, *api.SIC_CONFIG), rel=1e-15)


def test_native_rwg_table_matches_python(lib):
    """bemgpu_mesh_rwgs builds the reference's edge-creation order
    (src/ShapeMesh.cpp:857-928) as mesh.build_rwgs does, row for row."""
    from bem_gb300 import mesh
    cases = [mesh.cube(1.0, 3), mesh.icosphere(1.0, 2, jitter=0.02, seed=3), mesh.box(0.5, 10.0, 10.0, 2, 17, 17),
             mesh.cone_tip(0.5, 1.0, 0.1, n_around=13, n_side=5, n_cap=3, n_base=3)]
    for v, t in cases:
        want = mesh.build_rwgs(t)
        got = mesh.build_rwgs_native(t, v.shape[0])
        assert got.shape == (3 * t.shape[0] // 2, 4)
        assert np.array_equal(got, want)
        assert np.array_equal(mesh.Body.from_mesh(v, t, native=True).rwg, want)
    # a capacity below the count reports the count
    v, t = mesh.cube(1.0, 2)
    out = np.zeros((4, 4), np.int32)
    n = ctypes.c_int()
    rc = lib.bemgpu_mesh_rwgs(np.ascontiguousarray(t, np.int32).ctypes.data, t.shape[0], v.shape[0],
                              out.ctypes.data, 4, ctypes.byref(n))
    assert rc == -1 and n.value == 3 * t.shape[0] // 2
    # an open mesh (one triangle removed) and a bad vertex id are mesh errors
    with pytest.raises(ValueError):
        mesh.build_rwgs_native(t[1:], v.shape[0])
    bad = t.copy()
    bad[0, 0] = v.shape[0]
    with pytest.raises(ValueError):
        mesh.build_rwgs_native(bad, v.shape[0])


def test_solve_footprint_is_monotone_and_fits_the_slab_pair(lib):
    """bemgpu_solve_footprint (host only): grows with the bodies, the mixed
    path holds more than the FP64 path, and the largest workload (two
    8190-RWG slabs, N = 32760) stays below one GB300's 284,208 MiB with the
    default escalating solver (its complex64 and FP64-class stages are not
    held together)."""
    fp = lambda ns, nt, prec: lib.bemgpu_solve_footprint(ns, nt, prec)
    for prec in (0, 2):
        sizes = [fp(n, n, prec) for n in (288, 480, 1920, 4000, 8190)]
        assert all(a < b for a, b in zip(sizes, sizes[1:])), sizes
    assert fp(1920, 1920, 2) > fp(1920, 1920, 0)
    assert fp(8190, 8190, 2) < 284208 * 2 ** 20
    assert fp(0, 10, 2) == -1 and fp(10, -1, 0) == -1
