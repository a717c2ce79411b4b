"""The reference-side binding (bem_gb300/dropin/bem_gpu_dropin.cpp) is a
link-time drop-in: the reference's own objects, with Impedance.cpp and
HeatTransfer.cpp rebuilt so that their CPU Zts / CalcHeatTransfer / Theta keep
other names, link with the binding and libbemgpu.so into an executable with
every symbol resolved, and the public names resolve to the binding.  Needs the
reference checkout and its objects (built by __graft_entry__.build() where the
checkout exists); skipped elsewhere.  No GPU: the link is the check."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _reference_objects_present():
    import __graft_entry__ as g
    return os.path.isdir(g.REFERENCE_SRC) and os.path.isdir(os.path.join(ROOT, "oracle", "_ref", "obj"))


@pytest.mark.skipif(not shutil.which("make") or not shutil.which("nm"), reason="make and nm needed")
def test_binding_links_in_place_of_the_cpu_definitions():
    import sys
    sys.path.insert(0, ROOT)
    if not _reference_objects_present():
        pytest.skip("the reference checkout and its objects are not here")
    from bem_gb300 import build
    build.build()
    r = subprocess.run(["make", "-f", "oracle/Makefile.ref", "dropin"], cwd=ROOT, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    exe = os.path.join(ROOT, "oracle", "_ref", "dropin_harness")
    syms = subprocess.run(["nm", "-C", exe], capture_output=True, text=True, check=True).stdout
    defined = {ln.split(" T ", 1)[1] for ln in syms.splitlines() if " T " in ln}
    for name in ("Zts(RWGTree*, RWGTree*, GreensFunction*, Options&)",
                 "CalcHeatTransfer(double, double, double, double, RWGTree*, RWGTree*, RWGTree*, Options&)",
                 "Theta(double, double)"):
        assert name in defined, name                      # the binding's definition
        assert "bem_cpu_" + name in defined, name        # the reference's, renamed
    # the binding reaches the library through the C ABI only
    undefined = {ln.split()[-1] for ln in syms.splitlines() if ln.strip().startswith("U ")}
    assert {"bemgpu_heat_transfer", "bemgpu_zts_host", "bemgpu_tree_create", "bemgpu_geom_create"} <= undefined
