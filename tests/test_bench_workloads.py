"""The benchmark's synthetic workloads have the sizes their descriptions give
(the reference's cube4 case, the icosphere pair, the thin-slab pair, the tip
and the serving mix), and the reference arm prints the contract's JSON line.
No GPU."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _gap(b1, b2):
    return float(b1.verts[:, 0].min() - b2.verts[:, 0].max())


@pytest.mark.parametrize("name, nrwg, n_systems, steps", [
    ("cube4", 288, 1, 20), ("ico3", 1920, 6, 384), ("slab", 8190, 1, 8)])
def test_fixed_geometry_workloads(name, nrwg, n_systems, steps):
    wl = bench.WORKLOADS[name]
    bodies = bench.make_bodies(wl)
    grid = bench.step_grid(wl)
    assert len(bodies) == n_systems and len(grid) == steps
    for (b1, b2, cfg), gap in zip(bodies, wl["gaps"]):
        assert b1.nrwg == b2.nrwg == nrwg
        assert _gap(b1, b2) == pytest.approx(gap, abs=1e-12)
        assert cfg == bench.SIC
    assert all(T1 == 300.0 for (_, _, T1) in grid)


def test_mix_workload():
    wl = bench.WORKLOADS["mix"]
    reqs = bench.mix_requests(wl)
    assert len(reqs) == wl["requests"]
    ns = [2 * (b1.nrwg + b2.nrwg) for (b1, b2, _, _) in reqs]
    # bodies of 288 .. 4032 RWG edges (icosphere L2 480 is the smallest sphere)
    assert 4 * 288 <= min(ns) and max(ns) <= 4 * 4032
    assert {cfg for (_, _, cfg, _) in reqs} == {bench.SIC, bench.ALUMINA}
    for b1, b2, _, T1 in reqs:
        assert 0.01 - 1e-12 <= _gap(b1, b2) <= 1.0 + 1e-12
        assert 300.0 <= T1 <= 600.0
    grid = bench.step_grid(wl)
    assert len(grid) == wl["requests"] * wl["sweep"]
    # request-minor: the first `requests` steps are one frequency of every request
    assert [g for (g, _, _) in grid[:wl["requests"]]] == list(range(wl["requests"]))
    assert np.allclose(sorted({f for (_, f, _) in grid}), np.linspace(0.08, 0.13, wl["sweep"]))
    # the same seed gives the same requests
    again = bench.mix_requests(wl)
    assert all(np.array_equal(a[0].verts, b[0].verts) and a[3] == b[3] for a, b in zip(reqs, again))


def test_tip_workload():
    wl = bench.WORKLOADS["tip"]
    bodies = bench.make_bodies(wl)
    ns = [2 * (b1.nrwg + b2.nrwg) for (b1, b2, _) in bodies]
    assert len(bodies) == wl["requests"] and 4400 <= min(ns) and max(ns) <= 6800


def test_reference_arm_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--workload", "cube4", "--steps", "1", "--warmup", "3"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    d = json.loads(out.stdout.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["config"]["N"] == 1152
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    sp = d["cpu_baseline"]["spread"]
    assert sp["min"] <= d["value"] <= sp["max"] and sp["steps"] == 1
    assert "throughput mode" in d["cpu_baseline"]["sample"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]


def test_roofline_block_of_each_group():
    """The roofline block names the dominant kernel group with the contract's
    keys; the double-float fill is measured against the FP32 issue rate and
    the exact product against the bf16 peak, with the library's count of
    executed slice products."""
    pk = {"hbm_gbs": 7000.0, "bf16_tflops_sustained": 1715.7}
    fill = {"fill_near": dict(ms=38.0, flops=1.0e11, bytes=0.0, launches=3, tensor=0.0),
            "fill_far": dict(ms=17.8, flops=7.7e10, bytes=0.0, launches=3, tensor=0.0),
            "refine_gemm": dict(ms=33.0, flops=3.6e12, bytes=0.0, launches=10, tensor=3.1e13),
            "trace": dict(ms=17.0, flops=1.7e12, bytes=0.0, launches=10, tensor=1.5e13)}
    r = bench.roofline(fill, "mixed", pk, "measured", sm_mhz=2070.0)
    for k in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
        assert k in r, k
    assert r["kernel"] == "fill" and r["bound"].startswith("fp32 issue")
    assert r["peak"] == pytest.approx(152 * 128 * 2070e6 / 1e12)
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"]) and 0 < r["frac"] < 1
    tensor = dict(fill)
    tensor["fill_near"] = dict(fill["fill_near"], ms=1.0)
    tensor["fill_far"] = dict(fill["fill_far"], ms=1.0)
    r = bench.roofline(tensor, "mixed", pk, "measured", sm_mhz=2070.0)
    assert r["kernel"] == "ex_gemm" and r["bound"] == "tensor" and r["peak"] == 1715.7
    assert r["executed_bf16_tflops"] == pytest.approx(4.6e13 / 0.050 / 1e12)
    assert r["slice_products_per_mac"] == pytest.approx(4.6e13 / 5.3e12)
    # every group that ran, each with its own bound and its share of the time
    rs = bench.rooflines(fill, "mixed", pk, "measured", sm_mhz=2070.0)
    assert list(rs) == ["fill", "ex_gemm"]
    assert rs["fill"]["frac"] == pytest.approx(bench.roofline(fill, "mixed", pk, "measured", sm_mhz=2070.0)["frac"])
    assert rs["ex_gemm"]["bound"] == "tensor" and "executed_frac" in rs["ex_gemm"]
    assert sum(v["ms_share"] for v in rs.values()) == pytest.approx(1.0)
