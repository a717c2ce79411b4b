#!/usr/bin/env python3
"""Benchmark: spectral-power solves/s of the per-frequency hot path
(fill -> LU -> trace, CalcHeatTransfer) on one GB300, plus Z-fill entries/s.

Workload (default): two jittered icospheres, radius 1 um, subdivision level 3
(1280 triangles, 1920 RWG edges per body, N = 7680 complex unknowns), SiC
Lorentz model, gaps {20, 50, 100, 200, 500, 1000} nm x 64 frequencies in
0.08-0.13 eV; a step is one (gap, frequency) solve, steps walk that grid.
Synthetic meshes from bem_gb300.mesh (seeded), no dataset.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--precision fp64|mixed] [--workload ico3|ico2|cube4|tip] [--lanes L]

Requests go through the request farm (bem_gb300.api.Farm): L lanes (default
4), each a context with its own stream and host thread, keep L solves in
flight, as the reference's MPI task farm keeps one per servant.  The timed
region is bracketed by device synchronisations and CUDA events, so it is the
GPU's wall time for K solves.

--impl reference times the reference path's CPU implementation on the host
cores (the oracle port: oracle/bem_oracle.c fill + numpy LAPACK algebra), on a
bounded sample of each step's work.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "spectral-power solves/s"
SIC = (6.7, 0.0983, 0.120, 0.00059)

WORKLOADS = {
    # name: (generator kwargs, gaps um, freqs)
    "ico3": dict(kind="ico", level=3, gaps=[0.02, 0.05, 0.1, 0.2, 0.5, 1.0], freqs=np.linspace(0.08, 0.13, 64)),
    "ico2": dict(kind="ico", level=2, gaps=[0.02, 0.05, 0.1, 0.2, 0.5, 1.0], freqs=np.linspace(0.08, 0.13, 64)),
    "cube4": dict(kind="cube", nsub=4, gaps=[0.1], freqs=np.linspace(0.08, 0.13, 20)),
    # a tip over a plate: per request a cone (0.5 um base radius, 1 um high,
    # hemispherical apex 50-200 nm) of 300-1500 RWG edges drawn from a seed, a
    # 4 x 4 x 0.5 um plate of 1920 edges, gap log-uniform 10-1000 nm, frequency
    # uniform 0.08-0.13 eV: requests of uneven N (4400-6800 unknowns)
    "tip": dict(kind="tip", requests=64, seed=7),
}


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def tip_requests(wl):
    """(tip body, plate body, eV) per request of the tip workload."""
    from bem_gb300 import mesh
    rng = np.random.default_rng(wl["seed"])
    pv, pt = mesh.box(4.0, 4.0, 0.5, 16, 16, 2)
    out = []
    for _ in range(wl["requests"]):
        gap = float(np.exp(rng.uniform(np.log(0.01), np.log(1.0))))
        na = int(rng.integers(12, 21))
        nside = int(rng.integers(4, 20))
        tv, tt = mesh.cone_tip(0.5, 1.0, float(rng.uniform(0.05, 0.2)), n_around=na, n_side=nside, n_cap=3, n_base=3)
        plate = mesh.Body.from_mesh(pv + np.array([0.0, 0.0, -gap - 0.25]), pt)
        out.append((mesh.Body.from_mesh(tv, tt), plate, float(rng.uniform(0.08, 0.13))))
    return out


def make_bodies(wl):
    from bem_gb300 import mesh
    if wl["kind"] == "tip":
        return [(b1, b2) for (b1, b2, _) in tip_requests(wl)]
    if wl["kind"] == "ico":
        v, t = mesh.icosphere(1.0, wl["level"], jitter=0.02, seed=12345)
    else:
        v, t = mesh.cube(1.0, wl["nsub"])
    b2 = mesh.Body.from_mesh(v, t)
    bodies = []
    for gap in wl["gaps"]:
        b1 = b2.translated(mesh.gap_translation(v, v, gap))
        bodies.append((b1, b2))
    return bodies


def step_grid(wl):
    if wl["kind"] == "tip":
        return [(i, r[2]) for i, r in enumerate(tip_requests(wl))]
    return [(gi, float(f)) for gi in range(len(wl["gaps"])) for f in wl["freqs"]]


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


# Nominal GB300 FP64 rate (vector and tensor): MEASURED_PEAKS.json carries HBM and
# bf16 only, so FP64-bound kernels are compared with this nominal figure.
FP64_NOMINAL_TFLOPS = 1.25


def run_ours(args, rank, world):
    import ctypes
    import torch
    from bem_gb300 import api, _lib
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    wl = WORKLOADS[args.workload]
    prec = {"fp64": _lib.PREC_FP64, "mixed": _lib.PREC_MIXED_LA, "mixed-fp32fill": _lib.PREC_MIXED}[args.precision]
    ctx = api.Context(dev)
    L = _lib.load()
    diel = api.FixedLorentz(*SIC)
    bodies = make_bodies(wl)
    systems = [api.parseShapes(b1, b2, diel, diel, ctx) for (b1, b2) in bodies]
    grid = step_grid(wl)
    # each rank walks its own slice of the (gap, f) grid: independent solves, no collective
    order = grid[rank::world] if world > 1 else grid
    a = 1e-6
    # requests go through the farm: `lanes` contexts, each on its own stream
    # and host thread, so consecutive solves overlap on the GPU
    farm = api.Farm(args.lanes, dev)
    lane_ctx = farm.lane_contexts()

    def job(k, sysset=None):
        gi, f = order[k % len(order)]
        top, s, t = (sysset or systems)[gi]
        return (a, f, 300.0, 0.0, top, s, t)

    farm.map([job(k) for k in range(args.warmup)], precision=prec, strict=False)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = sum(L.bemgpu_ctx_launches(c) for c in lane_ctx)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    infos = []
    with ClockSampler(dev) as clk:
        # the GPU is idle here; ev1 is recorded after every lane has finished
        # (each collected result has synchronised its lane's stream)
        ev0.record()
        Ps = farm.map([job(args.warmup + k) for k in range(args.steps)], precision=prec, strict=False, infos=infos)
        torch.cuda.synchronize()
        ev1.record()
        torch.cuda.synchronize()
    launches = sum(L.bemgpu_ctx_launches(c) for c in lane_ctx) - launches0
    ms = ev0.elapsed_time(ev1)
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())

    # Serving: Poisson arrivals at 80 % of the measured throughput, each
    # request one (gap, frequency) solve; latency = submit -> result ready
    # (the farm's host clock), reported as p50 / p99.
    serving = None
    if args.serve_requests > 0:
        rate = 0.8 * args.steps * world / (ms / 1e3)
        rng = np.random.default_rng(2024)
        arrivals = np.cumsum(rng.exponential(1.0 / rate, args.serve_requests))
        t0s = time.perf_counter()
        tks = []
        for k, ta in enumerate(arrivals):
            dt = ta - (time.perf_counter() - t0s)
            if dt > 0:
                time.sleep(dt)
            tks.append(farm.submit(*job(args.warmup + args.steps + k), precision=prec))
        lat = []
        for tk in tks:
            info = {}
            farm.result(tk, info=info, strict=False)
            lat.append(info["ms_latency"])
        span = time.perf_counter() - t0s
        serving = {"arrivals": "poisson", "rate_per_s": rate, "requests": len(tks),
                   "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                   "mean_ms": float(np.mean(lat)), "solves_per_s": len(tks) / span, "lanes": args.lanes}

    # e2e through the public API from host buffers: each step uploads its
    # geometry and trees from host arrays inside the timed region, submits the
    # request to the farm and reads the spectral power back.
    from bem_gb300 import mesh as _mesh
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_ev0 = torch.cuda.Event(enable_timing=True)
    e2e_ev1 = torch.cuda.Event(enable_timing=True)
    e2e_ev0.record()
    h2d = 0
    tickets = []
    for k in range(args.steps):
        gi, f = order[(args.warmup + k) % len(order)]
        b1, b2 = bodies[gi]
        xyz, tris, rwg, ns = _mesh.two_body(b1, b2)
        sysk = api.parseShapes(b1, b2, diel, diel, ctx)
        h2d += xyz.nbytes + tris.nbytes + rwg.nbytes * 2
        tickets.append(farm.submit(a, f, 300.0, 0.0, *sysk, precision=prec))
        del sysk
    for tk in tickets:
        farm.result(tk, strict=False)
    torch.cuda.synchronize()
    e2e_ev1.record()
    torch.cuda.synchronize()
    e2e_ms = e2e_ev0.elapsed_time(e2e_ev1)
    e2e_wall = (time.perf_counter() - t0) * 1e3
    e2e_ms = max(e2e_ms, e2e_wall)
    farm.close()

    # Per-kernel times for the roofline: overlapped lanes inflate each other's
    # event-timed kernel durations, so the kernels are timed (CUDA events on
    # the launching stream, per kernel class) over solves run one at a time,
    # the same requests as the first timed steps.
    n_prof = min(args.steps, 4)
    prof_jobs = [job(args.warmup + k) for k in range(n_prof)]
    api.CalcHeatTransfer(*job(0), precision=prec, strict=False)  # workspace of this context
    torch.cuda.synchronize()
    L.bemgpu_prof_enable(ctx.handle, 1)
    prof_infos = []
    for j in prof_jobs:
        prof_infos.append({})
        api.CalcHeatTransfer(*j, precision=prec, strict=False, info=prof_infos[-1])
    stats = {}
    for kk, name in enumerate(_lib.K_NAMES):
        n = ctypes.c_int64()
        t_ms, fl, by = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        L.bemgpu_prof_query(ctx.handle, kk, ctypes.byref(n), ctypes.byref(t_ms), ctypes.byref(fl), ctypes.byref(by))
        stats[name] = dict(launches=n.value, ms=t_ms.value, flops=fl.value, bytes=by.value)
    L.bemgpu_prof_enable(ctx.handle, 0)

    n_unknowns = 2 * systems[0][0].rwgs
    ns2 = 2 * systems[0][1].rwgs
    nt2 = 2 * systems[0][2].rwgs
    entries = n_unknowns ** 2 + ns2 ** 2 + nt2 ** 2
    value = args.steps * world / (ms / 1e3)
    fill_ms = sum(i["ms_fill"] for i in prof_infos) / len(prof_infos)
    pk, pk_kind = peaks()
    roof = roofline(stats, args.precision, pk, pk_kind)
    out = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128" if args.precision == "fp64" else "c64+c128",
        "data": "synthetic (seeded jittered icospheres; no dataset)",
        "config": workload_config(args, n_unknowns, world),
        "fill_gentries_per_s": entries / (fill_ms / 1e3) / 1e9,
        "stage_ms": {k: sum(i[k] for i in prof_infos) / len(prof_infos)
                     for k in ("ms_fill", "ms_lu", "ms_solve", "ms_trace", "ms_refine")},
        "err_est": [i["err_est"] for i in infos], "refine_iters": [i["refine_iters"] for i in infos],
        "kernel_ms_per_step": {k: v["ms"] / n_prof for k, v in stats.items()},
        "kernel_ms_note": f"stage and kernel-class times (and the fill rate) over {n_prof} solves run one at "
                          f"a time, without lane overlap",
        "roofline": roof,
        "gpu_launches": int(launches),
        "e2e": {"value": args.steps / (e2e_ms / 1e3), "unit": "solves/s", "h2d_bytes_per_step": int(h2d / args.steps),
                "d2h_bytes_per_step": 8 + 16 + 4},
        "clocks": clk.summary(),
        "serving": serving,
        "P_sample": Ps[:2],
    }
    return out


# Kernel groups of the per-kind breakdown and the resource that bounds each.
# "ex_gemm": the exact complex128 tensor-core product (refinement residual and
# trace): 15 bf16 slice products per complex MAC; "tc_gemm": the bf16x3
# complex64 products (LU trailing updates, triangular inverses, correction
# solves): 6 bf16 products per complex MAC.
GROUPS = {
    "ex_gemm": (("refine_gemm", "trace"), "tensor", 15),
    "tc_gemm": (("lu_gemm", "solve_gemm", "trsm"), "tensor", 6),
    "fill": (("fill_near", "fill_far"), None, 0),
    "lu_panel": (("lu_panel",), "latency", 0),
    "memory": (("gather", "slice"), "hbm", 0),
}


def roofline(stats, precision, pk, pk_kind):
    """Roofline of the dominant kernel group of the timed region: algorithmic
    flops (or bytes) per CUDA-event second against the measured peak."""
    tot = {g: sum(stats[k]["ms"] for k in ks if k in stats) for g, (ks, _, _) in GROUPS.items()}
    dom = max(tot, key=tot.get)
    ks, bound, products = GROUPS[dom]
    ms = tot[dom]
    fl = sum(stats[k]["flops"] for k in ks if k in stats)
    by = sum(stats[k]["bytes"] for k in ks if k in stats)
    n = sum(stats[k]["launches"] for k in ks if k in stats)
    base = {"kernel": dom, "kinds": list(ks), "launches": n, "avg_launch_ms": ms / max(1, n), "traffic": None}
    if dom == "fill":
        if precision == "fp64":
            ach = fl / (ms / 1e3) / 1e12
            return dict(base, bound="fp64", achieved=ach, peak=FP64_NOMINAL_TFLOPS, unit="TFLOP/s",
                        frac=ach / FP64_NOMINAL_TFLOPS, peak_source="nominal GB300 FP64 (not in MEASURED_PEAKS.json)")
        ach = fl / (ms / 1e3) / 1e12
        return dict(base, bound="fp32 pipe (double-float)", achieved=ach, peak=FP64_NOMINAL_TFLOPS, unit="TFLOP/s",
                    frac=ach / FP64_NOMINAL_TFLOPS,
                    peak_source="FP64-class work in double-float; compared with the nominal FP64 rate it replaces",
                    note="algorithmic FP64-class flops of the fill (frozen count) per CUDA-event second; the FP32 "
                         "pipes run the double-float arithmetic at ~55 % of their issue rate (ncu, near-pair "
                         "kernel), so frac > 1 means faster than the FP64 pipe could be, not above a roofline")
    if bound == "tensor":
        ach = fl / (ms / 1e3) / 1e12
        peak = pk.get("bf16_tflops_sustained", 1700.0)
        return dict(base, bound="tensor", achieved=ach, peak=peak, unit="TFLOP/s", frac=ach / peak,
                    peak_source=f"{pk_kind} bf16 sustained",
                    executed_bf16_tflops=ach * products, executed_frac=ach * products / peak,
                    note=f"algorithmic complex flops (8 m n k); the kernel issues {products} bf16 slice products "
                         f"per complex MAC, so the tensor pipe runs {products}x the algorithmic rate")
    ach = by / (ms / 1e3) / 1e9
    out = dict(base, bound="hbm", achieved=ach, peak=pk["hbm_gbs"], unit="GB/s", frac=ach / pk["hbm_gbs"],
               peak_source=pk_kind)
    if bound == "latency":
        out["note"] = "latency-bound: one grid barrier per matrix column (cooperative panel); bytes are the panel's"
    return out


def workload_config(args, n_unknowns, world):
    wl = WORKLOADS[args.workload]
    if args.workload == "ico3":
        name = (f"{args.workload}: two r=1um icospheres L3 (1280 tris, 1920 RWGs each), N={n_unknowns}, SiC, "
                f"gaps {wl['gaps']} um x {len(wl['freqs'])} f in 0.08-0.13 eV")
    elif args.workload == "tip":
        name = (f"tip: {wl['requests']} requests, cone tip (300-1500 RWGs, apex 50-200 nm) over a 4x4x0.5 um "
                f"plate (1920 RWGs), gap log-uniform 10-1000 nm, f uniform 0.08-0.13 eV, seed {wl['seed']}; "
                f"N varies per request")
    else:
        name = args.workload
    return {"workload": name, "precision": args.precision, "N": n_unknowns, "parallelism": f"replicas x{world}",
            "lanes": getattr(args, "lanes", 1),
            "l2": "inputs larger than L2 (W alone is %.0f MB)" % (n_unknowns ** 2 * 16 / 1e6)}


def run_reference_sample(wl_name, threads=None, frac=None):
    """Times the oracle port (the reference path restated on the CPU) on a
    bounded sample of one solve: the three fills over a fraction of the test
    triangles (scaled up), and the dense algebra at full size."""
    from bem_gb300 import mesh
    from oracle import oracle
    wl = WORKLOADS[wl_name]
    (b1, b2) = make_bodies(wl)[0]
    xyz, tris, rwg, ns = mesh.two_body(b1, b2)
    ntri = b1.nt + b2.nt
    frac = frac or (1.0 if ntri <= 500 else 64.0 / ntri)
    threads = threads or os.cpu_count() or 1
    f = float(wl["freqs"][0])
    om = oracle.dimensionless_omega(1e-6, f)
    eps = oracle.lorentz_eps(f, *SIC)
    t0 = time.perf_counter()
    k = max(1, int(round(frac * ntri)))
    oracle.zts(xyz, tris, rwg, rwg, 1 + 0j, 1 + 0j, om, tri_range=(0, k), nthreads=threads)
    k1 = max(1, int(round(frac * b1.nt)))
    oracle.zts(xyz, tris, rwg[:ns], rwg[:ns], eps, 1 + 0j, om, tri_range=(0, k1), nthreads=threads)
    oracle.zts(xyz, tris, rwg[ns:], rwg[ns:], eps, 1 + 0j, om, tri_range=(0, k1), nthreads=threads)
    t_fill = (time.perf_counter() - t0) * (ntri / k)
    n = 2 * rwg.shape[0]
    rng = np.random.default_rng(0)
    W = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)) + n * np.eye(n)
    t0 = time.perf_counter()
    Wi = np.linalg.inv(W)
    ns2 = 2 * ns
    G = W[:ns2, :ns2]
    B1 = (G @ Wi[:ns2, :])[:, ns2:]
    B2 = (Wi[:, ns2:] @ W[ns2:, ns2:])[:ns2, :]
    _ = np.trace(B2.conj().T @ B1)
    t_la = time.perf_counter() - t0
    return {"solve_s": t_fill + t_la, "fill_s": t_fill, "la_s": t_la, "threads": threads, "n": n,
            "sample": f"fills over {k}/{ntri} test triangles (x{ntri / k:.1f}) + full-size inverse/products, "
                      f"n={n}, one frequency"}


def run_reference(args, rank, world):
    wl = WORKLOADS[args.workload]
    for _ in range(args.warmup if args.warmup < 1 else 1):
        pass
    samples = []
    for k in range(max(1, args.steps)):
        samples.append(run_reference_sample(args.workload))
    s = statistics.median(x["solve_s"] for x in samples)
    v = 1.0 / s
    return {"metric": METRIC, "value": v, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": s * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128", "data": "synthetic (seeded meshes; no dataset)",
            "config": workload_config(args, samples[0]["n"], world), "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "solves/s", "cores": samples[0]["threads"], "kind": "port",
                             "sample": samples[0]["sample"]},
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed", "mixed-fp32fill"])
    ap.add_argument("--workload", default="ico3", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--lanes", type=int, default=4, help="farm lanes: solves in flight at once on the GPU")
    ap.add_argument("--serve-requests", type=int, default=16,
                    help="requests of the Poisson-arrival serving measurement (0: skip)")
    args = ap.parse_args()
    rank, world, local = env_rank()
    if world > 1 and args.impl == "ours":
        import torch.distributed as dist
        dist.init_process_group("nccl")
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args, rank, world)))
        return
    out = run_ours(args, rank, world)
    if rank == 0:
        if not args.no_cpu_baseline and world == 1:
            r = run_reference_sample(args.workload)
            out["cpu_baseline"] = {"value": 1.0 / r["solve_s"], "unit": "solves/s", "cores": r["threads"],
                                   "kind": "port", "sample": r["sample"]}
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
