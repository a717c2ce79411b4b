#!/usr/bin/env python3
"""Benchmark: spectral-power solves/s of the per-frequency hot path
(fill -> LU -> trace, CalcHeatTransfer) on one GB300, plus Z-fill entries/s.

Workload (default): two jittered icospheres, radius 1 um, subdivision level 3
(1280 triangles, 1920 RWG edges per body, N = 7680 complex unknowns), SiC
Lorentz model, gaps {20, 50, 100, 200, 500, 1000} nm x 64 frequencies in
0.08-0.13 eV; a step is one (gap, frequency) solve, steps walk that grid.
Synthetic meshes from bem_gb300.mesh (seeded), no dataset.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--precision fp64|mixed] [--workload ico3|ico2|cube4|tip|slab|mix] [--lanes L]
                  [--batch B] [--solver escalate|c64|fp64class] [--serve-requests R] [--sweep F]
                  [--e2e-steps K2] [--prof-steps K3] [--fp64-steps K4] [--subs LIST]
                  [--tune cache|retune|off] [--ex-wide 0|1|2] [--panel-ctas C] [--lite]
                  [--no-cpu-baseline]

Other workloads: cube4 (two 1 um cubes, 4x4 squares per face, N = 1152, gap
100 nm, 20 f); tip (64 cone tips over a plate, each with a 64-frequency
sweep, uneven N per tip); slab (two 10 x 10 x 0.5 um slabs of 8190 RWGs each,
N = 32760, gap 50 nm, 8 f in 0.115-0.119 eV); mix (the serving mix: each
request a frequency sweep over a random pair of bodies drawn from cubes,
icospheres, thin slabs and cone tips, SiC or alumina, gap log-uniform
10-1000 nm, T1 uniform 300-600 K).  The default ico3 line also carries the
FP64 path's rate on its first timed requests with the measured error of the
mixed results against it, and sub-results of cube4, tip, slab and mix, each
run as its own process.

Requests go through the request farm (bem_gb300.api.Farm): L lanes (default
4), each a context with its own stream and host thread, keep L solves in
flight, as the reference's MPI task farm keeps one per servant.  The timed
region is bracketed by device synchronisations and CUDA events, so it is the
GPU's wall time for K solves.

--impl reference times the reference path's CPU implementation on the host
cores (the oracle port: oracle/bem_oracle.c fill + LAPACK zgetrf/zgetri and
the trace products) in the reference's throughput mode, one single-threaded
process per core, each on a bounded sample of a solve.
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
ALUMINA = (3.1, 0.0787, 0.111, 0.0020)

WORKLOADS = {
    # name: (generator kwargs, gaps um, freqs)
    "ico3": dict(kind="ico", level=3, gaps=[0.02, 0.05, 0.1, 0.2, 0.5, 1.0], freqs=np.linspace(0.08, 0.13, 64)),
    "ico2": dict(kind="ico", level=2, gaps=[0.02, 0.05, 0.1, 0.2, 0.5, 1.0], freqs=np.linspace(0.08, 0.13, 64)),
    "cube4": dict(kind="cube", nsub=4, gaps=[0.1], freqs=np.linspace(0.08, 0.13, 20)),
    # a tip over a plate: per geometry a cone (0.5 um base radius, 1 um high,
    # hemispherical apex 50-200 nm) of 300-1500 RWG edges drawn from a seed, a
    # 4 x 4 x 0.5 um plate of 1920 edges, gap log-uniform 10-1000 nm, and a
    # sweep of 64 frequencies uniform in 0.08-0.13 eV: 64 x 64 = 4096 solves of
    # uneven N (4400-6800 unknowns); the steps walk each geometry's sweep in turn
    "tip": dict(kind="tip", requests=64, seed=7, sweep=64),
    # two thin slabs facing each other across the gap (x is the 0.5 um side):
    # 2 x 35 x 35 squares per face, 8190 RWG edges each, N = 32760; W alone is
    # 17 GB in complex128
    "slab": dict(kind="slab", gaps=[0.05], freqs=np.linspace(0.115, 0.119, 8)),
    # the serving mix: per request a pair of bodies, each drawn from {cube of
    # 288-1152 edges, icosphere L2-L3 (480 / 1920 edges), 10 x 10 x 0.5 um slab
    # of 2142-4032 edges, cone tip of 300-1500 edges}, SiC or alumina, gap
    # log-uniform 10-1000 nm, T1 uniform 300-600 K, T2 = 0, and a sweep of
    # `sweep` frequencies in 0.08-0.13 eV
    "mix": dict(kind="mix", requests=64, sweep=32, seed=11),
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
        tv, tt = _tip_mesh(rng)
        plate = mesh.Body.from_mesh(pv + np.array([0.0, 0.0, -gap - 0.25]), pt)
        out.append((mesh.Body.from_mesh(tv, tt), plate, float(rng.uniform(0.08, 0.13))))
    return out


def tip_sweep(wl, i, eV0):
    """The frequencies of tip geometry i: its request's own eV, then
    sweep - 1 more drawn uniform in 0.08-0.13 eV (seeded per geometry)."""
    rng = np.random.default_rng([wl["seed"], i])
    return [eV0] + [float(x) for x in rng.uniform(0.08, 0.13, wl.get("sweep", 1) - 1)]


def _tip_mesh(rng):
    from bem_gb300 import mesh
    na = int(rng.integers(12, 21))
    nside = int(rng.integers(4, 20))
    return mesh.cone_tip(0.5, 1.0, float(rng.uniform(0.05, 0.2)), n_around=na, n_side=nside, n_cap=3, n_base=3)


def _mix_mesh(rng):
    from bem_gb300 import mesh
    kind = int(rng.integers(4))
    if kind == 0:
        return mesh.cube(1.0, int(rng.integers(4, 9)))
    if kind == 1:
        return mesh.icosphere(1.0, int(rng.integers(2, 4)), jitter=0.02, seed=int(rng.integers(1 << 30)))
    if kind == 2:
        m = int(rng.integers(17, 25))
        return mesh.box(0.5, 10.0, 10.0, 2, m, m)
    return _tip_mesh(rng)


def mix_requests(wl):
    """(body 1, body 2, Lorentz constants, T1) per request of the serving mix;
    body 1 sits the request's gap beyond body 2 along +x."""
    from bem_gb300 import mesh
    rng = np.random.default_rng(wl["seed"])
    out = []
    for _ in range(wl["requests"]):
        v1, t1 = _mix_mesh(rng)
        v2, t2 = _mix_mesh(rng)
        gap = float(np.exp(rng.uniform(np.log(0.01), np.log(1.0))))
        cfg = SIC if rng.integers(2) == 0 else ALUMINA
        T1 = float(rng.uniform(300.0, 600.0))
        b2 = mesh.Body.from_mesh(v2, t2)
        b1 = mesh.Body.from_mesh(v1 + mesh.gap_translation(v1, v2, gap), t1)
        out.append((b1, b2, cfg, T1))
    return out


def make_bodies(wl):
    """(body 1, body 2, Lorentz constants of both bodies) per system."""
    from bem_gb300 import mesh
    if wl["kind"] == "tip":
        return [(b1, b2, SIC) for (b1, b2, _) in tip_requests(wl)]
    if wl["kind"] == "mix":
        return [(b1, b2, cfg) for (b1, b2, cfg, _) in mix_requests(wl)]
    if wl["kind"] == "ico":
        v, t = mesh.icosphere(1.0, wl["level"], jitter=0.02, seed=12345)
    elif wl["kind"] == "slab":
        v, t = mesh.box(0.5, 10.0, 10.0, 2, 35, 35)
    else:
        v, t = mesh.cube(1.0, wl["nsub"])
    b2 = mesh.Body.from_mesh(v, t)
    bodies = []
    for gap in wl["gaps"]:
        b1 = b2.translated(mesh.gap_translation(v, v, gap))
        bodies.append((b1, b2, SIC))
    return bodies


def mix_freqs(wl):
    return np.linspace(0.08, 0.13, wl["sweep"])


def step_grid(wl):
    """(system index, eV, T1) per step.  The mix walks its requests' sweeps
    request-minor, so that consecutive steps are different requests."""
    if wl["kind"] == "tip":
        return [(i, f, 300.0) for i, r in enumerate(tip_requests(wl)) for f in tip_sweep(wl, i, r[2])]
    if wl["kind"] == "mix":
        reqs = mix_requests(wl)
        return [(i, float(f), reqs[i][3]) for f in mix_freqs(wl) for i in range(len(reqs))]
    return [(gi, float(f), 300.0) for gi in range(len(wl["gaps"])) for f in wl["freqs"]]


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
# FP32 lanes of the GPU (152 SMs x 128): the issue rate of the double-float fill.
FP32_LANES = 152 * 128
# FP32-pipe thread instructions per algorithmic FP64-class flop of the
# double-float fill kernels, from ncu's smsp__inst_executed on the ico2
# workload (one launch each over the three fills of a solve): near pairs 7.76
# (6.24e9 warp instructions, 16400 pairs x 1.57 Mflop), far pairs 7.2 (1.01e9
# warp instructions for 598000 pairs, 5 % more per pair than the 6.85 counted
# on the exterior fill alone with the rules' frozen flop counts).
DF_INSTR_PER_FLOP = {"fill_near": 7.76, "fill_far": 7.2}
# DRAM bytes of the fill (far and near launch together) per matrix entry of the
# three Zts outputs, from ncu on the ico2 workload: 246.7 MB (far 118.2 MB +
# near 128.5 MB) for 5.53 M entries; the half-pair blocks the fill writes are
# 32 B per entry (177 MB), so the measured traffic is 1.39x the algorithmic.
FILL_DRAM_BYTES_PER_ENTRY = 44.6
# The exact product's DRAM bytes against the library's operand-traffic model
# (its ProfScope bytes: A re-read once per band of N-tiles, B once, C written):
# ncu 313.7 MB against 327 MB modelled for ex_gemm_kernel<5, 3> at ico2.
EX_TRAFFIC_PER_MODEL_BYTE = 0.96


def shard_steps(grid, rank, world):
    """Replicas: rank r takes steps r, r + world, ... of the grid (independent
    solves, as the reference's task farm hands jobs to its servants)."""
    return grid[rank::world] if world > 1 else list(grid)


def max_over_ranks(x, world):
    """The slowest rank's value (the timed region ends when every replica has
    finished); the only cross-rank operation besides the barriers."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _check_rc(rc):
    if rc != 0:
        raise RuntimeError(f"bemgpu call failed with status {rc}")


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
    diels = {SIC: api.FixedLorentz(*SIC), ALUMINA: api.FixedLorentz(*ALUMINA)}
    bodies = make_bodies(wl)
    systems = [api.parseShapes(b1, b2, diels[c], diels[c], ctx) for (b1, b2, c) in bodies]
    grid = step_grid(wl)
    # each rank walks its own slice of the (gap, f) grid: independent solves, no collective
    order = shard_steps(grid, rank, world)
    a = 1e-6
    # requests go through the farm: `lanes` contexts, each on its own stream
    # and host thread, so consecutive solves overlap on the GPU
    farm = api.Farm(args.lanes, dev, batch=args.batch)
    lane_ctx = farm.lane_contexts()
    solver = {"escalate": 0, "c64": 1, "fp64class": 2}[args.solver]
    for c in lane_ctx:
        _check_rc(L.bemgpu_ctx_set_solver(c, solver))
    ctx.set_solver(solver)

    def job(k, sysset=None):
        gi, f, T1 = order[k % len(order)]
        top, s, t = (sysset or systems)[gi]
        return (a, f, T1, 0.0, top, s, t)

    # launch shapes from the project's autotuner (bem_gb300.tuning): cached per
    # GPU and size class, tuned on this workload's first request when missing
    tiles = None
    if args.tune != "off":
        from bem_gb300 import tuning
        t0t = time.perf_counter()
        params, source = tuning.tuned(lambda: api.CalcHeatTransfer(*job(0), precision=prec, strict=False),
                                      ctx.handle, 2 * systems[order[0][0]][0].rwgs, dev,
                                      retune=args.tune == "retune")
        for c in lane_ctx:
            tuning.apply(c, params)
        # the tuning solves ran on the main context: give back its workspace
        # before the lanes allocate theirs
        _check_rc(L.bemgpu_ctx_trim(ctx.handle))
        tiles = dict(params, source=source, seconds=time.perf_counter() - t0t)
    if args.panel_ctas:
        for c in lane_ctx + [ctx.handle]:
            _check_rc(L.bemgpu_ctx_set_tuning(c, _lib.TUNE_PANEL_CTAS, args.panel_ctas))
        tiles = dict(tiles or {}, panel_ctas=args.panel_ctas)
    if args.ex_wide is not None:
        for c in lane_ctx + [ctx.handle]:
            _check_rc(L.bemgpu_ctx_set_tuning(c, _lib.TUNE_EX_WIDE, args.ex_wide))
        tiles = dict(tiles or {}, ex_wide=args.ex_wide)
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
    ms = max_over_ranks(ev0.elapsed_time(ev1), world)

    # e2e through the public API from host buffers, right after the timed
    # region (the same requests): each step uploads its geometry and trees
    # from host arrays inside the timed region, submits the request to the
    # farm and reads the spectral power back.
    from bem_gb300 import mesh as _mesh
    e2e = None
    if not args.lite:
        with ClockSampler(dev) as e2e_clk:
            e2e = _e2e_segment(args, order, bodies, diels, ctx, farm, prec, _mesh, api, torch, a)
        e2e["clocks"] = e2e_clk.summary()

    # Serving: Poisson arrivals at 80 % of the measured throughput.  A request
    # is one (gap, frequency) solve, or for the mix a sweep of `sweep`
    # frequencies over one pair of bodies, all submitted at its arrival;
    # latency = arrival -> last result ready (the farm's host clock), p50 / p99.
    serving = None
    if args.serve_requests > 0:
        if wl["kind"] == "mix":
            t1_of = {gi: T1 for (gi, _, T1) in grid}
            mine = sorted({gi for (gi, _, _) in order})
            per_req = []
            for r in range(args.serve_requests):
                gi = mine[r % len(mine)]
                per_req.append([(a, float(f), t1_of[gi], 0.0, *systems[gi])
                                for f in np.linspace(0.08, 0.13, args.sweep or wl["sweep"])])
        else:
            per_req = [[job(args.warmup + args.steps + k)] for k in range(args.serve_requests)]
        solves = sum(len(r) for r in per_req)
        rate = 0.8 * args.steps * world / (ms / 1e3) * args.serve_requests / solves
        rng = np.random.default_rng(2024)
        arrivals = np.cumsum(rng.exponential(1.0 / rate, args.serve_requests))
        t0s = time.perf_counter()
        tks = []
        for k, ta in enumerate(arrivals):
            dt = ta - (time.perf_counter() - t0s)
            if dt > 0:
                time.sleep(dt)
            tks.append([farm.submit(*j, precision=prec) for j in per_req[k]])
        lat = []
        for req in tks:
            worst = 0.0
            for tk in req:
                info = {}
                farm.result(tk, info=info, strict=False)
                worst = max(worst, info["ms_latency"])
            lat.append(worst)
        span = time.perf_counter() - t0s
        serving = {"arrivals": "poisson", "rate_per_s": rate, "requests": len(tks),
                   "solves_per_request": solves / len(tks),
                   "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                   "mean_ms": float(np.mean(lat)), "solves_per_s": solves / span, "lanes": args.lanes}


    # The plain FP64 path on the first timed requests, through the same farm
    # (the rate the mixed path is compared with) and, request by request, the
    # measured error of the timed mixed-precision results against it.
    fp64_arm, accuracy = None, None
    n64 = min(args.fp64_steps, args.steps)
    if n64 > 0 and args.precision != "fp64":
        jobs64 = [job(args.warmup + k) for k in range(n64)]
        torch.cuda.synchronize()
        f_ev0 = torch.cuda.Event(enable_timing=True)
        f_ev1 = torch.cuda.Event(enable_timing=True)
        f_ev0.record()
        P64 = farm.map(jobs64, precision=_lib.PREC_FP64)
        torch.cuda.synchronize()
        f_ev1.record()
        torch.cuda.synchronize()
        ms64 = f_ev0.elapsed_time(f_ev1)
        errs = [abs(Ps[k] / P64[k] - 1) for k in range(n64)]
        fp64_arm = {"value": n64 / (ms64 / 1e3), "unit": "solves/s", "steps": n64, "ms_per_step": ms64 / n64,
                    "lanes": args.lanes, "note": "the plain FP64 path (complex128 fill, FP64 LU on the FMA pipes) "
                                                 "on the first timed requests, through the same farm"}
        accuracy = {"err_vs_fp64_max": max(errs), "err_vs_fp64": errs,
                    "err_est_same_solves": [infos[k]["err_est"] for k in range(n64)], "solves_checked": n64,
                    "note": "relative error of the timed mixed-precision spectral power against the FP64 path "
                            "on the same requests"}
    farm.close()

    n_all = sorted({2 * sy[0].rwgs for sy in systems})
    n_unknowns = n_all[0] if len(n_all) == 1 else f"{n_all[0]}-{n_all[-1]}"
    value = args.steps * world / (ms / 1e3)
    out = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128" if args.precision == "fp64" else "c64+c128",
        "data": "synthetic (seeded generated meshes; no dataset)",
        "config": workload_config(args, n_unknowns, world),
        "err_est": [i["err_est"] for i in infos], "refine_iters": [i["refine_iters"] for i in infos],
        "factorization": {"complex64": sum(i["solver"] == 1 for i in infos),
                          "fp64class": sum(i["solver"] == 2 for i in infos),
                          "fp64_fallback": sum(i["solver"] == 3 for i in infos)},
        "gpu_launches": int(launches),
        "tiles": tiles,
        "clocks": clk.summary(),
        "serving": serving,
        "P_sample": Ps[:2],
    }
    if fp64_arm:
        out["fp64_path"] = fp64_arm
        out["mixed_over_fp64"] = value / fp64_arm["value"]
        out["accuracy"] = accuracy
    if args.lite:
        out["stage_ms"] = {k: sum(i[k] for i in infos) / len(infos)
                           for k in ("ms_fill", "ms_lu", "ms_solve", "ms_trace", "ms_refine")}
        out["stage_ms_note"] = "per-solve stage times inside the timed region (lanes overlapping)"
        return out
    out["e2e"] = e2e
    out.update(_kernel_segment(args, job, prec, ctx, clk, L, api, torch, _lib, ctypes))
    return out


def _e2e_segment(args, order, bodies, diels, ctx, farm, prec, _mesh, api, torch, a):
    """e2e through the public API from host buffers: each step uploads its
    geometry and trees from host arrays inside the timed region, submits the
    request to the farm and reads the spectral power back."""
    e2e_steps = args.e2e_steps or args.steps
    steps = [order[(args.warmup + k) % len(order)] for k in range(e2e_steps)]
    # bytes each step uploads (vertices, triangles, and the RWG table of the
    # two-body tree and of the two bodies' trees), counted outside the timer
    up = {}
    for gi, _, _ in steps:
        if gi not in up:
            xyz, tris, rwg, ns = _mesh.two_body(*bodies[gi][:2])
            up[gi] = xyz.nbytes + tris.nbytes + rwg.nbytes * 2
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_ev0 = torch.cuda.Event(enable_timing=True)
    e2e_ev1 = torch.cuda.Event(enable_timing=True)
    e2e_ev0.record()
    h2d = 0
    tickets = []
    for gi, f, T1 in steps:
        b1, b2, c = bodies[gi]
        sysk = api.parseShapes(b1, b2, diels[c], diels[c], ctx)
        h2d += up[gi]
        tickets.append(farm.submit(a, f, T1, 0.0, *sysk, precision=prec))
        # the farm holds the trees until the result is collected; then they
        # are destroyed inside the timed region (their device memory goes to
        # the library's batch free, so no lane waits for it)
        del sysk
    for tk in tickets:
        farm.result(tk, strict=False)
    torch.cuda.synchronize()
    e2e_ev1.record()
    torch.cuda.synchronize()
    e2e_ms = e2e_ev0.elapsed_time(e2e_ev1)
    e2e_wall = (time.perf_counter() - t0) * 1e3
    e2e_ms = max(e2e_ms, e2e_wall)
    return {"value": e2e_steps / (e2e_ms / 1e3), "unit": "solves/s", "h2d_bytes_per_step": int(h2d / e2e_steps),
            "d2h_bytes_per_step": 8 + 16 + 4}


def _kernel_segment(args, job, prec, ctx, clk, L, api, torch, _lib, ctypes):
    """Per-kernel times for the roofline: overlapped lanes inflate each
    other's event-timed kernel durations, so the kernels are timed (CUDA
    events on the launching stream, per kernel class) over solves run one at
    a time, the same requests as the first timed steps."""
    n_prof = args.prof_steps or min(args.steps, 4)
    if args.batch > 1:
        # the farm solved batches: so do the profiled solves (whole batches)
        n_prof = max(n_prof, args.batch) // args.batch * args.batch
    prof_jobs = [job(args.warmup + k) for k in range(n_prof)]
    api.CalcHeatTransfer(*job(0), precision=prec, strict=False)  # workspace of this context
    if args.batch > 1:
        api.CalcHeatTransferBatch(prof_jobs[:args.batch], precision=prec, strict=False)
    torch.cuda.synchronize()
    L.bemgpu_prof_enable(ctx.handle, 1)
    prof_infos = []
    if args.batch > 1:
        for k in range(0, n_prof, args.batch):
            api.CalcHeatTransferBatch(prof_jobs[k:k + args.batch], precision=prec, strict=False, infos=prof_infos)
    else:
        for j in prof_jobs:
            prof_infos.append({})
            api.CalcHeatTransfer(*j, precision=prec, strict=False, info=prof_infos[-1])
    stats = {}
    for kk, name in enumerate(_lib.K_NAMES):
        n = ctypes.c_int64()
        t_ms, fl, by = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        L.bemgpu_prof_query(ctx.handle, kk, ctypes.byref(n), ctypes.byref(t_ms), ctypes.byref(fl), ctypes.byref(by))
        tf = ctypes.c_double()
        L.bemgpu_prof_query_tensor(ctx.handle, kk, ctypes.byref(tf))
        stats[name] = dict(launches=n.value, ms=t_ms.value, flops=fl.value, bytes=by.value, tensor=tf.value)
    L.bemgpu_prof_enable(ctx.handle, 0)

    def entries(j):
        n, ns2, nt2 = 2 * j[4].rwgs, 2 * j[5].rwgs, 2 * j[6].rwgs
        return n ** 2 + ns2 ** 2 + nt2 ** 2

    fill_s = sum(i["ms_fill"] for i in prof_infos) / 1e3
    pk, pk_kind = peaks()
    rargs = dict(fp64class=all(i.get("solver") == 2 for i in prof_infos), sm_mhz=clk.summary()["sm_mhz"],
                 entries=sum(entries(j) for j in prof_jobs))
    roof = roofline(stats, args.precision, pk, pk_kind, **rargs)
    roofs = rooflines(stats, args.precision, pk, pk_kind, **rargs)
    return {
        "fill_gentries_per_s": sum(entries(j) for j in prof_jobs) / fill_s / 1e9,
        # the three Zts outputs written as complex128 (16 B per entry)
        "fill_write_gbs": 16 * sum(entries(j) for j in prof_jobs) / fill_s / 1e9,
        "stage_ms": {k: sum(i[k] for i in prof_infos) / len(prof_infos)
                     for k in ("ms_fill", "ms_lu", "ms_solve", "ms_trace", "ms_refine")},
        "kernel_ms_per_step": {k: v["ms"] / n_prof for k, v in stats.items()},
        "kernel_ms_note": f"stage and kernel-class times (and the fill rate) over {n_prof} solves run one at "
                          f"a time, without lane overlap",
        "roofline": roof,
        # every kernel group's roofline (the dominant one above in full)
        "rooflines": roofs,
    }


# Kernel groups of the per-kind breakdown and the resource that bounds each.
# "ex_gemm": the exact complex128 tensor-core product (refinement residual and
# trace: 6 to 15 bf16 slice products per complex MAC, by the operands'
# slices); "tc_gemm": the bf16x3 complex64 products (LU trailing updates,
# triangular inverses, correction solves: 6 bf16 products per complex MAC),
# or with the FP64-class factorization its exact products.  The library
# reports the bf16 flops each kind executed (bemgpu_prof_query_tensor).
GROUPS = {
    "ex_gemm": (("refine_gemm", "trace"), "tensor"),
    "tc_gemm": (("lu_gemm", "solve_gemm", "trsm"), "tensor"),
    "fill": (("fill_near", "fill_far"), None),
    "lu_panel": (("lu_panel",), "latency"),
    "memory": (("gather", "slice"), "hbm"),
}


def _groups(fp64class):
    groups = dict(GROUPS)
    if fp64class:
        groups["ex_lu"] = groups.pop("tc_gemm")
    return groups


def roofline(stats, precision, pk, pk_kind, fp64class=False, sm_mhz=None, entries=None):
    """Roofline of the dominant kernel group of the timed region: algorithmic
    flops (or bytes) per CUDA-event second against the measured peak.
    entries: matrix entries the profiled solves filled (the fill's traffic)."""
    groups = _groups(fp64class)
    tot = {g: sum(stats[k]["ms"] for k in ks if k in stats) for g, (ks, _) in groups.items()}
    return group_roofline(max(tot, key=tot.get), stats, precision, pk, pk_kind, fp64class, sm_mhz, entries)


def rooflines(stats, precision, pk, pk_kind, fp64class=False, sm_mhz=None, entries=None):
    """The same roofline for every kernel group that ran, with its share of
    the profiled kernel time."""
    groups = _groups(fp64class)
    tot = {g: sum(stats[k]["ms"] for k in ks if k in stats) for g, (ks, _) in groups.items()}
    all_ms = sum(tot.values())
    out = {}
    for g in sorted(tot, key=tot.get, reverse=True):
        if tot[g] <= 0:
            continue
        r = group_roofline(g, stats, precision, pk, pk_kind, fp64class, sm_mhz, entries)
        out[g] = {k: r[k] for k in ("bound", "achieved", "peak", "unit", "frac", "avg_launch_ms", "launches",
                                    "traffic", "executed_frac", "alg_fp64class_tflops") if k in r}
        out[g]["ms_share"] = tot[g] / all_ms
        if groups[g][1] == "latency":
            out[g]["bound"] = "latency (panel bytes against HBM shown)"
    return out


def group_roofline(dom, stats, precision, pk, pk_kind, fp64class=False, sm_mhz=None, entries=None):
    """Roofline of kernel group `dom` (see GROUPS)."""
    ks, bound = _groups(fp64class)[dom]
    ms = sum(stats[k]["ms"] for k in ks if k in stats)
    fl = sum(stats[k]["flops"] for k in ks if k in stats)
    by = sum(stats[k]["bytes"] for k in ks if k in stats)
    n = sum(stats[k]["launches"] for k in ks if k in stats)
    base = {"kernel": dom, "kinds": list(ks), "launches": n, "avg_launch_ms": ms / max(1, n), "traffic": None}
    if dom == "fill":
        if entries:
            base["traffic"] = FILL_DRAM_BYTES_PER_ENTRY * entries / max(1, n)
            base["traffic_algorithmic"] = 32.0 * entries / max(1, n)
            base["traffic_source"] = ("ncu dram__bytes_read + dram__bytes_write of the far and near launches at ico2 "
                                      "per matrix entry, times this launch's entries")
        if precision == "fp64":
            ach = fl / (ms / 1e3) / 1e12
            return dict(base, bound="fp64", achieved=ach, peak=FP64_NOMINAL_TFLOPS, unit="TFLOP/s",
                        frac=ach / FP64_NOMINAL_TFLOPS, peak_source="nominal GB300 FP64 (not in MEASURED_PEAKS.json)")
        alg = fl / (ms / 1e3) / 1e12
        instr = sum(stats[k]["flops"] * DF_INSTR_PER_FLOP[k] for k in ks if k in stats)
        ach = instr / (ms / 1e3) / 1e12
        peak = FP32_LANES * (sm_mhz or 2070.0) * 1e6 / 1e12
        return dict(base, bound="fp32 issue (double-float)", achieved=ach, peak=peak,
                    unit="T thread-instructions/s", frac=ach / peak,
                    peak_source="nominal FP32 issue rate: 152 SMs x 128 lanes x the sampled SM clock",
                    alg_fp64class_tflops=alg, instr_per_alg_flop=DF_INSTR_PER_FLOP,
                    note="the fill is FP64-class arithmetic in double-float on the FP32 pipes: its algorithmic "
                         "FP64-class flops (frozen count, live) per CUDA-event second times the FP32-pipe "
                         "thread instructions per algorithmic flop that ncu counted on each fill kernel "
                         "(smsp__inst_executed, ico2)")
    if bound == "tensor":
        if dom == "ex_gemm":
            base["traffic"] = EX_TRAFFIC_PER_MODEL_BYTE * by / max(1, n)
            base["traffic_algorithmic"] = by / max(1, n)
            base["traffic_source"] = ("the library's operand-traffic model of each launch, scaled by ncu's "
                                      "dram__bytes / model on ex_gemm_kernel<5, 3> at ico2 (0.96)")
        ach = fl / (ms / 1e3) / 1e12
        peak = pk.get("bf16_tflops_sustained", 1700.0)
        tens = sum(stats[k].get("tensor", 0.0) for k in ks if k in stats)
        exe = tens / (ms / 1e3) / 1e12
        return dict(base, bound="tensor", achieved=ach, peak=peak, unit="TFLOP/s", frac=ach / peak,
                    peak_source=f"{pk_kind} bf16 sustained",
                    executed_bf16_tflops=exe, executed_frac=exe / peak,
                    slice_products_per_mac=tens / fl if fl else None,
                    note="achieved: algorithmic complex flops (8 m n k); executed: the bf16 slice products the "
                         "kernels issued (library count), against the same bf16 peak")
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
        name = (f"tip: {wl['requests']} geometries x {wl['sweep']} frequencies = {wl['requests'] * wl['sweep']} "
                f"solves, cone tip (300-1500 RWGs, apex 50-200 nm) over a 4x4x0.5 um plate (1920 RWGs), gap "
                f"log-uniform 10-1000 nm, f uniform 0.08-0.13 eV, seed {wl['seed']}; N varies per geometry; the "
                f"timed steps are the first {args.steps} of the geometry-major order")
    elif args.workload == "slab":
        name = (f"slab: two 10x10x0.5 um slabs (5460 tris, 8190 RWGs each), N={n_unknowns}, SiC, gap 50 nm, "
                f"{len(wl['freqs'])} f in 0.115-0.119 eV")
    elif args.workload == "mix":
        name = (f"mix: {wl['requests']} requests, each a pair of bodies from {{cube 288-1152, icosphere L2-L3, "
                f"10x10x0.5 um slab 2142-4032, cone tip 300-1500 RWGs}}, SiC or alumina, gap log-uniform "
                f"10-1000 nm, T1 300-600 K, sweep of {args.sweep or wl['sweep']} f in 0.08-0.13 eV "
                f"(timed steps: one f of each request in turn), seed {wl['seed']}; narrowed from icosphere L2-L4 "
                f"and slabs of 2000-8000 RWGs: L4 icospheres and slabs above 4032 RWGs take seconds per solve "
                f"(the slab workload measures that class)")
    else:
        name = args.workload
    n_max = n_unknowns if isinstance(n_unknowns, int) else int(str(n_unknowns).split("-")[-1])
    return {"workload": name, "precision": args.precision, "N": n_unknowns, "parallelism": f"replicas x{world}",
            "lanes": getattr(args, "lanes", 1), "batch": getattr(args, "batch", 1),
            "solver": getattr(args, "solver", "escalate"),
            "l2": "inputs larger than L2 (W alone is %.0f MB)" % (n_max ** 2 * 16 / 1e6)}


# CPU baseline: the reference path's CPU implementation (the oracle port,
# pinned to the reference binary) in the reference's throughput mode, the MPI
# task farm of src/transfer-mpi.cpp:91-190: one single-threaded process per
# host core (OPENBLAS_NUM_THREADS=1; the reference's fill has no threading,
# src/Impedance.cpp:388-413), all running at once.  Each process times a
# bounded sample of one solve and extrapolates it to the whole solve:
#   fill: the three Zts calls over CPU_FILL_UNITS far-pair equivalents of
#         test triangles (a near pair counts as CPU_NEAR_UNITS), x the
#         triangles / sampled triangles (the same fraction of each call);
#   algebra: zgetrf + zgetri (src/util/DenseMatrix.cpp:65-77), the two
#         products and B2^H B1 (src/HeatTransfer.cpp:36-52) at
#         n_la = min(n, CPU_LA_MAX) with the bodies' proportions, x (n/n_la)^3.
CPU_FILL_UNITS = 4.0e5
CPU_NEAR_UNITS = 150.0
NEAR_PER_TRIANGLE = 13.0
CPU_LA_MAX = 2048
# sample steps of the cpu_baseline block of the GPU arm's line
CPU_BASELINE_STEPS = 3

_CPU_SYSTEMS = {}


def _cpu_system(wl_name, gi):
    key = (wl_name, gi)
    if key not in _CPU_SYSTEMS:
        from bem_gb300 import mesh
        b1, b2, cfg = make_bodies(WORKLOADS[wl_name])[gi]
        xyz, tris, rwg, ns = mesh.two_body(b1, b2)
        _CPU_SYSTEMS[key] = (xyz, tris, rwg, ns, b1.nt, b2.nt, cfg)
    return _CPU_SYSTEMS[key]


def _cpu_solve_sample(task):
    """One process's bounded, single-threaded sample of one solve of the
    oracle port (see CPU_FILL_UNITS); returns its extrapolated seconds."""
    wl_name, gi, f, offset = task
    import scipy.linalg.lapack as lapack
    from oracle import oracle
    xyz, tris, rwg, ns, nt1, nt2, cfg = _cpu_system(wl_name, gi)
    ntri = nt1 + nt2
    units = (ntri + NEAR_PER_TRIANGLE * CPU_NEAR_UNITS) * ntri
    units += sum((m + NEAR_PER_TRIANGLE * CPU_NEAR_UNITS) * m for m in (nt1, nt2))
    frac = min(1.0, CPU_FILL_UNITS / units)
    om = oracle.dimensionless_omega(1e-6, f)
    eps = oracle.lorentz_eps(f, *cfg)
    t_fill = 0.0
    for rows, m, e in ((rwg, ntri, 1 + 0j), (rwg[:ns], nt1, eps), (rwg[ns:], nt2, eps)):
        k = max(1, int(round(frac * m)))
        lo = (offset * k) % m
        hi = min(m, lo + k)
        t0 = time.perf_counter()
        oracle.zts(xyz, tris, rows, rows, e, 1 + 0j, om, tri_range=(lo, hi), nthreads=1, timing_only=True)
        t_fill += (time.perf_counter() - t0) * m / (hi - lo)
    n = 2 * rwg.shape[0]
    n_la = min(n, CPU_LA_MAX)
    ns2 = 2 * max(1, int(round(ns * n_la / n)))
    rng = np.random.default_rng(offset)
    W = np.asfortranarray(rng.standard_normal((n_la, n_la)) + 1j * rng.standard_normal((n_la, n_la))
                          + n_la * np.eye(n_la))
    G1 = rng.standard_normal((ns2, ns2)) + 1j * rng.standard_normal((ns2, ns2))
    G2 = rng.standard_normal((n_la - ns2,) * 2) + 1j * rng.standard_normal((n_la - ns2,) * 2)
    t0 = time.perf_counter()
    lu, piv, info = lapack.zgetrf(W, overwrite_a=True)
    Wi, info = lapack.zgetri(lu, piv, overwrite_lu=True)
    B1 = ((G1 + G1.conj().T) @ Wi[:ns2, :])[:, ns2:]
    B2 = (Wi[:, ns2:] @ (G2 + G2.conj().T))[:ns2, :]
    _ = np.trace(B2.conj().T @ B1)
    t_la = (time.perf_counter() - t0) * (n / n_la) ** 3
    return {"solve_s": t_fill + t_la, "fill_s": t_fill, "la_s": t_la, "n": n, "n_la": n_la,
            "fill_scale": 1.0 / frac, "la_scale": (n / n_la) ** 3}


def _cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


class CpuFarm:
    """The throughput-mode CPU baseline: `procs` spawned single-threaded
    worker processes (spawned, so that they are safe after GPU work)."""

    def __init__(self, wl_name, procs=None):
        import multiprocessing as mp
        self.wl_name = wl_name
        self.procs = procs or _cpu_cores()
        self.grid = step_grid(WORKLOADS[wl_name])
        saved = {k: os.environ.get(k) for k in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS")}
        for k in saved:
            os.environ[k] = "1"
        try:
            self.pool = mp.get_context("spawn").Pool(self.procs)
        finally:
            for k, v in saved.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v

    def step(self, k):
        """One sample step: every process times its own solve sample at
        once; returns (solves/s of the farm, wall seconds, samples)."""
        tasks = []
        for p in range(self.procs):
            gi, f, _ = self.grid[(k * self.procs + p) % len(self.grid)]
            tasks.append((self.wl_name, gi, f, k * self.procs + p))
        t0 = time.perf_counter()
        res = self.pool.map(_cpu_solve_sample, tasks, chunksize=1)
        wall = time.perf_counter() - t0
        return sum(1.0 / r["solve_s"] for r in res), wall, res

    def close(self):
        self.pool.close()
        self.pool.join()


def cpu_baseline_run(wl_name, steps, procs=None):
    farm = CpuFarm(wl_name, procs)
    try:
        vals, walls, res = [], [], []
        for k in range(steps):
            v, w, r = farm.step(k)
            vals.append(v)
            walls.append(w)
            res.extend(r)
    finally:
        farm.close()
    fs = sorted(r["fill_scale"] for r in res)
    ls = sorted(r["la_scale"] for r in res)
    n_all = sorted({r["n"] for r in res})
    sample = (f"throughput mode: {farm.procs} single-threaded processes at once (OPENBLAS_NUM_THREADS=1), "
              f"each timing one solve of the oracle port per step: the three fills over sampled test triangles "
              f"(extrapolation x{fs[0]:.0f}-x{fs[-1]:.0f}) + zgetrf/zgetri and the trace products at "
              f"n_la={min(r['n_la'] for r in res)} (x{ls[0]:.1f}-x{ls[-1]:.1f} by (n/n_la)^3); "
              f"value = sum over processes of 1/(extrapolated solve time), median over {steps} steps")
    return {"value": statistics.median(vals), "spread": {"min": min(vals), "median": statistics.median(vals),
                                                        "max": max(vals), "steps": steps},
            "ms_per_step": 1e3 * statistics.median(walls), "cores": farm.procs,
            "n": n_all[0] if len(n_all) == 1 else f"{n_all[0]}-{n_all[-1]}", "sample": sample,
            "fill_s_per_solve": statistics.median(r["fill_s"] for r in res),
            "la_s_per_solve": statistics.median(r["la_s"] for r in res)}


def run_reference(args, rank, world):
    """The reference arm: the reference path's CPU implementation in its
    throughput mode (CpuFarm) on this host's cores, one bounded sample step
    per timed step (no warm-up: nothing is cached or compiled).  value is
    the median step's extrapolated solves/s; ms_per_step is a sample step's
    wall time."""
    r = cpu_baseline_run(args.workload, max(1, args.steps))
    return {"metric": METRIC, "value": r["value"], "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128", "data": "synthetic (seeded meshes; no dataset)",
            "config": workload_config(args, r["n"], world), "impl": "reference",
            "cpu_baseline": {"value": r["value"], "unit": "solves/s", "cores": r["cores"], "kind": "port",
                             "sample": r["sample"], "spread": r["spread"],
                             "fill_s_per_solve": r["fill_s_per_solve"], "la_s_per_solve": r["la_s_per_solve"]},
            "e2e": {"value": r["value"], "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# Sub-results of the default line: the other synthetic workloads, each run as
# its own bench process (its own GPU memory) after the main measurement, and
# summarised in the main line.  cube4: the reference's CPU case (N = 1152);
# tip: the first 256 solves (4 geometries x 64 frequencies) of the
# tip-over-plate sweep; slab: the large single solve (N = 32760, one
# FP64-class solve after one warm-up solve of the same size); mix: the
# serving mix (64 requests: closed-loop rate of one frequency per request,
# then 64 Poisson-arrival sweeps of SUB_MIX_SWEEP frequencies).
SUB_MIX_SWEEP = 8
SUBS = {
    "slab": ["--workload", "slab", "--solver", "fp64class", "--steps", "1", "--warmup", "1", "--lanes", "1",
             "--serve-requests", "0", "--fp64-steps", "0", "--tune", "off", "--lite"],
    "mix": ["--workload", "mix", "--steps", "64", "--warmup", "4", "--serve-requests", "64",
            "--sweep", str(SUB_MIX_SWEEP), "--lite"],
    "cube4": ["--workload", "cube4", "--steps", "128", "--warmup", "16", "--serve-requests", "0", "--lite"],
    "tip": ["--workload", "tip", "--steps", "256", "--warmup", "16", "--serve-requests", "0", "--lite"],
}
SUB_KEYS = ("value", "unit", "ms_per_step", "steps", "config", "err_est", "factorization", "serving", "stage_ms",
            "fp64_path", "accuracy", "mixed_over_fp64", "clocks", "gpu_launches", "fill_gentries_per_s", "tiles")


def run_subs(names):
    out = {}
    for nm in names:
        cmd = [sys.executable, os.path.abspath(__file__), *SUBS[nm], "--no-cpu-baseline", "--subs", "none"]
        t0 = time.perf_counter()
        r = subprocess.run(cmd, capture_output=True, text=True)
        wall = time.perf_counter() - t0
        lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
        if r.returncode != 0 or not lines:
            out[nm] = {"failed": f"rc={r.returncode}", "stderr_tail": r.stderr[-600:]}
            continue
        d = json.loads(lines[-1])
        sub = {k: d[k] for k in SUB_KEYS if k in d}
        sub["cmd"] = "python bench.py " + " ".join(SUBS[nm])
        sub["wall_s"] = wall
        out[nm] = sub
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    # 32 solves through 4 lanes (8 rounds: the ramp-down of the last round is
    # a small part of the timed region), after 8 warm-up solves
    ap.add_argument("--steps", type=int, default=32)
    ap.add_argument("--warmup", type=int, default=8)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed", "mixed-fp32fill"])
    ap.add_argument("--workload", default="ico3", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--lanes", type=int, default=4, help="farm lanes: solves in flight at once on the GPU")
    ap.add_argument("--batch", type=int, default=1,
                    help="continuous batching: queued requests of equal size a lane solves together")
    ap.add_argument("--serve-requests", type=int, default=64,
                    help="requests of the Poisson-arrival serving measurement (0: skip)")
    ap.add_argument("--solver", default="escalate", choices=["escalate", "c64", "fp64class"],
                    help="mixed-path factorization: complex64 LU escalating to the FP64-class LU when the "
                         "refinement does not converge (default), complex64 only, FP64-class only")
    ap.add_argument("--e2e-steps", type=int, default=0, help="solves of the end-to-end segment (default: --steps)")
    ap.add_argument("--prof-steps", type=int, default=0,
                    help="solves run one at a time for the kernel statistics (default: min(--steps, 4))")
    ap.add_argument("--sweep", type=int, default=0,
                    help="frequencies per serving request of the mix workload (default: the workload's 32)")
    ap.add_argument("--fp64-steps", type=int, default=4,
                    help="timed requests solved again on the plain FP64 path (rate and measured error; 0: skip)")
    ap.add_argument("--subs", default="default",
                    help="comma-separated sub-workloads summarised in the line (cube4, tip, slab, mix), 'none', or "
                         "'default' (all four for the default ico3 workload, none otherwise)")
    ap.add_argument("--tune", default="cache", choices=["cache", "retune", "off"],
                    help="launch shapes from the autotuner's cache (tuned first when missing), re-tuned, or the "
                         "library defaults")
    ap.add_argument("--ex-wide", type=int, default=None, choices=[0, 1, 2],
                    help="exact products' 128 x 128 tiles: 0 never, 1 grids of 4 waves or more (the library's "
                         "default), 2 always")
    ap.add_argument("--panel-ctas", type=int, default=0,
                    help="CTAs of a cooperative LU panel at most (0: one per SM)")
    ap.add_argument("--lite", action="store_true",
                    help="skip the end-to-end and per-kernel segments (sub-workload runs)")
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
    subs = (["cube4", "tip", "slab", "mix"] if args.workload == "ico3" else []) if args.subs == "default" else \
        [x for x in args.subs.split(",") if x and x != "none"]
    if rank == 0 and subs and world == 1:
        out["subs"] = run_subs(subs)
    if rank == 0:
        if not args.no_cpu_baseline and world == 1:
            r = cpu_baseline_run(args.workload, CPU_BASELINE_STEPS)
            out["cpu_baseline"] = {"value": r["value"], "unit": "solves/s", "cores": r["cores"], "kind": "port",
                                   "sample": r["sample"], "spread": r["spread"]}
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
