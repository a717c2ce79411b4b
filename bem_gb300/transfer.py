"""Job front ends of the reference, on the request farm.

``transfer`` (src/transfer.cpp:3-29): one solve from two X3D bodies,
    python -m bem_gb300.transfer single body1.x3d body2.x3d eV a T1 T2 gx gy gz

``transfer-mpi`` (src/transfer-mpi.cpp:91-241): the (T pair x a x gap x f) job
grid read from a.txt, gaps.txt, freqs.txt, temps.txt (pushFileLines,
src/FileUtils.h:8-20: whitespace-separated values, 1, 3 and 2 per entry),
bodies from body1.x3d / body2.x3d, results appended to ./output as each job
finishes, one line per job in the reference's own column layout,
    python -m bem_gb300.transfer sweep [--dir D] [--lanes L] [--precision mixed]
The MPI master/servant farm becomes a bem_gb300.api.Farm of L lanes on one GPU.

Output line: "%.15g %.15g %.15g %.15g %.15g %.14g" of (a, gap.x, gap.y, gap.z,
eV, P).  That is what the reference writes: its format names the columns
(a, feV, gap, T1, T2, S) but fills them from the job buffer (a, gap.x, gap.y,
gap.z, feV) and the result (src/transfer-mpi.cpp:163-171).  Temperatures are
not in the line.  An existing output file is resumed: jobs whose line is
already there (counted per (a, gap, eV) key, in job order) are skipped, the
checkpoint the reference's flushed output file allows but never uses.
"""
from __future__ import annotations

import argparse
import collections
import os
import sys

from . import _lib, api, dielectrics, x3d

FMT = "%.15g %.15g %.15g %.15g %.15g %.14g\n"


def push_file_values(path: str, arity: int) -> list:
    """Whitespace-separated numbers of a file, grouped by ``arity``; reading
    stops at the first token that is not a number (the reference's stream
    loop would stall there)."""
    out, cur = [], []
    with open(path) as fh:
        for tok in fh.read().split():
            try:
                cur.append(float(tok))
            except ValueError:
                break
            if len(cur) == arity:
                out.append(cur[0] if arity == 1 else tuple(cur))
                cur = []
    return out


def job_grid(as_, gaps, freqs, temps):
    """The Master's job order (src/transfer-mpi.cpp:115-131): T pairs, then a,
    then gaps, then frequencies."""
    return [(a, g, f, T) for T in temps for a in as_ for g in gaps for f in freqs]


def _key(a, g, f):
    """The job's first five output columns as they read back from the file."""
    return tuple(float("%.15g" % v) for v in (a, g[0], g[1], g[2], f))


def run_sweep(body1, body2, diel1, diel2, as_, gaps, freqs, temps, out_path="output", lanes=3,
              precision=_lib.PREC_MIXED_LA, ctx=None, options=None, log=None) -> int:
    """Solves every job of the grid not yet in ``out_path`` on a farm and
    appends one line per job.  Returns the number of jobs solved."""
    jobs = job_grid(as_, gaps, freqs, temps)
    done = collections.Counter()
    if os.path.exists(out_path):
        with open(out_path) as fh:
            for line in fh:
                v = line.split()
                if len(v) == 6:
                    done[tuple(float(x) for x in v[:5])] += 1
    todo = []
    for j in jobs:
        k = _key(j[0], j[1], j[2])
        if done[k] > 0:
            done[k] -= 1
        else:
            todo.append(j)
    ctx = ctx or api.Context(0)
    systems = {}
    n = 0
    with api.Farm(lanes, ctx.device) as farm, open(out_path, "a") as out:
        pending = []
        for (a, g, f, (T1, T2)) in todo:
            if g not in systems:
                systems[g] = api.parseShapes(body1.translated(g), body2, diel1, diel2, ctx)
            tk = farm.submit(a, f, T1, T2, *systems[g], options=options, precision=precision)
            pending.append((tk, a, g, f))
        for tk, a, g, f in pending:
            info = {}
            P = farm.result(tk, info=info, strict=False)
            out.write(FMT % (a, g[0], g[1], g[2], f, P))
            out.flush()
            n += 1
            if log:
                log(f"a={a:g} gap=({g[0]:g},{g[1]:g},{g[2]:g}) eV={f:g} P={P:.14g} err_est={info.get('err_est', 0):.1e}")
    return n


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m bem_gb300.transfer")
    sub = ap.add_subparsers(dest="cmd", required=True)
    s1 = sub.add_parser("single", help="one solve (transfer)")
    s1.add_argument("body1")
    s1.add_argument("body2")
    for k in ("eV", "a", "T1", "T2", "gx", "gy", "gz"):
        s1.add_argument(k, type=float)
    s1.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    s2 = sub.add_parser("sweep", help="the job grid of a.txt gaps.txt freqs.txt temps.txt (transfer-mpi)")
    s2.add_argument("--dir", default=".")
    s2.add_argument("--lanes", type=int, default=3)
    s2.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    for p in (s1, s2):
        p.add_argument("--table", help="eV n k columns for a tabulated material (SiN)")
        p.add_argument("--material", help="material of a body whose file has no Dielectric element")
    args = ap.parse_args(argv)
    table = None
    if args.table:
        cols = list(zip(*[tuple(map(float, ln.split()[:3])) for ln in open(args.table) if len(ln.split()) >= 3]))
        table = (cols[0], cols[1], cols[2])

    def body(path):
        b, d = x3d.body_from_x3d(path, table)
        if d is None:
            if not args.material:
                raise SystemExit(f"{path} has no Dielectric element; pass --material")
            d = dielectrics.getDielectric(args.material, None, table)
        return b, d
    prec = {"fp64": _lib.PREC_FP64, "mixed": _lib.PREC_MIXED_LA}[args.precision]
    if args.cmd == "single":
        b1, d1 = body(args.body1)
        b2, d2 = body(args.body2)
        top, s, t = api.parseShapes(b1.translated((args.gx, args.gy, args.gz)), b2, d1, d2)
        P = api.CalcHeatTransfer(args.a, args.eV, args.T1, args.T2, top, s, t, precision=prec)
        print(f"{P:.14g}")
        return 0
    d = args.dir
    b1, d1 = body(os.path.join(d, "body1.x3d"))
    b2, d2 = body(os.path.join(d, "body2.x3d"))
    n = run_sweep(b1, b2, d1, d2, push_file_values(os.path.join(d, "a.txt"), 1),
                  push_file_values(os.path.join(d, "gaps.txt"), 3), push_file_values(os.path.join(d, "freqs.txt"), 1),
                  push_file_values(os.path.join(d, "temps.txt"), 2), os.path.join(d, "output"), args.lanes, prec,
                  log=lambda m: sys.stderr.write(m + "\n"))
    print(f"{n} jobs solved")
    return 0


if __name__ == "__main__":
    sys.exit(main())
