#!/usr/bin/env python3
"""Generates the golden fixtures in tests/golden/ from the reference itself.

Runs the reference's own C++ (built from its sources by oracle/Makefile.ref
into oracle/_ref/ref_harness) on seeded synthetic meshes, and stores for each
case: the meshes, the RWG order the reference chose, reference matrices (whole
for the small case, a seeded sample of entries for the larger ones) and the
reference's CalcHeatTransfer output per frequency.

The reference publishes no golden vectors for this path (its examples/output
does not reproduce with its current code), so these fixtures are the pin.

Usage (where the reference checkout is present):
    make -f oracle/Makefile.ref -j8
    python tests/golden/make_golden.py [case names]   # all cases, or only the named ones
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from bem_gb300 import mesh  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
OUT = os.path.dirname(os.path.abspath(__file__))

SIC = (6.7, 0.0983, 0.120, 0.00059)
ALUMINA = (3.1, 0.0787, 0.111, 0.0020)


def run_case(name, v1, t1, v2, t2, gap_vec, freqs, lor1, lor2, a=1e-6, T1=300.0, T2=0.0, full_z=False,
             n_sample=4096, seed=7):
    with tempfile.TemporaryDirectory() as td:
        m1, m2 = os.path.join(td, "m1.txt"), os.path.join(td, "m2.txt")
        mesh.write_mesh_txt(m1, v1, t1)
        mesh.write_mesh_txt(m2, v2, t2)
        order = os.path.join(td, "order.txt")
        zp = os.path.join(td, "z")
        cmd = [HARNESS, "--mesh1", m1, "--mesh2", m2, "--gap", ",".join(repr(float(x)) for x in gap_vec),
               "--a", repr(a), "--T1", repr(T1), "--T2", repr(T2),
               "--lorentz1", ",".join(map(repr, lor1)), "--lorentz2", ",".join(map(repr, lor2)),
               "--freqs", ",".join(repr(float(f)) for f in freqs), "--order", order, "--dumpz", zp]
        r = subprocess.run(cmd, capture_output=True, text=True, check=True)
        P = np.array([[float(x) for x in line.split()[1:]] for line in r.stdout.splitlines() if line.startswith("P ")])
        assert P.shape == (len(freqs), 2) and np.allclose(P[:, 0], freqs)
        o1, o2 = mesh.read_reference_order(order)
        ns, nt = o1.shape[0], o2.shape[0]
        n = 2 * (ns + nt)
        Zext = np.fromfile(zp + "_ext.bin", dtype=np.complex128).reshape(n, n).T
        G1 = np.fromfile(zp + "_int1.bin", dtype=np.complex128).reshape(2 * ns, 2 * ns).T
        G2 = np.fromfile(zp + "_int2.bin", dtype=np.complex128).reshape(2 * nt, 2 * nt).T
    rec = dict(v1=v1, t1=t1, v2=v2, t2=t2, gap=np.asarray(gap_vec, float), order1=o1, order2=o2,
               freqs=np.asarray(freqs, float), P=P[:, 1], lorentz1=np.asarray(lor1), lorentz2=np.asarray(lor2),
               a=a, T1=T1, T2=T2, z_eV=float(freqs[0]))
    if full_z:
        rec.update(Zext=Zext, G1=G1, G2=G2)
    else:
        rng = np.random.default_rng(seed)
        for key, M in (("Zext", Zext), ("G1", G1), ("G2", G2)):
            k = n_sample if key == "Zext" else n_sample // 4
            ii = rng.integers(0, M.shape[0], k)
            jj = rng.integers(0, M.shape[1], k)
            rec[key + "_idx"] = np.stack([ii, jj], 1).astype(np.int32)
            rec[key + "_val"] = M[ii, jj]
            rec[key + "_rowabs"] = np.abs(M).sum(1)
    path = os.path.join(OUT, name + ".npz")
    np.savez_compressed(path, **rec)
    print(f"{name}: n={n} P={P[:, 1]} -> {os.path.relpath(path, ROOT)} ({os.path.getsize(path)} B)")


def main():
    if not os.path.exists(HARNESS):
        sys.exit("build the reference harness first: make -f oracle/Makefile.ref -j8")
    # 1. tiny: two unit cubes, one square per face (12 triangles, 18 RWGs each)
    v, t = mesh.cube(1.0, 1)
    run_case("cube1_gap100nm", v, t, v, t, mesh.gap_translation(v, v, 0.1), [0.1, 0.08, 0.115, 0.13], SIC, SIC,
             full_z=True)
    # 2. the plain-FP64 workload: two 1 um cubes, 4x4 squares per face, gap 100 nm, 20 frequencies
    v, t = mesh.cube(1.0, 4)
    run_case("cube4_gap100nm", v, t, v, t, mesh.gap_translation(v, v, 0.1), np.linspace(0.08, 0.13, 20), SIC, SIC)
    # 3. jittered icospheres at 20 nm: the cross-gap pairs select the 10..36-point far rules
    v, t = mesh.icosphere(1.0, 1, jitter=0.02, seed=12345)
    run_case("ico1_gap20nm", v, t, v, t, mesh.gap_translation(v, v, 0.02), [0.0983, 0.11, 0.12], SIC, SIC)
    # 4. alumina cubes, 2x2 squares per face, gap 50 nm
    v, t = mesh.cube(1.0, 2)
    run_case("cube2_alumina_gap50nm", v, t, v, t, mesh.gap_translation(v, v, 0.05), [0.09, 0.1, 0.12], ALUMINA,
             ALUMINA)
    # 5. jittered icospheres L2 (N = 1920) at 50 nm, below, at and above SiC's surface-phonon resonance
    v, t = mesh.icosphere(1.0, 2, jitter=0.02, seed=12345)
    run_case("ico2_gap50nm", v, t, v, t, mesh.gap_translation(v, v, 0.05), [0.0983, 0.116, 0.125], SIC, SIC)
    # 6. the precision-form workload itself: jittered icospheres L3 (N = 7680) at its smallest gap, 20 nm,
    #    at omega_TO and in the surface-phonon band
    v, t = mesh.icosphere(1.0, 3, jitter=0.02, seed=12345)
    run_case("ico3_gap20nm", v, t, v, t, mesh.gap_translation(v, v, 0.02), [0.0983, 0.116], SIC, SIC)


def main_only(names):
    """Regenerates the named cases only (each case is independent)."""
    saved = globals()["run_case"]

    def pick(name, *a, **k):
        if name in names:
            saved(name, *a, **k)
    globals()["run_case"] = pick
    try:
        main()
    finally:
        globals()["run_case"] = saved


if __name__ == "__main__":
    if len(sys.argv) > 1:
        main_only(set(sys.argv[1:]))
    else:
        main()
