"""Closed triangle meshes for the two-body heat-transfer problem, and their RWG tables.

Host-side set-up only (runs once per geometry).  The generators produce the
synthetic bodies the workloads are defined on: a structured cube, a jittered
icosphere, a structured slab, a cone tip with a hemispherical apex, and a plate.

The RWG builder follows the edge-creation rule of the reference's mesh builder
(``ShapeMesh::ShapeMesh``, src/ShapeMesh.cpp:857-928): triangles are visited in
order; each of a triangle's edges 12, 23, 31 that has an unvisited neighbour
becomes one RWG whose positive triangle (``t1``) is the current triangle and
whose negative triangle (``t2``) is the neighbour (src/RWG.cpp:5).  The
reference then permutes RWGs by a recursive segment partition
(src/RWGTree.cpp:602-761); that partition is not rebuilt here, so an RWG order
taken from the reference is passed in explicitly where entry-by-entry parity
with the reference's matrices is wanted (see ``Body.from_reference_order``).
"""
from __future__ import annotations

import dataclasses
import numpy as np


@dataclasses.dataclass
class Body:
    """One closed surface: vertices, triangles (vertex order kept as given),
    and the RWG table in the order the impedance matrix uses.

    ``rwg[i] = (pos_triangle, neg_triangle, edge_v1, edge_v2)``.
    """
    verts: np.ndarray          # (nv, 3) float64
    tris: np.ndarray           # (nt, 3) int32
    rwg: np.ndarray            # (nrwg, 4) int32

    @property
    def nv(self) -> int:
        return int(self.verts.shape[0])

    @property
    def nt(self) -> int:
        return int(self.tris.shape[0])

    @property
    def nrwg(self) -> int:
        return int(self.rwg.shape[0])

    def translated(self, d) -> "Body":
        return Body(self.verts + np.asarray(d, dtype=np.float64)[None, :], self.tris.copy(), self.rwg.copy())

    def max_edge(self) -> float:
        v = self.verts
        t = self.tris
        e = np.concatenate([v[t[:, 1]] - v[t[:, 0]], v[t[:, 2]] - v[t[:, 1]], v[t[:, 0]] - v[t[:, 2]]])
        return float(np.sqrt((e * e).sum(1)).max())

    @staticmethod
    def from_mesh(verts, tris, native: bool = False) -> "Body":
        """``native``: build the RWG table in the C++ library
        (``bemgpu_mesh_rwgs``, same rows) instead of in Python."""
        verts = np.ascontiguousarray(verts, dtype=np.float64)
        tris = np.ascontiguousarray(tris, dtype=np.int32)
        rwg = build_rwgs_native(tris, verts.shape[0]) if native else build_rwgs(tris)
        return Body(verts, tris, rwg)

    @staticmethod
    def from_reference_order(verts, tris, order) -> "Body":
        """``order`` rows are (edge p1, edge p2, pos tri, neg tri) as exported
        by the reference harness for this body."""
        order = np.asarray(order, dtype=np.int64)
        rwg = np.stack([order[:, 2], order[:, 3], order[:, 0], order[:, 1]], axis=1).astype(np.int32)
        return Body(np.ascontiguousarray(verts, np.float64), np.ascontiguousarray(tris, np.int32), rwg)


def build_rwgs(tris: np.ndarray) -> np.ndarray:
    """Edge extraction with the reference's first-visit rule (see module doc)."""
    tris = np.asarray(tris)
    edge_tris: dict[tuple[int, int], list[int]] = {}
    for ti, (a, b, c) in enumerate(tris.tolist()):
        for u, v in ((a, b), (b, c), (c, a)):
            edge_tris.setdefault((min(u, v), max(u, v)), []).append(ti)
    for k, ts in edge_tris.items():
        if len(ts) != 2:
            raise ValueError(f"mesh is not a closed 2-manifold: edge {k} has {len(ts)} triangles")
    touched = np.zeros(len(tris), dtype=bool)
    out = []
    for ti, (a, b, c) in enumerate(tris.tolist()):
        for u, v in ((a, b), (b, c), (c, a)):
            t1, t2 = edge_tris[(min(u, v), max(u, v))]
            nb = t2 if t1 == ti else t1
            if not touched[nb]:
                out.append((ti, nb, u, v))
        touched[ti] = True
    return np.asarray(out, dtype=np.int32)


def build_rwgs_native(tris: np.ndarray, nv: int) -> np.ndarray:
    """The same table as ``build_rwgs`` from libbemgpu's host-side builder
    (``bemgpu_mesh_rwgs``: a sort of the directed edges, no Python loop)."""
    import ctypes
    from . import _lib
    tris = np.ascontiguousarray(tris, dtype=np.int32)
    nt = tris.shape[0]
    cap = (3 * nt) // 2
    out = np.zeros((max(cap, 1), 4), dtype=np.int32)
    n = ctypes.c_int()
    rc = _lib.load().bemgpu_mesh_rwgs(tris.ctypes.data, nt, int(nv), out.ctypes.data, cap, ctypes.byref(n))
    if rc == _lib.ERR_MESH:
        raise ValueError("mesh is not a closed 2-manifold (an edge without exactly two triangles)")
    if rc != 0:
        raise _lib.BemGpuError(rc, f"bemgpu_mesh_rwgs: {n.value} RWGs for {nt} triangles")
    return out[:n.value].copy()


def _dedup(verts: np.ndarray, tris: np.ndarray, decimals: int = 12):
    key = np.round(verts, decimals)
    _, first, inv = np.unique(key, axis=0, return_index=True, return_inverse=True)
    # keep first-appearance order so that meshes are stable
    order = np.argsort(first)
    remap = np.empty_like(order)
    remap[order] = np.arange(len(order))
    new_verts = verts[first[order]]
    new_tris = remap[inv.reshape(-1)[tris]]
    return new_verts, new_tris


def box(lx: float, ly: float, lz: float, nx: int, ny: int, nz: int, center=(0.0, 0.0, 0.0)):
    """Axis-aligned box, each face a structured grid of squares split into two
    triangles, outward-oriented.  Returns (verts, tris)."""
    cx, cy, cz = center
    hx, hy, hz = lx / 2, ly / 2, lz / 2
    verts = []
    tris = []

    def face(origin, du, dv, nu, nv):
        base = len(verts)
        for j in range(nv + 1):
            for i in range(nu + 1):
                verts.append(origin + du * (i / nu) + dv * (j / nv))
        for j in range(nv):
            for i in range(nu):
                a = base + j * (nu + 1) + i
                b = a + 1
                c = a + (nu + 1)
                d = c + 1
                tris.append((a, b, d))
                tris.append((a, d, c))

    o = np.array([cx - hx, cy - hy, cz - hz])
    X = np.array([lx, 0, 0.0]); Y = np.array([0, ly, 0.0]); Z = np.array([0, 0, lz])
    # (du x dv) points outward on each face
    face(o, Y, X, ny, nx)                 # z = -hz, normal -z
    face(o + Z, X, Y, nx, ny)             # z = +hz
    face(o, X, Z, nx, nz)                 # y = -hy, normal -y
    face(o + Y, Z, X, nz, nx)             # y = +hy
    face(o, Z, Y, nz, ny)                 # x = -hx, normal -x
    face(o + X, Y, Z, ny, nz)             # x = +hx
    v, t = _dedup(np.asarray(verts, dtype=np.float64), np.asarray(tris, dtype=np.int64))
    return v, t.astype(np.int32)


def cube(side: float = 1.0, nsub: int = 4):
    """Cube of the given side centred at the origin, nsub x nsub squares per face."""
    return box(side, side, side, nsub, nsub, nsub)


def icosphere(radius: float = 1.0, level: int = 3, jitter: float = 0.0, seed: int = 12345):
    """Subdivided icosahedron projected to the sphere (20 * 4**level triangles).
    ``jitter`` is the uniform per-coordinate displacement bound as a fraction of
    the mean edge length, drawn from ``numpy.random.default_rng(seed)``."""
    p = (1 + 5 ** 0.5) / 2
    v = [(-1, p, 0), (1, p, 0), (-1, -p, 0), (1, -p, 0), (0, -1, p), (0, 1, p), (0, -1, -p), (0, 1, -p),
         (p, 0, -1), (p, 0, 1), (-p, 0, -1), (-p, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5),
         (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = [np.array(x, dtype=np.float64) / np.linalg.norm(x) for x in v]
    faces = list(f)
    for _ in range(level):
        mid = {}

        def midpoint(a, b):
            k = (min(a, b), max(a, b))
            if k not in mid:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                mid[k] = len(verts) - 1
            return mid[k]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    V = np.asarray(verts) * radius
    T = np.asarray(faces, dtype=np.int32)
    if jitter > 0:
        e = np.concatenate([V[T[:, 1]] - V[T[:, 0]], V[T[:, 2]] - V[T[:, 1]], V[T[:, 0]] - V[T[:, 2]]])
        lmean = float(np.sqrt((e * e).sum(1)).mean())
        rng = np.random.default_rng(seed)
        V = V + rng.uniform(-1.0, 1.0, size=V.shape) * jitter * lmean
    return V, T


def cone_tip(base_radius: float = 0.5, height: float = 1.0, apex_radius: float = 0.1,
             n_around: int = 24, n_side: int = 8, n_cap: int = 4, n_base: int = 4):
    """Closed cone standing on the z=0 plane pointing down to a hemispherical
    apex whose lowest point is at z = 0 (the body extends upward to z=height).
    Triangle counts grow with n_around * (n_side + n_cap + n_base)."""
    # profile: from the apex bottom point up along the cap, then along the
    # cone side to the base rim, then across the flat base to the axis.
    ra = apex_radius
    rb = base_radius
    # cone half-angle
    alpha = np.arctan2(rb, height)
    # tangent point of the sphere of radius ra centred on the axis at z=zc
    zc = ra / np.sin(alpha) if alpha > 0 else ra
    # choose zc so that the lowest sphere point is z=0
    zc = ra
    # tangency: the side line through the rim (rb, height) tangent to the sphere
    # (solve for the tangent point angle numerically)
    def tangent_gap(th):
        # point on sphere at polar angle th from -z axis
        px, pz = ra * np.sin(th), zc - ra * np.cos(th)
        # tangent direction
        tx, tz = np.cos(th), np.sin(th)
        # rim point must lie on the tangent line: cross((rim - p), t) = 0
        return (rb - px) * tz - (height - pz) * tx
    lo, hi = 1e-6, np.pi / 2 - 1e-6
    for _ in range(200):
        mid_ = 0.5 * (lo + hi)
        if tangent_gap(lo) * tangent_gap(mid_) <= 0:
            hi = mid_
        else:
            lo = mid_
    th_t = 0.5 * (lo + hi)
    prof = []  # (r, z) from bottom point to the base centre, excluding the two axis points
    for k in range(1, n_cap + 1):
        th = th_t * k / n_cap
        prof.append((ra * np.sin(th), zc - ra * np.cos(th)))
    r0, z0 = prof[-1]
    for k in range(1, n_side + 1):
        s = k / n_side
        prof.append((r0 + (rb - r0) * s, z0 + (height - z0) * s))
    for k in range(1, n_base):
        s = k / n_base
        prof.append((rb * (1 - s), height))
    verts = [(0.0, 0.0, 0.0)]
    for r, z in prof:
        for j in range(n_around):
            ph = 2 * np.pi * j / n_around
            verts.append((r * np.cos(ph), r * np.sin(ph), z))
    verts.append((0.0, 0.0, height))
    nring = len(prof)
    tris = []
    ring = lambda k, j: 1 + k * n_around + (j % n_around)
    top = len(verts) - 1
    for j in range(n_around):
        tris.append((0, ring(0, j + 1), ring(0, j)))
    for k in range(nring - 1):
        for j in range(n_around):
            a, b = ring(k, j), ring(k, j + 1)
            c, d = ring(k + 1, j), ring(k + 1, j + 1)
            tris.append((a, b, d))
            tris.append((a, d, c))
    for j in range(n_around):
        tris.append((top, ring(nring - 1, j), ring(nring - 1, j + 1)))
    return np.asarray(verts, dtype=np.float64), np.asarray(tris, dtype=np.int32)


def write_mesh_txt(path: str, verts: np.ndarray, tris: np.ndarray) -> None:
    """Plain-text mesh: 'nv nt', then vertices, then triangles (vertex ids)."""
    with open(path, "w") as f:
        f.write(f"{len(verts)} {len(tris)}\n")
        for x, y, z in verts:
            f.write(f"{float(x)!r} {float(y)!r} {float(z)!r}\n")
        for a, b, c in tris:
            f.write(f"{a} {b} {c}\n")


def gap_translation(body1_verts: np.ndarray, body2_verts: np.ndarray, gap: float) -> np.ndarray:
    """Translation along +x for body 1 that leaves a surface-to-surface gap of
    ``gap`` between body 2's largest x and body 1's smallest x."""
    dx = float(body2_verts[:, 0].max() - body1_verts[:, 0].min()) + gap
    return np.array([dx, 0.0, 0.0])


def two_body(body1: Body, body2: Body):
    """Concatenates two bodies into one geometry index space (body 1 first), as
    the two-body RWG tree orders its unknowns (src/RWGTree.cpp:748-761).
    Returns (xyz, tris, rwg_top, n_s)."""
    xyz = np.concatenate([body1.verts, body2.verts]).astype(np.float64)
    tris = np.concatenate([body1.tris, body2.tris + body1.nv]).astype(np.int32)
    r2 = body2.rwg.copy()
    r2[:, 0:2] += body1.nt
    r2[:, 2:4] += body1.nv
    rwg = np.concatenate([body1.rwg, r2]).astype(np.int32)
    return np.ascontiguousarray(xyz), np.ascontiguousarray(tris), np.ascontiguousarray(rwg), body1.nrwg


def read_reference_order(path: str):
    """Reads the RWG order written by the reference harness; returns the
    (edge p1, edge p2, pos tri, neg tri) rows of body 1 and of body 2."""
    with open(path) as f:
        ntop, ns, nt = (int(x) for x in f.readline().split())
        rows = np.loadtxt(f, dtype=np.int64).reshape(-1, 5)
    assert rows.shape[0] == ntop == ns + nt
    b = rows[:, 0]
    assert (b[:ns] == 0).all() and (b[ns:] == 1).all()
    return rows[:ns, 1:], rows[ns:, 1:]
