"""X3D shape files, as the reference's ShapeParser reads them
(src/ShapeParser.cpp:83-153, with Transform src/util/Transform.cpp:43-72 and
Rotation src/util/Rotation.cpp:64-78), without Xerces: the standard library's
XML parser walks the same elements.

  * ``Coordinate point="x y z, x y z, ..."``: vertices, each mapped through the
    stack of enclosing Transform elements.  The reference applies the stack
    from the OUTERMOST element inwards (``transform(vector<Transform>, v)``
    loops from index 0, the document root); that order is kept.
  * ``IndexedFaceSet coordIndex="a b c -1, ..."``: faces of 3 vertex ids
    (FaceIndex reads four integers, the fourth the -1 terminator); a face with
    a fourth id is split into (a b c), (a c d).
  * ``Dielectric material="..." key="value"``: the body's material, through
    dielectrics.getDielectric.
  * A Transform is P' = T + C + R (SR (S (-SR (P - C)))), with Rotation.rotate
    as the reference writes it (the matrix of a rotation by -phi about the
    unnormalised axis, src/util/Rotation.cpp:70-77).

The reference then remeshes the shape (ShapeMesh with edge refinement); this
reader returns the file's own triangles, from which mesh.Body.from_mesh builds
the RWG table.
"""
from __future__ import annotations

import math
import xml.etree.ElementTree as ET

import numpy as np

from . import dielectrics, mesh


def _vec(s: str, n: int):
    v = [float(x) for x in s.replace(",", " ").split()]
    if len(v) < n:
        raise ValueError(f"expected {n} numbers in {s!r}")
    return v[:n]


class Rotation:
    def __init__(self, x=0.0, y=0.0, z=1.0, phi=0.0):
        self.x, self.y, self.z, self.phi = x, y, z, phi
        self.s, self.c = math.sin(phi), math.cos(phi)
        self.t = 1.0 - self.c

    def __neg__(self):
        return Rotation(self.x, self.y, self.z, -self.phi)

    def matrix(self) -> np.ndarray:
        x, y, z, s, c, t = self.x, self.y, self.z, self.s, self.c, self.t
        return np.array([[t * x * x + c, t * x * y + s * z, t * x * z - s * y],
                         [t * x * y - s * z, t * y * y + c, t * y * z + s * x],
                         [t * x * z + s * y, t * y * z - s * x, t * z * z + c]])


class Transform:
    def __init__(self, el=None):
        self.C = np.zeros(3)
        self.R = Rotation()
        self.S = np.ones(3)
        self.SR = Rotation()
        self.T = np.zeros(3)
        self.null = True
        if el is None:
            return
        a = el.attrib
        if "center" in a:
            self.C = np.array(_vec(a["center"], 3))
        if "rotation" in a:
            self.R = Rotation(*_vec(a["rotation"], 4))
        if "scale" in a:
            self.S = np.array(_vec(a["scale"], 3))
        if "scaleOrientation" in a:
            self.SR = Rotation(*_vec(a["scaleOrientation"], 4))
        if "translation" in a:
            self.T = np.array(_vec(a["translation"], 3))
        self.null = (not self.C.any() and self.R.phi == 0.0 and (self.S == 1.0).all() and self.SR.phi == 0.0
                     and not self.T.any())

    def apply(self, P: np.ndarray) -> np.ndarray:
        if self.null:
            return P
        r = P - self.C
        r = r @ (-self.SR).matrix().T
        r = r * self.S
        r = r @ self.SR.matrix().T
        r = r @ self.R.matrix().T
        return r + self.C + self.T


class Shape:
    def __init__(self):
        self.coord = []
        self.faces = []
        self.dielectric = None


def _walk(el, stack, shape, table):
    stack = stack + [Transform(el) if el.tag == "Transform" else Transform()]
    if el.tag == "Dielectric":
        params = {k: dielectrics.parse_param(v) for k, v in el.attrib.items() if k != "material"}
        shape.dielectric = dielectrics.getDielectric(el.attrib.get("material", ""), params, table)
    elif el.tag == "IndexedFaceSet" and "coordIndex" in el.attrib:
        for face in el.attrib["coordIndex"].split(","):
            ids = [int(x) for x in face.split()]
            if len(ids) < 4:
                continue  # FaceIndex needs four integers
            a, b, c, d = ids[:4]
            shape.faces.append((a, b, c))
            if d >= 0:
                shape.faces.append((a, c, d))
    elif el.tag == "Coordinate" and "point" in el.attrib:
        pts = []
        for p in el.attrib["point"].split(","):
            v = p.split()
            if len(v) >= 3:
                pts.append([float(v[0]), float(v[1]), float(v[2])])
        P = np.array(pts, dtype=np.float64).reshape(-1, 3)
        for t in stack:  # outermost first, as the reference does
            P = t.apply(P)
        shape.coord.extend(P.tolist())
    for child in el:
        _walk(child, stack, shape, table)


def read_x3d(path: str, table=None) -> Shape:
    """Parses an X3D file into vertices, triangles and the Dielectric (None if
    the file names none).  ``table`` feeds tabulated materials (SiN)."""
    root = ET.parse(path).getroot()
    shape = Shape()
    _walk(root, [], shape, table)
    return shape


def body_from_x3d(path: str, table=None):
    """(mesh.Body, dielectric) of an X3D file."""
    sh = read_x3d(path, table)
    verts = np.array(sh.coord, dtype=np.float64).reshape(-1, 3)
    tris = np.array(sh.faces, dtype=np.int32).reshape(-1, 3)
    if len(tris) == 0 or tris.min() < 0 or tris.max() >= len(verts):
        raise ValueError(f"{path}: coordIndex names vertices outside the Coordinate list")
    return mesh.Body.from_mesh(verts, tris), sh.dielectric
