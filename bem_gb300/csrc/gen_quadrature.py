#!/usr/bin/env python3
"""Regenerates quadrature_tables.h from the reference's rule tables.

The impedance fill must integrate with exactly the nodes and weights the
reference uses (src/TriangleQuadrature.h: Gauss6 :31-43, Gauss10 :45-65,
Gauss15 :67-92, Gauss21 :94-121, Gauss36 :162-204, Gauss91 :330-427,
Gauss105 :429-540, line rule QuadratureGauss15 :620-655), otherwise matrix
entries differ from the reference's at the 1e-7 level instead of 1e-15.
This script reads the numbers out of that header and writes them as plain
(xi1, xi2, weight) arrays; it is run by hand where the reference checkout is
present and its output is committed.

Usage: python bem_gb300/csrc/gen_quadrature.py [path/to/TriangleQuadrature.h]
(default: $BEM_REFERENCE_SRC/TriangleQuadrature.h, BEM_REFERENCE_SRC defaulting
to /root/reference/src)
"""
import re
import sys

TRI_RULES = [6, 10, 15, 21, 36, 91, 105]
NUM = r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?"


def parse(text):
    rules = {}
    for n in TRI_RULES:
        m = re.search(r"class TriangleQuadratureGauss%d\b.*?\n\};" % n, text, re.S)
        body = m.group(0)
        pts = []
        for line in body.splitlines():
            line = line.strip()
            if not line.startswith("v = v0"):
                continue
            expr, w = re.match(r"v = (v0[^;]*); integrand\.weighPoint\((%s),v\);" % NUM, line).groups()
            a = b = 0.0
            for coef, var in re.findall(r"\+\s*(?:(%s)\s*\*\s*)?(v[12])" % NUM, expr):
                c = float(coef) if coef else 1.0
                if var == "v1":
                    a = c
                else:
                    b = c
            pts.append((a, b, float(w), line))
        assert len(pts) == n, (n, len(pts))
        rules[n] = pts
    m = re.search(r"class QuadratureGauss15\b.*?\n\};", text, re.S)
    body = m.group(0)
    xs = [float(x) for x in re.findall(r"v = v0 \+\s*(%s) \* v1;" % NUM, body)]
    ws = [float(x) for x in re.findall(r"weighPoint\(\s*(%s),v\);" % NUM, body)]
    assert len(xs) == 15 and len(ws) == 15
    return rules, list(zip(xs, ws))


def emit(rules, line15):
    out = []
    out.append("// Generated by gen_quadrature.py from the reference's src/TriangleQuadrature.h.")
    out.append("// Node r = p0 + xi1*(p1-p0) + xi2*(p2-p0); weights sum to 1 (the rules")
    out.append("// integrate the mean over the triangle).  Do not edit by hand.")
    out.append("#pragma once")
    out.append("")
    for n, pts in rules.items():
        out.append("#define BEMGPU_TRI_RULE%d_N %d" % (n, n))
        out.append("static const double bemgpu_tri_rule%d[%d][3] = {" % (n, n))
        for a, b, w, _ in pts:
            out.append("  {%r, %r, %r}," % (a, b, w))
        out.append("};")
        out.append("")
    out.append("#define BEMGPU_LINE_RULE15_N 15")
    out.append("static const double bemgpu_line_rule15[15][2] = {")
    for x, w in line15:
        out.append("  {%r, %r}," % (x, w))
    out.append("};")
    return "\n".join(out) + "\n"


if __name__ == "__main__":
    import os
    src = sys.argv[1] if len(sys.argv) > 1 else os.path.join(
        os.environ.get("BEM_REFERENCE_SRC", "/root/reference/src"), "TriangleQuadrature.h")
    rules, line15 = parse(open(src).read())
    dst = __file__.replace("gen_quadrature.py", "quadrature_tables.h")
    open(dst, "w").write(emit(rules, line15))
    for n, pts in rules.items():
        print(n, "sum w = %.15f" % sum(p[2] for p in pts))
