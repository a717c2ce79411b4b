"""Writes df_constants.h: the double-float Taylor coefficients 1/n! (FP32 hi
part and FP32 remainder) and the FP64 Cody-Waite constants, computed exactly
with sympy.  Run from this directory: python gen_df_constants.py"""
import numpy as np
import sympy as sp

N = 21
H, L = [], []
for n in range(N):
    v = sp.Rational(1, sp.factorial(n))
    h = np.float32(float(v))
    H.append(float(h))
    L.append(float(np.float32(float(v - sp.Rational(float(h))))))


def two(val):
    hi = float(sp.N(val, 50))
    return hi, float(sp.N(val - sp.Rational(hi), 50))


def four(val, bits=(16, 16, 16, 24)):
    """FP32 Cody-Waite parts: the first three carry 16 significant bits, so that
    n * part is exact for integers |n| < 2^8; the fourth carries 24."""
    rem, out = sp.N(val, 80), []
    for b in bits:
        x = float(rem)
        e = int(np.floor(np.log2(abs(x))))
        p = round(x / 2.0 ** (e - b + 1)) * 2.0 ** (e - b + 1)
        assert float(np.float32(p)) == p
        out.append(p)
        rem = rem - sp.Rational(p)
    return out


pio2 = two(sp.pi / 2)
ln2 = two(sp.log(2))
lines = ["// Generated by gen_df_constants.py (exact values from sympy); do not edit.", "#pragma once", "",
         f"#define DF_NFACT {N}",
         "// 1/n! = DF_FACT_HI[n] + DF_FACT_LO[n] (FP32 parts)",
         "static __constant__ const float DF_FACT_HI[DF_NFACT] = {" + ", ".join(f"{x!r}f" for x in H) + "};",
         "static __constant__ const float DF_FACT_LO[DF_NFACT] = {" + ", ".join(f"{x!r}f" for x in L) + "};",
         f"#define DF_PIO2_HI {pio2[0]!r}", f"#define DF_PIO2_LO {pio2[1]!r}",
         f"#define DF_TWO_OVER_PI {float(sp.N(2 / sp.pi, 50))!r}",
         f"#define DF_LN2_HI {ln2[0]!r}", f"#define DF_LN2_LO {ln2[1]!r}",
         f"#define DF_LOG2E {float(sp.N(1 / sp.log(2), 50))!r}",
         "// FP32 Cody-Waite parts of pi/2 and ln 2 (n * part exact for |n| < 2^8 in the first three)"]
for nm, parts in (("DF_PIO2_F", four(sp.pi / 2)), ("DF_LN2_F", four(sp.log(2)))):
    for i, x in enumerate(parts):
        lines.append(f"#define {nm}{i} {x!r}f")
lines += [f"#define DF_TWO_OVER_PI_F {float(np.float32(float(sp.N(2 / sp.pi, 30))))!r}f",
          f"#define DF_LOG2E_F {float(np.float32(float(sp.N(1 / sp.log(2), 30))))!r}f", ""]
open("df_constants.h", "w").write("\n".join(lines))
