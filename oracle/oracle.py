"""ORACLE — test infrastructure only (tests/, __graft_entry__.smoke(), bench.py's
CPU-baseline leg).  The product never imports this module.

Python side of the oracle: builds and binds oracle/bem_oracle.c (the fill
restatement) and restates the per-frequency driver CalcHeatTransfer
(src/HeatTransfer.cpp:8-59) with numpy's LAPACK for the dense algebra, as the
reference does with system LAPACK (zgetrf + zgetri, src/util/DenseMatrix.cpp:65-77).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

# src/util/SI.cpp:3-9
HBAR = 1.05457148e-34
KB = 1.3806503e-23
EV = 1.60217646e-19
C0 = 2.99792458e8

# Options::Options far-rule thresholds, src/Options.cpp:23-26
FAR_THRESH = (12.0, 8.0, 4.0, 2.0)


def build(force: bool = False) -> str:
    """Compiles bem_oracle.c into liboracle.so (plain gcc, no CUDA)."""
    src = os.path.join(HERE, "bem_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        tmp = LIB_PATH + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", "-O3", "-std=gnu11", "-fPIC", "-shared", src, "-o", tmp, "-lm", "-lpthread"])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        L.oracle_zts.restype = ctypes.c_int
        L.oracle_zts.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                 ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                 ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                 ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        L.oracle_green.restype = None
        L.oracle_green.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        _lib = L
    return _lib


def lorentz_eps(feV: float, epsinf: float, wTO_eV: float, wLO_eV: float, gamma_eV: float) -> complex:
    """SiC::eps's functional form with fixed parameters (src/util/SiC.cpp:16-19)."""
    wT = wTO_eV * EV / HBAR
    wL = wLO_eV * EV / HBAR
    gamma = gamma_eV * EV / HBAR
    w = feV * EV / HBAR
    return epsinf * (wL * wL - w * w - 1j * gamma * w) / (wT * wT - w * w - 1j * gamma * w)


def theta(omega: float, T: float) -> float:
    """Theta, src/HeatTransfer.cpp:3-6 (called with the dimensionless omega)."""
    with np.errstate(divide="ignore", over="ignore"):
        x = np.float64(HBAR * omega) / (np.float64(KB) * np.float64(T))
        return float(HBAR * omega / (np.exp(x) - 1))


def dimensionless_omega(a: float, eV: float) -> float:
    """src/HeatTransfer.cpp:10-11."""
    omegaSI = eV * EV / HBAR
    return omegaSI * a / C0


def green_constants(eps: complex, mu: complex, omega: complex) -> dict:
    out = np.zeros(12)
    emo = np.array([eps.real, eps.imag, mu.real, mu.imag, omega.real, omega.imag], dtype=np.float64)
    lib().oracle_green(emo.ctypes.data, out.ctypes.data)
    names = ["ksquared", "k", "ik", "k2", "Zeps", "Zmu"]
    return {n: complex(out[2 * i], out[2 * i + 1]) for i, n in enumerate(names)}


def zts(xyz, tris, rwg_t, rwg_s, eps: complex, mu: complex, omega: complex, far=FAR_THRESH,
        tri_range=(0, -1), nthreads: int | None = None, counts: bool = False, timing_only: bool = False):
    """Zts(t, s, g) (src/Impedance.cpp:388-413) on one shared geometry.
    Returns the (2*Nt x 2*Ns) complex128 matrix in column-major (Fortran) order.
    timing_only: integrate the same pairs without an output matrix (a CPU
    timing sample of a fill too large to hold per process); returns None."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    tris = np.ascontiguousarray(tris, dtype=np.int32)
    rwg_t = np.ascontiguousarray(rwg_t, dtype=np.int32)
    rwg_s = np.ascontiguousarray(rwg_s, dtype=np.int32)
    nt_rwg, ns_rwg = rwg_t.shape[0], rwg_s.shape[0]
    Z = None if timing_only else np.zeros((2 * nt_rwg, 2 * ns_rwg), dtype=np.complex128, order="F")
    emo = np.array([eps.real, eps.imag, mu.real, mu.imag, complex(omega).real, complex(omega).imag])
    far = np.asarray(far, dtype=np.float64)
    cnt = np.zeros(7, dtype=np.int64)
    if nthreads is None:
        nthreads = os.cpu_count() or 1
    rc = lib().oracle_zts(xyz.ctypes.data, xyz.shape[0], tris.ctypes.data, tris.shape[0],
                          rwg_t.ctypes.data, nt_rwg, rwg_s.ctypes.data, ns_rwg, emo.ctypes.data,
                          far.ctypes.data, None if Z is None else Z.ctypes.data, 2 * nt_rwg,
                          int(tri_range[0]), int(tri_range[1]),
                          int(nthreads), cnt.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"oracle_zts failed: {rc}")
    if counts:
        return Z, dict(zip(["same", "neighbour", "g6", "g10", "g15", "g21", "g36"], cnt.tolist()))
    return Z


def symm(A: np.ndarray) -> np.ndarray:
    """symm, src/util/DenseMatrix.cpp:477-486: A + A^H (diagonal 2 Re)."""
    return A + A.conj().T


def calc_heat_transfer(a: float, eV: float, T1: float, T2: float, xyz, tris, rwg_top, n_s: int,
                       eps1: complex, eps2: complex, mu1: complex = 1.0 + 0j, mu2: complex = 1.0 + 0j,
                       nthreads: int | None = None, return_parts: bool = False):
    """CalcHeatTransfer, src/HeatTransfer.cpp:8-59.

    ``rwg_top`` is the two-body RWG table in matrix order (body 1's ``n_s``
    RWGs first); eps1/eps2 are the bodies' permittivities at ``eV`` (the
    reference evaluates Dielectric::eps at this point, :17-20)."""
    omega = dimensionless_omega(a, eV)
    rwg_top = np.asarray(rwg_top, dtype=np.int32)
    rwg_s = rwg_top[:n_s]
    rwg_t = rwg_top[n_s:]
    W = zts(xyz, tris, rwg_top, rwg_top, 1.0 + 0j, 1.0 + 0j, omega, nthreads=nthreads)
    G1 = zts(xyz, tris, rwg_s, rwg_s, complex(eps1), complex(mu1), omega, nthreads=nthreads)
    G2 = zts(xyz, tris, rwg_t, rwg_t, complex(eps2), complex(mu2), omega, nthreads=nthreads)
    ns2, nt2 = 2 * n_s, 2 * rwg_t.shape[0]
    W[:ns2, :ns2] += G1
    W[ns2:, ns2:] += G2
    Winv = np.linalg.inv(W)                       # inverse(*W), :36
    W1 = Winv[:ns2, :]                            # :37
    B1 = (symm(G1) @ W1)[:, ns2:]                 # :39-41
    W2 = Winv[:, ns2:]                            # :44
    B2 = (W2 @ symm(G2))[:ns2, :]                 # :45-47
    S = 0.25 * np.trace(B2.conj().T @ B1)         # :50-52
    P = S.real * (theta(omega, T1) - theta(omega, T2))
    if return_parts:
        return P, dict(S=S, W=W, G1=G1, G2=G2, omega=omega)
    return P
