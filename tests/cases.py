"""Shared helpers for the parity tests: rebuild a golden case's two-body
geometry in the reference's RWG order."""
import numpy as np

from bem_gb300 import mesh


def golden_geometry(rec):
    b1 = mesh.Body.from_reference_order(rec["v1"] + rec["gap"], rec["t1"], rec["order1"])
    b2 = mesh.Body.from_reference_order(rec["v2"], rec["t2"], rec["order2"])
    return b1, b2


def row_scaled_err(Z, Zref):
    """max_ij |Z - Zref| / max_j |Zref_ij|: entry errors relative to their row's scale
    (entries that are zero up to rounding in the reference have no relative error)."""
    scale = np.abs(Zref).max(axis=1, keepdims=True)
    scale[scale == 0] = 1.0
    return float((np.abs(np.asarray(Z) - Zref) / scale).max())


def lorentz_eps(rec_lorentz, eV):
    from oracle import oracle
    return oracle.lorentz_eps(eV, *[float(x) for x in rec_lorentz])
