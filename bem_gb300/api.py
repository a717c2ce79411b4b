"""Host-side mirror of the reference's per-frequency interface, over the C ABI.

Same names, argument meaning and error behaviour as the reference's surface
(claytonotey/bem):

  GreensFunction(eps, mu, omega, bExternal)   src/GreensFunction.h:7-28, .cpp:17-30
  Options()                                   src/Options.h, src/Options.cpp:3-27
  Zts(t, s, g, options)                       src/Impedance.h:21
  CalcHeatTransfer(a, eV, T1, T2, top, s, t, options)   src/HeatTransfer.h:33
  Theta(omega, T)                             src/HeatTransfer.cpp:3-6
  FrequencySweep(file).f                      src/FrequencySweep.h:8-12
  parseShapes(...) -> (top, s, t)             src/HeatTransfer.cpp:61-109 (with the
                                              trees kept alive, which the reference's
                                              by-value out-parameters do not do)
  Farm(lanes).submit / result / cancel        the MPI task farm, src/transfer-mpi.cpp:25-190
                                              (several solves in flight on one GPU)

Materials beyond FixedLorentz / SiC live in bem_gb300.dielectrics, the X3D
reader in bem_gb300.x3d, the transfer / transfer-mpi front ends in
bem_gb300.transfer.

All compute runs in libbemgpu.so on the GPU; there is no CPU path.
"""
from __future__ import annotations

import ctypes
import math
import threading

import numpy as np

from . import _lib
from .mesh import Body, two_body

HBAR = 1.05457148e-34   # src/util/SI.cpp:3-9
KB = 1.3806503e-23
EV = 1.60217646e-19
C0 = 2.99792458e8


def _check(rc: int, ctx=None):
    if rc != _lib.OK:
        msg = _lib.load().bemgpu_ctx_last_error(ctx.handle if ctx else None).decode()
        raise _lib.BemGpuError(rc, msg)


class Context:
    """One CUDA device, its stream and workspace (bemgpu_ctx_t)."""

    def __init__(self, device: int = 0):
        L = _lib.load()
        h = ctypes.c_void_p()
        rc = L.bemgpu_ctx_create(int(device), ctypes.byref(h))
        if rc != _lib.OK:
            raise _lib.BemGpuError(rc, f"cannot create a context on CUDA device {device}")
        self.handle = h
        self.device = device

    def set_solver(self, mode: int):
        """Mixed-path factorization: 0 complex64 LU escalating to the FP64-class
        tensor-core LU when refinement does not converge, 1 complex64 only, 2
        FP64-class only."""
        _check(_lib.load().bemgpu_ctx_set_solver(self.handle, int(mode)), self)

    def close(self):
        if self.handle:
            _lib.load().bemgpu_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = None
_ctx_lock = threading.Lock()


def default_context() -> Context:
    global _default_ctx
    with _ctx_lock:
        if _default_ctx is None:
            _default_ctx = Context(0)
        return _default_ctx


class Options:
    """Options fields on the fill path (src/Options.cpp:23-26 defaults)."""

    def __init__(self):
        self.farThresh6 = 12.0
        self.farThresh10 = 8.0
        self.farThresh15 = 4.0
        self.farThresh21 = 2.0
        self.minSegmentSize = 32

    def _c(self) -> _lib.Options:
        return _lib.Options(self.farThresh6, self.farThresh10, self.farThresh15, self.farThresh21)


class GreensFunction:
    """GreensFunction(eps, mu, omega, bExternal); init() recomputes the constants."""

    def __init__(self, eps=1.0, mu=1.0, omega=0.0, bExternal: bool = False):
        self.bExternal = bool(bExternal)
        self.init(eps, mu, omega)

    def init(self, eps, mu, omega):
        g = _lib.Green()
        e = (ctypes.c_double * 2)(complex(eps).real, complex(eps).imag)
        m = (ctypes.c_double * 2)(complex(mu).real, complex(mu).imag)
        w = (ctypes.c_double * 2)(complex(omega).real, complex(omega).imag)
        _check(_lib.load().bemgpu_green_init(e, m, w, int(self.bExternal), ctypes.byref(g)))
        self._g = g
        c = lambda a: complex(a[0], a[1])
        self.eps, self.mu, self.omega = c(g.eps), c(g.mu), c(g.omega)
        self.ksquared, self.k, self.ik, self.k2 = c(g.ksquared), c(g.k), c(g.ik), c(g.k2)
        self.Zeps, self.Zmu = c(g.Zeps), c(g.Zmu)
        self.normk = abs(self.k)

    def isExternal(self) -> bool:
        return self.bExternal


class FixedLorentz:
    """Single Lorentz oscillator with SiC::eps's form (src/util/SiC.cpp:16-19),
    parameters in eV and independent of temperature."""

    def __init__(self, epsinf: float, wTO_eV: float, wLO_eV: float, gamma_eV: float):
        self.epsinf = epsinf
        self.wT = wTO_eV * EV / HBAR
        self.wL = wLO_eV * EV / HBAR
        self.gamma = gamma_eV * EV / HBAR

    def setTemperature(self, T: float):
        pass

    def eps(self, feV: float) -> complex:
        w = feV * EV / HBAR
        return self.epsinf * (self.wL * self.wL - w * w - 1j * self.gamma * w) / (
            self.wT * self.wT - w * w - 1j * self.gamma * w)

    def mu(self, feV: float) -> complex:
        return 1.0 + 0j


class SiC(FixedLorentz):
    """Temperature-dependent SiC (src/util/SiC.cpp:4-14)."""

    def __init__(self):
        self.setTemperature(300.0)

    def setTemperature(self, T: float):
        self.epsinf = 6.7 * math.exp(5e-5 * (T - 300))
        self.wL = 182.7e12 - 5.463e9 * (T - 300)
        self.wT = 149.5e12 - 4.106e9 * (T - 300)
        self.gamma = 6.6e11 * (1 + 2.0 / (math.exp(HBAR * self.wT / (2 * KB * T)) - 1))


# Material models of the workloads (single Lorentz oscillators, eV units).
SIC_CONFIG = (6.7, 0.0983, 0.120, 0.00059)
ALUMINA_CONFIG = (3.1, 0.0787, 0.111, 0.0020)


class Geometry:
    """Resident vertices + triangles (bemgpu_geom_t)."""

    def __init__(self, xyz, tris, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        self.tris = np.ascontiguousarray(tris, dtype=np.int32)
        h = ctypes.c_void_p()
        _check(_lib.load().bemgpu_geom_create(self.ctx.handle, self.xyz.ctypes.data, self.xyz.shape[0],
                                              self.tris.ctypes.data, self.tris.shape[0], ctypes.byref(h)), self.ctx)
        self.handle = h

    def __del__(self):
        try:
            if self.handle:
                _lib.load().bemgpu_geom_destroy(self.handle)
        except Exception:
            pass


class RWGTree:
    """An RWG table over a Geometry (bemgpu_tree_t); ``rwgs`` unknown pairs."""

    def __init__(self, geom: Geometry, rwg, diel=None):
        self.geom = geom
        self.rwg = np.ascontiguousarray(rwg, dtype=np.int32)
        self.rwgs = int(self.rwg.shape[0])
        self.diel = diel
        self.g = GreensFunction(1.0, 1.0, 0.0, False)
        h = ctypes.c_void_p()
        _check(_lib.load().bemgpu_tree_create(geom.handle, self.rwg.ctypes.data, self.rwgs, ctypes.byref(h)), geom.ctx)
        self.handle = h

    @classmethod
    def _adopt(cls, geom: Geometry, handle: ctypes.c_void_p, diel=None) -> "RWGTree":
        """A tree the library built (device set-up); its table read back."""
        L = _lib.load()
        n = L.bemgpu_tree_size(handle)
        rwg = np.empty((n, 4), dtype=np.int32)
        L.bemgpu_tree_rwgs(handle, rwg.ctypes.data, n)
        self = cls.__new__(cls)
        self.geom, self.rwg, self.rwgs, self.diel = geom, rwg, n, diel
        self.g = GreensFunction(1.0, 1.0, 0.0, False)
        self.handle = handle
        return self

    def __del__(self):
        try:
            if self.handle:
                _lib.load().bemgpu_tree_destroy(self.handle)
        except Exception:
            pass


def parseShapes(body1: Body, body2: Body, diel1, diel2, ctx: Context | None = None, setup: str = "host"):
    """Builds the two-body tree and the one-body trees over one geometry.
    ``body1`` is expected already translated by the gap vector (as
    parseShapes translates body 1, src/HeatTransfer.cpp:67-69).
    Returns (top, s, t).

    setup="host": the trees take the bodies' own RWG tables.  setup="device":
    only the vertices and triangles are uploaded; each body's RWG table (the
    reference's edge-creation order, ShapeMesh.cpp:857-928) and half-RWG
    frames are built by kernels (bemgpu_tree_create_body_device), and the
    two-body tree is their concatenation (bemgpu_tree_concat)."""
    xyz, tris, rwg, ns = two_body(body1, body2)
    geom = Geometry(xyz, tris, ctx)
    if setup == "device":
        L = _lib.load()
        hs, ht, htop = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        _check(L.bemgpu_tree_create_body_device(geom.handle, 0, body1.nt, ctypes.byref(hs)), geom.ctx)
        s = RWGTree._adopt(geom, hs, diel1)
        _check(L.bemgpu_tree_create_body_device(geom.handle, body1.nt, body2.nt, ctypes.byref(ht)), geom.ctx)
        t = RWGTree._adopt(geom, ht, diel2)
        _check(L.bemgpu_tree_concat(hs, ht, ctypes.byref(htop)), geom.ctx)
        return RWGTree._adopt(geom, htop), s, t
    if setup != "host":
        raise ValueError(f"setup must be 'host' or 'device', not {setup!r}")
    top = RWGTree(geom, rwg)
    s = RWGTree(geom, rwg[:ns], diel1)
    t = RWGTree(geom, rwg[ns:], diel2)
    return top, s, t


def Zts(t: RWGTree, s: RWGTree, g: GreensFunction, options: Options | None = None, precision: int = _lib.PREC_FP64):
    """Zts(t, s, g, options): the (2 t.rwgs x 2 s.rwgs) complex128 block,
    column-major like ComplexDenseMatrix."""
    options = options or Options()
    ctx = t.geom.ctx
    m, n = 2 * t.rwgs, 2 * s.rwgs
    Z = np.empty((m, n), dtype=np.complex128, order="F")
    _check(_lib.load().bemgpu_zts_host(ctx.handle, t.handle, s.handle, ctypes.byref(g._g), ctypes.byref(options._c()),
                                       int(precision), Z.ctypes.data, m), ctx)
    return Z


def Theta(omega: float, T: float) -> float:
    return _lib.load().bemgpu_theta(float(omega), float(T))


def dimensionless_omega(a: float, eV: float) -> float:
    return _lib.load().bemgpu_dimensionless_omega(float(a), float(eV))


def _solve_req(a: float, eV: float, T1: float, T2: float, s: RWGTree, t: RWGTree) -> _lib.SolveReq:
    """The material constants of one request at eV, as CalcHeatTransfer reads
    them (src/HeatTransfer.cpp:15-24: setTemperature, then eps/mu)."""
    s.diel.setTemperature(T1)
    t.diel.setTemperature(T2)
    e1, m1, e2, m2 = s.diel.eps(eV), s.diel.mu(eV), t.diel.eps(eV), t.diel.mu(eV)
    c2 = ctypes.c_double * 2
    return _lib.SolveReq(a, eV, T1, T2, c2(e1.real, e1.imag), c2(m1.real, m1.imag), c2(e2.real, e2.imag),
                         c2(m2.real, m2.imag))


def CalcHeatTransfer(a: float, eV: float, T1: float, T2: float, top: RWGTree, s: RWGTree, t: RWGTree,
                     options: Options | None = None, precision: int = _lib.PREC_FP64, info: dict | None = None,
                     strict: bool = True) -> float:
    """Spectral power Re(S) (Theta(omega,T1) - Theta(omega,T2)) at eV.

    With strict=False a mixed-precision solve whose refinement stalls returns
    its result anyway; info['err_est'] then states the estimated error."""
    options = options or Options()
    req = _solve_req(a, eV, T1, T2, s, t)
    P = ctypes.c_double()
    si = _lib.SolveInfo()
    ctx = top.geom.ctx
    rc = _lib.load().bemgpu_heat_transfer(ctx.handle, top.handle, s.handle, t.handle, ctypes.byref(req),
                                          ctypes.byref(options._c()), int(precision), ctypes.byref(P),
                                          ctypes.byref(si))
    if not (rc == _lib.ERR_NO_CONVERGE and not strict):
        _check(rc, ctx)
    if info is not None:
        for k, _ in _lib.SolveInfo._fields_:
            info[k] = getattr(si, k)
    return P.value


def CalcHeatTransferBatch(jobs, options: Options | None = None, precision: int = _lib.PREC_FP64,
                          infos: list | None = None, strict: bool = True) -> list:
    """CalcHeatTransfer for several (a, eV, T1, T2, top, s, t) at once
    (bemgpu_heat_transfer_batch): one fill launch pair for all of them and,
    for requests of equal size, one cooperative LU panel launch per block
    column.  The results equal CalcHeatTransfer's one by one, bit for bit."""
    options = options or Options()
    jobs = list(jobs)
    n = len(jobs)
    if n == 0:
        return []
    ctx = jobs[0][4].geom.ctx
    reqs = (_lib.SolveReq * n)(*[_solve_req(a, eV, T1, T2, s, t) for (a, eV, T1, T2, top, s, t) in jobs])
    vp = ctypes.c_void_p * n
    tops, ss, ts = vp(*[j[4].handle for j in jobs]), vp(*[j[5].handle for j in jobs]), vp(*[j[6].handle for j in jobs])
    P = (ctypes.c_double * n)()
    si = (_lib.SolveInfo * n)()
    st = (ctypes.c_int * n)()
    rc = _lib.load().bemgpu_heat_transfer_batch(ctx.handle, n, tops, ss, ts, reqs, ctypes.byref(options._c()),
                                                int(precision), P, si, st)
    if rc == _lib.ERR_ARG and all(st[i] == _lib.OK for i in range(n)):
        _check(rc, ctx)
    for i in range(n):
        if not (st[i] == _lib.ERR_NO_CONVERGE and not strict) and st[i] != _lib.OK:
            _check(st[i], ctx)
    if infos is not None:
        for i in range(n):
            infos.append({k: getattr(si[i], k) for k, _ in _lib.SolveInfo._fields_})
    return list(P)


class FrequencySweep:
    """FrequencySweep(file): one frequency (eV) per line (src/FrequencySweep.cpp:4-16)."""

    def __init__(self, filename: str):
        self.f = []
        try:
            with open(filename) as fh:
                for line in fh:
                    try:
                        self.f.append(float(line.split()[0]) if line.split() else 0.0)
                    except ValueError:
                        self.f.append(0.0)
        except OSError as e:
            import sys
            sys.stderr.write(f"{filename}: {e.strerror}\n")


def solve_footprint(s: RWGTree, t: RWGTree, precision: int = _lib.PREC_FP64, ctx: Context | None = None) -> int:
    """Device bytes one CalcHeatTransfer solve of these bodies needs at most
    (under ``ctx``'s solver mode when a context is given, else the default)."""
    if ctx is not None:
        return int(_lib.load().bemgpu_ctx_solve_footprint(ctx.handle, s.rwgs, t.rwgs, int(precision)))
    return int(_lib.load().bemgpu_solve_footprint(s.rwgs, t.rwgs, int(precision)))


def _check_farm(rc: int, farm):
    if rc != _lib.OK:
        raise _lib.BemGpuError(rc, _lib.load().bemgpu_farm_last_error(farm.handle).decode())


class Farm:
    """In-process request farm: the counterpart of the reference's MPI task
    farm (src/transfer-mpi.cpp:25-190), where a Master queues
    (a, gap, f, T1, T2) jobs and Servants run CalcHeatTransfer.  Here
    ``lanes`` contexts on one GPU, each driven by its own native thread, take
    requests from a FIFO, so several solves overlap on the device.

    ``submit`` takes CalcHeatTransfer's arguments and returns a ticket;
    ``result`` waits for it and returns the spectral power with
    CalcHeatTransfer's error behaviour.  The farm keeps the trees of every
    uncollected request alive."""

    def __init__(self, lanes: int = 2, device: int = 0, batch: int = 1):
        L = _lib.load()
        h = ctypes.c_void_p()
        rc = L.bemgpu_farm_create(int(device), int(lanes), ctypes.byref(h))
        if rc != _lib.OK:
            raise _lib.BemGpuError(rc, f"cannot create a {lanes}-lane farm on CUDA device {device}")
        self.handle = h
        self.lanes = lanes
        self.device = device
        self._held = {}
        self.set_batch(batch)

    def set_batch(self, max_requests: int):
        """Continuous batching: each lane solves up to ``max_requests`` queued
        requests of equal sizes together (bemgpu_farm_set_batch)."""
        rc = _lib.load().bemgpu_farm_set_batch(self.handle, int(max_requests))
        if rc != _lib.OK:
            raise _lib.BemGpuError(rc, f"batch size {max_requests} not in 1..64")
        self.batch = max_requests

    def _err(self) -> str:
        return _lib.load().bemgpu_farm_last_error(self.handle).decode()

    @property
    def budget(self) -> int:
        """Device bytes the lanes may hold together (admission by footprint)."""
        return int(_lib.load().bemgpu_farm_budget(self.handle))

    @budget.setter
    def budget(self, nbytes: int):
        _check_farm(_lib.load().bemgpu_farm_set_budget(self.handle, int(nbytes)), self)

    def lane_contexts(self) -> list:
        """Raw context handles of the lanes (for bemgpu_prof_* statistics)."""
        out = []
        for i in range(self.lanes):
            c = ctypes.c_void_p()
            _lib.load().bemgpu_farm_lane_ctx(self.handle, i, ctypes.byref(c))
            out.append(c)
        return out

    def submit(self, a: float, eV: float, T1: float, T2: float, top: RWGTree, s: RWGTree, t: RWGTree,
               options: Options | None = None, precision: int = _lib.PREC_FP64) -> int:
        options = options or Options()
        req = _solve_req(a, eV, T1, T2, s, t)
        tk = ctypes.c_int64()
        rc = _lib.load().bemgpu_farm_submit(self.handle, top.handle, s.handle, t.handle, ctypes.byref(req),
                                           ctypes.byref(options._c()), int(precision), ctypes.byref(tk))
        if rc != _lib.OK:
            raise _lib.BemGpuError(rc, self._err())
        self._held[tk.value] = (top, s, t)
        return tk.value

    def poll(self, ticket: int, timeout: float | None = 0.0, info: dict | None = None, strict: bool = True):
        """The request's spectral power, or None while it runs.  ``timeout``
        in seconds (None: wait until it finishes)."""
        P = ctypes.c_double()
        si = _lib.SolveInfo()
        ms = -1.0 if timeout is None else 1e3 * float(timeout)
        rc = _lib.load().bemgpu_farm_poll(self.handle, int(ticket), ms, ctypes.byref(P), ctypes.byref(si))
        if rc == _lib.PENDING:
            return None
        self._held.pop(int(ticket), None)
        if info is not None:
            for k, _ in _lib.SolveInfo._fields_:
                info[k] = getattr(si, k)
        if rc != _lib.OK and not (rc == _lib.ERR_NO_CONVERGE and not strict):
            raise _lib.BemGpuError(rc, self._err())
        return P.value

    def result(self, ticket: int, info: dict | None = None, strict: bool = True) -> float:
        return self.poll(ticket, None, info, strict)

    def cancel(self, ticket: int) -> bool:
        """True if the request was still queued and is now dropped."""
        rc = _lib.load().bemgpu_farm_cancel(self.handle, int(ticket))
        if rc < 0:
            raise _lib.BemGpuError(rc, self._err())
        return rc == _lib.OK

    def map(self, jobs, options: Options | None = None, precision: int = _lib.PREC_FP64, strict: bool = True,
            infos: list | None = None) -> list:
        """Solves every (a, eV, T1, T2, top, s, t) of ``jobs``; results in job order."""
        tickets = [self.submit(*j, options=options, precision=precision) for j in jobs]
        out = []
        for tk in tickets:
            info = {} if infos is not None else None
            out.append(self.result(tk, info, strict))
            if infos is not None:
                infos.append(info)
        return out

    def close(self):
        if self.handle:
            _lib.load().bemgpu_farm_destroy(self.handle)
            self.handle = None
            self._held.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

