"""Material models and the registry CalcHeatTransfer's callers pick them from.

Mirrors the reference's dielectric layer (claytonotey/bem):

  Dielectric.eps(eV), .mu(eV), .setTemperature(T)   src/util/Dielectric.h:7-14
  ConstantDielectric(eps, mu), Vacuum                src/util/Dielectric.h:33-47
  SiC (temperature dependent)                        src/util/SiC.cpp:4-19 (api.SiC)
  Al (one Lorentz pole on a constant)                src/util/Al.cpp:4-12
  Au (Drude)                                         src/util/Au.cpp:4-11
  SiliconDoped(N) (Drude with carrier mobility)      src/util/SiliconDoped.cpp:4-41
  Tabulated n + ik (SiN's form, linear interpolation) src/util/SiN.cpp (eps), MathUtils.cpp:9-21,351-366
  getDielectric(name, params)                        src/util/Dielectrics.cpp:15-63

The SiN table itself is measured data shipped with the reference; it is not
repeated here: ``Tabulated`` takes the (eV, n, k) columns from the caller, and
``getDielectric("SiN", table=...)`` requires them.  All values are evaluated on
the host once per request (a handful of flops); nothing here runs on the GPU.
"""
from __future__ import annotations

import bisect
import math

from .api import EV, HBAR, FixedLorentz, SiC

ME = 9.109e-31           # electron mass, kg (the reference's value, src/util/SI.cpp:8)
EPS0 = 8.85418782e-12    # vacuum permittivity, F/m (src/util/SI.cpp:9)


def _omega(feV: float) -> float:
    return feV * EV / HBAR


class ConstantDielectric:
    def __init__(self, eps: complex = 1.0, mu: complex = 1.0):
        self._eps, self._mu = complex(eps), complex(mu)

    def setTemperature(self, T: float):
        pass

    def eps(self, feV: float) -> complex:
        return self._eps

    def mu(self, feV: float) -> complex:
        return self._mu


class Vacuum(ConstantDielectric):
    def __init__(self):
        super().__init__(1.0, 1.0)


class Al(ConstantDielectric):
    """eps = eps_inf + eps_L w0^2 / (w0^2 - w^2 - 2 i w g0)."""
    EPS_INF, EPS_LORENTZ, OMEGA0, GAMMA0 = 2.2281, 1.30601, 1.50690679e14, 3.76734192e13

    def __init__(self):
        super().__init__()

    def eps(self, feV: float) -> complex:
        w = _omega(feV)
        w0 = self.OMEGA0
        return self.EPS_INF + self.EPS_LORENTZ * w0 * w0 / (w0 * w0 - w * w - 2j * w * self.GAMMA0)


class Au(ConstantDielectric):
    """Drude: eps = eps0 - wp^2 / (w (w + i wc))."""
    EPS0, OMEGAP, OMEGAC = 1.0, 1.366592804e16, 4.08407045e13

    def __init__(self):
        super().__init__()

    def eps(self, feV: float) -> complex:
        w = _omega(feV)
        return self.EPS0 - self.OMEGAP ** 2 / (w * (w + 1j * self.OMEGAC))


class SiliconDoped(ConstantDielectric):
    """Doped silicon, N carriers per m^3 (N < 0: n-type, N > 0: p-type, 0:
    intrinsic): eps = 11.7 - wp^2 / (w (w + i g)) with wp^2 = e^2 |N| / (m eps0)
    and g = e / (m mobility), the mobility from the doping-dependent fits the
    reference uses (src/util/SiliconDoped.cpp:9-38)."""

    def __init__(self, N: float = 0.0):
        super().__init__()
        self.N = float(N)

    def eps(self, feV: float) -> complex:
        N = self.N
        if N == 0.0:
            return 11.7 + 0j
        w = _omega(feV)
        if N < 0.0:
            mu1, mumax, mu2, Cr, Cs, alpha, beta, m = .00685, .1414, .00561, 9.20e22, 3.41e26, .711, 1.98, .27 * ME
            mob = mu1 + (mumax - mu1) / (1 + (abs(N) / Cr) ** alpha) - mu2 / (1 + (Cs / abs(N)) ** beta)
        else:
            mu1, mumax, mu2, Cr, Cs, alpha, beta, pc, m = (.00449, .04705, .0029, 2.23e23, 6.10e26, .719, 2.00,
                                                           9.23e24, .37 * ME)
            mob = mu1 * math.exp(-pc / N) + mumax / (1 + (N / Cr) ** alpha) - mu2 / (1 + (Cs / N) ** beta)
        wp = EV * math.sqrt(abs(N) / m / EPS0)
        g = EV / m / mob
        return 11.7 - wp * wp / (w * (w + 1j * g))


class Tabulated(ConstantDielectric):
    """eps = (n + i k)^2 with n, k linearly interpolated in a table over eV
    (SiN's model); outside the table the end segments are extended."""

    def __init__(self, eV, n, k):
        super().__init__()
        if not (len(eV) == len(n) == len(k)) or len(eV) < 2:
            raise ValueError("Tabulated: eV, n, k need equal lengths >= 2")
        if any(b <= a for a, b in zip(eV, eV[1:])):
            raise ValueError("Tabulated: eV must increase")
        self.f, self.n, self.k = [float(x) for x in eV], [float(x) for x in n], [float(x) for x in k]

    def _interp(self, y, x):
        j = min(max(bisect.bisect_right(self.f, x) - 1, 0), len(self.f) - 2)
        h = self.f[j + 1] - self.f[j]
        return y[j] + (y[j + 1] - y[j]) / h * (x - self.f[j])

    def eps(self, feV: float) -> complex:
        s = complex(self._interp(self.n, feV), self._interp(self.k, feV))
        return s * s


def parse_param(s: str):
    """A Dielectric element's attribute value: complex ("(a,b)", "a+bj"),
    int, float, or the string itself (Params::parseParam's order)."""
    t = s.strip()
    if t.startswith("(") and t.endswith(")") and "," in t:
        a, b = t[1:-1].split(",", 1)
        try:
            return complex(float(a), float(b))
        except ValueError:
            pass
    for conv in (int, float):
        try:
            return conv(t)
        except ValueError:
            pass
    try:
        return complex(t.replace("i", "j"))
    except ValueError:
        return t


_registry: dict = {}


def getDielectric(name: str, params: dict | None = None, table=None):
    """The registry lookup of src/util/Dielectrics.cpp:15-53: a named model
    (SiC, Al, Au, SiN), SiliconDoped with params["N"], or else a
    ConstantDielectric from params["eps"] / params["mu"] (default 1).  One
    instance per (name, params), as the reference caches them."""
    params = dict(params or {})
    key = (name, tuple(sorted((k, str(v)) for k, v in params.items())))
    if key in _registry:
        return _registry[key]
    if name == "SiC" and not params:
        d = SiC()
    elif name == "Al" and not params:
        d = Al()
    elif name == "Au" and not params:
        d = Au()
    elif name == "SiN" and not params:
        if table is None:
            raise ValueError("SiN is a tabulated model: pass table=(eV, n, k)")
        d = Tabulated(*table)
    elif name == "SiliconDoped":
        N = params.get("N", 0.0)
        d = SiliconDoped(float(N.real if isinstance(N, complex) else N) if not isinstance(N, str) else 0.0)
    elif name == "Lorentz":
        d = FixedLorentz(float(params["epsinf"]), float(params["wTO"]), float(params["wLO"]), float(params["gamma"]))
    else:
        e, m = params.get("eps", 1.0), params.get("mu", 1.0)
        d = ConstantDielectric(complex(e) if not isinstance(e, str) else 1.0,
                               complex(m) if not isinstance(m, str) else 1.0)
    _registry[key] = d
    return d


__all__ = ["ConstantDielectric", "Vacuum", "Al", "Au", "SiliconDoped", "Tabulated", "SiC", "FixedLorentz",
           "getDielectric", "parse_param"]
