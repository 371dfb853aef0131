"""Host-side mirror of the reference's Config, scatterer and geometry types.

Field names follow the reference with ASCII spellings of its Unicode names
(``τ₀ -> tau0``, ``Nθ -> Ntheta``, ``Nϕ -> Nphi``, ``θb -> thetab``, ``ω -> omega``).
The defaults are the reference's (src/config.jl:55-124).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from . import _lib

# DEFAULT_THEB (src/config.jl:3-53), degrees converted to radians.
DEFAULT_THEB_DEG = np.array([
    0.00, 0.02, 0.04, 0.06, 0.08, 0.10, 0.15, 0.20, 0.25, 0.30, 0.35, 0.40, 0.45, 0.50, 0.60,
    0.70, 0.80, 0.90, 1.00, 1.50, 2.00, 2.50, 3.00, 4.00, 5.00, 6.00, 7.00, 8.00, 9.00, 12.0,
    15.0, 18.0, 21.0, 24.0, 27.0, 30.0, 40.0, 50.0, 60.0, 70.0, 80.0, 90.0, 100.0, 110.0,
    120.0, 130.0, 140.0, 150.0, 160.0, 170.0, 180.0])
DEFAULT_THEB = math.pi / 180.0 * DEFAULT_THEB_DEG


# ------------------------------------------------------------------ scatterers
class RayleighScatterer:
    """RayleighScatterer(ω, kl) (src/scatterers/rayleigh.jl:3-6)."""

    kind = _lib.RAYLEIGH

    def __init__(self, omega: float, kl: float):
        self.omega = float(omega)
        self.kl = float(kl)

    def __repr__(self) -> str:
        return f"RayleighScatterer(omega={self.omega}, kl={self.kl})"


class MieScatterer:
    """MieScatterer(r, m, λ, ν; Nθ=181, random_points=1000) (src/scatterers/mie.jl:36-44).

    The Mie tables (bhmie) and the inverse CDF (calculate_csrn) are produced by the
    library's host code. ``from_tables`` builds one from given tables instead.
    """

    kind = _lib.MIE

    def __init__(self, r: float, m: complex, lam: float = 1.0, nu: float = 0.1, *,
                 Ntheta: int = 181, random_points: int = 1000):
        n = int(Ntheta)
        rp = int(random_points)
        L = _lib.lib()
        om = np.zeros(1)
        kl = np.zeros(1)
        F = [np.zeros(n) for _ in range(4)]
        S = [np.zeros(2 * n) for _ in range(2)]
        cs = np.zeros(rp + 1)
        q = np.zeros(5)
        m = complex(m)
        _lib.check(L.mcrt_mie_tables(float(r), m.real, m.imag, float(lam), float(nu), n, rp,
                                     _lib.dptr(om), _lib.dptr(kl), *[_lib.dptr(f) for f in F],
                                     *[_lib.dptr(s) for s in S], _lib.dptr(cs), _lib.dptr(q)))
        self.r, self.m, self.lam, self.nu = float(r), m, float(lam), float(nu)
        self.x = 2 * math.pi * self.r / self.lam
        self.omega = float(om[0])
        self.kl = float(kl[0])
        self.F11, self.F12, self.F33, self.F34 = F
        self.S11 = S[0][0::2] + 1j * S[0][1::2]
        self.S22 = S[1][0::2] + 1j * S[1][1::2]
        self.csrn = cs
        self.Ntheta = n
        self.random_points = rp
        self.q_ext, self.q_sca, self.q_abs, self.q_back, self.asymm = (float(v) for v in q)

    @classmethod
    def from_tables(cls, omega, kl, F11, F12, F33, F34, S11, S22, csrn) -> "MieScatterer":
        self = cls.__new__(cls)
        self.omega, self.kl = float(omega), float(kl)
        self.F11, self.F12, self.F33, self.F34 = (np.ascontiguousarray(a, float) for a in (F11, F12, F33, F34))
        self.S11 = np.asarray(S11, complex)
        self.S22 = np.asarray(S22, complex)
        self.csrn = np.ascontiguousarray(csrn, float)
        self.Ntheta = len(self.F11)
        self.random_points = len(self.csrn) - 1
        return self

    def rounded_fp32(self) -> "MieScatterer":
        """The same scatterer with its tables rounded to FP32 (what the device stores)."""
        f = lambda a: np.asarray(a, np.float32).astype(np.float64)
        c = lambda z: f(z.real) + 1j * f(z.imag)
        return MieScatterer.from_tables(self.omega, self.kl, f(self.F11), f(self.F12), f(self.F33),
                                        f(self.F34), c(self.S11), c(self.S22), f(self.csrn))

    def __repr__(self) -> str:
        return f"MieScatterer(omega={self.omega:.6g}, kl={self.kl:.6g}, Ntheta={self.Ntheta})"


def mean_free_path(s) -> float:
    return s.kl  # src/scatterers/index.jl:1


def single_scattering_albedo(s) -> float:
    return s.omega  # src/scatterers/index.jl:3


# ------------------------------------------------------------------ geometries
@dataclass
class Layer:
    """Layer(d, n=1, scatterer, τ=d/kl, ω=ω(scatterer)) (src/geometries/plane.jl:6-21).

    A negative thickness ``d`` marks a semi-infinite layer (plane.jl:23)."""

    d: float
    scatterer: object
    n: float = 1.0
    tau: Optional[float] = None
    omega: Optional[float] = None

    def __post_init__(self):
        if self.tau is None:
            self.tau = self.d / mean_free_path(self.scatterer)
        if self.omega is None:
            self.omega = single_scattering_albedo(self.scatterer)

    @property
    def infinite(self) -> bool:
        return self.d < 0


@dataclass
class PlaneGeometry:
    """PlaneGeometry(θ, ϕ, layers) (src/geometries/plane.jl:28-38)."""

    theta: float
    phi: float
    layers: List[Layer]
    kind: int = field(default=_lib.PLANE, init=False)

    def validate(self) -> None:  # plane.jl:52-62
        if not (math.pi / 2 < self.theta <= math.pi):
            raise ValueError("θ must be in (π/2, π]")
        if not (0 <= self.phi < 2 * math.pi):
            raise ValueError("ϕ must be in [0, 2π)")
        if not self.layers:
            raise ValueError("There needs to be at least one layer")
        for i, l in enumerate(self.layers):
            if i != len(self.layers) - 1 and l.infinite:
                raise ValueError("Only the last layer can be infinite")

    def incidence_angle(self):
        return self.theta, self.phi

    def initial_I(self) -> np.ndarray:  # plane.jl:70-75
        return np.array([[1.0, 1.0, 1.0, 1.0, 1.0, 1.0],
                         [-1.0, 1.0, 0.0, 0.0, 0.0, 0.0],
                         [0.0, 0.0, -1.0, 1.0, 0.0, 0.0],
                         [0.0, 0.0, 0.0, 0.0, -1.0, 1.0]])

    def initial_weights(self, Ntheta: int, Nphi: int):  # plane.jl:131-142
        h = Ntheta // 2
        x, w = np.polynomial.legendre.leggauss(h)
        cos = np.zeros(Ntheta)
        inorm = np.zeros(Ntheta)
        cos[:h] = (x - 1.0) / 2.0
        inorm[:h] = w / 2.0
        cos[h:] = -cos[:h][::-1]
        inorm[h:] = inorm[:h][::-1]
        inorm *= 1.0 / (2 * Nphi)
        return cos, np.sqrt(1.0 - cos ** 2), inorm

    def scatterers(self):
        return [l.scatterer for l in self.layers]


@dataclass
class SphereGeometry:
    """SphereGeometry(R, n=1, scatterer, τ=R/kl, ω) (src/geometries/sphere.jl:6-21)."""

    R: float
    scatterer: object
    n: float = 1.0
    tau: Optional[float] = None
    omega: Optional[float] = None
    kind: int = field(default=_lib.SPHERE, init=False)

    def __post_init__(self):
        if self.tau is None:
            self.tau = self.R / mean_free_path(self.scatterer)
        if self.omega is None:
            self.omega = single_scattering_albedo(self.scatterer)

    def validate(self) -> None:  # sphere.jl:35-37
        if not self.R > 0:
            raise ValueError("Radius must be positive")

    def incidence_angle(self):
        return math.pi, 0.0

    def initial_I(self) -> np.ndarray:  # sphere.jl:49-52
        return np.array([[1.0, 1.0], [-1.0, 0.0], [0.0, 0.0], [0.0, -1.0]])

    def initial_weights(self, Ntheta: int, Nphi: int):  # sphere.jl:85-90
        cos, w = np.polynomial.legendre.leggauss(Ntheta)
        return cos, np.sqrt(1.0 - cos ** 2), w / (2 * Nphi)

    def scatterers(self):
        return [self.scatterer]


# ------------------------------------------------------------------ configuration
class Config:
    """Config (src/config.jl:55-124) with its defaults; the arrays derive from the
    counts unless given."""

    def __init__(self, geometry, *, number_of_rays: int = 1000, minimum_intensity: float = 1e-6,
                 maximum_scattering_times: int = 10000, maximum_threads: int = 8192,
                 compute_cb: bool = True, tau0: float = 50.0, Nphi: int = 48,
                 phi: Optional[Sequence[float]] = None, Ntheta: int = 64,
                 thetab: Optional[Sequence[float]] = None, Nphib: int = 8,
                 phib: Optional[Sequence[float]] = None):
        self.geometry = geometry
        self.number_of_rays = int(number_of_rays)
        self.minimum_intensity = float(minimum_intensity)
        self.maximum_scattering_times = int(maximum_scattering_times)
        self.maximum_threads = int(maximum_threads)
        self.compute_cb = bool(compute_cb)
        self.tau0 = float(tau0)
        self.Nphi = int(Nphi)
        self.phi = (np.asarray(phi, float) if phi is not None
                    else np.linspace(0.0, 2 * math.pi * (self.Nphi - 1) / self.Nphi, self.Nphi))
        self.cosphi, self.sinphi = np.cos(self.phi), np.sin(self.phi)
        self.Ntheta = int(Ntheta)
        self.costheta, self.sintheta, self.inorm = geometry.initial_weights(self.Ntheta, self.Nphi)
        self.thetab = np.asarray(thetab if thetab is not None else DEFAULT_THEB, float)
        self.Nthetab = len(self.thetab)
        self.costhetab, self.sinthetab = np.cos(self.thetab), np.sin(self.thetab)
        self.Nphib = int(Nphib)
        self.phib = (np.asarray(phib, float) if phib is not None
                     else np.linspace(0.0, 2 * math.pi * (self.Nphib - 1) / self.Nphib, self.Nphib))
        self.cosphib, self.sinphib = np.cos(self.phib), np.sin(self.phib)

    def replace(self, **kw) -> "Config":
        args = dict(number_of_rays=self.number_of_rays, minimum_intensity=self.minimum_intensity,
                    maximum_scattering_times=self.maximum_scattering_times,
                    maximum_threads=self.maximum_threads, compute_cb=self.compute_cb,
                    tau0=self.tau0, Nphi=self.Nphi, phi=self.phi, Ntheta=self.Ntheta,
                    thetab=self.thetab, Nphib=self.Nphib, phib=self.phib)
        geometry = kw.pop("geometry", self.geometry)
        args.update(kw)
        return Config(geometry, **args)

    def to_c(self) -> _lib.ConfigC:
        """C view of the config; the numpy arrays stay referenced by this object."""
        self._keep = [np.ascontiguousarray(a, float) for a in (
            self.cosphi, self.sinphi, self.costheta, self.sintheta, self.inorm,
            self.costhetab, self.sinthetab, self.cosphib, self.sinphib)]
        k = self._keep
        return _lib.ConfigC(self.number_of_rays, self.minimum_intensity,
                            self.maximum_scattering_times, self.maximum_threads,
                            int(self.compute_cb), self.tau0,
                            self.Nphi, _lib.dptr(k[0]), _lib.dptr(k[1]),
                            self.Ntheta, _lib.dptr(k[2]), _lib.dptr(k[3]), _lib.dptr(k[4]),
                            self.Nthetab, _lib.dptr(k[5]), _lib.dptr(k[6]),
                            self.Nphib, _lib.dptr(k[7]), _lib.dptr(k[8]))
