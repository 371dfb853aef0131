"""ctypes binding of the CPU oracle (oracle/mcrt_oracle.cpp) and the oracle's own
restatement of the reference's input types.

TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's CPU
baseline and reference arm use it as the checker; the library and its Python host
code never do. This module imports nothing from the library: the Mie tables come from
the oracle's own bhmie / calculate_csrn (orc_mie_tables), and Config, the geometries and
the scatterers are restated here from src/config.jl, src/geometries/*.jl and
src/scatterers/*.jl. Parity is unpinned by the reference (it ships no golden vectors
and Julia is not installed); see the header of mcrt_oracle.cpp for how the oracle is
pinned instead.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmcrt_oracle.so")
_dp = C.POINTER(C.c_double)


class OrcScatterer(C.Structure):
    _fields_ = [("kind", C.c_int), ("omega", C.c_double), ("kl", C.c_double), ("n_theta", C.c_int),
                ("F11", _dp), ("F12", _dp), ("F33", _dp), ("F34", _dp), ("S11", _dp), ("S22", _dp),
                ("random_points", C.c_int), ("csrn", _dp)]


class OrcLayer(C.Structure):
    _fields_ = [("tau", C.c_double), ("omega", C.c_double), ("infinite", C.c_int), ("scatterer", C.c_int)]


class OrcGeometry(C.Structure):
    _fields_ = [("kind", C.c_int), ("theta", C.c_double), ("phi", C.c_double), ("n_layers", C.c_int),
                ("layers", C.POINTER(OrcLayer)), ("n_scatterers", C.c_int),
                ("scatterers", C.POINTER(OrcScatterer))]


class OrcConfig(C.Structure):
    _fields_ = [("number_of_rays", C.c_int64), ("minimum_intensity", C.c_double),
                ("maximum_scattering_times", C.c_int64), ("compute_cb", C.c_int), ("tau0", C.c_double),
                ("n_phi", C.c_int), ("cos_phi", _dp), ("sin_phi", _dp),
                ("n_theta", C.c_int), ("cos_theta", _dp), ("sin_theta", _dp), ("inorm", _dp),
                ("n_theta_b", C.c_int), ("cos_theta_b", _dp), ("sin_theta_b", _dp),
                ("n_phi_b", C.c_int), ("cos_phi_b", _dp), ("sin_phi_b", _dp)]


class OrcRun(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("instance", C.c_uint32), ("rng_mode", C.c_int), ("cb_form", C.c_int),
                ("n_threads", C.c_int), ("photon_begin", C.c_int64), ("photon_count", C.c_int64)]


_lib = None


def build() -> str:
    """Compiles the oracle with the Makefile beside this file."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_simulate.argtypes = [C.POINTER(OrcConfig), C.POINTER(OrcGeometry), _dp, C.POINTER(OrcRun),
                                   _dp, _dp, _dp, _dp, _dp, _dp]
        L.orc_simulate.restype = C.c_int
        L.orc_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.orc_rayleigh_sample.argtypes = [C.c_double]
        L.orc_rayleigh_sample.restype = C.c_double
        L.orc_kepler_solver.argtypes = [C.c_double, C.c_double]
        L.orc_kepler_solver.restype = C.c_double
        L.orc_mie_tables.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int, C.c_int] + [_dp] * 8
        L.orc_mie_tables.restype = C.c_int
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(_dp)


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, o)
    return list(o)


def simulate(cfg, g, I0, *, seed=1, instance=0, rng_mode=0, cb_form=0, threads=0, photon_begin=0,
             photon_count=None, fp32_tables=True):
    """Runs the oracle on a config/geometry built with the host package's types.

    Returns raw sums (not divided by the number of rays) as a dict with A, Irt
    (4, Ntheta, Nphi), Icb (4, Ntheta_b, Nphi_b), ladder, stats and counters. With
    ``fp32_tables`` the Mie tables are rounded to FP32 first, as the device stores them.
    """
    L = lib()
    keep = []

    def arr(a):
        a = np.ascontiguousarray(a, float)
        keep.append(a)
        return _p(a)

    if g.kind == 0:
        layers_in = [(l.tau, l.omega, int(l.infinite), l.scatterer) for l in g.layers]
    else:
        layers_in = [(g.tau, g.omega, 0, g.scatterer)]
    scats = []
    layers = (OrcLayer * len(layers_in))()
    for i, (tau, om, inf, s) in enumerate(layers_in):
        k = next((j for j, t in enumerate(scats) if t is s), None)
        if k is None:
            scats.append(s)
            k = len(scats) - 1
        layers[i] = OrcLayer(tau, om, inf, k)
    sarr = (OrcScatterer * len(scats))()
    for j, s in enumerate(scats):
        o = OrcScatterer()
        o.kind, o.omega, o.kl = s.kind, s.omega, s.kl
        if s.kind == 1:
            t = s.rounded_fp32() if fp32_tables else s
            o.n_theta = len(t.F11)
            o.F11, o.F12, o.F33, o.F34 = arr(t.F11), arr(t.F12), arr(t.F33), arr(t.F34)
            o.S11 = arr(np.column_stack([t.S11.real, t.S11.imag]).ravel())
            o.S22 = arr(np.column_stack([t.S22.real, t.S22.imag]).ravel())
            o.random_points = len(t.csrn) - 1
            o.csrn = arr(t.csrn)
        sarr[j] = o
    gc = OrcGeometry(g.kind, getattr(g, "theta", np.pi), getattr(g, "phi", 0.0), len(layers_in), layers,
                     len(scats), sarr)
    cc = OrcConfig(cfg.number_of_rays, cfg.minimum_intensity, cfg.maximum_scattering_times, int(cfg.compute_cb),
                   cfg.tau0, cfg.Nphi, arr(cfg.cosphi), arr(cfg.sinphi), cfg.Ntheta, arr(cfg.costheta),
                   arr(cfg.sintheta), arr(cfg.inorm), cfg.Nthetab, arr(cfg.costhetab), arr(cfg.sinthetab),
                   cfg.Nphib, arr(cfg.cosphib), arr(cfg.sinphib))
    n = cfg.number_of_rays if photon_count is None else photon_count
    run = OrcRun(int(seed), int(instance), int(rng_mode), int(cb_form), int(threads), int(photon_begin), int(n))
    A = np.zeros(5)
    Irt = np.zeros(4 * cfg.Ntheta * cfg.Nphi)
    Icb = np.zeros(4 * cfg.Nthetab * cfg.Nphib)
    lad = np.zeros(cfg.Nthetab * cfg.Nphib)
    st = np.zeros(3)
    ct = np.zeros(7)
    I = np.ascontiguousarray(I0, float)
    rc = L.orc_simulate(C.byref(cc), C.byref(gc), _p(I), C.byref(run), _p(A), _p(Irt), _p(Icb), _p(lad),
                        _p(st), _p(ct))
    if rc != 0:
        raise RuntimeError(f"oracle failed with {rc}")
    return {
        "A": A,
        "Irt": Irt.reshape(cfg.Nphi, cfg.Ntheta, 4).transpose(2, 1, 0),
        "Icb": Icb.reshape(cfg.Nphib, cfg.Nthetab, 4).transpose(2, 1, 0),
        "ladder": lad.reshape(cfg.Nphib, cfg.Nthetab).T,
        "stats": {"cb_peak_sum": st[0], "cb_peak_sumsq": st[1], "photons": st[2]},
        "counters": dict(zip(["events", "attempts", "rt_evals", "cb1_evals", "cbn_evals", "kepler_capped",
                              "attempts_capped"], ct)),
    }


# ------------------------------------------------------------------ reference input types
# Restated from the reference, independently of the library's host package, so that the
# oracle and the reference arm build their inputs without loading the library.

RAYLEIGH, MIE = 0, 1
PLANE, SPHERE = 0, 1

# DEFAULT_THEB of src/config.jl:3-53, in degrees.
DEFAULT_THEB_DEG = [0.0, 0.02, 0.04, 0.06, 0.08, 0.1, 0.15, 0.2, 0.25, 0.3, 0.35, 0.4, 0.45, 0.5, 0.6, 0.7,
                    0.8, 0.9, 1.0, 1.5, 2.0, 2.5, 3.0, 4.0, 5.0, 6.0, 7.0, 8.0, 9.0, 12.0, 15.0, 18.0, 21.0,
                    24.0, 27.0, 30.0, 40.0, 50.0, 60.0, 70.0, 80.0, 90.0, 100.0, 110.0, 120.0, 130.0, 140.0,
                    150.0, 160.0, 170.0, 180.0]


def mie_tables(x, m, n_theta=181, random_points=1000):
    """bhmie (src/scatterers/mie.jl:129-216) and calculate_csrn (src/utils.jl:263-287) in
    the oracle: dict with F11, F12, F33, F34, S11, S22 (complex), csrn, q_ext, q_sca,
    q_abs, q_back, asymm."""
    n, rp = int(n_theta), int(random_points)
    F = [np.zeros(n) for _ in range(4)]
    S = [np.zeros(2 * n) for _ in range(2)]
    cs = np.zeros(rp + 1)
    q = np.zeros(5)
    m = complex(m)
    rc = lib().orc_mie_tables(float(x), m.real, m.imag, n, rp, *[_p(f) for f in F], _p(S[0]), _p(S[1]),
                              _p(cs), _p(q))
    if rc != 0:
        raise ValueError("orc_mie_tables: invalid arguments")
    out = dict(zip(("F11", "F12", "F33", "F34"), F))
    out["S11"] = S[0][0::2] + 1j * S[0][1::2]
    out["S22"] = S[1][0::2] + 1j * S[1][1::2]
    out["csrn"] = cs
    out.update(zip(("q_ext", "q_sca", "q_abs", "q_back", "asymm"), (float(v) for v in q)))
    return out


class RayleighScatterer:
    """RayleighScatterer(ω, kl) (src/scatterers/rayleigh.jl:3-6)."""

    kind = RAYLEIGH

    def __init__(self, omega, kl):
        self.omega, self.kl = float(omega), float(kl)


class MieScatterer:
    """MieScatterer(r, m, λ, ν; Nθ=181, random_points=1000) (src/scatterers/mie.jl:36-44):
    x = 2πr/λ, ω = q_sca/q_ext, kl = (4/3 r)/(ν q_ext), tables from the oracle's bhmie."""

    kind = MIE

    def __init__(self, r, m, lam=1.0, nu=0.1, *, Ntheta=181, random_points=1000):
        self.r, self.m, self.lam, self.nu = float(r), complex(m), float(lam), float(nu)
        self.x = 2 * math.pi * self.r / self.lam
        t = mie_tables(self.x, self.m, Ntheta, random_points)
        self.q_ext, self.q_sca, self.q_abs, self.q_back, self.asymm = (
            t["q_ext"], t["q_sca"], t["q_abs"], t["q_back"], t["asymm"])
        self.omega = self.q_sca / self.q_ext
        self.kl = (4.0 / 3.0) * self.r / (self.nu * self.q_ext)
        self.F11, self.F12, self.F33, self.F34 = t["F11"], t["F12"], t["F33"], t["F34"]
        self.S11, self.S22, self.csrn = t["S11"], t["S22"], t["csrn"]
        self.Ntheta, self.random_points = int(Ntheta), int(random_points)

    def rounded_fp32(self):
        """A view with every table rounded to FP32, as a device that stores FP32 tables sees it."""
        f = lambda a: np.asarray(a, np.float32).astype(np.float64)
        c = lambda z: f(z.real) + 1j * f(z.imag)
        o = MieScatterer.__new__(MieScatterer)
        o.__dict__.update(self.__dict__)
        o.F11, o.F12, o.F33, o.F34 = f(self.F11), f(self.F12), f(self.F33), f(self.F34)
        o.S11, o.S22, o.csrn = c(self.S11), c(self.S22), f(self.csrn)
        return o


class Layer:
    """Layer(d, n=1, scatterer, τ=d/kl, ω) (src/geometries/plane.jl:6-21); d < 0 is a
    semi-infinite layer."""

    def __init__(self, d, scatterer, n=1.0, tau=None, omega=None):
        self.d, self.scatterer, self.n = float(d), scatterer, float(n)
        self.tau = float(tau) if tau is not None else self.d / scatterer.kl
        self.omega = float(omega) if omega is not None else scatterer.omega
        self.infinite = self.d < 0


class PlaneGeometry:
    """PlaneGeometry(θ, ϕ, layers) (src/geometries/plane.jl:28-38)."""

    kind = PLANE

    def __init__(self, theta, phi, layers):
        self.theta, self.phi, self.layers = float(theta), float(phi), list(layers)

    def initial_weights(self, Ntheta, Nphi):  # plane.jl:131-142, half-range Gauss-Legendre
        h = Ntheta // 2
        x, w = np.polynomial.legendre.leggauss(h)
        cos = np.concatenate([(x - 1.0) / 2.0, -((x - 1.0) / 2.0)[::-1]])
        inorm = np.concatenate([w / 2.0, (w / 2.0)[::-1]]) * (1.0 / (2 * Nphi))
        return cos, np.sqrt(1.0 - cos ** 2), inorm


class SphereGeometry:
    """SphereGeometry(R, n=1, scatterer, τ=R/kl, ω) (src/geometries/sphere.jl:6-21)."""

    kind = SPHERE
    theta, phi = math.pi, 0.0

    def __init__(self, R, scatterer, n=1.0, tau=None, omega=None):
        self.R, self.scatterer, self.n = float(R), scatterer, float(n)
        self.tau = float(tau) if tau is not None else self.R / scatterer.kl
        self.omega = float(omega) if omega is not None else scatterer.omega

    def initial_weights(self, Ntheta, Nphi):  # sphere.jl:85-90
        cos, w = np.polynomial.legendre.leggauss(Ntheta)
        return cos, np.sqrt(1.0 - cos ** 2), w / (2 * Nphi)


class Config:
    """Config (src/config.jl:55-124): the reference's defaults and derived trig tables."""

    def __init__(self, geometry, *, number_of_rays=1000, minimum_intensity=1e-6, maximum_scattering_times=10000,
                 compute_cb=True, tau0=50.0, Nphi=48, Ntheta=64, thetab=None, Nphib=8):
        self.number_of_rays = int(number_of_rays)
        self.minimum_intensity = float(minimum_intensity)
        self.maximum_scattering_times = int(maximum_scattering_times)
        self.compute_cb, self.tau0 = bool(compute_cb), float(tau0)
        self.Nphi, self.Ntheta, self.Nphib = int(Nphi), int(Ntheta), int(Nphib)
        phi = np.linspace(0.0, 2 * math.pi * (self.Nphi - 1) / self.Nphi, self.Nphi)  # config.jl:81
        self.cosphi, self.sinphi = np.cos(phi), np.sin(phi)
        self.costheta, self.sintheta, self.inorm = geometry.initial_weights(self.Ntheta, self.Nphi)
        tb = np.asarray(thetab, float) if thetab is not None else math.pi / 180.0 * np.array(DEFAULT_THEB_DEG)
        self.Nthetab = len(tb)
        self.costhetab, self.sinthetab = np.cos(tb), np.sin(tb)
        phib = np.linspace(0.0, 2 * math.pi * (self.Nphib - 1) / self.Nphib, self.Nphib)  # config.jl:117
        self.cosphib, self.sinphib = np.cos(phib), np.sin(phib)
