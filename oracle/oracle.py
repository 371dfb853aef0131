"""ctypes binding of the CPU oracle (oracle/mcrt_oracle.cpp).

TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's CPU
baseline use it as the checker; the library and its Python host code never do.
Parity is unpinned by the reference (it ships no golden vectors and Julia is not
installed); see the header of mcrt_oracle.cpp for how the oracle is pinned instead.
"""
from __future__ import annotations

import ctypes as C
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
