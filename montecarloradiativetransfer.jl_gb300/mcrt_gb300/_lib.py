"""ctypes binding of libmcrt.so (the C ABI declared in include/mcrt.h).

The library is built in-tree by ``build.py`` into ``_lib/libmcrt.so``. There is no
fallback: if the library is missing or fails to load, :func:`lib` raises.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libmcrt.so")

MCRT_OK, MCRT_EINVAL, MCRT_ENOMEM, MCRT_ECUDA, MCRT_ENONCONV = 0, 1, 2, 3, 4
MCRT_ETIMEDOUT, MCRT_EBUSY, MCRT_ENOTFOUND, MCRT_ENODEV = 5, 6, 7, 8
RAYLEIGH, MIE = 0, 1
PLANE, SPHERE = 0, 1
FP32, FP64 = 0, 1
KERNEL_PERSISTENT, KERNEL_PLAIN = 0, 1
RNG_PHILOX, RNG_STRATIFIED_DEPTH = 0, 1

_dp = C.POINTER(C.c_double)


class ScattererDesc(C.Structure):
    _fields_ = [
        ("kind", C.c_int), ("omega", C.c_double), ("kl", C.c_double),
        ("n_theta", C.c_int),
        ("F11", _dp), ("F12", _dp), ("F33", _dp), ("F34", _dp),
        ("S11", _dp), ("S22", _dp),
        ("random_points", C.c_int), ("csrn", _dp),
    ]


class ConfigC(C.Structure):
    _fields_ = [
        ("number_of_rays", C.c_int64), ("minimum_intensity", C.c_double),
        ("maximum_scattering_times", C.c_int64), ("maximum_threads", C.c_int64),
        ("compute_cb", C.c_int), ("tau0", C.c_double),
        ("n_phi", C.c_int), ("cos_phi", _dp), ("sin_phi", _dp),
        ("n_theta", C.c_int), ("cos_theta", _dp), ("sin_theta", _dp), ("inorm", _dp),
        ("n_theta_b", C.c_int), ("cos_theta_b", _dp), ("sin_theta_b", _dp),
        ("n_phi_b", C.c_int), ("cos_phi_b", _dp), ("sin_phi_b", _dp),
    ]


class LayerC(C.Structure):
    _fields_ = [("tau", C.c_double), ("omega", C.c_double), ("infinite", C.c_int),
                ("scatterer", C.c_void_p)]


class GeometryC(C.Structure):
    _fields_ = [("kind", C.c_int), ("theta", C.c_double), ("phi", C.c_double),
                ("n_layers", C.c_int), ("layers", C.POINTER(LayerC))]


class RunOpts(C.Structure):
    _fields_ = [
        ("precision", C.c_int), ("kernel", C.c_int), ("seed", C.c_uint64),
        ("instance", C.c_uint32), ("rng_mode", C.c_int), ("photon_begin", C.c_int64),
        ("block_size", C.c_int), ("blocks_per_sm", C.c_int), ("plain_threads", C.c_int),
        ("table_staging", C.c_int), ("max_attempts", C.c_int64),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("cb_peak_sum", C.c_double), ("cb_peak_sumsq", C.c_double), ("photons", C.c_double),
        ("events", C.c_double), ("attempts", C.c_double), ("rt_evals", C.c_double),
        ("cb1_evals", C.c_double), ("cbn_evals", C.c_double), ("kernel_ms", C.c_double),
        ("status_flags", C.c_int), ("block_size", C.c_int), ("blocks", C.c_int),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class ServerOpts(C.Structure):
    _fields_ = [("memory_cap_bytes", C.c_double), ("max_active", C.c_int), ("wave_photons", C.c_int64),
                ("min_quantum", C.c_int64), ("precision", C.c_int), ("use_graphs", C.c_int),
                ("wave_work", C.c_double)]


class RequestC(C.Structure):
    _fields_ = [("config", C.POINTER(ConfigC)), ("geometry", C.POINTER(GeometryC)), ("I0", C.c_double * 4),
                ("seed", C.c_uint64), ("instance", C.c_uint32), ("n_photons", C.c_int64)]


class TicketInfo(C.Structure):
    _fields_ = [("submitted_s", C.c_double), ("admitted_s", C.c_double), ("completed_s", C.c_double),
                ("footprint_bytes", C.c_double), ("photons", C.c_int64), ("waves", C.c_int),
                ("status_flags", C.c_int)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class InstanceC(C.Structure):
    _fields_ = [("geometry", C.POINTER(GeometryC)), ("I0", C.c_double * 4),
                ("seed", C.c_uint64), ("instance", C.c_uint32), ("n_photons", C.c_int64)]


# (name, argtypes) of every entry point include/mcrt.h declares.
_VP = C.c_void_p
SIGNATURES = {
    "mcrt_abi_version": [],
    "mcrt_last_error": [],
    "mcrt_device_count": [],
    "mcrt_ctx_create": [C.c_int, C.POINTER(_VP)],
    "mcrt_ctx_destroy": [_VP],
    "mcrt_scatterer_create": [_VP, C.POINTER(ScattererDesc), C.POINTER(_VP)],
    "mcrt_scatterer_destroy": [_VP],
    "mcrt_mie_tables": [C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int,
                        _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp],
    "mcrt_simulate": [_VP, C.POINTER(ConfigC), C.POINTER(GeometryC), _dp, C.POINTER(RunOpts),
                      _dp, _dp, _dp, _dp, C.POINTER(Stats)],
    "mcrt_solve_create": [_VP, C.POINTER(ConfigC), C.POINTER(GeometryC), _dp, C.POINTER(RunOpts),
                          C.POINTER(_VP)],
    "mcrt_solve_launch": [_VP, C.c_int64, C.c_int64],
    "mcrt_solve_read": [_VP, _dp, _dp, _dp, _dp, C.POINTER(Stats)],
    "mcrt_solve_destroy": [_VP],
    "mcrt_batch_create": [_VP, C.POINTER(ConfigC), C.POINTER(InstanceC), C.c_int,
                          C.POINTER(RunOpts), C.POINTER(_VP)],
    "mcrt_batch_launch": [_VP],
    "mcrt_batch_read": [_VP, C.c_int, _dp, _dp, _dp, _dp, C.POINTER(Stats)],
    "mcrt_batch_timing": [_VP, _dp, _dp],
    "mcrt_batch_destroy": [_VP],
    "mcrt_scatterer_params": [_VP, _dp, _dp],
    "mcrt_mie_scatterers_create": [_VP, C.c_int, _dp, _dp, _dp, _dp, _dp, C.c_int, C.c_int, C.POINTER(_VP), _dp],
    "mcrt_run_rt": [_VP, C.POINTER(ConfigC), C.POINTER(GeometryC), C.POINTER(RunOpts), _dp, _dp, _dp,
                    C.POINTER(Stats)],
    "mcrt_measure_fp32_peak": [_VP, _dp],
    "mcrt_simulate_noalloc": [_VP, C.POINTER(ConfigC), C.POINTER(GeometryC), _dp, C.POINTER(RunOpts),
                              _dp, _dp, _dp, _dp, C.POINTER(Stats)],
    "mcrt_server_create": [_VP, C.POINTER(ServerOpts), C.POINTER(_VP)],
    "mcrt_server_submit": [_VP, C.POINTER(RequestC), C.POINTER(C.c_uint64)],
    "mcrt_server_wait": [_VP, C.c_uint64, C.c_double],
    "mcrt_server_result": [_VP, C.c_uint64, _dp, _dp, _dp, _dp, C.POINTER(TicketInfo)],
    "mcrt_server_stats": [_VP, _dp],
    "mcrt_server_destroy": [_VP],
}

_lib = None


class MCRTError(RuntimeError):
    """A libmcrt call returned a non-zero status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"libmcrt error {code}: {msg}")
        self.code = code


def lib() -> C.CDLL:
    """Loads libmcrt.so once; raises if it is missing (there is no CPU fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"libmcrt.so not found at {LIB_PATH}; build it with "
                "`python montecarloradiativetransfer.jl_gb300/build.py`")
        L = C.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = C.c_char_p if name == "mcrt_last_error" else C.c_int
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != MCRT_OK:
        raise MCRTError(rc, lib().mcrt_last_error().decode("utf-8", "replace"))


def dptr(a):
    """Pointer to a contiguous float64 numpy array (or None)."""
    if a is None:
        return None
    return a.ctypes.data_as(_dp)
