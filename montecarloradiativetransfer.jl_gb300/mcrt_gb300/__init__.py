"""GB300 engine for polarised Monte Carlo radiative transfer with coherent
backscattering — the host-side mirror of MonteCarloRadiativeTransfer.jl's types and
driver, running the transport in libmcrt (hand-written CUDA for sm_103a).

    from mcrt_gb300 import Config, RayleighScatterer, Layer, PlaneGeometry, simulate
"""
from ._lib import MCRTError, LIB_PATH, lib
from .engine import (Batch, Context, DeviceMieScatterer, Server, Solve, cb_peak_batch_means, default_context,
                     peak_error_estimates, run_opts, run_rt, simulate, simulate_to_stderr, write_arrow,
                     write_csv)
from .model import (DEFAULT_THEB, Config, Layer, MieScatterer, PlaneGeometry, RayleighScatterer,
                    SphereGeometry, mean_free_path, single_scattering_albedo)

__all__ = [
    "Batch", "cb_peak_batch_means", "Config", "Context", "default_context", "DEFAULT_THEB",
    "DeviceMieScatterer", "Layer", "lib", "LIB_PATH", "MCRTError", "mean_free_path", "MieScatterer",
    "peak_error_estimates", "PlaneGeometry", "RayleighScatterer", "run_opts", "run_rt", "Server", "simulate",
    "simulate_to_stderr", "single_scattering_albedo", "Solve", "SphereGeometry", "write_arrow", "write_csv",
]
