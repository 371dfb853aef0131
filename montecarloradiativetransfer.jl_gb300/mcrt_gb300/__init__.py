"""GB300 engine for polarised Monte Carlo radiative transfer with coherent
backscattering — the host-side mirror of MonteCarloRadiativeTransfer.jl's types and
driver, running the transport in libmcrt (hand-written CUDA for sm_103a).

    from mcrt_gb300 import Config, RayleighScatterer, Layer, PlaneGeometry, simulate
"""
from ._lib import MCRTError, LIB_PATH, lib
from .engine import (Batch, Context, DeviceMieScatterer, Server, Solve, default_context, run_opts, run_rt, simulate,
                     simulate_to_stderr, write_csv)
from .model import (DEFAULT_THEB, Config, Layer, MieScatterer, PlaneGeometry, RayleighScatterer,
                    SphereGeometry, mean_free_path, single_scattering_albedo)

__all__ = [
    "Batch", "Config", "Context", "DEFAULT_THEB", "DeviceMieScatterer", "Layer", "LIB_PATH", "MCRTError", "MieScatterer",
    "PlaneGeometry", "RayleighScatterer", "Server", "Solve", "SphereGeometry", "default_context", "lib",
    "mean_free_path", "run_opts", "run_rt", "simulate", "simulate_to_stderr", "single_scattering_albedo",
    "write_csv",
]
