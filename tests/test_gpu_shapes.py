"""Parity of every compiled launch shape of the persistent kernel, forced past the
autotuner: FP32 with 128, 256 (one and two blocks per SM), 512 and 768 threads per
block; FP64 with 128 (one and two blocks per SM) and 256; Mie tables staged in shared
memory and read from global memory through L1. Each shape runs a Mie slab at oblique
incidence with polarised light, a Mie sphere, and a Rayleigh slab (whose RT tally takes
the azimuthal Fourier path), small enough that the oracle finishes in seconds.

Gates: FP64 shapes against the oracle on identical Philox streams at 1e-9 of the tally
scale; FP32 shapes against the oracle on the same streams at 1e-4 of the scale (the
FP32 transport's stated bound)."""
import math

import numpy as np
import pytest

from helpers import scaled_err, sim_arrays

pytestmark = pytest.mark.gpu

SHAPES = [("fp32", 128, 4), ("fp32", 256, 1), ("fp32", 256, 2), ("fp32", 512, 1), ("fp32", 768, 1),
          ("fp64", 128, 1), ("fp64", 128, 2), ("fp64", 256, 1)]


def cases(M, mie5, mie2):
    ray = M.RayleighScatterer(0.99, 100.0)
    th = np.deg2rad(np.linspace(0.0, 3.0, 12))
    out = []
    g = M.PlaneGeometry(math.radians(150), 0.4, [M.Layer(d=3 * mie5.kl, scatterer=mie5)])
    out.append(("mie_slab", g, [1.0, 0.0, 1.0, 0.0], M.Config(g, number_of_rays=700, Ntheta=16, Nphi=8, Nphib=4,
                                                              thetab=th, maximum_scattering_times=500)))
    g = M.SphereGeometry(R=4 * mie2.kl, scatterer=mie2)
    out.append(("mie_sphere", g, [1.0, 0.0, 0.0, -1.0], M.Config(g, number_of_rays=500, Ntheta=16, Nphi=8,
                                                                 Nphib=4, thetab=th,
                                                                 maximum_scattering_times=500)))
    g = M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=4 * ray.kl, scatterer=ray)])
    out.append(("rayleigh_slab", g, [1.0, 0.0, 0.0, 0.0], M.Config(g, number_of_rays=900, Ntheta=16, Nphi=12,
                                                                   Nphib=4, thetab=th,
                                                                   maximum_scattering_times=500)))
    return out


@pytest.fixture(scope="module")
def references(M, O, mie5, mie2):
    return {name: O.simulate(cfg, g, I0, seed=17, threads=0) for name, g, I0, cfg in cases(M, mie5, mie2)}


@pytest.mark.parametrize("prec,bs,bps", SHAPES)
@pytest.mark.parametrize("staging", ["shared", "global"])
def test_every_launch_shape_matches_the_oracle(M, gpu_ctx, mie5, mie2, references, prec, bs, bps, staging):
    tol = 1e-9 if prec == "fp64" else 1e-4
    for name, g, I0, cfg in cases(M, mie5, mie2):
        if staging == "global" and name == "rayleigh_slab":
            continue  # no tables to stage
        ref = references[name]
        n = cfg.number_of_rays
        out = M.simulate(cfg, g, I0, precision=prec, seed=17, block_size=bs, blocks_per_sm=bps,
                         table_staging=staging, with_extras=True)
        st = out[7]["stats"]
        assert st["block_size"] == bs, (st["block_size"], bs)
        assert st["status_flags"] & 5 == 0 and st["photons"] == n
        A, Irt, Icb = sim_arrays(out)
        errs = {"A": scaled_err(A, ref["A"] / n), "Irt": scaled_err(Irt, ref["Irt"] / n),
                "Icb": scaled_err(Icb, ref["Icb"] / n), "ladder": scaled_err(out[7]["ladder"], ref["ladder"] / n)}
        for k, e in errs.items():
            assert e < tol, (name, prec, bs, bps, staging, k, e)
        if prec == "fp64":
            assert st["events"] == ref["counters"]["events"], (name, bs, bps, staging)
