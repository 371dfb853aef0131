"""The device Mie table producer (mcrt_mie_scatterers_create) against the host one
(mcrt_mie_tables), both restating bhmie (src/scatterers/mie.jl:129-216) and
calculate_csrn (src/utils.jl:263-287).

Tolerance: 1e-10 of each table's scale. Both are FP64; they differ by the GPU's fused
multiply-adds, its elementary functions and complex division (Smith's algorithm here,
libgcc's on the host), i.e. by a few ulps propagated through the recurrences.
"""
import math
import time

import numpy as np
import pytest

from helpers import scaled_err, sim_arrays

pytestmark = pytest.mark.gpu

PARAMS = [  # (r, m, lambda, nu): x = 2 pi r / lambda
    (5.0 / (2 * math.pi), 1.5 + 0.001j, 1.0, 0.1),   # the Mie slab workload, x = 5
    (2.0 / (2 * math.pi), 1.31 + 0.0j, 1.0, 0.1),    # the sphere workload, x = 2
    (0.5 / (2 * math.pi), 1.33 + 1e-5j, 1.0, 0.2),   # small particle
    (30.0 / (2 * math.pi), 1.6 + 0.01j, 1.0, 0.05),  # large, absorbing
    (1.3, 1.45 + 0.1j, 0.9, 0.3),
]


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(b)))


@pytest.mark.parametrize("nt,rp", [(181, 1000), (1801, 1000), (64, 37)])
def test_device_tables_match_host_tables(M, gpu_ctx, nt, rp):
    dev = gpu_ctx.mie_scatterers(PARAMS, Ntheta=nt, random_points=rp, with_tables=True)
    for p, d in zip(PARAMS, dev):
        h = M.MieScatterer(p[0], p[1], p[2], p[3], Ntheta=nt, random_points=rp)
        assert abs(d.omega / h.omega - 1) < 1e-12, p
        assert abs(d.kl / h.kl - 1) < 1e-12, p
        for k in ("q_ext", "q_sca", "q_back", "asymm"):
            assert abs(getattr(d, k) - getattr(h, k)) <= 1e-11 * max(abs(getattr(h, k)), 1e-300), (p, k)
        for k in ("F11", "F12", "F33", "F34", "S11", "S22", "csrn"):
            assert rel(getattr(d, k), getattr(h, k)) < 1e-10, (p, k, rel(getattr(d, k), getattr(h, k)))


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-9), ("fp32", 1e-5)])
def test_simulate_with_device_tables_matches_host_tables(M, gpu_ctx, prec, tol):
    p = PARAMS[0]
    (dev,) = gpu_ctx.mie_scatterers([p], Ntheta=1801)
    host = M.MieScatterer(*p, Ntheta=1801)
    outs = []
    for sc in (dev, host):
        g = M.PlaneGeometry(math.radians(150.0), 0.2, [M.Layer(d=3 * sc.kl, scatterer=sc)])
        cfg = M.Config(g, number_of_rays=2000, Ntheta=16, Nphi=8, Nphib=4,
                       thetab=np.deg2rad(np.linspace(0, 3, 12)), maximum_scattering_times=500)
        outs.append(M.simulate(cfg, g, [1, 0, 0, 0], precision=prec, seed=13, ctx=gpu_ctx))
    (A1, R1, C1), (A2, R2, C2) = (sim_arrays(o) for o in outs)
    assert scaled_err(A1, A2) < tol
    assert scaled_err(R1, R2) < tol
    assert scaled_err(C1, C2) < tol


def test_a_batch_of_new_scatterers_in_one_launch(M, gpu_ctx):
    rng = np.random.default_rng(4)
    n = 256
    params = [(float(x) / (2 * math.pi), complex(rng.uniform(1.3, 1.6), 10 ** rng.uniform(-5, -2)), 1.0, 0.1)
              for x in rng.uniform(0.5, 10.0, n)]
    t0 = time.perf_counter()
    dev = gpu_ctx.mie_scatterers(params, Ntheta=1801, with_tables=True)
    t_dev = time.perf_counter() - t0
    t0 = time.perf_counter()
    host = [M.MieScatterer(*p, Ntheta=1801) for p in params[:16]]
    t_host = (time.perf_counter() - t0) * n / 16
    print(f"{n} Mie scatterers (1801 angles): device {t_dev * 1e3:.1f} ms, host (extrapolated) {t_host * 1e3:.1f} ms")
    for d, h in zip(dev[:16], host):
        assert rel(d.F11, h.F11) < 1e-10 and rel(d.csrn, h.csrn) < 1e-10
    assert all(0 < d.omega <= 1 and d.kl > 0 for d in dev)
