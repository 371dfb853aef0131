"""GPU parity on the benchmark configurations at their own parameters and bin grids:

  * Rayleigh slab: omega 0.99, kl 100, tau 10, normal incidence, Ntheta 180, 200 CB
    phase angles over 0-2 degrees, Nphi 48, Nphi_b 8, at most 1000 orders;
  * Mie slab: x 5, m 1.5+0.001i, 1801-angle tables, tau 5, incidence zenith 30 degrees,
    the reference's default grids (Ntheta 64, Nphi 48, 51 CB angles, Nphi_b 8);
  * Mie sphere: tau 20, x 2, m 1.31, 500 CB phase angles over 0-5 degrees, default
    Ntheta and Nphi.

For each, three comparisons against the oracle (the CPU restatement of the reference's
src/cpu.jl:162-273, with the CB bin body of src/gpu.jl:41-175):
  (a) the FP64 persistent and FP64 plain kernels on identical Philox streams: 1e-9 of
      the tally scale on every element of every tally, and 1e-8 relative on every
      element above 1e-6 of the scale;
  (b) the FP32 kernel against the FP64 kernel on identical streams: 1e-4 of the tally
      scale on every tally; the per-element relative error above floors of 1e-3 and 1e-2
      of the scale is printed (noise-limited on small elements, gated loosely at 2e-2
      above the 1e-2 floor). The Mie slab runs 2^17 photons; FP64 on this GPU runs at
      about 1/64 of the FP32 rate, so the long-path Rayleigh slab (850 FP64 paths/s) and
      Mie sphere (270 FP64 paths/s) run 2^14 and 2^15. On identical streams the
      difference is dominated by the few paths whose FP32 and FP64 forms take different
      branches (a boundary test or the termination threshold decided the other way) and
      are independent samples from then on, so it falls as N^-1/2;
  (c) independent streams: the oracle's estimate scored element by element against the
      GPU's batch means (16 batches), with the score's null distribution calibrated by
      199 GPU estimates of the same size on independent photon ranges (the docstring of
      helpers.calibrated_independent_streams says why a fixed per-element sigma rule is
      not valid here); also every batch finite and the CB enhancement factor in (1, 2].
  (d) run_rt: the device Mueller assembly of all incident polarisation states against the
      same assembly of the oracle's per-state results, 1e-9.

The Mie tables come from the oracle's own bhmie and calculate_csrn (tests/conftest.py).
"""
import math

import numpy as np
import pytest

from helpers import calibrated_independent_streams, per_element_err, scaled_err, sim_arrays

pytestmark = pytest.mark.gpu
N0 = [1.0, 0.0, 0.0, 0.0]


def workload(M, name, mie5, mie2, n):
    if name == "rayleigh_slab":
        ray = M.RayleighScatterer(0.99, 100.0)
        g = M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=10.0 * ray.kl, scatterer=ray)])
        return g, M.Config(g, number_of_rays=n, Ntheta=180, thetab=np.deg2rad(np.linspace(0.0, 2.0, 200)),
                           maximum_scattering_times=1000)
    if name == "mie_slab":
        g = M.PlaneGeometry(math.radians(150.0), 0.0, [M.Layer(d=5.0 * mie5.kl, scatterer=mie5)])
        return g, M.Config(g, number_of_rays=n)
    if name == "mie_sphere":
        g = M.SphereGeometry(R=20.0 * mie2.kl, scatterer=mie2)
        return g, M.Config(g, number_of_rays=n, thetab=np.deg2rad(np.linspace(0.0, 5.0, 500)))
    raise ValueError(name)


NAMES = ["rayleigh_slab", "mie_slab", "mie_sphere"]
# photons of the identical-stream comparison: persistent kernel, plain kernel (one
# thread per photon, FP64: the long Rayleigh-slab and sphere paths keep it short)
SAME_STREAM = {"rayleigh_slab": (128, 32), "mie_slab": (512, 128), "mie_sphere": (128, 32)}
# photons of the FP32-against-FP64 comparison
FP32_VS_FP64 = {"rayleigh_slab": 1 << 14, "mie_slab": 1 << 17, "mie_sphere": 1 << 15}
# independent streams: (GPU photons per batch, oracle photons)
INDEPENDENT = {"rayleigh_slab": (1 << 14, 1024), "mie_slab": (1 << 16, 8192), "mie_sphere": (1 << 14, 768)}


@pytest.mark.parametrize("name", NAMES)
def test_fp64_kernels_match_the_oracle_on_identical_streams(M, O, gpu_ctx, mie5, mie2, name):
    n_pers, n_plain = SAME_STREAM[name]
    for kernel, n in (("persistent", n_pers), ("plain", n_plain)):
        g, cfg = workload(M, name, mie5, mie2, n)
        ref = O.simulate(cfg, g, N0, seed=31, threads=0)
        out = M.simulate(cfg, g, N0, precision="fp64", kernel=kernel, seed=31, with_extras=True)
        A, Irt, Icb = sim_arrays(out)
        st = out[7]["stats"]
        assert st["status_flags"] & 5 == 0 and st["photons"] == n
        assert st["events"] == ref["counters"]["events"], (kernel, st["events"], ref["counters"]["events"])
        pairs = {"A": (A, ref["A"] / n), "Irt": (Irt, ref["Irt"] / n), "Icb": (Icb, ref["Icb"] / n),
                 "ladder": (out[7]["ladder"], ref["ladder"] / n)}
        for k, (a, b) in pairs.items():
            assert scaled_err(a, b) < 1e-9, (name, kernel, k, scaled_err(a, b))
            e, used, total, _ = per_element_err(a, b, 1e-6)
            assert e < 1e-8, (name, kernel, k, e, used, total)
        assert abs(st["cb_peak_sum"] / ref["stats"]["cb_peak_sum"] - 1) < 1e-9
        assert abs(A.sum() - 1) < 1e-12


@pytest.mark.parametrize("name", NAMES)
def test_fp32_matches_fp64_on_identical_streams(M, gpu_ctx, mie5, mie2, name):
    n = FP32_VS_FP64[name]
    g, cfg = workload(M, name, mie5, mie2, n)
    o64 = M.simulate(cfg, g, N0, precision="fp64", seed=7, with_extras=True)
    o32 = M.simulate(cfg, g, N0, precision="fp32", seed=7, with_extras=True)
    A64, R64, C64 = sim_arrays(o64)
    A32, R32, C32 = sim_arrays(o32)
    pairs = {"A": (A32, A64), "Irt": (R32, R64), "Icb": (C32, C64), "ladder": (o32[7]["ladder"], o64[7]["ladder"])}
    report = {}
    for k, (a, b) in pairs.items():
        report[k] = {"scaled": scaled_err(a, b)}
        for floor in (1e-3, 1e-2):
            e, used, total, _ = per_element_err(a, b, floor)
            report[k][f"per_element_max_above_{floor:g}"] = e
            report[k][f"elements_above_{floor:g}"] = f"{used}/{total}"
    print(name, "FP32 vs FP64 on identical streams,", n, "photons:", report)
    for k, r in report.items():
        assert r["scaled"] < 1e-4, (name, k, r)
        # per element the difference is noise-limited on small elements (it is the
        # divergent paths' share of each element); a loose sanity bound above 1e-2 of
        # the scale
        assert r["per_element_max_above_0.01"] < 2e-2, (name, k, r)
    assert abs(A32.sum() - 1) < 1e-5
    assert o32[7]["stats"]["status_flags"] & 5 == 0


@pytest.mark.parametrize("name", NAMES)
def test_statistics_agree_with_the_oracle_on_independent_streams(M, O, gpu_ctx, mie5, mie2, name):
    """The oracle on its own Philox streams against the GPU's batch means, calibrated by 199
    GPU estimates of the oracle's sample size (helpers.calibrated_independent_streams)."""
    n_b, n_ref = INDEPENDENT[name]
    g, cfg = workload(M, name, mie5, mie2, n_b)
    pv = calibrated_independent_streams(M, O, cfg, g, N0, n_b, n_ref, label=name)
    for k, p in pv.items():
        assert p > 1.0 / 200, (name, k, p)


# photons per incident state for run_rt against the oracle (6 states on a slab, 2 on a sphere)
RUN_RT_PHOTONS = {"rayleigh_slab": 48, "mie_slab": 256, "mie_sphere": 96}


@pytest.mark.parametrize("name", NAMES)
def test_run_rt_matches_the_oracle_at_the_benchmark_grids(M, O, gpu_ctx, mie5, mie2, name):
    """run_rt (src/MonteCarloRadiativeTransfer.jl:87-291) as one batched FP64 launch with the
    Mueller assembly on the device (mcrt_run_rt), against the same assembly (the numpy
    restatement in helpers.assemble_run_rt) fed by the oracle's simulate of each incident
    polarisation state on the same Philox streams (state i is instance i): every Mueller
    element of the RT and CB tables and the energy budget at 1e-9 of their scale."""
    from helpers import assemble_run_rt, table_of

    n = RUN_RT_PHOTONS[name]
    g, cfg = workload(M, name, mie5, mie2, n)
    plane = g.kind == 0
    sm_rt, sm_cb, energy, st = M.run_rt(cfg, g, seed=41, precision="fp64", with_stats=True)
    assert st["status_flags"] & 5 == 0 and st["photons"] == n * (6 if plane else 2)

    def sim(I, i):
        r = O.simulate(cfg, g, I, seed=41, instance=i, threads=0)
        return tuple(r["A"] / n) + (r["Irt"] / n, r["Icb"] / n)

    MRT, MCB, G = assemble_run_rt(cfg, g, sim)
    ref_rt, ref_cb = table_of(MRT, plane), table_of(MCB, plane)
    scale_rt = max(np.max(np.abs(v)) for v in ref_rt.values())
    scale_cb = max(np.max(np.abs(v)) for v in ref_cb.values())
    for k in ref_rt:
        assert np.max(np.abs(sm_rt[k] - ref_rt[k])) <= 1e-9 * scale_rt, (name, "RT", k)
        assert np.max(np.abs(sm_cb[k] - ref_cb[k])) <= 1e-9 * scale_cb, (name, "CB", k)
    E = [energy["direct_transmission"], energy["absorption"], energy["reflection"],
         energy.get("transmission", 0.0), energy["remaining"]]
    assert np.allclose(E, G, rtol=1e-9, atol=1e-15)


def more_geometry(M, name, mie5, mie2):
    ray = M.RayleighScatterer(0.99, 100.0)
    if name == "two_layers":
        # Rayleigh over Mie: layer crossings, CB tied to layer 1. The upper layer is the
        # thicker: moving up, the reference resets z to minus the thickness of the layer
        # left (src/gpu.jl:238), which stays inside a thicker upper layer (a thinner one
        # gives negative boundary distances, and NaN at the grid's horizontal CB bins,
        # in the reference, the oracle and the kernels alike).
        return M.PlaneGeometry(math.radians(160), 0.5, [M.Layer(d=2.0 * ray.kl, scatterer=ray),
                                                        M.Layer(d=1.0 * mie5.kl, scatterer=mie5)]), [1, 0, 0, 1]
    if name == "semi_infinite":  # a finite layer over a semi-infinite one
        return M.PlaneGeometry(math.radians(140), 0.0, [M.Layer(d=0.5 * ray.kl, scatterer=ray),
                                                        M.Layer(d=-1.0, scatterer=mie5, tau=math.inf)]), [1, 1, 0, 0]
    if name == "sphere_circular":
        return M.SphereGeometry(R=8.0 * mie2.kl, scatterer=mie2), [1, 0, 0, -1]
    raise ValueError(name)


@pytest.mark.parametrize("name", ["two_layers", "semi_infinite", "sphere_circular"])
def test_fp64_and_fp32_on_more_geometries_at_default_grids(M, O, gpu_ctx, mie5, mie2, name):
    """Geometries beside the benchmark configurations, at the reference's default grids
    (Ntheta 64, Nphi 48, 51 CB angles, Nphi_b 8) and polarised incident light: the FP64
    kernel against the oracle on identical streams (1e-9 of the scale, equal event
    counts), and FP32 against FP64 (1e-4 of the scale)."""
    g, I0 = more_geometry(M, name, mie5, mie2)
    n = 256
    cfg = M.Config(g, number_of_rays=n, maximum_scattering_times=2000)
    ref = O.simulate(cfg, g, I0, seed=57, threads=0)
    out = M.simulate(cfg, g, I0, precision="fp64", seed=57, with_extras=True)
    A, Irt, Icb = sim_arrays(out)
    st = out[7]["stats"]
    assert st["status_flags"] & 5 == 0 and st["photons"] == n
    assert st["events"] == ref["counters"]["events"]
    for k, (a, b) in {"A": (A, ref["A"] / n), "Irt": (Irt, ref["Irt"] / n), "Icb": (Icb, ref["Icb"] / n),
                      "ladder": (out[7]["ladder"], ref["ladder"] / n)}.items():
        assert scaled_err(a, b) < 1e-9, (name, k, scaled_err(a, b))
    n32 = 1 << 14
    c32 = cfg.replace(number_of_rays=n32)
    o64 = M.simulate(c32, g, I0, precision="fp64", seed=58, with_extras=True)
    o32 = M.simulate(c32, g, I0, precision="fp32", seed=58, with_extras=True)
    for i, k in ((5, "Irt"), (6, "Icb")):
        assert scaled_err(o32[i], o64[i]) < 1e-4, (name, k, scaled_err(o32[i], o64[i]))
    assert scaled_err(o32[7]["ladder"], o64[7]["ladder"]) < 1e-4
