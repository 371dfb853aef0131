"""GPU parity tests: the CUDA kernels (through the C ABI) against the CPU oracle.

Tolerances (scaled errors as defined in helpers.scaled_err):
  * FP64 kernels vs the FP64 oracle on identical Philox streams: 1e-9 on every tally
    (both restate the same arithmetic; only rounding order differs).
  * FP32 persistent kernel vs its FP64 form on identical streams: 1e-4 on every tally.
  * Independent streams: the oracle's per-element z against the GPU's batch means (mean
    z^2 and max z per tally, and the CB enhancement) inside the distribution of the same
    scores for 199 GPU estimates of equal size on independent photon ranges.
  * First scattering order vs the analytic single-scattering slab result: 1e-6 (FP64),
    1e-5 (FP32).
"""
import math

import numpy as np
import pytest

from helpers import calibrated_independent_streams, cb_peak_stats, reciprocity_z, scaled_err, sim_arrays

pytestmark = pytest.mark.gpu
N0 = [1.0, 0.0, 0.0, 0.0]


def small_cfg(M, g, n, **kw):
    kw.setdefault("Ntheta", 16)
    kw.setdefault("Nphi", 8)
    kw.setdefault("Nphib", 4)
    kw.setdefault("thetab", np.deg2rad(np.linspace(0, 3, 12)))
    kw.setdefault("maximum_scattering_times", 500)
    return M.Config(g, number_of_rays=n, **kw)


def geometry(M, case, mie5, mie2):
    ray = M.RayleighScatterer(0.99, 100.0)
    if case in ("plane_rayleigh", "plane_rayleigh_nphi4", "plane_rayleigh_full_bins", "plane_rayleigh_uneven_phi",
                "plane_rayleigh_short_tau0"):
        return M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=5 * ray.kl, scatterer=ray)]), N0
    if case == "plane_rayleigh_V":
        return M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=5 * ray.kl, scatterer=ray)]), [1, 0, 0, -1]
    if case in ("plane_mie_oblique", "plane_mie_short_tau0", "plane_mie_ragged_bins"):
        return M.PlaneGeometry(math.radians(150), 0.4, [M.Layer(d=3 * mie5.kl, scatterer=mie5)]), [1, 0, 1, 0]
    if case == "sphere_rayleigh":
        return M.SphereGeometry(R=3 * ray.kl, scatterer=ray), [1, 0, 0, -1]
    if case == "sphere_mie":
        return M.SphereGeometry(R=6 * mie2.kl, scatterer=mie2), N0
    if case == "two_layers":
        return M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=1 * ray.kl, scatterer=ray),
                                              M.Layer(d=2 * mie5.kl, scatterer=mie5)]), N0
    if case == "two_layers_rayleigh":  # Fourier RT tally across layers of different albedo
        ray2 = M.RayleighScatterer(0.9, 50.0)
        return M.PlaneGeometry(math.radians(160), 0.7, [M.Layer(d=1 * ray.kl, scatterer=ray),
                                                        M.Layer(d=2 * ray2.kl, scatterer=ray2)]), [1, 0, 1, 0]
    if case == "semi_infinite":
        return M.PlaneGeometry(math.radians(170), 0.0, [M.Layer(d=1 * ray.kl, scatterer=ray),
                                                        M.Layer(d=-1.0, scatterer=ray, tau=math.inf)]), [1, 1, 0, 0]
    raise ValueError(case)


CASES = ["plane_rayleigh", "plane_rayleigh_V", "plane_mie_oblique", "sphere_mie", "two_layers", "semi_infinite",
         "plane_rayleigh_nphi4", "plane_rayleigh_full_bins", "plane_rayleigh_uneven_phi", "two_layers_rayleigh",
         "plane_rayleigh_short_tau0", "plane_mie_short_tau0", "sphere_rayleigh", "plane_mie_ragged_bins"]
# Bin grids other than small_cfg's. A slab of Rayleigh scatterers tallies RT through
# azimuthal Fourier modes when Nphi >= 5; Nphi = 4 keeps the per-bin evaluation, and the
# full grid is the reference's default (64 x 48 RT bins).
CASE_BINS = {"plane_rayleigh_nphi4": {"Nphi": 4}, "plane_rayleigh_full_bins": {"Ntheta": 64, "Nphi": 48},
             # an irregular azimuth grid: the Fourier tally is expanded at the given angles
             "plane_rayleigh_uneven_phi": {"Nphi": 7, "phi": [0.0, 0.3, 1.1, 2.0, 3.5, 4.4, 6.0]},
             # tau0 below the slab depth: the peel-off and CB cut-offs (t <= tau0) decide many bins
             "plane_rayleigh_short_tau0": {"tau0": 0.7}, "plane_mie_short_tau0": {"tau0": 0.7},
             # grids that leave lanes and bin pairs partly empty in every tile
             "plane_mie_ragged_bins": {"Ntheta": 10, "Nphi": 3, "Nphib": 3,
                                       "thetab": np.deg2rad([0.0, 0.4, 1.1, 1.9, 2.5])}}


@pytest.mark.parametrize("case", CASES)
def test_fp64_kernels_match_oracle_on_same_streams(M, O, gpu_ctx, mie5, mie2, case):
    g, I0 = geometry(M, case, mie5, mie2)
    cfg = small_cfg(M, g, 600, **CASE_BINS.get(case, {}))
    n = cfg.number_of_rays
    ref = O.simulate(cfg, g, I0, seed=21, threads=0)
    for kernel in ("persistent", "plain"):
        out = M.simulate(cfg, g, I0, precision="fp64", kernel=kernel, seed=21, with_extras=True)
        A, Irt, Icb = sim_arrays(out)
        st = out[7]["stats"]
        assert st["status_flags"] & 5 == 0
        assert st["photons"] == n
        assert st["events"] == ref["counters"]["events"], kernel
        assert scaled_err(A, ref["A"] / n) < 1e-9, kernel
        assert scaled_err(Irt, ref["Irt"] / n) < 1e-9, kernel
        assert scaled_err(Icb, ref["Icb"] / n) < 1e-9, kernel
        assert scaled_err(out[7]["ladder"], ref["ladder"] / n) < 1e-9, kernel
        if ref["stats"]["cb_peak_sum"] != 0:
            assert abs(st["cb_peak_sum"] / ref["stats"]["cb_peak_sum"] - 1) < 1e-9
        assert abs(A.sum() - 1) < 1e-12


@pytest.mark.parametrize("case", ["plane_rayleigh", "plane_mie_oblique", "sphere_mie", "plane_rayleigh_full_bins",
                                  "plane_mie_short_tau0", "plane_mie_ragged_bins"])
def test_fp32_matches_fp64_on_same_streams(M, gpu_ctx, mie5, mie2, case):
    g, I0 = geometry(M, case, mie5, mie2)
    cfg = small_cfg(M, g, 1 << 14, **CASE_BINS.get(case, {}))
    o64 = M.simulate(cfg, g, I0, precision="fp64", seed=5, with_extras=True)
    o32 = M.simulate(cfg, g, I0, precision="fp32", seed=5, with_extras=True)
    A64, R64, C64 = sim_arrays(o64)
    A32, R32, C32 = sim_arrays(o32)
    errs = {"A": scaled_err(A32, A64), "Irt": scaled_err(R32, R64), "Icb": scaled_err(C32, C64),
            "ladder": scaled_err(o32[7]["ladder"], o64[7]["ladder"])}
    print(case, "FP32 vs FP64 scaled errors:", errs)
    for k, e in errs.items():
        assert e < 1e-4, (k, e)
    assert abs(A32.sum() - 1) < 1e-5


def _batch_means(M, cfg, g, I0, prec, seed, nb):
    """nb independent sub-runs on consecutive photon ranges of one stream."""
    n = cfg.number_of_rays
    s = M.Solve(cfg, g, I0, precision=prec, seed=seed)
    outs = []
    for b in range(nb):
        s.launch(b * n, n)
        r = s.read()
        outs.append((r["Irt"] / n, r["Icb"] / n, r["ladder"] / n))
    s.close()
    return [np.array([o[i] for o in outs]) for i in range(3)]


def test_statistics_agree_with_oracle_on_independent_streams(M, O, gpu_ctx):
    """A small Rayleigh slab: the oracle on its own Philox streams against the GPU's batch
    means, calibrated by 199 GPU estimates of the oracle's sample size
    (helpers.calibrated_independent_streams)."""
    ray = M.RayleighScatterer(0.99, 100.0)
    g = M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=4 * ray.kl, scatterer=ray)])
    cfg = small_cfg(M, g, 2000)
    pv = calibrated_independent_streams(M, O, cfg, g, N0, 2000, 8000, label="small rayleigh slab")
    for k, p in pv.items():
        assert p > 1.0 / 200, (k, p)


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-6), ("fp32", 1e-5)])
def test_first_order_matches_analytic_single_scattering(M, gpu_ctx, prec, tol):
    ray = M.RayleighScatterer(0.9, 1.0)
    g = M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=1.0, scatterer=ray)])
    cfg = small_cfg(M, g, 1 << 16, maximum_scattering_times=1)
    out = M.simulate(cfg, g, N0, precision=prec, seed=3, rng_mode=1)
    got = out[5][0]
    tau, mu0 = 1.0, 1.0
    exp = np.zeros_like(got)
    for j1 in range(cfg.Ntheta):
        mu = cfg.costheta[j1]
        c = -mu  # cos of the scattering angle for normal incidence
        if mu > 0:
            f = mu * (1 - math.exp(-tau * (1 / mu0 + 1 / mu))) / (mu + mu0)
        else:
            a = 1 - mu0 / -mu
            f = math.exp(-tau / -mu) * (1 - math.exp(-tau / mu0 * a)) / a
        exp[j1, :] = 0.9 * 0.75 * (1 + c * c) * cfg.inorm[j1] * f
    assert np.max(np.abs(got - exp) / exp) < tol
    cb = out[6][0, 0, 0]
    assert abs(cb / (0.9 * 1.5 * (1 - math.exp(-2.0)) / 2) - 1) < tol


def test_batch_matches_individual_solves(M, gpu_ctx, mie5, mie2):
    ray = M.RayleighScatterer(0.95, 50.0)
    geos = [(M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=2 * ray.kl, scatterer=ray)]), N0, 3000),
            (M.PlaneGeometry(math.radians(140), 1.0, [M.Layer(d=1 * mie5.kl, scatterer=mie5)]), [1, 0, 0, 1], 500),
            (M.SphereGeometry(R=2 * mie2.kl, scatterer=mie2), N0, 1200),
            (M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=0.3 * ray.kl, scatterer=ray)]), [1, -1, 0, 0], 7)]
    cfg = small_cfg(M, geos[0][0], 1)
    inst = [{"geometry": g, "I0": I, "n_photons": n, "seed": 40 + i, "instance": i}
            for i, (g, I, n) in enumerate(geos)]
    b = M.Batch(cfg, inst, precision="fp64")
    b.launch()
    for i, (g, I, n) in enumerate(geos):
        r = b.read(i)
        # the batch shares the config's bin grids, so the solo run reuses the same arrays
        solo = M.simulate(cfg.replace(number_of_rays=n), g, I, precision="fp64", seed=40 + i,
                          instance=i, with_extras=True)
        assert r["stats"]["photons"] == n
        assert scaled_err(r["A"] / n, np.array(solo[:5])) < 1e-12
        assert scaled_err(r["Irt"] / n, solo[5]) < 1e-12
        assert scaled_err(r["Icb"] / n, solo[6]) < 1e-12
    b.close()


def test_edge_cases(M, gpu_ctx, mie5):
    ray = M.RayleighScatterer(0.99, 10.0)
    g = M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=3 * ray.kl, scatterer=ray)])
    # zero photons: all-zero tallies
    out = M.simulate(small_cfg(M, g, 0), g, N0, with_extras=True)
    assert np.all(np.array(out[:5]) == 0) and not np.any(out[5]) and not np.any(out[6])
    # one photon and an odd count
    for n in (1, 37):
        out = M.simulate(small_cfg(M, g, n), g, N0, precision="fp64", with_extras=True)
        assert abs(sum(out[:5]) - 1) < 1e-12 and out[7]["stats"]["photons"] == n
    # no CB: the CB tallies stay zero, RT unchanged
    a = M.simulate(small_cfg(M, g, 300), g, N0, precision="fp64", seed=4)
    b = M.simulate(small_cfg(M, g, 300, compute_cb=False), g, N0, precision="fp64", seed=4)
    assert not np.any(b[6]) and scaled_err(b[5], a[5]) < 1e-12
    # no scattering allowed: only direct transmission and the remaining weight
    out = M.simulate(small_cfg(M, g, 100, maximum_scattering_times=0), g, N0, precision="fp64")
    assert out[1] == 0 and out[2] == 0 and not np.any(out[5])
    assert abs(out[0] - math.exp(-3)) < 1e-12 and abs(out[4] - (1 - math.exp(-3))) < 1e-12
    # optically very thin and very thick slabs (tau beyond tau0 disables the lower peel-off)
    for tau in (0.01, 60.0):
        gt = M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=tau * ray.kl, scatterer=ray)])
        out = M.simulate(small_cfg(M, gt, 200), gt, N0, precision="fp64", with_extras=True)
        assert abs(sum(out[:5]) - 1) < 1e-12
        assert out[7]["stats"]["status_flags"] & 5 == 0
    # invalid input is rejected with the reference's message
    bad = M.PlaneGeometry(1.0, 0.0, [M.Layer(d=1.0, scatterer=ray)])
    with pytest.raises(ValueError, match="θ must be in"):
        M.simulate(small_cfg(M, g, 10), bad, N0)


@pytest.mark.parametrize("prec,kernel", [("fp32", "persistent"), ("fp64", "persistent"), ("fp64", "plain")])
def test_rejection_cap_is_reported_and_the_context_survives(M, gpu_ctx, prec, kernel):
    """Failure injected from the host: a rejection-loop cap of one attempt makes every
    rejected free path hit the cap. The kernel ends those photons, sets
    MCRT_FLAG_REJECT_LIMIT and returns; the call reports MCRT_ENONCONV; the device stays
    usable for the next call."""
    ray = M.RayleighScatterer(0.99, 10.0)
    g = M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=0.3 * ray.kl, scatterer=ray)])
    cfg = small_cfg(M, g, 500)
    with pytest.raises(M.MCRTError, match="rejection loop hit its iteration cap"):
        M.simulate(cfg, g, N0, precision=prec, kernel=kernel, seed=3, max_attempts=1)
    out = M.simulate(cfg, g, N0, precision=prec, kernel=kernel, seed=3, with_extras=True)
    assert out[7]["stats"]["status_flags"] & 5 == 0
    assert abs(sum(out[:5]) - 1) < 1e-5


def test_full_size_workload_properties(M, gpu_ctx, mie5):
    """At the benchmark workload's size: size-independent properties of the result."""
    g = M.PlaneGeometry(math.radians(150), 0.0, [M.Layer(d=5 * mie5.kl, scatterer=mie5)])
    cfg = M.Config(g, number_of_rays=1 << 21)
    out = M.simulate(cfg, g, N0, precision="fp32", seed=2, with_extras=True)
    A = np.array(out[:5])
    st = out[7]["stats"]
    assert abs(A.sum() - 1) < 1e-5
    assert st["photons"] == cfg.number_of_rays and st["status_flags"] & 5 == 0
    assert np.all(np.isfinite(out[5])) and np.all(np.isfinite(out[6]))
    assert np.all(out[5][0] >= 0) and np.all(out[7]["ladder"] >= 0)
    enh = out[6][0, 0, 0] / out[7]["ladder"][0, 0]
    assert 1.0 < enh <= 2.0
    mu, sd = cb_peak_stats(st)
    assert mu > 0 and abs(mu - out[6][0, 0, 0]) < 1e-6 * mu
    # splitting the photons into two launches on the same stream gives the same sums
    s = M.Solve(cfg, g, N0, precision="fp32", seed=2)
    half = cfg.number_of_rays // 2
    s.launch(0, half)
    r1 = s.read()
    s.launch(half, half)
    r2 = s.read()
    s.close()
    tot = (r1["Irt"] + r2["Irt"]) / cfg.number_of_rays
    assert scaled_err(tot, out[5]) < 1e-6


@pytest.mark.parametrize("geom", ["plane_rayleigh", "plane_mie", "sphere_mie"])
def test_run_rt_matches_per_state_simulate(M, gpu_ctx, mie5, mie2, geom):
    """mcrt_run_rt (one batched launch + device Mueller assembly) against the numpy
    restatement of run_rt fed by one FP64 simulate per incident state on the same
    Philox streams."""
    from helpers import assemble_run_rt, table_of

    ray = M.RayleighScatterer(0.99, 100.0)
    if geom == "plane_rayleigh":
        g = M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=2 * ray.kl, scatterer=ray)])
    elif geom == "plane_mie":
        g = M.PlaneGeometry(math.radians(160), 0.3, [M.Layer(d=2 * mie5.kl, scatterer=mie5)])
    else:
        g = M.SphereGeometry(R=2 * mie2.kl, scatterer=mie2)
    cfg = small_cfg(M, g, 2000)
    plane = g.kind == 0
    sm_rt, sm_cb, energy, st = M.run_rt(cfg, g, seed=9, precision="fp64", with_stats=True)
    assert st["status_flags"] & 5 == 0
    assert st["photons"] == cfg.number_of_rays * (6 if plane else 2)

    def sim(I, i):
        return M.simulate(cfg, g, I, seed=9, instance=i, precision="fp64")

    MRT, MCB, G = assemble_run_rt(cfg, g, sim)
    ref_rt, ref_cb = table_of(MRT, plane), table_of(MCB, plane)
    scale_rt = max(np.max(np.abs(v)) for v in ref_rt.values())
    scale_cb = max(np.max(np.abs(v)) for v in ref_cb.values())
    for k in ref_rt:
        assert np.max(np.abs(sm_rt[k] - ref_rt[k])) <= 1e-9 * scale_rt, k
        assert np.max(np.abs(sm_cb[k] - ref_cb[k])) <= 1e-9 * scale_cb, k
    E = [energy["direct_transmission"], energy["absorption"], energy["reflection"],
         energy.get("transmission", 0.0), energy["remaining"]]
    assert np.allclose(E, G, rtol=1e-12, atol=1e-15)
    assert np.all(np.isfinite(sm_rt["s11"]))
    if plane:
        s11 = sm_rt["s11"].reshape(cfg.Nphi, cfg.Ntheta).T
        assert np.all(s11[cfg.costheta > 0] > 0)
        assert abs(sum(energy.values()) - 1) < 1e-9
    else:
        assert np.all(sm_rt["s11"] > 0)


def test_simulate_to_stderr_stops_at_the_target_and_equals_one_run(M, gpu_ctx):
    """The 1% stopping rule of the CB-peak metric: consecutive launches on one Philox
    stream until the per-path standard error of the CB peak reaches the target; the sum
    equals one simulate() of the same photons."""
    ray = M.RayleighScatterer(0.99, 100.0)
    g = M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=3 * ray.kl, scatterer=ray)])
    cfg = small_cfg(M, g, 1)
    res, info = M.simulate_to_stderr(cfg, g, N0, rel_err=0.02, batch=2048, precision="fp64", seed=12)
    assert info["rel_err"] <= 0.02 and info["launches"] >= 1
    assert info["photons"] == 2048 * info["launches"]
    one = M.simulate(cfg.replace(number_of_rays=info["photons"]), g, N0, precision="fp64", seed=12)
    A, Irt, Icb = sim_arrays(res)
    A1, Irt1, Icb1 = sim_arrays(one)
    assert scaled_err(A, A1) < 1e-9 and scaled_err(Irt, Irt1) < 1e-9 and scaled_err(Icb, Icb1) < 1e-9


def test_simulate_to_stderr_resumes_from_a_checkpoint(M, gpu_ctx):
    """A run stopped early and resumed from its checkpoint equals one uninterrupted run."""
    ray = M.RayleighScatterer(0.99, 100.0)
    g = M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=3 * ray.kl, scatterer=ray)])
    cfg = small_cfg(M, g, 1)
    _, first = M.simulate_to_stderr(cfg, g, N0, rel_err=1e-9, batch=1024, max_photons=2048,
                                    precision="fp64", seed=7)
    assert first["photons"] == 2048
    saved = {k: np.array(v) for k, v in first["state"].items()}  # what numpy.savez would keep
    res, info = M.simulate_to_stderr(cfg, g, N0, rel_err=1e-9, batch=1024, max_photons=4096,
                                     precision="fp64", seed=7, state=saved)
    assert info["photons"] == 4096
    one = M.simulate(cfg.replace(number_of_rays=4096), g, N0, precision="fp64", seed=7)
    A, Irt, Icb = sim_arrays(res)
    A1, Irt1, Icb1 = sim_arrays(one)
    assert scaled_err(A, A1) < 1e-9 and scaled_err(Irt, Irt1) < 1e-9 and scaled_err(Icb, Icb1) < 1e-9


def test_cb_peak_batch_means_agree_with_the_per_path_error(M, gpu_ctx):
    """The CB peak's standard error from batch means over 32 photon sub-ranges against
    the per-path estimate: their ratio follows sqrt(chi2_31 / 31), inside [0.39, 1.77]
    with probability 1 - 2e-8. The sub-ranges tile one stream, so the mean equals one
    simulate() of all their photons."""
    ray = M.RayleighScatterer(0.99, 100.0)
    g = M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=3 * ray.kl, scatterer=ray)])
    cfg = small_cfg(M, g, 1)
    r = M.cb_peak_batch_means(cfg, g, N0, batches=32, photons_per_batch=2048, precision="fp64", seed=4)
    mu = r["mean_per_path"]
    assert mu > 0 and 0.39 < r["rel_err_batch_means"] / r["rel_err_per_path"] < 1.77
    one = M.simulate(cfg.replace(number_of_rays=32 * 2048), g, N0, precision="fp64", seed=4)
    assert abs(mu - one[6][0, 0, 0]) < 1e-9 * mu


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_plane_reflection_is_reciprocal(M, gpu_ctx, mie5, prec):
    """Reciprocity of the plane reflection matrix (s11, unpolarised light) on the Mie
    scatterer x = 5 in a slab of tau = 1, all orders: 8 incidence nodes, 28 node pairs x
    48 azimuths, batch means over 16 independent seeds per incidence.

    The reference lowers a photon's weight after each event by the escape probability
    that its bin quadrature estimates (src/gpu.jl:285-294). With a forward-peaked Mie
    phase function, 8 azimuths estimate it poorly at grazing angles: grazing reflection
    is then off by about 10% at mu = 0.02, and reciprocity fails in the oracle as well.
    The reference's default 48 azimuths make that error small against the noise here."""
    n = 4096

    def cfg_for(g):
        return small_cfg(M, g, n, Nphi=48)

    def run(theta, seed):
        g = M.PlaneGeometry(theta, 0.0, [M.Layer(d=1.0 * mie5.kl, scatterer=mie5)])
        cfg = cfg_for(g)
        return cfg, M.simulate(cfg, g, N0, precision=prec, seed=seed)[5]

    g0 = M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=1.0 * mie5.kl, scatterer=mie5)])
    z = reciprocity_z(run, cfg_for(g0).costheta, 16)
    assert z.size == 28 * 48
    assert np.max(np.abs(z)) < 5.5 and np.mean(np.abs(z) > 3.0) < 0.03
