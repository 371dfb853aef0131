"""CPU tests of the library's host side: the exported C ABI, the Mie table producer,
Config defaults and quadratures, validation, and the run_rt Mueller assembly."""
import json
import math
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def header_symbols():
    text = open(os.path.join(ROOT, "include", "mcrt.h")).read()
    return sorted(set(re.findall(r"\b(mcrt_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(M):
    L = M.lib()
    syms = header_symbols()
    assert len(syms) >= 19
    for s in syms:
        assert hasattr(L, s), s
    assert set(syms) <= set(M._lib.SIGNATURES), "ctypes signatures missing for: %s" % (
        set(syms) - set(M._lib.SIGNATURES))
    assert L.mcrt_abi_version() == 1


def test_no_device_is_reported_not_faked(M):
    # Without a GPU the library must refuse to compute rather than fall back to a CPU path.
    L = M.lib()
    if L.mcrt_device_count() > 0:
        pytest.skip("a GPU is visible")
    import ctypes

    h = ctypes.c_void_p()
    assert L.mcrt_ctx_create(0, ctypes.byref(h)) == M._lib.MCRT_ENODEV
    with pytest.raises(M.MCRTError):
        M.Context(0)


@pytest.mark.parametrize("case", range(4))
def test_mie_tables_match_an_independent_mie_evaluation(M, case):
    c = json.load(open(os.path.join(GOLDEN, "mie_scipy.json")))[case]
    x, m = c["x"], complex(*c["m"])
    ang = np.array(c["angles_deg"])
    # Angles 0, 30, ..., 180 lie on the uniform grid of 7 points.
    s = M.MieScatterer(x / (2 * math.pi), m, 1.0, 0.1, Ntheta=7)
    assert np.allclose(np.rad2deg(np.linspace(0, math.pi, 7)), ang)
    assert abs(s.q_ext / c["q_ext"] - 1) < 1e-10
    assert abs(s.q_sca / c["q_sca"] - 1) < 1e-10
    assert abs(s.asymm / c["asymm"] - 1) < 1e-9
    S1 = np.array([complex(*v) for v in c["S1"]])
    S2 = np.array([complex(*v) for v in c["S2"]])
    assert np.max(np.abs(s.S11 - S1)) < 1e-10 * np.max(np.abs(S1))
    assert np.max(np.abs(s.S22 - S2)) < 1e-10 * np.max(np.abs(S2))
    assert abs(s.omega - c["q_sca"] / c["q_ext"]) < 1e-10  # mie.jl:39


def test_mie_phase_function_is_normalised_and_csrn_is_an_inverse_cdf(M):
    mie5 = M.MieScatterer(5.0 / (2 * math.pi), 1.5 + 0.001j, 1.0, 0.1, Ntheta=1801)  # the library's producer
    th = np.linspace(0, math.pi, mie5.Ntheta)
    assert abs(np.trapezoid(mie5.F11 * np.sin(th), th) / 2 - 1) < 1e-4
    cs = mie5.csrn
    assert len(cs) == 1001
    assert np.all(np.diff(cs) >= 0)
    assert cs[-1] == 1.0 and -1.0 <= cs[0] < -0.99
    # the median of cos(theta) under F11 sin(theta)
    cdf = np.cumsum(mie5.F11 * np.sin(th))
    cdf /= cdf[-1]
    med = math.cos(th[np.searchsorted(cdf, 0.5)])
    assert abs(cs[500] - med) < 0.01
    assert abs(mie5.kl - (4 / 3) * mie5.r / (mie5.nu * mie5.q_ext)) < 1e-12  # mie.jl:40


def test_fp32_arccos_meets_its_published_error_bound():
    """The FP32 kernels' arccos is Hastings' approximation (Abramowitz & Stegun 4.4.46,
    |error| <= 2e-8 in exact arithmetic); evaluated in FP32 with the same operation order
    as acos_as4446 in csrc/mcrt_device.cuh it stays within 5e-7 rad of arccos, about two
    FP32 ulps of pi, the resolution of angles near pi."""
    f = np.float32
    a = [f(-0.0012624911), f(0.0066700901), f(-0.0170881256), f(0.0308918810), f(-0.0501743046),
         f(0.0889789874), f(-0.2145988016), f(1.5707963050)]
    x = np.linspace(-1, 1, 200001).astype(np.float32)
    ax = np.abs(x)
    p = np.full_like(ax, a[0])
    for c in a[1:]:
        p = (p * ax + c).astype(np.float32)
    y = np.maximum(f(1) - ax, f(0))
    with np.errstate(divide="ignore", invalid="ignore"):  # y = 0 takes the other branch
        r = np.where(y > 0, (y * (f(1) / np.sqrt(y)) * p).astype(np.float32), f(0))
    th = np.where(x < 0, f(3.14159265358979) - r, r).astype(np.float32)
    err = np.abs(th.astype(np.float64) - np.arccos(x.astype(np.float64)))
    assert err.max() < 5e-7, err.max()


def test_config_defaults_mirror_the_reference(M):
    ray = M.RayleighScatterer(0.99, 1.0)
    g = M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=10.0, scatterer=ray)])
    cfg = M.Config(g)
    assert (cfg.number_of_rays, cfg.minimum_intensity, cfg.maximum_scattering_times) == (1000, 1e-6, 10000)
    assert (cfg.maximum_threads, cfg.compute_cb, cfg.tau0) == (8192, True, 50.0)
    assert (cfg.Nphi, cfg.Ntheta, cfg.Nthetab, cfg.Nphib) == (48, 64, 51, 8)
    assert abs(cfg.thetab[-1] - math.pi) < 1e-15 and cfg.thetab[0] == 0.0
    assert abs(cfg.phi[1] - 2 * math.pi / 48) < 1e-15
    # half-range Gauss-Legendre: each hemisphere's inorm sums to 1 / (2 Nphi) * 1
    h = cfg.Ntheta // 2
    assert np.all(cfg.costheta[:h] < 0) and np.all(cfg.costheta[h:] > 0)
    assert abs(cfg.inorm[:h].sum() * 2 * cfg.Nphi - 1) < 1e-14
    assert abs(np.sum(cfg.inorm[h:] * cfg.costheta[h:]) * 2 * cfg.Nphi - 0.5) < 1e-14
    s = M.SphereGeometry(R=2.0, scatterer=ray)
    cs = M.Config(s)
    assert abs(cs.inorm.sum() * 2 * cs.Nphi - 2) < 1e-14
    assert s.tau == 2.0 and s.omega == 0.99
    assert g.layers[0].tau == 10.0 and not g.layers[0].infinite


def test_validation_messages(M):
    ray = M.RayleighScatterer(0.99, 1.0)
    with pytest.raises(ValueError, match="θ must be in"):
        M.PlaneGeometry(1.0, 0.0, [M.Layer(d=1.0, scatterer=ray)]).validate()
    with pytest.raises(ValueError, match="ϕ must be in"):
        M.PlaneGeometry(math.pi, 7.0, [M.Layer(d=1.0, scatterer=ray)]).validate()
    with pytest.raises(ValueError, match="at least one layer"):
        M.PlaneGeometry(math.pi, 0.0, []).validate()
    with pytest.raises(ValueError, match="Only the last layer"):
        M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=-1, scatterer=ray, tau=math.inf),
                                       M.Layer(d=1, scatterer=ray)]).validate()
    with pytest.raises(ValueError, match="Radius must be positive"):
        M.SphereGeometry(R=0.0, scatterer=ray).validate()


def test_cpu_path_is_not_offered(M):
    ray = M.RayleighScatterer(0.99, 1.0)
    g = M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=1.0, scatterer=ray)])
    with pytest.raises(NotImplementedError):
        M.simulate(M.Config(g), g, [1, 0, 0, 0], use_gpu=False)


def _fake_sim(cfg, calls):
    """A stand-in for one simulate() per incident state, with tallies that encode the state."""

    def sim(I, i):
        calls.append(np.array(I))
        k = len(calls)
        irt = np.zeros((4, cfg.Ntheta, cfg.Nphi))
        icb = np.zeros((4, cfg.Nthetab, cfg.Nphib))
        for s in range(4):
            irt[s] = (s + 1) * 10.0 ** k + np.arange(cfg.Ntheta)[:, None] + 0.1 * np.arange(cfg.Nphi)[None, :]
            icb[s] = (s + 1) * 10.0 ** k + np.arange(cfg.Nthetab)[:, None]
        return 0.1 * k, 0.2, 0.3, 0.05, 0.01, irt, icb

    return sim


def test_run_rt_plane_assembly_restatement(M):
    """The checker's plane Mueller assembly (MonteCarloRadiativeTransfer.jl:186-291)
    against hand-derived columns."""
    from helpers import assemble_run_rt, table_of

    ray = M.RayleighScatterer(0.99, 1.0)
    g = M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=1.0, scatterer=ray)])
    cfg = M.Config(g, Ntheta=4, Nphi=2, Nphib=2, thetab=[0.0, 0.1, math.pi / 2])
    calls = []
    MRT, MCB, G = assemble_run_rt(cfg, g, _fake_sim(cfg, calls))
    sm_rt, sm_cb = table_of(MRT, True), table_of(MCB, True)
    assert len(calls) == 6
    # column 1 = (R(-Q) + R(+Q)) / 2, column 2 = (R(+Q) - R(-Q)) / 2 of the raw tallies
    norm = np.abs(1 / (4 * cfg.costheta * cfg.inorm))
    s11 = sm_rt["s11"].reshape(cfg.Nphi, cfg.Ntheta).T
    s12 = sm_rt["s12"].reshape(cfg.Nphi, cfg.Ntheta).T
    raw = lambda k, s: (s + 1) * 10.0 ** k + np.arange(cfg.Ntheta)[:, None] + 0.1 * np.arange(cfg.Nphi)[None, :]
    assert np.allclose(s11, (raw(1, 0) + raw(2, 0)) / 2 * norm[:, None])
    assert np.allclose(s12, (raw(2, 0) - raw(1, 0)) / 2 * norm[:, None])
    s44 = sm_rt["s44"].reshape(cfg.Nphi, cfg.Ntheta).T
    assert np.allclose(s44, (raw(6, 3) - raw(5, 3)) / 2 * norm[:, None])
    assert G[0] == pytest.approx((0.1 + 0.2) / 2)
    cb = sm_cb["s11"].reshape(cfg.Nphib, cfg.Nthetab).T
    rawb = lambda k, s: (s + 1) * 10.0 ** k + np.arange(cfg.Nthetab)[:, None]
    assert np.allclose(cb, (rawb(1, 0) + rawb(2, 0)) / 2 / np.abs(4 * cfg.costhetab)[:, None])


def test_run_rt_sphere_assembly_restatement(M):
    """The checker's sphere Mueller assembly (MonteCarloRadiativeTransfer.jl:87-184)."""
    from helpers import assemble_run_rt

    ray = M.RayleighScatterer(0.99, 1.0)
    g = M.SphereGeometry(R=1.0, scatterer=ray)
    cfg = M.Config(g, Ntheta=4, Nphi=8, Nphib=8, thetab=[0.0, 0.1])
    calls = []
    MRT, MCB, G = assemble_run_rt(cfg, g, _fake_sim(cfg, calls))
    assert len(calls) == 2
    raw1 = lambda s, j2: (s + 1) * 10.0 + np.arange(cfg.Ntheta) + 0.1 * j2
    renorm = 1 / (0.1 + 0.3)
    exp11 = (raw1(0, 0) + raw1(0, 2) + raw1(0, 4) + raw1(0, 6)) * 0.25 * renorm / cfg.inorm
    assert np.allclose(MRT[0, 0], exp11)
    exp44 = -np.mean([(4 * 100.0 + np.arange(cfg.Ntheta) + 0.1 * j2) for j2 in range(8)], axis=0)
    assert np.allclose(MRT[3, 3], exp44 * renorm / cfg.inorm)
    assert G[2] == pytest.approx(0.3)


def test_run_rt_needs_a_device(M):
    """run_rt has no CPU path: without a GPU it reports the missing device."""
    L = M.lib()
    if L.mcrt_device_count() > 0:
        pytest.skip("a CUDA device is visible")
    ray = M.RayleighScatterer(0.99, 1.0)
    g = M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=1.0, scatterer=ray)])
    with pytest.raises(M.MCRTError):
        M.run_rt(M.Config(g, number_of_rays=10), g)
    with pytest.raises(NotImplementedError):
        M.run_rt(M.Config(g, number_of_rays=10), g, use_gpu=False)


def test_csv_writer_uses_the_reference_columns(M, tmp_path):
    tab = {"theta": np.array([10.0, 20.0]), "phi": np.array([0.0, 0.0])}
    for a in range(1, 5):
        for b in range(1, 5):
            tab[f"s{a}{b}"] = np.array([a + 0.1 * b, -(a + 0.1 * b)])
    p = tmp_path / "rt.csv"
    M.write_csv(tab, str(p))
    lines = p.read_text(encoding="utf-8").splitlines()
    head = lines[0].split(",")
    assert head[:3] == ["θ", "ϕ", "s11"] and head[-1] == "s44" and len(head) == 18
    row = [float(v) for v in lines[2].split(",")]
    assert row[0] == 20.0 and row[2] == pytest.approx(-1.1) and row[-1] == pytest.approx(-4.4)


def test_peak_error_estimates_batch_means_and_per_path_agree(M):
    """The two standard errors of the CB peak agree on independent draws: their ratio
    follows sqrt(chi2_31 / 31), inside [0.46, 1.64] with probability 1 - 2e-6. A
    hand-computed case pins the formulas."""
    rng = np.random.default_rng(3)
    x = rng.exponential(2.0, size=(32, 4096))
    mean, se_bm, se_pp = M.peak_error_estimates(x.sum(1), (x * x).sum(1), 4096)
    assert abs(mean - x.mean()) < 1e-12
    assert 0.46 < se_bm / se_pp < 1.64
    assert abs(se_pp - x.std() / math.sqrt(x.size)) < 1e-12 * se_pp
    # two batches of two paths: x = (1, 3 | 5, 7)
    mean, se_bm, se_pp = M.peak_error_estimates([4.0, 12.0], [10.0, 74.0], 2)
    assert mean == 4.0
    assert abs(se_bm - np.std([2.0, 6.0], ddof=1) / math.sqrt(2)) < 1e-15
    assert abs(se_pp - math.sqrt((84.0 / 4 - 16.0) / 4)) < 1e-15
    with pytest.raises(ValueError):
        M.peak_error_estimates([1.0], [1.0], 10)


def test_arrow_writer_uses_the_reference_columns(M, tmp_path):
    pa = pytest.importorskip("pyarrow")
    import pyarrow.ipc as ipc

    tab = {"theta": np.array([10.0, 20.0])}  # a sphere table has no phi column
    for a in range(1, 5):
        for b in range(1, 5):
            tab[f"s{a}{b}"] = np.array([a + 0.1 * b, -(a + 0.1 * b)])
    p = tmp_path / "rt.arrow"
    M.write_arrow(tab, str(p))
    with pa.memory_map(str(p)) as src:
        t = ipc.open_file(src).read_all()
    assert t.column_names == ["θ"] + [f"s{a}{b}" for a in range(1, 5) for b in range(1, 5)]
    assert all(f.type == pa.float64() for f in t.schema)
    assert t.column("θ").to_pylist() == [10.0, 20.0] and t.column("s44").to_pylist() == [4.4, -4.4]


def test_host_mirrors_match_the_reference_source(M, O):
    """The Python mirrors of the reference's types (the library's host package and the
    oracle's own) against the reference's text, as extracted into
    tests/golden/reference_fields.json by make_reference_fields.py: Config's literal
    defaults, the default CB angles (DEFAULT_THEB, src/config.jl:3-53) and the exact
    ArgumentError messages of validate (src/geometries/plane.jl:52-62, sphere.jl:35-37)."""
    import mcrt_gb300.model as model

    ref = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                                      "reference_fields.json"), encoding="utf-8"))
    d = ref["config_defaults"]
    names = {"number_of_rays": "number_of_rays", "minimum_intensity": "minimum_intensity",
             "maximum_scattering_times": "maximum_scattering_times", "compute_cb": "compute_cb",
             "τ₀": "tau0", "Nϕ": "Nphi", "Nθ": "Ntheta", "Nϕb": "Nphib"}
    deg = np.array(ref["default_theb_degrees"])
    for Mod in (M, O):
        ray = Mod.RayleighScatterer(0.99, 1.0)
        cfg = Mod.Config(Mod.PlaneGeometry(math.pi, 0.0, [Mod.Layer(d=1.0, scatterer=ray)]))
        for jl, py in names.items():
            assert getattr(cfg, py) == d[jl], (Mod.__name__, jl)
        assert cfg.Nthetab == len(deg)
        assert np.allclose(np.arccos(np.clip(cfg.costhetab, -1, 1)), np.pi / 180.0 * deg, rtol=0, atol=2e-8)
    assert M.Config(M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=1.0, scatterer=M.RayleighScatterer(0.99, 1.0))])
                    ).maximum_threads == d["maximum_threads"]
    assert list(model.DEFAULT_THEB_DEG) == list(deg) and list(O.DEFAULT_THEB_DEG) == list(deg)

    ray = M.RayleighScatterer(0.99, 1.0)
    bad = [M.PlaneGeometry(1.0, 0.0, [M.Layer(d=1.0, scatterer=ray)]),
           M.PlaneGeometry(math.pi, 7.0, [M.Layer(d=1.0, scatterer=ray)]),
           M.PlaneGeometry(math.pi, 0.0, []),
           M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=-1, scatterer=ray, tau=math.inf), M.Layer(d=1, scatterer=ray)])]
    got = []
    for g in bad:
        with pytest.raises(ValueError) as e:
            g.validate()
        got.append(str(e.value))
    assert got == ref["validate_messages"]["PlaneGeometry"]
    with pytest.raises(ValueError) as e:
        M.SphereGeometry(R=0.0, scatterer=ray).validate()
    assert [str(e.value)] == ref["validate_messages"]["SphereGeometry"]
