"""The oracle against an exact deterministic solution at every bin and every order: the
vector adding-doubling solver of tests/doubling.py (Hansen & Travis 1974; de Haan, Bosma
& Hovenier 1987), written apart from the oracle, gives the reflection and diffuse
transmission matrices of a homogeneous slab to quadrature accuracy.

The oracle's RT tally of a run with incident Stokes vector I0 estimates, per bin,
Irt[:, j, k] / n = 4 |mu_j| inorm_j D R(mu_j, mu0, phi_k - phi0) D I0 (T in place of R
for the lower hemisphere), where R is in the normalisation of those papers and
D = diag(1, 1, -1, -1): the oracle takes Stokes vectors in the frame (e_theta, -e_phi)
(the reference's get_basis, src/utils.jl:52-62, gives Eh = (sin phi, -cos phi, 0)),
which is left-handed about the direction of travel, so its U and V are the negatives
of the right-handed meridian frame's. The first-order test fixes D, with the oracle's
exact single-scattering mode (one order, first-collision depth on a midpoint grid);
the all-orders test then runs the four incident states [1,0,0,0], [1,1,0,0], [1,0,1,0],
[1,0,0,1], which give all 16 elements of the matrices, and scores every bin of both
hemispheres against the exact values with standard errors from batch means.

This pins what the analog Monte Carlo of tests/analog_mc.py does not: the angular
distribution and the polarisation of every Mueller element at multiple orders, for
oblique incidence, in Rayleigh and in Mie slabs, through the reference's own scheme
(forced collisions, peel-off into the Gauss-Legendre bins, weights lowered by the
bin-quadrature escape estimate of src/gpu.jl:285-294; at the reference's default 64 x 48
grid that estimate's error stays below the noise here).

The same runs pin the coherent-backscattering tallies at exact backscatter, where
reciprocity fixes the interference of reciprocal paths as a linear function of the
exact ladder matrix (doubling.cyclical): the ladder, the CB intensity and the CB
enhancement factor for each incident state."""
import math

import numpy as np
import pytest

import doubling as D

STATES = np.array([[1.0, 0, 0, 0], [1, 1, 0, 0], [1, 0, 1, 0], [1, 0, 0, 1]])
FRAME = np.diag([1.0, 1.0, -1.0, -1.0])
THETA0 = math.radians(150.0)  # 30 degrees from the normal, travelling downwards
TAU = 1.0


def _case(O, kind):
    """(scatterer, F, azimuthal modes, azimuth samples) of a case."""
    if kind.startswith("rayleigh"):
        s = O.RayleighScatterer(0.8 if kind == "rayleigh_semi_infinite" else 0.9, 1.0)
        return s, D.rayleigh_matrix, 2, 16
    s = O.MieScatterer(2.0 / (2 * math.pi), 1.5 + 0.01j, 1.0, 0.1, Ntheta=1801)  # omega 0.951, g 0.63
    t = s.rounded_fp32()  # the oracle interpolates the FP32-rounded tables, as the device does
    return s, D.TabulatedMatrix(t.F11, t.F12, t.F33, t.F34), 24, 128


def _expected(sol, cfg, mu0):
    """4 |mu| inorm D R D I0 per incident state, Stokes parameter and bin."""
    phi = np.arctan2(cfg.sinphi, cfg.cosphi)
    out = np.zeros((4, 4, cfg.Ntheta, cfg.Nphi))
    for j, mu in enumerate(cfg.costheta):
        M = sol.reflection(mu, mu0, phi) if mu > 0 else sol.transmission(-mu, mu0, phi)
        M = FRAME @ M @ FRAME * (4 * abs(mu) * cfg.inorm[j])  # (Nphi, 4, 4)
        out[:, :, j, :] = np.einsum("kab,sb->sak", M, STATES)
    return out


def _solve(O, kind, cfg, n_doublings=30):
    s, F, n_modes, n_az = _case(O, kind)
    h = cfg.Ntheta // 2
    mu0 = abs(math.cos(THETA0))
    q, w = D.half_range_gauss(h)  # the bins' own half-range Gauss-Legendre nodes
    tau = TAU
    if kind == "rayleigh_semi_infinite":  # 60 optical depths: e^-46 of the light gets through
        tau, n_doublings = 60.0, n_doublings + 6 if n_doublings else 0
    sol = D.solve(tau, s.omega, F, q, w, extra_mu=[mu0], n_modes=n_modes, n_azimuth=n_az,
                  n_doublings=n_doublings)
    assert sol.dropped_mode_norm < 1e-6  # the azimuthal modes left out are negligible
    return sol, mu0


def _geometry(O, kind, s):
    if kind == "rayleigh_semi_infinite":
        return O.PlaneGeometry(THETA0, 0.0, [O.Layer(d=-1.0, scatterer=s, tau=math.inf)])
    return O.PlaneGeometry(THETA0, 0.0, [O.Layer(d=TAU * s.kl, scatterer=s)])


def test_doubling_solver_conserves_energy_and_obeys_reciprocity(O):
    """The solver's own checks: at omega = 1 reflected + diffusely transmitted + direct
    flux is 1 for every incidence node; Rayleigh phase matrices have no azimuthal modes
    beyond 2; and for a Mie phase matrix, at all orders, the reciprocity relation
    R(mu_a, mu_b, dphi) = Q R(mu_b, mu_a, dphi)^T Q with Q = diag(1, 1, 1, -1) and the
    mirror relation R(mu, mu0, -dphi) = P R(mu, mu0, dphi) P with P = diag(1, 1, -1, -1)
    (the reciprocity and mirror-symmetry relations of polarised reflection, e.g. Hovenier,
    van der Mee & Domke, Transfer of Polarized Light in Planetary Atmospheres, 2004; the
    signs are those of a right-handed meridian frame)."""
    q, w = D.half_range_gauss(16)
    sol = D.solve(1.0, 1.0, D.rayleigh_matrix, q, w, n_modes=2, n_azimuth=32)
    assert sol.dropped_mode_norm < 1e-14
    n = len(sol.nodes)
    R0 = sol.R[0].real.reshape(n, 4, n, 4)[:, 0, :, 0]
    T0 = sol.T[0].real.reshape(n, 4, n, 4)[:, 0, :, 0]
    flux = 2 * (sol.nodes * sol.weights) @ (R0 + T0) + np.exp(-1.0 / sol.nodes)
    assert np.max(np.abs(flux - 1.0)) < 1e-7

    mie = O.MieScatterer(2.0 / (2 * math.pi), 1.5 + 0.01j, 1.0, 0.1, Ntheta=1801)
    sol = D.solve(1.0, 0.9, D.TabulatedMatrix(mie.F11, mie.F12, mie.F33, mie.F34), q, w, n_modes=24,
                  n_azimuth=128, n_doublings=24)
    dphi = np.array([0.3, 1.1, 2.5])
    Qm, Pm = np.diag([1.0, 1, 1, -1]), np.diag([1.0, 1, -1, -1])
    for a, b in ((q[3], q[11]), (q[0], q[15]), (q[7], q[8])):
        Rab = sol.reflection(a, b, dphi)
        scale = np.abs(Rab).max()
        assert np.abs(Rab - Qm @ np.swapaxes(sol.reflection(b, a, dphi), 1, 2) @ Qm).max() < 1e-12 * scale
        assert np.abs(sol.reflection(a, b, -dphi) - Pm @ Rab @ Pm).max() < 1e-12 * scale
        # and the polarisation is not trivial: the off-diagonal blocks carry weight
        assert np.abs(Rab[:, 0, 1]).max() > 1e-2 * scale and np.abs(Rab[:, 2, 3]).max() > 1e-4 * scale

    # the interference map of exact backscatter: its (1, 1) element is Mishchenko's
    # (L11 + L22 - L33 + L44) / 2 for any ladder matrix L
    L = np.random.default_rng(1).normal(size=(4, 4))
    assert abs(D.cyclical(L)[0, 0] - (L[0, 0] + L[1, 1] - L[2, 2] + L[3, 3]) / 2) < 1e-12


@pytest.mark.parametrize("kind", ["rayleigh", "mie"])
def test_oracle_first_order_equals_the_exact_single_scattering_matrix(O, kind):
    """With one order and the first-collision depth on a midpoint grid the oracle's tally
    is the single-scattering matrix to 1e-6 for all four incident states, which fixes
    the frame relation D = diag(1, 1, -1, -1); the other sign of V fails for the Mie
    matrix (its F34 couples U and V)."""
    s = _case(O, kind)[0]
    g = _geometry(O, kind, s)
    n = 1 << 14
    cfg = O.Config(g, number_of_rays=n, compute_cb=False, maximum_scattering_times=1)
    sol, mu0 = _solve(O, kind, cfg, n_doublings=0)  # no doubling: the layer's single scattering
    got = np.array([O.simulate(cfg, g, I0, seed=3, rng_mode=1, threads=0)["Irt"] / n for I0 in STATES])
    exp = _expected(sol, cfg, mu0)
    scale = np.abs(exp).max()
    err = np.abs(got - exp).max() / scale
    print(f"{kind} first order: max |oracle - exact| / scale = {err:.2e}")
    assert err < 1e-6
    if kind == "mie":
        # the same matrix with V of the other sign on both sides: the states' flipped
        # vectors are combinations C of the states themselves, STATES Vflip = C STATES
        Vflip = np.diag([1.0, 1, 1, -1])
        C = STATES @ Vflip @ np.linalg.inv(STATES)
        alt = np.einsum("ab,cs,sbjk->cajk", Vflip, C, exp)
        assert np.abs(got - alt).max() / scale > 1e-2


@pytest.fixture(scope="module", params=["rayleigh", "mie", "rayleigh_semi_infinite"])
def all_orders(request, O):
    """Slab tau = 1 at 30 degrees incidence with the reference's default 64 x 48 RT grid;
    Rayleigh scatterers (omega 0.9) or Mie spheres x = 2, m = 1.5+0.01i (omega 0.951,
    asymmetry 0.63); or a semi-infinite layer of Rayleigh scatterers (omega 0.8, the
    reference's infinite Layer: unforced first flight, no lower boundary), whose exact
    solution is the doubling carried to tau = 60. Per incident state 16 batches of 1 000
    photons on disjoint Philox ranges, with CB bins at theta_b = 0 and 0.001 rad (the
    incremental reciprocal-path form, which equals the reference's walks to 1e-12); the
    RT tallies do not depend on the CB settings."""
    kind = request.param
    s = _case(O, kind)[0]
    g = _geometry(O, kind, s)
    nb, photons = 16, 1000
    cfg = O.Config(g, number_of_rays=photons, compute_cb=True, thetab=np.array([0.0, 1e-3]), Nphib=2)
    sol, mu0 = _solve(O, kind, cfg)
    sol1 = _solve(O, kind, cfg, n_doublings=0)[0]  # the layer's single scattering, R1
    runs = [[O.simulate(cfg, g, I0, seed=11 + i, threads=0, cb_form=1, photon_begin=b * photons,
                        photon_count=photons) for i, I0 in enumerate(STATES)] for b in range(nb)]
    return {"kind": kind, "cfg": cfg, "sol": sol, "sol1": sol1, "mu0": mu0, "nb": nb, "photons": photons,
            "runs": runs}


def test_oracle_rt_matches_the_exact_doubling_solution_at_all_orders(all_orders):
    """Every bin, Stokes parameter and incident state (up to 49 152 comparisons) is scored
    by z = (oracle - exact) / se: all |z| < 6, and mean z^2 < 2 as a loose gate against
    a bias shared by many bins (about 1.15 is expected from 16 batch means, but all bins
    see the same events, so the z are strongly correlated and their mean square
    fluctuates far more than independent z's would: 1.36 is seen on the semi-infinite
    layer at both 1.6e4 and 3.2e4 photons per state); the reflected and transmitted
    fractions within 4 se; elements that are exactly zero in the oracle (V from linear
    states in Rayleigh scattering, every transmission bin of the semi-infinite layer) are
    zero in the exact solution too."""
    a = all_orders
    kind, cfg, nb, photons = a["kind"], a["cfg"], a["nb"], a["photons"]
    exp = _expected(a["sol"], cfg, a["mu0"])
    bat = np.array([[r["Irt"] / photons for r in row] for row in a["runs"]])
    mean = bat.mean(0)
    se = bat.std(0, ddof=1) / math.sqrt(nb)
    scale = np.abs(exp[:, 0]).max()
    live = se > 0
    z = (mean - exp)[live] / se[live]
    print(f"{kind}: {live.sum()} comparisons, max |z| {np.abs(z).max():.2f}, mean z^2 {np.mean(z * z):.3f}, "
          f"max |oracle - exact| / scale {np.abs(mean - exp).max() / scale:.2e}")
    assert np.abs(z).max() < 6.0
    assert np.mean(z * z) < 2.0
    assert np.abs(exp[~live]).max(initial=0.0) < 1e-10 * scale
    assert np.all(mean[~live] == 0.0)
    h = cfg.Ntheta // 2
    for name, sl in (("reflected", slice(h, None)), ("transmitted", slice(0, h))):
        f = bat[:, 0, 0, sl].sum(axis=(1, 2))
        if not np.any(f):  # the semi-infinite layer transmits nothing
            assert abs(exp[0, 0, sl].sum()) < 1e-10
            continue
        zf = (f.mean() - exp[0, 0, sl].sum()) / (f.std(ddof=1) / math.sqrt(nb))
        print(f"{kind} {name}: oracle {f.mean():.5f}, exact {exp[0, 0, sl].sum():.5f}, z {zf:.2f}")
        assert abs(zf) < 4.0


def test_oracle_cb_at_exact_backscatter_matches_reciprocity(all_orders):
    """The CB tallies at theta_b = 0 against exact values. There the reciprocal paths'
    phase difference vanishes, and the ensemble sum of their interference is fixed by
    reciprocity: C = cyclical(L) with L = R - R1 at (mu0, mu0, pi) from the doubling
    solution (tests/doubling.py). Per photon the ladder tally estimates
    4 mu0 [R D I0]_1 and the CB intensity 4 mu0 [(R + C) D I0]_1 (the peel-off
    normalisation of the RT bins without the quadrature weight). This checks the
    reference's whole reciprocal-path machinery (src/cpu.jl:38-160: forward and backward
    fields, the amplitude matrices, the scaling of the fields to the incoherent intensity
    and the Ia / (Ia + Ib) share) at all orders, and the CB enhancement factor
    Icb / ladder, for linearly and circularly polarised light and for unpolarised light
    (which the reference carries as a circularly polarised field, src/utils.jl:122-134;
    the bias that leaves, 0.25% on the benchmark's Mie slab and none on Rayleigh slabs,
    is below these samples' resolution and is measured on the GPU, test_gpu_exact.py):
    each within 4 se from the batch means."""
    a = all_orders
    kind, nb, photons, mu0 = a["kind"], a["nb"], a["photons"], a["mu0"]
    sol = a["sol"]
    R = sol.reflection(mu0, mu0, np.array([math.pi]))[0]
    R1 = a["sol1"].reflection(mu0, mu0, np.array([math.pi]))[0]
    C = D.cyclical(R - R1)
    for i, I0 in enumerate(STATES):
        lad = np.array([row[i]["ladder"][0, 0] / photons for row in a["runs"]])
        icb = np.array([row[i]["Icb"][0, 0, 0] / photons for row in a["runs"]])
        e_lad = 4 * mu0 * (R @ FRAME @ I0)[0]
        e_icb = 4 * mu0 * ((R + C) @ FRAME @ I0)[0]
        se = lambda v: v.std(ddof=1) / math.sqrt(nb)
        zeta = icb / lad
        z = [(lad.mean() - e_lad) / se(lad), (icb.mean() - e_icb) / se(icb),
             (zeta.mean() - e_icb / e_lad) / se(zeta)]
        print(f"{kind} I0 {I0}: ladder {lad.mean():.5f} (exact {e_lad:.5f}), CB {icb.mean():.5f} "
              f"(exact {e_icb:.5f}), enhancement {zeta.mean():.4f} (exact {e_icb / e_lad:.4f}), "
              f"z {np.round(z, 2)}")
        assert np.all(np.abs(z) < 4.0)
        assert 1.0 < e_icb / e_lad < 2.0


def test_oracle_cb_enhancement_on_the_headline_mie_slab_is_exact(O):
    """The benchmark's Mie slab itself: spheres x = 5, m = 1.5+0.001i with 1801-angle
    tables (omega 0.9925, asymmetry 0.71), a slab of tau = 5 at 30 degrees incidence, the
    default 64 x 48 RT grid; about 71 events per path. The exact solution takes 32 nodes
    and 32 azimuthal modes (converged to 6e-5 of the tally scale against 64 and 64).

    At sizes the CPU runs in seconds, single bins here are heavy tailed: photons kept near
    a surface for many events inside the forward lobe (F11 up to 25) contribute rarely but
    much, and batches that miss them are low in both mean and spread. At 3.2e4 photons a
    region of reflection bins came out 6% low with z = -9 while its mirror image, equal in
    exact arithmetic, was 0.3% high; the circular state's ladder was 4% low (z = -3) at
    4 800 photons and agrees at 6.4e4 (z = -0.5). So the gates are relative: the CB
    enhancement factor at exact backscatter, a ratio in which the tails largely cancel,
    within 1% of the exact value for unpolarised light (the metric's CB peak) and for
    linearly polarised light (a CB that ignored reciprocity's structure, C = L, would
    give 1.83 against the exact 1.71); the ladder and CB intensities within 8%; the
    reflected and transmitted fractions within 4 se. (The circularly polarised and U
    states' CB elements are checked on the Mie slab of tau = 1 above.)"""
    mie = O.MieScatterer(5.0 / (2 * math.pi), 1.5 + 0.001j, 1.0, 0.1, Ntheta=1801)
    tau = 5.0
    t = mie.rounded_fp32()
    F = D.TabulatedMatrix(t.F11, t.F12, t.F33, t.F34)
    g = O.PlaneGeometry(THETA0, 0.0, [O.Layer(d=tau * mie.kl, scatterer=mie)])
    nb, photons = 16, 300
    cfg = O.Config(g, number_of_rays=photons, compute_cb=True, thetab=np.array([0.0, 1e-3]), Nphib=2)
    mu0 = abs(math.cos(THETA0))
    q, w = D.half_range_gauss(cfg.Ntheta // 2)
    kw = dict(extra_mu=[mu0], n_modes=32, n_azimuth=128)
    sol = D.solve(tau, mie.omega, F, q, w, n_doublings=28, **kw)
    sol1 = D.solve(tau, mie.omega, F, q, w, n_doublings=0, **kw)
    assert sol.dropped_mode_norm < 1e-6 * mie.F11.max()
    R = sol.reflection(mu0, mu0, np.array([math.pi]))[0]
    C = D.cyclical(R - sol1.reflection(mu0, mu0, np.array([math.pi]))[0])
    exp = _expected(sol, cfg, mu0)
    states = STATES[:2]  # [1,0,0,0] and [1,1,0,0]
    runs = [[O.simulate(cfg, g, I0, seed=11 + i, threads=0, cb_form=1, photon_begin=b * photons,
                        photon_count=photons) for i, I0 in enumerate(states)] for b in range(nb)]
    h = cfg.Ntheta // 2
    for name, sl in (("reflected", slice(h, None)), ("transmitted", slice(0, h))):
        f = np.array([row[0]["Irt"][0, sl].sum() / photons for row in runs])
        zf = (f.mean() - exp[0, 0, sl].sum()) / (f.std(ddof=1) / math.sqrt(nb))
        print(f"headline Mie slab {name}: oracle {f.mean():.5f}, exact {exp[0, 0, sl].sum():.5f}, z {zf:.2f}")
        assert abs(zf) < 4.0
    for i, I0 in enumerate(states):
        lad = np.array([row[i]["ladder"][0, 0] / photons for row in runs])
        icb = np.array([row[i]["Icb"][0, 0, 0] / photons for row in runs])
        e_lad = 4 * mu0 * (R @ FRAME @ I0)[0]
        e_icb = 4 * mu0 * ((R + C) @ FRAME @ I0)[0]
        zeta = icb.mean() / lad.mean()
        print(f"headline Mie slab I0 {I0}: ladder {lad.mean():.4f} (exact {e_lad:.4f}), CB {icb.mean():.4f} "
              f"(exact {e_icb:.4f}), enhancement {zeta:.4f} (exact {e_icb / e_lad:.4f})")
        assert abs(zeta / (e_icb / e_lad) - 1) < 0.01
        assert abs(lad.mean() / e_lad - 1) < 0.08 and abs(icb.mean() / e_icb - 1) < 0.08
        assert 1.0 < e_icb / e_lad < 2.0


def test_run_rt_assembly_of_the_exact_tallies_is_the_exact_matrix(M, O):
    """run_rt's Mueller assembly for a plane (src/MonteCarloRadiativeTransfer.jl:186-291:
    half differences of the six polarised states' tallies, scaled by
    1 / |4 cos(theta) inorm|), restated in tests/helpers.py and matched by the device
    epilogue at 1e-9 in the GPU tests, applied to the exact expected tallies
    4 |mu| inorm D R D I0 (the doubling solution, all orders), returns exactly
    s_ab = (D R D)_ab, the reflection and transmission matrices in the doubling papers'
    normalisation, in the reference's frame. Deterministic: 1e-12. With the oracle's
    tallies matching the exact ones (the tests above), this fixes what run_rt's
    s11 ... s44 columns are."""
    from helpers import assemble_run_rt

    for kind in ("rayleigh", "mie"):
        s = _case(O, kind)[0]
        g = _geometry(O, kind, s)
        cfg = O.Config(g, number_of_rays=1, compute_cb=False)
        sol, mu0 = _solve(O, kind, cfg)
        phi = np.arctan2(cfg.sinphi, cfg.cosphi)
        exact = np.zeros((4, 4, cfg.Ntheta, cfg.Nphi))
        for j, mu in enumerate(cfg.costheta):
            Rj = sol.reflection(mu, mu0, phi) if mu > 0 else sol.transmission(-mu, mu0, phi)
            exact[:, :, j, :] = np.moveaxis(FRAME @ Rj @ FRAME, 0, -1)
        tally = exact * (4 * np.abs(cfg.costheta) * cfg.inorm)[None, None, :, None]

        def sim(I, _):
            Irt = np.einsum("abjk,b->ajk", tally, np.asarray(I, float))
            return (0.0, 0.0, Irt[0, cfg.Ntheta // 2:].sum(), Irt[0, :cfg.Ntheta // 2].sum(), 0.0, Irt,
                    np.zeros((4, cfg.Nthetab, cfg.Nphib)))

        shape_g = M.PlaneGeometry(THETA0, 0.0, [M.Layer(d=1.0, scatterer=M.RayleighScatterer(0.9, 1.0))])
        MRT = assemble_run_rt(cfg, shape_g, sim)[0]
        assert np.abs(MRT - exact).max() < 1e-12 * np.abs(exact).max(), kind
