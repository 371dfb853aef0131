"""The oracle's sphere geometry against an exact first-order integral.

Light falls along -z on a sphere of optical radius tau (src/geometries/sphere.jl). A
photon enters at a point uniform over the projected disk (sphere.jl:43-47), is
attenuated along its chord (the direct part is counted apart, src/cpu.jl:175-183), has
its first collision at depth t along the chord with density e^{-t}, and peels off into
each bin direction k with the attenuation e^{-d(x, k)} of the path to the surface
(sphere.jl:69-73). At one order the expected RT tally per photon is therefore

    Irt[:, j, k] / n = omega inorm_j G(mu_j) D Z(k_jk <- k0) D I0,
    G(mu) = 1/(pi tau^2) int_disk dA int_0^chord e^{-t - d(x(t), k)} dt,

where Z is the phase matrix in meridian frames (tests/doubling.py) and
D = diag(1, 1, -1, -1) the reference's Stokes frame, as for the plane. G depends only on
the exit cosine (the sphere is symmetric about z); it is evaluated here by Gauss-Legendre
quadrature with the substitution r = tau sqrt(1 - s^2), which removes the square-root
edge of the chord. The CB tally at theta_b (one order, src/cpu.jl:132-156) has the
intensity omega P11(pi - theta_b) G(cos theta_b) for unpolarised light, the same without
the quadrature weight.

Nothing here shares code with the oracle: this pins its entry-point distribution, its
chord and exit distances, its first flight and the CB bins' directions for the sphere,
which the plane-parallel anchors (analog Monte Carlo, adding-doubling) cannot reach."""
import math

import numpy as np
import pytest

import doubling as D

STATES = np.array([[1.0, 0, 0, 0], [1, 1, 0, 0], [1, 0, 1, 0], [1, 0, 0, 1]])
FRAME = np.diag([1.0, 1.0, -1.0, -1.0])


def geometric_factor(tau, mu_out, n=96):
    """G(mu) for each exit cosine in `mu_out` (exit azimuth 0; G does not depend on it)."""
    xs, ws = np.polynomial.legendre.leggauss(n)
    s, w = (xs + 1) / 2, ws / 2                      # s in (0, 1): r = tau sqrt(1 - s^2), chord 2 tau s
    psi = (np.arange(2 * n) + 0.5) * (math.pi / n)   # azimuth of the entry point
    S, P, U = np.meshgrid(s, psi, s, indexing="ij")  # U: depth as a fraction of the chord
    W = w[:, None, None] * (math.pi / n) * w[None, None, :]
    h = tau * S
    r = tau * np.sqrt(1 - S * S)
    t = 2 * h * U
    x = np.stack([r * np.cos(P), r * np.sin(P), h - t], -1)
    xx = (x * x).sum(-1)
    out = []
    for m in np.atleast_1d(mu_out):
        k = np.array([math.sqrt(max(1 - m * m, 0.0)), 0.0, m])
        kx = x @ k
        d = -kx + np.sqrt(np.maximum(kx * kx + tau * tau - xx, 0.0))
        # dA = r dr dpsi = tau^2 s ds dpsi, dt = 2 tau s du; divided by pi tau^2
        out.append(np.sum(W * S * (2 * tau * S) * np.exp(-t - d)) / math.pi)
    return np.array(out)


def _case(O, kind):
    if kind == "rayleigh":
        s = O.RayleighScatterer(0.9, 1.0)
        return s, D.rayleigh_matrix, 2.0
    # the benchmark sphere: x = 2, m = 1.31 (omega 1), tau = 20
    s = O.MieScatterer(2.0 / (2 * math.pi), 1.31 + 0j, 1.0, 0.1, Ntheta=1801)
    t = s.rounded_fp32()
    return s, D.TabulatedMatrix(t.F11, t.F12, t.F33, t.F34), 20.0


def test_geometric_factor_converges_and_knows_the_thin_limit():
    """G converges with the quadrature order, and for a thin sphere it tends to the mean
    chord times e^0: (1/pi tau^2) int 2 h dA = 4 tau / 3."""
    for tau in (2.0, 20.0):
        mu = np.array([-0.9, -0.2, 0.3, 0.95, 1.0])
        a, b = geometric_factor(tau, mu, 96), geometric_factor(tau, mu, 128)
        assert np.max(np.abs(a - b) / b) < 2e-5
    tau = 1e-4
    assert abs(geometric_factor(tau, [0.5])[0] / (4 * tau / 3) - 1) < 1e-3


@pytest.mark.parametrize("kind", ["rayleigh", "mie"])
def test_oracle_sphere_first_order_matches_the_exact_integral(O, kind):
    """One order, 16 independent runs of 65 536 photons per incident state, each with its
    first-collision depth on its own midpoint grid (so the runs are independent samples
    of the entry points): every RT bin and Stokes parameter within 5 se of the exact
    value (mean z^2 < 2: the bins share the entry points), and the unpolarised CB
    intensity at ten angles from exact backscatter within 5 se."""
    s, F, tau = _case(O, kind)
    g = O.SphereGeometry(R=tau * s.kl, scatterer=s)
    nb, m = 16, 1 << 16
    thetab = np.radians(np.linspace(0.0, 5.0, 10))
    cfg = O.Config(g, number_of_rays=m, compute_cb=True, maximum_scattering_times=1, Ntheta=16, Nphi=8,
                   thetab=thetab, Nphib=2)
    runs = [[O.simulate(cfg, g, I0, seed=1000 * b + 7 + i, rng_mode=1, threads=0) for i, I0 in enumerate(STATES)]
            for b in range(nb)]
    bat = np.array([[r["Irt"] / m for r in row] for row in runs])
    mean = bat.mean(0)
    se = bat.std(0, ddof=1) / math.sqrt(nb)

    Gv = geometric_factor(tau, cfg.costheta)
    phi = np.arctan2(cfg.sinphi, cfg.cosphi)
    Z = np.array([[D.phase_matrix(mu, p, -1.0, 0.0, F) for p in phi] for mu in cfg.costheta])
    M = FRAME @ Z @ FRAME * (s.omega * cfg.inorm * Gv)[:, None, None, None]
    exp = np.einsum("jkab,sb->sajk", M, STATES)
    scale = np.abs(exp).max()
    live = (se > 0) & (np.maximum(np.abs(mean), np.abs(exp)) > 1e-12 * scale)
    z = (mean - exp)[live] / se[live]
    print(f"{kind} sphere: {live.sum()} comparisons, max |z| {np.abs(z).max():.2f}, mean z^2 "
          f"{np.mean(z * z):.2f}, max |oracle - exact| / scale {np.abs(mean - exp).max() / scale:.2e}")
    assert np.abs(z).max() < 5.0
    assert np.mean(z * z) < 2.0
    assert np.abs(mean - exp)[~live].max(initial=0.0) < 1e-12 * scale

    cb = np.array([row[0]["Icb"][0] / m for row in runs])  # (nb, Nthetab, Nphib), unpolarised
    exp_cb = s.omega * F(-np.cos(thetab))[0] * geometric_factor(tau, np.cos(thetab))
    zc = (cb.mean(0) - exp_cb[:, None]) / (cb.std(0, ddof=1) / math.sqrt(nb))
    print(f"{kind} sphere CB: max |z| {np.abs(zc).max():.2f}, at exact backscatter oracle "
          f"{cb.mean(0)[0, 0]:.5f}, exact {exp_cb[0]:.5f}")
    assert np.abs(zc).max() < 5.0


@pytest.mark.parametrize("kind", ["rayleigh", "mie"])
def test_run_rt_sphere_assembly_of_the_exact_first_order(M, O, kind):
    """run_rt's assembly for a sphere (src/MonteCarloRadiativeTransfer.jl:87-184: the two
    states [1,-1,0,0] and [1,0,0,-1], the azimuths 0, 45, ..., 315 degrees combined into
    the columns, renormalised by the scattered fraction Gdt + Gref and the quadrature
    weight), restated in tests/helpers.py and matched by the device epilogue at 1e-9 in
    the GPU tests, applied to the exact first-order tallies above, returns exactly
    omega G(mu) / (Gdt + Gref) F(Theta): the scattering matrix [[F11, F12, 0, 0],
    [F12, F11, 0, 0], [0, 0, F33, F34], [0, 0, -F34, F33]] in the scattering plane,
    which the reference's frame leaves as it is (D F D = F). Deterministic: 1e-12."""
    from helpers import assemble_run_rt

    s, F, tau = _case(O, kind)
    g = O.SphereGeometry(R=tau * s.kl, scatterer=s)
    cfg = O.Config(g, number_of_rays=1, compute_cb=False, Ntheta=16, Nphi=8)
    Gv = geometric_factor(tau, cfg.costheta)
    phi = np.arctan2(cfg.sinphi, cfg.cosphi)
    Z = np.array([[D.phase_matrix(mu, p, -1.0, 0.0, F) for p in phi] for mu in cfg.costheta])
    tally = np.einsum("ab,jkbc,cd->adjk", FRAME, Z, FRAME) * (s.omega * cfg.inorm * Gv)[None, None, :, None]
    direct = (1 - (1 + 2 * tau) * math.exp(-2 * tau)) / (2 * tau * tau)  # mean e^{-chord} over the disk

    def sim(I, _):
        Irt = np.einsum("abjk,b->ajk", tally, np.asarray(I, float))
        return (direct, 0.0, Irt[0].sum(), 0.0, 0.0, Irt, np.zeros((4, cfg.Nthetab, cfg.Nphib)))

    shape_g = M.SphereGeometry(R=2.0, scatterer=M.RayleighScatterer(0.9, 1.0))
    MRT, _, G = assemble_run_rt(cfg, shape_g, sim)
    c = -cfg.costheta  # cos(Theta) for the exit cosine mu, light incident along -z
    F11, F12, F33, F34 = F(c)
    Fm = np.zeros((4, 4, cfg.Ntheta))
    Fm[0, 0] = Fm[1, 1] = F11
    Fm[0, 1] = Fm[1, 0] = F12
    Fm[2, 2] = Fm[3, 3] = F33
    Fm[2, 3], Fm[3, 2] = F34, -F34
    expect = Fm * (s.omega * Gv / (G[0] + G[2]))[None, None, :]
    assert np.abs(MRT - expect).max() < 1e-12 * np.abs(expect).max()
