"""An independent multiple-scattering anchor for the oracle: the oracle (forced collisions,
peel-off into Gauss-Legendre bins, weight renormalised by the escape estimate, as the
reference's cpu.jl/gpu.jl do) against an analog polarised Monte Carlo written apart from
it (tests/analog_mc.py: free flights, escape counting, exact sampling of the polarised
phase matrix), on Rayleigh slabs, on a slab of absorbing Mie spheres, and on a
Rayleigh sphere and the benchmark Mie sphere (analog_mc.run_sphere).

Both estimate the same integrals of the escaping light at all scattering orders: the
reflected and diffusely transmitted fractions, their first moments in the exit cosine,
the second reflected moment, and the reflected Q in the exit meridian frame (for a
sphere: the escaping fraction over all directions and the same moments). Each must
agree within 4 combined standard errors from batch means, and the single-scattering
parts within 2%. The analog run also fixes the sign convention of Q independently
(Q = I_par - I_perp with respect to the meridian plane)."""
import math

import numpy as np
import pytest

import analog_mc

QUANTITIES = ("R", "T", "R_mu", "R_mu2", "T_mu", "R_Q")


def _oracle(O, g, n, nb, max_scat=10000):
    cfg = O.Config(g, number_of_rays=n, compute_cb=False, maximum_scattering_times=max_scat)
    h = cfg.Ntheta // 2
    mu = cfg.costheta
    res = {k: [] for k in QUANTITIES}
    m = n // nb
    for b in range(nb):
        r = O.simulate(cfg, g, [1, 0, 0, 0], seed=9, threads=0, photon_begin=b * m, photon_count=m)
        I = r["Irt"][0].sum(1) / m  # sum over azimuths: per polar node, quadrature weight included
        Q = r["Irt"][1].sum(1) / m
        res["R"].append(I[h:].sum())
        res["T"].append(I[:h].sum())
        res["R_mu"].append((I[h:] * mu[h:]).sum())
        res["R_mu2"].append((I[h:] * mu[h:] ** 2).sum())
        res["T_mu"].append((I[:h] * np.abs(mu[:h])).sum())
        res["R_Q"].append(Q[h:].sum())
        assert abs(r["A"][2] / m - res["R"][-1]) < 1e-12  # Aref is the upper bins' sum
    return {k: np.array(v) for k, v in res.items()}


def _compare(O, g, a, n_oracle, label):
    o = _oracle(O, g, n_oracle, 10)
    for k in QUANTITIES:
        ma, sa = a[k].mean(), a[k].std(ddof=1) / math.sqrt(len(a[k]))
        mo, so = o[k].mean(), o[k].std(ddof=1) / math.sqrt(len(o[k]))
        z = (ma - mo) / math.hypot(sa, so)
        print(f"{label} {k}: analog {ma:.5f} +- {sa:.5f}, oracle {mo:.5f} +- {so:.5f}, z {z:.2f}")
        assert abs(z) < 4.0, (k, ma, mo, z)
    o1 = _oracle(O, g, 8000, 4, max_scat=1)
    for ka, ko in (("R1", "R"), ("R1_Q", "R_Q")):
        print(f"{label} {ka}: analog {a[ka].mean():.5f}, oracle {o1[ko].mean():.5f}")
        assert abs(a[ka].mean() / o1[ko].mean() - 1) < 0.02, (ka, a[ka].mean(), o1[ko].mean())


@pytest.mark.parametrize("tau,omega,n_analog,n_oracle", [(1.0, 0.95, 1_000_000, 20000), (3.0, 0.99, 1_000_000, 10000)])
def test_oracle_agrees_with_an_analog_polarised_monte_carlo(O, tau, omega, n_analog, n_oracle):
    ray = O.RayleighScatterer(omega, 1.0)
    g = O.PlaneGeometry(math.pi, 0.0, [O.Layer(d=tau, scatterer=ray)])
    a = analog_mc.run(tau, omega, n_analog, np.random.default_rng(5), batches=20)
    _compare(O, g, a, n_oracle, f"rayleigh tau {tau}")


def test_oracle_agrees_with_an_analog_monte_carlo_on_a_mie_slab(O):
    """Spheres x = 2, m = 1.5+0.01i (omega 0.951, asymmetry 0.63) in a slab of tau = 1. This
    exercises the oracle's Mie path: Theta drawn from calculate_csrn's inverse CDF
    (utils.jl:263-287), the Kepler azimuth, and the interpolated phase matrix in update_I
    (mie.jl:46-74). The analog run uses the same tables, which test_oracle.py pins to an
    independent Mie evaluation, but none of the oracle's sampling or transport."""
    tau = 1.0
    mie = O.MieScatterer(2.0 / (2 * math.pi), 1.5 + 0.01j, 1.0, 0.1, Ntheta=1801)
    g = O.PlaneGeometry(math.pi, 0.0, [O.Layer(d=tau * mie.kl, scatterer=mie)])
    phase = analog_mc.TabulatedPhase(mie.F11, mie.F12, mie.F33, mie.F34)
    a = analog_mc.run(tau, mie.omega, 1_000_000, np.random.default_rng(6), batches=20, phase=phase)
    _compare(O, g, a, 20000, "mie x=2 tau 1")


SPHERE_QUANTITIES = ("E", "E_mu", "E_mu2", "E_Q")


@pytest.mark.parametrize("kind,tau,n_analog,n_oracle", [("rayleigh", 2.0, 1_000_000, 20000),
                                                        ("mie", 20.0, 100_000, 3000)])
def test_oracle_agrees_with_an_analog_monte_carlo_on_spheres(O, kind, tau, n_analog, n_oracle):
    """Spheres lit along -z (src/geometries/sphere.jl) at all orders: the analog run
    (analog_mc.run_sphere: entry uniform over the disk, free flights, escape when a
    flight outruns the chord) against the oracle's forced collisions and peel-off over
    the full-range Gauss-Legendre grid, on the escaping fraction, its first and second
    moments in the exit cosine and its Q in the exit meridian frame, within 4 combined
    standard errors; the single-scattering fraction within 2%. Cases: a Rayleigh sphere
    (tau 2, omega 0.9) and the benchmark sphere (x = 2, m = 1.31, omega 1, tau 20: about
    174 events per path)."""
    if kind == "rayleigh":
        s, phase = O.RayleighScatterer(0.9, 1.0), None
    else:
        s = O.MieScatterer(2.0 / (2 * math.pi), 1.31 + 0j, 1.0, 0.1, Ntheta=1801)
        phase = analog_mc.TabulatedPhase(s.F11, s.F12, s.F33, s.F34)
    a = analog_mc.run_sphere(tau, s.omega, n_analog, np.random.default_rng(8), batches=20, phase=phase)
    g = O.SphereGeometry(R=tau * s.kl, scatterer=s)
    nb = 10
    m = n_oracle // nb
    cfg = O.Config(g, number_of_rays=m, compute_cb=False)
    mu = cfg.costheta
    o = {k: [] for k in SPHERE_QUANTITIES}
    for b in range(nb):
        r = O.simulate(cfg, g, [1, 0, 0, 0], seed=9, threads=0, photon_begin=b * m, photon_count=m)
        I, Q = r["Irt"][0].sum(1) / m, r["Irt"][1].sum(1) / m  # all bins: a sphere tallies every exit
        o["E"].append(I.sum())
        o["E_mu"].append((I * mu).sum())
        o["E_mu2"].append((I * mu * mu).sum())
        o["E_Q"].append(Q.sum())
        assert abs(r["A"][2] / m - o["E"][-1]) < 1e-12 and r["A"][3] == 0.0
    for k in SPHERE_QUANTITIES:
        ov = np.array(o[k])
        ma, sa = a[k].mean(), a[k].std(ddof=1) / math.sqrt(len(a[k]))
        mo, so = ov.mean(), ov.std(ddof=1) / math.sqrt(nb)
        z = (ma - mo) / math.hypot(sa, so)
        print(f"{kind} sphere {k}: analog {ma:.5f} +- {sa:.5f}, oracle {mo:.5f} +- {so:.5f}, z {z:.2f}")
        assert abs(z) < 4.0, (k, ma, mo, z)
    cfg1 = O.Config(g, number_of_rays=8192, compute_cb=False, maximum_scattering_times=1)
    r1 = O.simulate(cfg1, g, [1, 0, 0, 0], seed=3, rng_mode=1, threads=0)
    e1 = r1["Irt"][0].sum() / 8192
    print(f"{kind} sphere E1: analog {a['E1'].mean():.5f}, oracle {e1:.5f}")
    assert abs(a["E1"].mean() / e1 - 1) < 0.02
