"""The oracle's coherent-backscattering cone against exact second-order results.

A Rayleigh scatterer radiates the field P(k) E, P(k) = I - k k^T, into direction k, so a
double-scattering path (x1 then x2, exit direction k_b) and its reversal (x2 then x1)
carry the same field P(k_b) P(k1) E0, whatever the polarisation. Two exact consequences
for the second order (the tallies of a run of two orders minus those of a run of one
order on the same streams):

- At exact backscatter the reversed paths are in phase and equally attenuated, so the
  CB intensity is exactly twice the ladder, path by path: a deterministic identity of
  the reference's reciprocal-path sum (src/cpu.jl:38-126: the forward and backward
  fields, the scaling to the incoherent intensity, the Ia / (Ia + Ib) share), for the
  plane and the sphere and every incident state.
- Off backscatter the interference is the ladder's integrand times
  cos(kl (k0 + k_b).(x2 - x1)) with the geometric mean of the two paths' attenuations.
  Both expectations are four-dimensional integrals (first depth, scattering direction,
  second flight) evaluated here by quadrature, at the reference's own CB bin directions
  (the bin grid in the frame of the exact backscatter direction, src/cpu.jl:85-90).
  This pins the interference phase, the cone's shape and anisotropy, the bin
  directions and the reversed path's attenuation, none of which the exact-backscatter
  checks can see (the phase vanishes there)."""
import math

import numpy as np
import pytest

STATES = ([1.0, 0, 0, 0], [1, 1, 0, 0], [1, 0, 1, 0], [1, 0, 0, 1])


def cb_direction(kf, theta_b, phi_b):
    """The CB bin (theta_b, phi_b) as a direction: (sin theta_b cos phi_b,
    sin theta_b sin phi_b, cos theta_b) in the frame whose pole is kf, the exact
    backscatter direction, with the reference's orientation of that frame."""
    ct = kf[2]
    st = math.sqrt(max(1 - ct * ct, 0.0))
    si = 1 / math.hypot(kf[0], kf[1])
    cp, sp = kf[0] * si, kf[1] * si
    v = (math.sin(theta_b) * math.cos(phi_b), math.sin(theta_b) * math.sin(phi_b), math.cos(theta_b))
    return np.array([v[0] * ct * cp - v[1] * sp + v[2] * st * cp, v[0] * ct * sp + v[1] * cp + v[2] * st * sp,
                     -v[0] * st + v[2] * ct])


def second_order_cb(tau, omega, theta0, kl, kbs, n1=32, nmu=64, nphi=64, n2=32):
    """Expected second-order ladder and CB intensity per photon (no quadrature weight, as
    the CB tallies) in each direction of `kbs`, for unpolarised light on a Rayleigh slab
    of optical thickness tau, incident from above at polar angle theta0 and azimuth 0.

    Per ordered path the ladder integrand is
        omega^2 / 4pi * (9/8) |P(kb) P(k1) Pi0|_F^2 * e^{-s1} e^{-s2} e^{-d(x2, kb)},
    (Pi0 the projector normal to k0: the average over two orthogonal incident fields),
    and the interference replaces e^{-s1 - d(x2, kb)} by
        e^{-(s1 + d(x2, kb) + d_in(x2) + d(x1, kb)) / 2} cos(kl (k0 + kb).(x2 - x1)).
    s1 and s2 are drawn through truncated-exponential substitutions, so the quadrature
    sees smooth integrands."""
    k0 = np.array([math.sin(theta0), 0.0, math.cos(theta0)])
    mu0 = -k0[2]
    g1, gw1 = np.polynomial.legendre.leggauss(n1)
    u1, w1 = (g1 + 1) / 2, gw1 / 2
    gm, gwm = np.polynomial.legendre.leggauss(nmu)
    ph = (np.arange(nphi) + 0.5) * 2 * math.pi / nphi
    g2, gw2 = np.polynomial.legendre.leggauss(n2)
    u2, w2 = (g2 + 1) / 2, gw2 / 2
    J1 = -np.expm1(-tau / mu0)
    s1 = -np.log1p(-u1 * J1)
    Pi0 = np.eye(3) - np.outer(k0, k0)
    st = np.sqrt(1 - gm ** 2)
    K1 = np.stack([st[:, None] * np.cos(ph), st[:, None] * np.sin(ph), np.repeat(gm[:, None], nphi, 1)], -1)
    WK = gwm[:, None] * (2 * math.pi / nphi)
    P1 = np.eye(3) - K1[..., :, None] * K1[..., None, :]
    kz = K1[..., 2]
    out = []
    for kb in kbs:
        Pf = np.eye(3) - np.outer(kb, kb)
        M = np.einsum("ij,abjk,kl->abil", Pf, P1, Pi0)
        w = 9.0 / 8.0 * (M ** 2).sum((-1, -2)) * WK
        q = ((k0 + kb) @ K1.reshape(-1, 3).T).reshape(kz.shape)
        lad = intf = 0.0
        for i in range(n1):
            z1 = s1[i] * k0[2]
            smax = np.where(kz > 0, -z1 / np.where(kz > 0, kz, 1), (z1 + tau) / np.where(kz < 0, -kz, 1))
            J2 = -np.expm1(-smax)
            s2 = -np.log1p(-u2 * J2[..., None])
            z2 = z1 + s2 * kz[..., None]
            dout2, dout1, din2 = -z2 / kb[2], -z1 / kb[2], -z2 / mu0
            base = (w * J2)[..., None] * w2 * (w1[i] * J1)
            lad += np.sum(base * np.exp(-dout2))
            intf += np.sum(base * np.exp(0.5 * s1[i] - 0.5 * (dout2 + din2 + dout1)) * np.cos(kl * s2 * q[..., None]))
        out.append((lad, lad + intf))
    return np.array(out) * omega ** 2 / (4 * math.pi)


def _second_order(O, cfg_for, g, I0, seed, n):
    r = {ms: O.simulate(cfg_for(ms), g, I0, seed=seed, threads=0, cb_form=1) for ms in (1, 2)}
    return (r[2]["ladder"] - r[1]["ladder"]) / n, (r[2]["Icb"] - r[1]["Icb"]) / n


@pytest.mark.parametrize("geom", ["plane", "sphere"])
def test_second_order_rayleigh_cb_is_twice_the_ladder_at_exact_backscatter(O, geom):
    ray = O.RayleighScatterer(0.9, 10.0)
    if geom == "plane":
        g = O.PlaneGeometry(math.radians(150.0), 0.0, [O.Layer(d=1.0 * ray.kl, scatterer=ray)])
    else:
        g = O.SphereGeometry(R=2.0 * ray.kl, scatterer=ray)
    n = 4096
    cfg_for = lambda ms: O.Config(g, number_of_rays=n, compute_cb=True, maximum_scattering_times=ms, Ntheta=16,
                                  Nphi=8, thetab=np.radians([0.0, 2.0, 5.0]), Nphib=2)
    for I0 in STATES:
        lad, icb = _second_order(O, cfg_for, g, I0, 3, n)
        assert lad[0, 0] > 0
        assert np.max(np.abs(icb[0, 0, :] / lad[0, :] - 2.0)) < 1e-12, (I0, icb[0, 0, :] / lad[0, :])
        assert np.all(icb[0, 1:, :] < 2.0 * lad[1:, :])  # off backscatter the paths dephase


def test_second_order_rayleigh_cb_cone_matches_the_exact_integral(O):
    """Slab tau = 1, omega 0.9, kl = 10 (a cone some 10 degrees wide), unpolarised light at
    30 degrees incidence, the default RT grid; CB bins at theta_b = 0..20 degrees and
    phi_b = 0 and 90 degrees (the cone is not round at oblique incidence); 16 batches of
    8 192 photons. Ladder and CB intensity within 4 se of the exact values in every bin,
    and the enhancement within 0.2% (the quadrature is converged to 2e-4)."""
    tau, omega, theta0, kl = 1.0, 0.9, math.radians(150.0), 10.0
    tbs = np.radians([0.0, 2, 4, 6, 8, 10, 15, 20])
    pbs = np.radians([0.0, 90.0, 180.0, 270.0])
    kf = -np.array([math.sin(theta0), 0.0, math.cos(theta0)])
    kbs = [cb_direction(kf, tb, pb) for pb in pbs[:2] for tb in tbs]
    exact = second_order_cb(tau, omega, theta0, kl, kbs)
    ray = O.RayleighScatterer(omega, kl)
    g = O.PlaneGeometry(theta0, 0.0, [O.Layer(d=tau * kl, scatterer=ray)])
    nb, n = 16, 8192
    cfg_for = lambda ms: O.Config(g, number_of_rays=n, compute_cb=True, maximum_scattering_times=ms, thetab=tbs,
                                  Nphib=len(pbs))
    bat = []
    for b in range(nb):
        lad, icb = _second_order(O, cfg_for, g, [1, 0, 0, 0], 70 + b, n)
        bat.append(np.stack([lad[:, :2].T.ravel(), icb[0][:, :2].T.ravel()], -1))
    bat = np.array(bat)
    mean = bat.mean(0)
    z = (mean - exact) / (bat.std(0, ddof=1) / math.sqrt(nb))
    enh, enh_exact = mean[:, 1] / mean[:, 0], exact[:, 1] / exact[:, 0]
    for i in range(len(kbs)):
        print(f"theta_b {math.degrees(tbs[i % len(tbs)]):4.1f} phi_b {math.degrees(pbs[i // len(tbs)]):3.0f}: "
              f"enhancement {enh[i]:.4f} (exact {enh_exact[i]:.4f}), z {z[i, 0]:+.2f} {z[i, 1]:+.2f}")
    assert np.abs(z).max() < 4.0
    assert np.max(np.abs(enh / enh_exact - 1)) < 2e-3
    assert enh_exact[0] == pytest.approx(2.0, abs=1e-12) and enh_exact[len(tbs) - 1] < 1.6
