"""A deterministic vector adding-doubling solver for a homogeneous plane-parallel layer,
written for the tests independently of the oracle and of the library.

It gives the exact (to quadrature accuracy) reflection and diffuse transmission matrices
R(mu, mu0, phi - phi0) and T(mu, mu0, phi - phi0) of polarised light at all scattering
orders, by the published adding-doubling method: Hansen & Travis, "Light scattering in
planetary atmospheres", Space Sci. Rev. (1974) (the adding equations in kernel form),
and de Haan, Bosma & Hovenier, "The adding method for multiple scattering calculations
of polarized light", Astron. Astrophys. (1987) (the same for the full Stokes vector,
mode by mode in azimuth). The normalisation is theirs: for a parallel beam of net flux
pi F per unit area normal to the beam, incident at cosine mu0, the reflected radiance
is I(mu, phi) = mu0 R(mu, mu0, phi - phi0) F.

How it is built:
- Directions are (mu, phi), k = (sqrt(1 - mu^2) cos phi, sqrt(1 - mu^2) sin phi, mu),
  mu > 0 upwards. Stokes vectors are taken in the meridian frame (e1, e2) =
  (d k / d theta, d k / d phi normalised), which is right-handed with k, with
  Q = I_1 - I_2 and U = 2 Re(E1 conj(E2)).
- The phase matrix Z(k <- k') in those frames is assembled by explicit vector geometry:
  the incident Stokes vector is rotated into the scattering-plane frame
  (n x k', n), n = k' x k / |k' x k|, multiplied by the scattering matrix
  [[F11, F12, 0, 0], [F12, F11, 0, 0], [0, 0, F33, F34], [0, 0, -F34, F33]] and rotated
  into the exit meridian frame. No closed-form Fourier decomposition is used: each
  azimuthal mode Z_m = (1/2 pi) int Z e^{-i m dphi} d dphi is a discrete Fourier sum over
  an azimuth grid offset by half a step (so exact forward and backward scattering,
  where the scattering plane is undefined, are never evaluated).
- Each complex mode m >= 0 is doubled on its own from a layer of optical thickness
  tau / 2^n_doublings, initialised with its exact single-scattering kernels. The adding
  equations are applied in kernel form (products A o B = 2 int A B mu' dmu' through the
  quadrature weights), with the direct beam attenuation exp(-tau / mu) kept apart, so
  that output and incidence cosines can be nodes of zero weight: they take no part in
  the internal integrals but get exact kernels. Reflection and transmission from below
  are doubled alongside those from above (no symmetry relation is assumed).
- R(dphi) = Re R_0 + 2 Re sum_{m >= 1} R_m e^{i m dphi}.
"""
from __future__ import annotations

import math

import numpy as np


def rayleigh_matrix(c):
    """F11, F12, F33, F34 of Rayleigh scattering (normalised to a sphere average of 1)."""
    c = np.asarray(c, float)
    return 0.75 * (1 + c * c), -0.75 * (1 - c * c), 1.5 * c, np.zeros_like(c)


class TabulatedMatrix:
    """F11, F12, F33, F34 tabulated on uniform scattering angles over [0, pi], linear in the
    angle between nodes (the form in which the transport code interpolates its tables)."""

    def __init__(self, F11, F12, F33, F34):
        self.F = [np.asarray(f, float) for f in (F11, F12, F33, F34)]
        self.theta = np.linspace(0.0, math.pi, len(self.F[0]))

    def __call__(self, c):
        th = np.arccos(np.clip(c, -1.0, 1.0))
        return tuple(np.interp(th, self.theta, f) for f in self.F)


def _frame(mu, phi):
    mu = np.asarray(mu, float)
    st = np.sqrt(np.maximum(1.0 - mu * mu, 0.0))
    cp, sp = np.cos(phi), np.sin(phi)
    k = np.stack([st * cp, st * sp, mu * np.ones_like(cp)], -1)
    e1 = np.stack([mu * cp, mu * sp, -st * np.ones_like(cp)], -1)
    e2 = np.stack([-sp * np.ones_like(mu), cp * np.ones_like(mu), np.zeros_like(mu * cp)], -1)
    return k, e1, e2


def _rot(c, s):
    """Stokes rotation matrices for frames turned by chi, given cos chi and sin chi."""
    c2, s2 = c * c - s * s, 2 * s * c
    L = np.zeros(c.shape + (4, 4))
    L[..., 0, 0] = 1.0
    L[..., 3, 3] = 1.0
    L[..., 1, 1] = c2
    L[..., 1, 2] = s2
    L[..., 2, 1] = -s2
    L[..., 2, 2] = c2
    return L


def phase_matrix(mu_out, phi_out, mu_in, phi_in, F):
    """Z(k_out <- k_in) in meridian frames; the arguments broadcast against each other.
    `F` maps cos(Theta) to (F11, F12, F33, F34)."""
    ko, e1o, e2o = _frame(mu_out, phi_out)
    ki, e1i, e2i = _frame(mu_in, phi_in)
    ko, e1o, e2o, ki, e1i, e2i = np.broadcast_arrays(ko, e1o, e2o, ki, e1i, e2i)
    c = np.clip(np.einsum("...i,...i", ki, ko), -1.0, 1.0)
    n = np.cross(ki, ko)
    nn = np.linalg.norm(n, axis=-1)
    deg = nn < 1e-12
    n = np.where(deg[..., None], e2i, n / np.where(deg, 1.0, nn)[..., None])
    par_i = np.cross(n, ki)
    par_o = np.cross(n, ko)
    # into the scattering-plane frame: e1' = par_i, measured in (e1i, e2i)
    Lin = _rot(np.einsum("...i,...i", e1i, par_i), np.einsum("...i,...i", e2i, par_i))
    # out of it: e1' = e1o, measured in (par_o, n)
    Lout = _rot(np.einsum("...i,...i", par_o, e1o), np.einsum("...i,...i", n, e1o))
    F11, F12, F33, F34 = F(c)
    S = np.zeros(c.shape + (4, 4))
    S[..., 0, 0] = S[..., 1, 1] = F11
    S[..., 0, 1] = S[..., 1, 0] = F12
    S[..., 2, 2] = S[..., 3, 3] = F33
    S[..., 2, 3] = F34
    S[..., 3, 2] = -F34
    return Lout @ S @ Lin


def fourier_modes(mu_out, mu_in, F, n_modes, n_azimuth):
    """Z_m(mu_out <- mu_in), m = 0..n_modes, shape (n_modes + 1, len(mu_out), len(mu_in), 4, 4),
    complex; also the largest |Z_m| over the modes n_modes+1 .. n_azimuth/2 - 1 (what the
    truncation drops)."""
    K = int(n_azimuth)
    if n_modes >= K // 2:
        raise ValueError("n_azimuth must exceed twice the number of modes")
    dphi = (np.arange(K) + 0.5) * (2 * math.pi / K)
    mu_out = np.asarray(mu_out, float)
    mi = np.asarray(mu_in, float)[None, :, None]
    # the grid's half-step offset turns the DFT into e^{-i pi m / K} times an FFT
    shift = np.exp(-1j * math.pi * np.arange(K // 2) / K)
    out = np.zeros((n_modes + 1, len(mu_out), mi.shape[1], 4, 4), complex)
    drop = 0.0
    step = max(1, int(2e6 // (mi.shape[1] * K)))
    for a in range(0, len(mu_out), step):
        mo = mu_out[a:a + step, None, None]
        Z = phase_matrix(mo, dphi[None, None, :], mi, 0.0, F)  # (no, ni, K, 4, 4)
        Zm = np.fft.rfft(Z, axis=2)[:, :, : K // 2] / K
        Zm = np.moveaxis(Zm * shift[None, None, :, None, None], 2, 0)
        out[:, a:a + step] = Zm[: n_modes + 1]
        if n_modes + 1 < K // 2:
            drop = max(drop, float(np.abs(Zm[n_modes + 1:]).max()))
    return out, drop


class DoublingSolution:
    """R and T (with R* and T* from below) per azimuthal mode at the node cosines
    `nodes` (quadrature `weights`, zero for the added cosines); `dropped_mode_norm` is the
    largest azimuthal mode of the phase matrix left out."""

    def __init__(self, nodes, weights, modes_R, modes_T, modes_Rs, modes_Ts, tau, dropped_mode_norm):
        self.nodes, self.weights, self.tau = nodes, weights, tau
        self.R, self.T, self.Rs, self.Ts = modes_R, modes_T, modes_Rs, modes_Ts
        self.dropped_mode_norm = dropped_mode_norm

    def _index(self, m):
        i = np.flatnonzero(np.isclose(self.nodes, m, rtol=0, atol=1e-14))
        if len(i) == 0:
            raise KeyError(f"cosine {m} is not a node of this solution")
        return int(i[0])

    def _eval(self, modes, mu_out, mu_in, dphi):
        i, j = self._index(mu_out), self._index(mu_in)
        blk = modes[:, 4 * i:4 * i + 4, 4 * j:4 * j + 4]  # (M+1, 4, 4)
        m = np.arange(blk.shape[0])
        ph = np.exp(1j * np.multiply.outer(np.atleast_1d(dphi), m))  # (n, M+1)
        w = np.where(m == 0, 1.0, 2.0)
        return np.real(np.einsum("nm,mij->nij", ph * w, blk))

    def reflection(self, mu, mu0, dphi):
        """R(mu, mu0, dphi): light incident from above at cosine mu0 (travelling downwards),
        reflected upwards at cosine mu; shape (len(dphi), 4, 4)."""
        return self._eval(self.R, mu, mu0, dphi)

    def transmission(self, mu, mu0, dphi):
        """Diffuse T(mu, mu0, dphi): incident from above at mu0, leaving the bottom
        downwards at cosine mu (given as a positive number)."""
        return self._eval(self.T, mu, mu0, dphi)


def solve(tau, omega, F, quad_mu, quad_w, extra_mu=(), n_modes=2, n_azimuth=16, n_doublings=30):
    """Reflection and transmission matrices of a homogeneous layer of optical thickness
    `tau` and single-scattering albedo `omega`.

    quad_mu, quad_w: a quadrature on (0, 1] for the internal integrals (weights summing to
    1); extra_mu: further cosines (incidence, outputs) carried with zero weight."""
    qm = np.asarray(quad_mu, float)
    ex = np.array([m for m in np.atleast_1d(np.asarray(extra_mu, float))
                   if not np.any(np.isclose(qm, m, rtol=0, atol=1e-14))])
    ex = np.unique(ex) if len(ex) else ex
    u = np.concatenate([qm, ex])
    W = np.concatenate([np.asarray(quad_w, float), np.zeros(len(ex))])
    n = len(u)
    d = tau / 2.0 ** n_doublings
    # mode decomposition of the phase matrix for the four hemisphere pairs
    Zr, dr = fourier_modes(u, -u, F, n_modes, n_azimuth)    # up <- down (reflection from above)
    Zt, dt = fourier_modes(-u, -u, F, n_modes, n_azimuth)   # down <- down
    Zrs, drs = fourier_modes(-u, u, F, n_modes, n_azimuth)  # down <- up (reflection from below)
    Zts, dts = fourier_modes(u, u, F, n_modes, n_azimuth)   # up <- up
    dropped = max(dr, dt, drs, dts)
    ui, uj = u[:, None], u[None, :]
    r0 = omega / 4.0 * -np.expm1(-d * (1 / ui + 1 / uj)) / (ui + uj)
    # (e^{-d/ui} - e^{-d/uj}) / (ui - uj) = e^{-d/max(.)} (1 - e^{-y}) / y * d / (ui uj),
    # y = d |ui - uj| / (ui uj): no cancellation for close cosines, no overflow for thick layers
    y = d * np.abs(ui - uj) / (ui * uj)
    ys = np.where(y == 0.0, 1.0, y)
    g = np.where(y == 0.0, 1.0, -np.expm1(-ys) / ys)
    t0 = omega / 4.0 * np.exp(-d / np.maximum(ui, uj)) * g * d / (ui * uj)
    expand = lambda s, Zm: np.einsum("ab,mabij->maibj", s, Zm).reshape(Zm.shape[0], 4 * n, 4 * n)
    R, T, Rs, Ts = expand(r0, Zr), expand(t0, Zt), expand(r0, Zrs), expand(t0, Zts)
    Mw = np.repeat(2.0 * W * u, 4)  # kernel products A o B = A diag(Mw) B
    I = np.eye(4 * n)
    for _ in range(n_doublings):
        e = np.repeat(np.exp(-d / u), 4)
        R, T, Rs, Ts = [np.stack(v) for v in zip(*[_double(R[m], T[m], Rs[m], Ts[m], e, Mw, I)
                                                   for m in range(R.shape[0])])]
        d *= 2.0
    return DoublingSolution(u, W, R, T, Rs, Ts, tau, dropped)


def _double(R, T, Rs, Ts, e, Mw, I):
    """One doubling step with the adding equations in kernel form (Hansen & Travis
    1974), for incidence from above and, with the roles of the two sides exchanged, from
    below: layers a and b are the same layer."""
    def add(Ra, Ta, Rsa, Tsa):
        # light from above on a, then b = the same layer
        Q = (Rsa * Mw) @ Ra
        S = np.linalg.solve(I - Q * Mw, Q)
        D = Ta + (S * Mw) @ Ta + S * e[None, :]
        U = (Ra * Mw) @ D + Ra * e[None, :]
        R2 = Ra + e[:, None] * U + (Tsa * Mw) @ U
        T2 = e[:, None] * D + Ta * e[None, :] + (Ta * Mw) @ D
        return R2, T2

    R2, T2 = add(R, T, Rs, Ts)
    Rs2, Ts2 = add(Rs, Ts, R, T)
    return R2, T2, Rs2, Ts2


def _cross_stokes(u, v):
    """The Stokes parameters of the cross term of fields u and v (u = v gives the Stokes
    vector of u): Re(u1 v1* + u2 v2*), Re(u1 v1* - u2 v2*), Re(u1 v2* + v1 u2*),
    Im(u1 v2* + v1 u2*)."""
    a, b = u[0] * np.conj(v[0]), u[1] * np.conj(v[1])
    c = u[0] * np.conj(v[1]) + v[0] * np.conj(u[1])
    return np.array([(a + b).real, (a - b).real, c.real, c.imag])


def cyclical_map():
    """The linear map C = cyclical(L) of coherent backscattering in exactly the
    backscattering direction, as a 16 x 16 matrix acting on L.ravel().

    L is the multiple-scattering (ladder) part of the reflection matrix at
    (mu0, mu0, dphi = pi), with the incident Stokes vector in its meridian frame (e1, e2)
    and the reflected one in the exit meridian frame, which is (e1, -e2) because the
    exit direction is the reverse of the incident one. By reciprocity (the scattering
    dyadic of a path equals the transpose of its time-reversed path's,
    A(k_b, k_a) = A^T(-k_a, -k_b)), a path with Jones matrix S in those frames has a
    reversed partner with Jones matrix J S^T J, J = diag(1, -1). The interference of the
    two adds, per path, the cross term of S E and J S^T J E to the reflected Stokes
    vector; C is the ensemble sum of those cross terms as L is the sum of the paths'
    Mueller matrices. Both are linear in the paths' coherency S (x) S*, so C is a linear
    function of L, found here by least squares over random Jones matrices. Its (1, 1)
    element is (L11 + L22 - L33 + L44) / 2, the relation Mishchenko derived for exact
    backscattering (J. Opt. Soc. Am. A, 1992)."""
    E = [np.array([1, 0], complex), np.array([0, 1], complex), np.array([1, 1], complex) / math.sqrt(2),
         np.array([1, 1j], complex) / math.sqrt(2)]
    Sv_inv = np.linalg.inv(np.array([_cross_stokes(e, e) for e in E]).T)
    J = np.diag([1.0, -1.0])
    rng = np.random.default_rng(0)
    A, B = [], []
    for _ in range(64):
        S = rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2))
        Sr = J @ S.T @ J
        A.append((np.array([_cross_stokes(S @ e, S @ e) for e in E]).T @ Sv_inv).ravel())
        B.append((np.array([_cross_stokes(S @ e, Sr @ e) for e in E]).T @ Sv_inv).ravel())
    A, B = np.array(A), np.array(B)
    Phi, _, rank, _ = np.linalg.lstsq(A, B, rcond=None)
    assert rank == 16 and np.abs(A @ Phi - B).max() < 1e-10  # exactly linear in the coherency
    return Phi


def cyclical(L):
    """C from L (4 x 4), see cyclical_map."""
    return (np.asarray(L, float).ravel() @ cyclical_map()).reshape(4, 4)


def half_range_gauss(n):
    """Gauss-Legendre nodes and weights on (0, 1], weights summing to 1, nodes ascending."""
    x, w = np.polynomial.legendre.leggauss(int(n))
    return (x + 1.0) / 2.0, w / 2.0
