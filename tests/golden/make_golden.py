"""Generates the golden fixtures in this directory (run once; the outputs are committed).

* philox_kat.json: published known-answer vectors of Philox4x32-10 (Salmon et al.,
  SC'11; the Random123 distribution's kat_vectors).
* mie_scipy.json: Mie efficiencies, asymmetry and amplitude functions S1, S2 computed
  independently of bhmie's logarithmic-derivative recurrence, from Riccati-Bessel
  functions built on scipy.special.spherical_jn / spherical_yn, for the size
  parameters and refractive indices of the benchmark configurations.

    python tests/golden/make_golden.py
"""
import json
import math
import os

import numpy as np
from scipy.special import spherical_jn, spherical_yn

HERE = os.path.dirname(os.path.abspath(__file__))

PHILOX_KAT = [
    {"ctr": [0, 0, 0, 0], "key": [0, 0], "out": [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]},
    {"ctr": [0xFFFFFFFF] * 4, "key": [0xFFFFFFFF] * 2,
     "out": [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]},
    {"ctr": [0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], "key": [0xA4093822, 0x299F31D0],
     "out": [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]},
]


def riccati(n, z):
    """psi_n(z) = z j_n(z), xi_n(z) = z h1_n(z) and their derivatives."""
    j = spherical_jn(n, z)
    jd = spherical_jn(n, z, derivative=True)
    psi = z * j
    dpsi = j + z * jd
    return psi, dpsi


def mie_coefficients(x, m, nstop):
    n = np.arange(1, nstop + 1)
    mx = m * x
    psi_x, dpsi_x = riccati(n, x)
    y = spherical_yn(n, x)
    yd = spherical_yn(n, x, derivative=True)
    xi_x = psi_x + 1j * x * y
    dxi_x = dpsi_x + 1j * (y + x * yd)
    psi_m, dpsi_m = riccati(n, mx)
    a = (m * psi_m * dpsi_x - psi_x * dpsi_m) / (m * psi_m * dxi_x - xi_x * dpsi_m)
    b = (psi_m * dpsi_x - m * psi_x * dpsi_m) / (psi_m * dxi_x - m * xi_x * dpsi_m)
    return n, a, b


def mie(x, m, angles_deg):
    nstop = int(math.floor(max(x + 4 * x ** (1 / 3) + 2, x * abs(m))))
    n, a, b = mie_coefficients(x, m, nstop)
    qext = 2 / x ** 2 * np.sum((2 * n + 1) * (a + b).real)
    qsca = 2 / x ** 2 * np.sum((2 * n + 1) * (abs(a) ** 2 + abs(b) ** 2))
    g = np.sum(n[:-1] * (n[:-1] + 2) / (n[:-1] + 1) * (a[:-1] * np.conj(a[1:]) + b[:-1] * np.conj(b[1:])).real)
    g += np.sum((2 * n + 1) / (n * (n + 1)) * (a * np.conj(b)).real)
    g *= 4 / (x ** 2 * qsca)
    S1, S2 = [], []
    for th in np.deg2rad(angles_deg):
        mu = math.cos(th)
        pi = np.zeros(nstop + 1)
        tau = np.zeros(nstop + 1)
        pi[1] = 1.0
        tau[1] = mu
        for k in range(2, nstop + 1):
            pi[k] = ((2 * k - 1) * mu * pi[k - 1] - k * pi[k - 2]) / (k - 1)
            tau[k] = k * mu * pi[k] - (k + 1) * pi[k - 1]
        f = (2 * n + 1) / (n * (n + 1))
        S1.append(np.sum(f * (a * pi[1:] + b * tau[1:])))
        S2.append(np.sum(f * (a * tau[1:] + b * pi[1:])))
    return {"x": x, "m": [m.real, m.imag], "nstop": nstop, "q_ext": qext, "q_sca": qsca, "asymm": g,
            "angles_deg": list(angles_deg), "S1": [[s.real, s.imag] for s in S1],
            "S2": [[s.real, s.imag] for s in S2]}


def main():
    with open(os.path.join(HERE, "philox_kat.json"), "w") as f:
        json.dump(PHILOX_KAT, f, indent=1)
    angles = [0.0, 30.0, 60.0, 90.0, 120.0, 150.0, 180.0]
    cases = [mie(5.0, 1.5 + 0.001j, angles), mie(2.0, 1.31 + 0.0j, angles), mie(0.5, 1.3 + 1e-5j, angles),
             mie(10.0, 1.6 + 0.01j, angles)]
    with open(os.path.join(HERE, "mie_scipy.json"), "w") as f:
        json.dump(cases, f, indent=1)


if __name__ == "__main__":
    main()
