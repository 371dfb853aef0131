"""Shared comparison helpers for the parity tests."""
import math
import socket

import numpy as np


def free_port() -> int:
    """A TCP port on 127.0.0.1 that the OS reports free, for a process group's store."""
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def scaled_err(a, b):
    """Max |a - b| of a tally array relative to its scale.

    Tallies of Stokes vectors (leading axis of length 4) are scaled per bin-array by
    the largest intensity |I| of the second operand, since |Q|, |U|, |V| <= I for each
    contribution; other arrays by their own largest magnitude."""
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    if b.ndim >= 1 and b.shape[0] == 4 and b.ndim == 3:
        scale = np.max(np.abs(b[0]))
    else:
        scale = np.max(np.abs(b))
    if scale == 0:
        return float(np.max(np.abs(a)))
    return float(np.max(np.abs(a - b)) / scale)


def sim_arrays(out):
    """(A, Irt, Icb) from a simulate() tuple."""
    return np.array(out[:5]), out[5], out[6]


def cb_peak_stats(stats):
    n = stats["photons"]
    mu = stats["cb_peak_sum"] / n
    var = max(stats["cb_peak_sumsq"] / n - mu * mu, 0.0)
    return mu, math.sqrt(var)


# ------------------------------------------------------------------ reciprocity
def reciprocity_z(run, costheta, n_batches):
    """Plane-slab reciprocity R(mu, mu0, phi) = R(mu0, mu, phi) for unpolarised light.

    ``run(theta, seed)`` returns ``(cfg, Irt)`` for incidence zenith ``theta`` (propagation
    azimuth 0), Irt of shape (4, Ntheta, Nphi) divided by the photon count. Incidence is
    put at each upward Gauss-Legendre node of ``costheta``. The reflection function is
    Irt[0] / (inorm mu): the normalisation under which the single-scattering result
    omega P11 [1 - exp(-tau (1/mu0 + 1/mu))] / (mu + mu0) is symmetric. Returns the
    z-scores of R(a -> b, phi_k) - R(b -> a, phi_k) over every node pair and azimuth, from
    batch means over independent seeds."""
    up = np.where(np.asarray(costheta) > 0)[0]
    R = {}
    for i in up:
        batches = []
        for k in range(n_batches):
            cfg, irt = run(math.pi - math.acos(costheta[i]), 1000 * int(i) + k)
            batches.append(irt[0] / (cfg.inorm[:, None] * cfg.costheta[:, None]))
        b = np.array(batches)
        R[i] = (b.mean(0), b.std(0, ddof=1) / math.sqrt(n_batches))
    z = []
    for a in up:
        for b in up:
            if a < b:
                z.extend(((R[a][0][b] - R[b][0][a]) / np.hypot(R[a][1][b], R[b][1][a])).tolist())
    return np.array(z)


# ------------------------------------------------------------------ run_rt restatement
# The checker for mcrt_run_rt: the Mueller assembly of src/MonteCarloRadiativeTransfer.jl
# :87-291 in numpy, fed by one simulate-like call per incident state. ``sim(I, i)``
# returns (Adt, Aabs, Aref, Atrans, Arem, Irt (4, Ntheta, Nphi), Icb (4, Ntheta_b, Nphi_b))
# already divided by number_of_rays.
def first_polarisation(I):
    for j1 in range(1, 4):  # MonteCarloRadiativeTransfer.jl:208-215
        if abs(I[j1]) > 1.0 - np.finfo(float).eps:
            return j1, float(I[j1])
    return 0, 0.0


def assemble_run_rt(cfg, g, sim):
    """(Mrt, Mcb, energy[5]) with Mrt of shape (4, 4, Ntheta, Nphi) for a plane and
    (4, 4, Ntheta) for a sphere (Mcb likewise), energy = (dt, abs, ref, trans, rem)."""
    IS = g.initial_I()
    if g.kind == 1:  # sphere, :87-184
        NFI = [i * cfg.Nphi // 8 for i in range(8)]
        NFIB = [i * cfg.Nphib // 8 for i in range(8)]
        G = np.zeros(5)
        MRT = np.zeros((4, 4, cfg.Ntheta))
        MCB = np.zeros((4, 4, cfg.Nthetab))
        for i in range(IS.shape[1]):
            I = IS[:, i]
            Adt, Aabs, Aref, _, Arem, IRT, ICB = sim(I, i)
            if I[3] == 0:
                G += [Adt, Aabs, Aref, 0.0, Arem]
                for M, X, N in ((MRT, IRT, NFI), (MCB, ICB, NFIB)):
                    M[:, 0, :] += (X[:, :, N[0]] + X[:, :, N[2]] + X[:, :, N[4]] + X[:, :, N[6]]) * 0.25
                    M[:, 1, :] += (-X[:, :, N[0]] + X[:, :, N[2]] - X[:, :, N[4]] + X[:, :, N[6]]) * 0.25
                    M[:, 2, :] += (X[:, :, N[1]] - X[:, :, N[3]] + X[:, :, N[5]] - X[:, :, N[7]]) * 0.25
            else:
                for M, X, N, n in ((MRT, IRT, NFI, cfg.Nphi), (MCB, ICB, NFIB, cfg.Nphib)):
                    M[2, 3, :] -= (X[2, :, N[0]] + X[2, :, N[4]]) * 0.5
                    M[3, 3, :] -= X[3, :, :].sum(axis=1) / n
        renorm = 1.0 / (G[0] + G[2])
        MRT *= renorm * (1.0 / cfg.inorm)[None, None, :]
        MCB *= renorm
        return MRT, MCB, G
    G = np.zeros(5)  # plane, :186-291
    MRT = np.zeros((4, 4, cfg.Ntheta, cfg.Nphi))
    MCB = np.zeros((4, 4, cfg.Nthetab, cfg.Nphib))
    for i in range(IS.shape[1]):
        I = IS[:, i]
        Adt, Aabs, Aref, Atrans, Arem, IRT, ICB = sim(I, i)
        k1, k2 = first_polarisation(I)
        if k1 == 1:
            G += np.array([Adt, Aabs, Aref, Atrans, Arem]) / 2.0
            MRT[:, 0] += IRT / 2.0
            MCB[:, 0] += ICB / 2.0
        MRT[:, k1] += k2 * IRT / 2.0
        MCB[:, k1] += k2 * ICB / 2.0
    MRT *= np.abs(1.0 / (4.0 * cfg.costheta * cfg.inorm))[None, None, :, None]  # :259
    MCB *= (1.0 / np.abs(4.0 * cfg.costhetab))[None, None, :, None]  # :273-278
    return MRT, MCB, G


def table_of(M, plane):
    """The s_ab columns of an assembled matrix in run_rt's row order (theta fastest)."""
    return {f"s{a + 1}{b + 1}": (M[a, b].reshape(-1, order="F") if plane else M[a, b])
            for a in range(4) for b in range(4)}


def tally_scale(b):
    """The scale of scaled_err: the largest |I| of a Stokes tally, else the largest |b|."""
    b = np.asarray(b, float)
    return float(np.max(np.abs(b[0]))) if b.ndim == 3 and b.shape[0] == 4 else float(np.max(np.abs(b)))


def per_element_err(a, b, floor_frac):
    """Per-element relative error max |a - b| / |b| over the elements with
    |b| >= floor_frac * scale (scale as in scaled_err). Returns (max error, elements
    compared, elements in the tally, the floor)."""
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    floor = floor_frac * tally_scale(b)
    m = np.abs(b) >= floor
    if not np.any(m):
        return 0.0, 0, int(b.size), floor
    return float(np.max(np.abs(a[m] - b[m]) / np.abs(b[m]))), int(m.sum()), int(b.size), floor


def _zstats(mean, ref, se):
    """(mean z^2, max z) of ref against mean over the elements with se > 0."""
    m = se > 0
    z = np.abs(ref - mean)[m] / se[m]
    return float(np.mean(z * z)), float(np.max(z))


def calibrated_independent_streams(M, O, cfg, g, I0, n_b, n_ref, *, nb=16, K=199, seed_gpu=101, seed_ref=202,
                                   seed_null=10000, label=""):
    """Independent-stream comparison of the FP32 kernel with the oracle, calibrated on the GPU.

    The oracle's estimate from n_ref photons on its own Philox streams is scored against
    the GPU's mean over nb batches of n_b photons: per Stokes element of Irt and Icb, z =
    |oracle - GPU| / se with se combining the GPU's batch means and the oracle's sample
    size (same per-path variance under the hypothesis tested). Per-path contributions are
    heavy tailed (a few events close to a surface dominate grazing and near-backscatter
    bins) and all bins of a tally share the same events, so these z are neither normal
    nor independent, and a fixed rule such as "at most 1% beyond 3 sigma" is broken by two
    GPU runs on different seeds. So K further GPU estimates from n_ref photons each (K
    disjoint photon ranges of a third stream) are scored the same way, and the oracle's
    mean z^2 and max z per tally, and the CB enhancement factor's |z|, must each lie within
    that reference distribution: the Monte Carlo p-value (1 + #{GPU scores >= oracle's}) /
    (K + 1) must exceed 1 / (K + 1), i.e. the oracle's score may not exceed every GPU
    score. Returns the p-values; asserts every batch is finite and free of error flags."""
    s = M.Solve(cfg.replace(number_of_rays=n_b), g, I0, precision="fp32", seed=seed_gpu)
    R, Cb, L = [], [], []
    for b in range(nb):
        s.launch(b * n_b, n_b)
        r = s.read()
        assert r["stats"]["status_flags"] & 5 == 0, r["stats"]["status_flags"]
        R.append(r["Irt"] / n_b)
        Cb.append(r["Icb"] / n_b)
        L.append(r["ladder"] / n_b)
    s.close()
    R, Cb, L = np.array(R), np.array(Cb), np.array(L)
    for t in (R, Cb, L):
        assert np.all(np.isfinite(t)), label
    f = math.sqrt(1.0 / nb + n_b / n_ref)
    mean = {"Irt": R.mean(0), "Icb": Cb.mean(0)}
    se = {"Irt": R.std(0, ddof=1) * f, "Icb": Cb.std(0, ddof=1) * f}
    enh_b = Cb[:, 0, 0, 0] / L[:, 0, 0]
    enh, se_enh = float(enh_b.mean()), float(enh_b.std(ddof=1) * f)

    def score(irt, icb, lad):
        return {"Irt": _zstats(mean["Irt"], irt, se["Irt"]), "Icb": _zstats(mean["Icb"], icb, se["Icb"]),
                "enh": (abs(icb[0, 0, 0] / lad[0, 0] - enh) / se_enh,)}

    cfg_ref = cfg.replace(number_of_rays=n_ref)
    ref = O.simulate(cfg_ref, g, I0, seed=seed_ref, threads=0)
    got = score(ref["Irt"] / n_ref, ref["Icb"] / n_ref, ref["ladder"] / n_ref)
    null = []
    s = M.Solve(cfg_ref, g, I0, precision="fp32", seed=seed_null)
    for k in range(K):
        s.launch(k * n_ref, n_ref)
        r = s.read()
        assert r["stats"]["status_flags"] & 5 == 0, r["stats"]["status_flags"]
        null.append(score(r["Irt"] / n_ref, r["Icb"] / n_ref, r["ladder"] / n_ref))
    s.close()
    pv = {}
    for key, names in (("Irt", ("mean z^2", "max z")), ("Icb", ("mean z^2", "max z")), ("enh", ("|z|",))):
        for i, stat in enumerate(names):
            vals = np.array([nz[key][i] for nz in null])
            p = (1 + int(np.sum(vals >= got[key][i]))) / (K + 1)
            lo, hi = np.percentile(vals, [1, 99])
            print(f"{label} {key} {stat}: oracle {got[key][i]:.3g}, GPU samples 1-99% [{lo:.3g}, {hi:.3g}], p {p:.3f}")
            pv[(key, stat)] = p
    enh_ref = ref["Icb"][0, 0, 0] / ref["ladder"][0, 0]
    print(f"{label} CB enhancement GPU {enh:.5f} oracle {enh_ref:.5f}")
    assert 1.0 < enh <= 2.0 and 1.0 < enh_ref <= 2.0
    return pv
