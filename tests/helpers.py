"""Shared comparison helpers for the parity tests."""
import math

import numpy as np


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
