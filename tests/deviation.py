"""Deviation measures shared by the GPU parity tests."""

import numpy as np

PLANES = ((6, 8), (7, 9), (10, 12))  # (x, px), (y, py), (zeta, delta) rows


def f64(block, row):
    return block[row].view(np.float64)


def amplitude_dev(got, exp, init):
    """Per-particle deviation normalised by that particle's phase-space
    amplitude, for the three planes (x, px), (y, py), (zeta, delta): with
    r = rms(u) / rms(pu) of the sample, the amplitude is
    A = max over the initial and final state of sqrt(u^2 + (r pu)^2), and
    the deviation is max(|du|, r |dpu|) / A.  Returns the median, the 99th
    percentile and the maximum over particles."""
    worst = np.zeros(got.shape[1])
    for u, pu in PLANES:
        eu, epu = f64(exp, u), f64(exp, pu)
        iu, ipu = f64(init, u), f64(init, pu)
        r = np.std(eu) / max(np.std(epu), 1e-300)
        amp = np.maximum(np.hypot(eu, r * epu), np.hypot(iu, r * ipu))
        amp = np.maximum(amp, 1e-6 * np.max(amp))
        d = np.maximum(np.abs(f64(got, u) - eu), r * np.abs(f64(got, pu) - epu)) / amp
        worst = np.maximum(worst, d)
    return float(np.median(worst)), float(np.percentile(worst, 99)), float(np.max(worst))
