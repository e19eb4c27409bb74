"""The statistic tolerance of the GPU parity tests.

Every score (raw, APC- or ASC-corrected) must be within 1e-5 relative of the
FP64 oracle on each pair whose magnitude is at least 1e-3 of the largest
magnitude of that score matrix; the smaller ones within 1e-8 of that largest
magnitude, absolute (the relative bound taken at the threshold).  There is
no term scaled by the raw, uncorrected scores: a corrected score is held to
its own size.
"""
import numpy as np

RTOL = 1e-5
FLOOR = 1e-3


def stat_errors(gpu, ref):
    """(max relative error over the pairs at or above the floor, max absolute
    error below it divided by the largest |ref|)."""
    gpu = np.asarray(gpu, dtype=np.float64).ravel()
    ref = np.asarray(ref, dtype=np.float64).ravel()
    if ref.size == 0:
        return 0.0, 0.0
    m = float(np.max(np.abs(ref)))
    if m == 0.0:
        return 0.0, float(np.max(np.abs(gpu)))
    big = np.abs(ref) >= FLOOR * m
    err = np.abs(gpu - ref)
    rel = float(np.max(err[big] / np.abs(ref[big]), initial=0.0))
    small = float(np.max(err[~big], initial=0.0)) / m
    return rel, small


def stat_close(gpu, ref, rtol=RTOL):
    """True when gpu meets the bound against ref; also returns the two error
    figures of stat_errors."""
    rel, small = stat_errors(gpu, ref)
    return (rel <= rtol and small <= rtol * FLOOR), rel, small
