"""The reference's deconvolved density profile solve, restated with numpy/scipy (TEST INFRASTRUCTURE).

Restates ``bbarolo/profile.py``: ``_second_differences`` (:60-62), ``_second_difference_rows`` (:68-85),
``_relative_rows`` (:141-151) and ``solve_profile`` (:91-138): the non-negative least-squares densities of
``A dens = b`` (QR of A, then scipy's NNLS on the small system) with the smoothness prior on the second
differences of the profile, in two solves (a relative prior first, then a prior scaled by the first solution
and its reduced chi2). The same numpy/scipy calls in the same order as the reference, so the result is the
reference's on the same machine (checked against ``tests/golden/profile.npz``).

Used only by the tests (as the checker of the device solve) and by the CPU-baseline leg of ``bench.py``.
"""

import math

import numpy as np

DENSPROF_SMOOTH = 0.3
DENSPROF_FLOOR = 0.05


def second_differences(d1, d2):
    """Weights of the second difference at distance d1 from the previous radius and d2 from the next."""
    return np.array([1. / d1, -1. / d1 - 1. / d2, 1. / d2]) * 2. / (d1 + d2)


def second_difference_rows(R):
    """(L, o, Rs, tiny, dmin): the rows of the second differences at the radii R in order of radius."""
    R = np.asarray(R, float)
    n = R.size
    o = np.argsort(R, kind="stable")
    Rs = R[o]
    tiny = 1e-6 * max(float(np.ptp(R)), 1e-300)
    dmin = max(0.25 * float(np.min(np.diff(np.sort(R[:-1])))), tiny) if n > 2 else tiny
    L = np.zeros((n - 2, n))
    for i in range(1, n - 1):
        d1, d2 = (max(float(d), tiny) for d in (Rs[i] - Rs[i - 1], Rs[i + 1] - Rs[i]))
        L[i - 1, o[i - 1:i + 2]] = second_differences(d1, d2)
    return L, o, Rs, tiny, dmin


def relative_norm(radii):
    """The sum of the squared second-difference weights of the relative prior (distances at least dmin)."""
    L, o, Rs, tiny, dmin = second_difference_rows(radii)
    norm = 0.
    for i in range(1, len(Rs) - 1):
        d1, d2 = (max(float(d), tiny) for d in (Rs[i] - Rs[i - 1], Rs[i + 1] - Rs[i]))
        norm += float(np.sum(second_differences(max(d1, dmin), max(d2, dmin)) ** 2))
    return L, norm, o


def relative_rows(radii, traa, alpha):
    """(L, srel, o): the prior rows, the scale sqrt(alpha trace(A^T A) / norm) and the order of the radii."""
    L, norm, o = relative_norm(radii)
    return L, math.sqrt(alpha * traa / max(norm, 1e-300)), o


def solve_profile(A, b, radii, smooth=DENSPROF_SMOOTH, corr=1., floor=None):
    """The reference's solve_profile (two NNLS solves with the smoothness prior; smooth 0: plain NNLS)."""
    from scipy.optimize import nnls
    n = A.shape[1]
    q, r = np.linalg.qr(A)
    c = q.T @ b
    if not smooth or n < 3:
        return nnls(r, c)[0]
    L, srel, o = relative_rows(radii, float(np.sum(A * A)), 0.1)
    zeros = np.zeros(n - 2)
    x0 = nnls(np.vstack([r, srel * L]), np.r_[c, zeros])[0]
    xm = float(np.mean(x0[:-1]))
    if not xm > 0:
        return x0
    chi2 = float(np.sum((b - A @ x0) ** 2)) / max(A.shape[0] - n, 1)
    corr = max(float(corr), 1.) * max(chi2, 1.)
    d = float(np.median(np.diff(np.sort(np.asarray(radii, float)[:-1]))))
    xc = np.maximum(x0[o[1:-1]], 0.1 * xm)
    w = math.sqrt(corr) * d * d / (float(smooth) * xc)
    w = np.maximum(w, math.sqrt(DENSPROF_FLOOR if floor is None else float(floor)) * srel)
    Rs = np.asarray(radii, float)[o]
    near = np.minimum(np.diff(Rs)[:-1], np.diff(Rs)[1:]) < 0.25 * d
    w[near] = srel
    return nnls(np.vstack([r, w[:, None] * L]), np.r_[c, zeros])[0]
