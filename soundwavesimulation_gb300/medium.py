"""Slowness-squared parameterisation, interior mask and host regularisers.

Same functions and conventions as the reference's fdtd2d/inversion/medium.py
and the regularisers of fdtd2d/inversion/misfit.py: the inversion variable is
m = 1 / c^2; only pixels inside ``radius - margin`` are free.
"""

from __future__ import annotations

import numpy as np


def m_from_c(c):
    c = np.asarray(c, dtype=float)
    return 1.0 / (c * c)


def c_from_m(m):
    return 1.0 / np.sqrt(np.asarray(m, dtype=float))


def clip_m(m, c_min, c_max):
    """Clip m so that c stays within [c_min, c_max]."""
    return np.clip(m, 1.0 / float(c_max) ** 2, 1.0 / float(c_min) ** 2)


def interior_mask(x_m, y_m, radius_m, margin_m, center=(0.0, 0.0)):
    """True where (x, y) lies strictly inside radius - margin."""
    r = float(radius_m) - float(margin_m)
    if r <= 0.0:
        raise ValueError("Interior radius must be positive; reduce the margin.")
    x, y = np.meshgrid(np.asarray(x_m, float) - center[0], np.asarray(y_m, float) - center[1],
                       indexing="xy")
    return x * x + y * y < r * r


def mute_transmitter(traces, tx):
    """Copy of the traces with the transmitter channel zeroed."""
    out = np.array(traces, dtype=float, copy=True)
    out[tx] = 0.0
    return out


def waveform_misfit(predicted, observed, tx):
    """0.5 * ||P u - d||^2 without the transmitter channel."""
    r = mute_transmitter(np.asarray(predicted) - np.asarray(observed), tx)
    return 0.5 * float(np.sum(r * r))


def tikhonov(m, mask, alpha):
    """0.5 * alpha * sum of squared forward differences inside the mask, and its gradient.

    A difference counts only when both of its pixels are in the mask, so the
    fixed exterior adds no penalty (fdtd2d/inversion/misfit.py:19-44).
    """
    g = np.zeros_like(m, dtype=float)
    if alpha <= 0.0:
        return 0.0, g
    value = 0.0
    for axis in (1, 0):
        d = np.diff(m, axis=axis)
        both = np.logical_and(np.take(mask, range(1, m.shape[axis]), axis=axis),
                              np.take(mask, range(0, m.shape[axis] - 1), axis=axis))
        value += 0.5 * alpha * float(np.sum(d[both] ** 2))
        flux = np.where(both, alpha * d, 0.0)
        if axis == 1:
            g[:, 1:] += flux
            g[:, :-1] -= flux
        else:
            g[1:, :] += flux
            g[:-1, :] -= flux
    g[~mask] = 0.0
    return value, g


def total_variation(m, mask, alpha, eps):
    """Smoothed isotropic TV alpha * sum(sqrt(|grad m|^2 + eps^2) - eps) and its gradient
    (fdtd2d/inversion/misfit.py:47-71)."""
    g = np.zeros_like(m, dtype=float)
    if alpha <= 0.0:
        return 0.0, g
    gx = np.zeros_like(m, dtype=float)
    gy = np.zeros_like(m, dtype=float)
    gx[:, :-1] = np.where(mask[:, 1:] & mask[:, :-1], np.diff(m, axis=1), 0.0)
    gy[:-1, :] = np.where(mask[1:, :] & mask[:-1, :], np.diff(m, axis=0), 0.0)
    norm = np.sqrt(gx * gx + gy * gy + eps * eps)
    value = alpha * float(np.sum(norm - eps))
    px = alpha * gx / norm
    py = alpha * gy / norm
    g -= px + py
    g[:, 1:] += px[:, :-1]
    g[1:, :] += py[:-1, :]
    g[~mask] = 0.0
    return value, g
