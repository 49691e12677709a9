"""Slowness-squared variable, the interior mask and the regularisers.

The inversion works on m = 1 / c^2 and frees only the pixels strictly inside
``radius - margin`` of the ring centre; the functions keep the names and
argument meaning of the reference's fdtd2d/inversion/medium.py and
fdtd2d/inversion/misfit.py, so a caller can swap the import.

``tikhonov`` and ``total_variation`` evaluate on the GPU through the engine
library's ``fdtd_regularization`` kernel (float64, NumPy's operation order per
element); they take and return NumPy arrays like the reference's host versions.
There is no CPU path: without a CUDA device they raise.
"""

from __future__ import annotations

import numpy as np
import torch


def m_from_c(c):
    """Slowness squared of a sound-speed map."""
    return np.reciprocal(np.square(np.asarray(c, dtype=float)))


def c_from_m(m):
    """Sound speed of a slowness-squared map."""
    return np.reciprocal(np.sqrt(np.asarray(m, dtype=float)))


def clip_m(m, c_min, c_max):
    """m limited to the slowness-squared interval of speeds [c_min, c_max]."""
    lo, hi = m_from_c(float(c_max)), m_from_c(float(c_min))
    return np.minimum(np.maximum(m, lo), hi)


def interior_mask(x_m, y_m, radius_m, margin_m, center=(0.0, 0.0)):
    """Boolean (ny, nx) map of the pixels closer than ``radius - margin`` to ``center``."""
    inner = float(radius_m) - float(margin_m)
    if inner <= 0.0:
        raise ValueError("Interior radius must be positive; reduce the margin.")
    ry = np.square(np.asarray(y_m, dtype=float) - float(center[1]))
    rx = np.square(np.asarray(x_m, dtype=float) - float(center[0]))
    return np.add.outer(ry, rx) < inner * inner


def mute_transmitter(traces, tx):
    """Float64 copy of a gather (receivers first) with channel ``tx`` set to zero."""
    out = np.array(traces, dtype=float)
    out[tx] = 0.0
    return out


def waveform_misfit(predicted, observed, tx):
    """Half the squared residual norm of one gather, channel ``tx`` left out."""
    r = mute_transmitter(np.subtract(predicted, observed, dtype=float), tx)
    return 0.5 * float(np.vdot(r, r))


def regularizers(m, mask, alpha, tv, tv_eps, device="cuda"):
    """Tikhonov (weight ``alpha``) plus total variation (weight ``tv``) of m: the
    summed value and gradient, zero outside the mask, in one call on ``device``."""
    from .engine import require_cuda
    from .optim import regularization_device
    dev = require_cuda(device)
    m_d = torch.as_tensor(np.ascontiguousarray(m, dtype=float), device=dev)
    mask_d = torch.as_tensor(np.ascontiguousarray(mask, dtype=bool), device=dev).to(torch.uint8)
    grad = torch.zeros_like(m_d)
    value = torch.zeros(1, dtype=torch.float64, device=dev)
    regularization_device(m_d, mask_d, alpha, tv, tv_eps, grad, value)
    return float(value.item()), grad.cpu().numpy()


def tikhonov(m, mask, alpha):
    """0.5 * alpha * (sum of squared forward differences of m whose two pixels are
    inside the mask) and its gradient, zero outside the mask. Computed on the GPU."""
    if alpha <= 0.0:
        return 0.0, np.zeros(np.shape(m))
    return regularizers(m, mask, float(alpha), 0.0, 1.0)


def total_variation(m, mask, alpha, eps):
    """alpha * sum(sqrt(|grad m|^2 + eps^2) - eps) over in-mask forward differences,
    and its gradient, zero outside the mask. Computed on the GPU."""
    if alpha <= 0.0:
        return 0.0, np.zeros(np.shape(m))
    return regularizers(m, mask, 0.0, float(alpha), float(eps))
