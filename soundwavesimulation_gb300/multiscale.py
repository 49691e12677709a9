"""Multiscale FWI stage transfer (invert_ring.py:1037-1068).

``multiscale_stages`` is the reference's coarse-to-fine ladder (grid size,
spacing, chirp band, chirp duration); ``resize_slowness`` moves the slowness
squared between two grid levels in physical coordinates with the library's
bicubic kernel (``fdtd_resize_slowness``, the border-padded, corner-aligned
bicubic the reference gets from ``torch.nn.functional.grid_sample``).
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .engine import ptr, require_cuda, stream_handle

# Single-stage defaults of the ring FWI driver (invert_ring.py:59-70).
NX = 401
DX = 0.50e-3
F_START_HZ = 1.00e5
F_END_HZ = 2.50e5
CHIRP_DURATION = 20.0e-6


def multiscale_stages(enabled, coarse_band_hz=(25.0e3, 75.0e3)):
    """(grid size, spacing, start Hz, end Hz, chirp duration) per stage (invert_ring.py:1037-1045)."""
    if enabled:
        return (
            (101, 2.0e-3, *coarse_band_hz, 80.0e-6),
            (201, 1.0e-3, 50.0e3, 125.0e3, 40.0e-6),
            (401, 0.5e-3, F_START_HZ, F_END_HZ, CHIRP_DURATION),
        )
    return ((NX, DX, F_START_HZ, F_END_HZ, CHIRP_DURATION),)


def resize_slowness(m, source_axes, target_axes, background_m, device=None):
    """Bicubically transfer slowness squared to the next grid level (invert_ring.py:1048-1068).

    ``source_axes`` / ``target_axes`` are the (x_m, y_m) cell-centre axes of the
    two grids (they need not cover the same field of view); target points outside
    the source grid get ``background_m``. A NumPy ``m`` returns a NumPy array; a
    CUDA tensor returns a float64 tensor on its device.
    """
    as_numpy = not isinstance(m, torch.Tensor)
    dev = require_cuda(device if device is not None else (m.device if not as_numpy else "cuda"))
    src = torch.as_tensor(m, dtype=torch.float64).to(dev).contiguous()
    if src.ndim != 2:
        raise ValueError("m must be a 2D array (ny, nx)")
    sx, sy = (torch.as_tensor(np.asarray(a, dtype=float)).to(dev) for a in source_axes)
    tx, ty = (torch.as_tensor(np.asarray(a, dtype=float)).to(dev) for a in target_axes)
    if (sy.numel(), sx.numel()) != tuple(src.shape):
        raise ValueError("source axes do not match the shape of m")
    out = torch.empty((ty.numel(), tx.numel()), dtype=torch.float64, device=dev)
    _lib.check(_lib.load().fdtd_resize_slowness(ptr(src), src.shape[0], src.shape[1], ptr(sx), ptr(sy), ptr(out),
                                                out.shape[0], out.shape[1], ptr(tx), ptr(ty),
                                                float(background_m), stream_handle(dev)), "resize_slowness")
    return out.cpu().numpy() if as_numpy else out
