"""Source waveforms: the reference's Hann-windowed linear chirp and a Ricker wavelet.

``linear_chirp`` follows the torch backend's definition
(fdtd2d/torch_backend.py:80-102; the sweep uses (n_pulse - 1) * dt). The Ricker
wavelet is not in the reference; it enters the engine the same way any
waveform does, as per-step source values (fdtd2d/torch_backend.py:744-759).
"""

from __future__ import annotations

import math

import numpy as np


def hann_window(n):
    """Symmetric Hann window of n samples (fdtd2d/sources.py:6-9)."""
    if n <= 1:
        return np.ones(max(n, 0))
    return 0.5 - 0.5 * np.cos(2.0 * np.pi * np.arange(n) / (n - 1))


def linear_chirp(dt, duration_s, f_start_hz, f_end_hz, *, device=None, dtype=None):
    """Hann-windowed linear FM pulse sampled at k * dt, k < round(duration / dt).

    Returns a torch tensor when ``device`` or ``dtype`` is given (the torch
    backend's signature), otherwise a float64 NumPy array.
    """
    if duration_s <= 0.0:
        raise ValueError("Chirp duration must be positive.")
    if f_start_hz <= 0.0 or f_end_hz <= 0.0:
        raise ValueError("Chirp frequencies must be positive.")
    n = max(int(round(duration_s / dt)), 2)
    t = np.arange(n) * dt
    rate = (f_end_hz - f_start_hz) / ((n - 1) * dt)
    pulse = hann_window(n) * np.sin(2.0 * math.pi * (f_start_hz * t + 0.5 * rate * t * t))
    if device is None and dtype is None:
        return pulse
    import torch
    return torch.as_tensor(pulse, device=device, dtype=dtype or torch.float32)


def ricker(f0_hz, dt, n_steps, delay_s=None):
    """Ricker wavelet (1 - 2 a) exp(-a), a = (pi f0 (t - t0))^2, at t = k * dt.

    The default delay t0 = 1.5 / f0 starts the wavelet at ~2e-10 of its peak.
    """
    t0 = 1.5 / f0_hz if delay_s is None else float(delay_s)
    a = (math.pi * f0_hz * (np.arange(n_steps) * dt - t0)) ** 2
    return (1.0 - 2.0 * a) * np.exp(-a)
