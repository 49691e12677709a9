"""GB300 (sm_103a) engine for the 2-D ring-array wave simulation and its FWI gradient.

A drop-in for the reference's ``fdtd2d.torch_backend`` engine and the device
part of ``TorchLeastSquaresFWI`` (scjoshi/SoundWaveSimulation): the same class
and function names, backed by hand-written CUDA kernels in ``libfdtd_gb300.so``
(C ABI: ``include/fdtd_gb300.h``).
"""

from .geometry import ArcArray, RingArray, axis_centers, n_steps_for_crossing, stable_dt
from .medium import (c_from_m, clip_m, interior_mask, m_from_c, mute_transmitter, regularizers,
                     tikhonov, total_variation, waveform_misfit)
from .waveforms import linear_chirp, ricker

__all__ = [
    "ArcArray", "RingArray", "axis_centers", "n_steps_for_crossing", "stable_dt",
    "c_from_m", "clip_m", "interior_mask", "m_from_c", "mute_transmitter", "regularizers", "tikhonov",
    "total_variation", "waveform_misfit", "linear_chirp", "ricker",
]
