"""Variable density: sound-speed and density maps in; traces, misfit and the
gradients with respect to slowness squared and density out.

No reference counterpart in 2-D: the reference propagates with constant density
(its density maps are written but unused) and only plans the conservative form
rho c^2 div((1/rho) grad u) (fdtd2d/wave.py:61-63), which its 1-D solver uses with
1/rho on the faces as 2 / (rho_a + rho_b) (1DWaveSimulation.py:116-143). Here
that operator runs on the one-step engine (one launch per step and kernel,
shot after shot): ``fdtd_forward_plain_density`` / ``fdtd_gradient_plain_density``
and the device chain rule ``fdtd_density_chain_rule``. The edges are the
reference's Mur edges, the adjoint is the reference's l-form with the forward Mur
(invert_ring.py:683-701), and at constant density the operator is the
reference's stencil.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .engine import ProblemTables, padded_width, ptr, require_cuda, stream_handle


class DensityMedium:
    """Device arrays of one grid with sound speed c and density rho (both (ny, nx)):
    kappa = rho c^2 dt^2, the face coefficients 1/rho and the Mur table."""

    def __init__(self, c, rho, dx, dy, dt, device):
        self.device = require_cuda(device)
        self.c64 = torch.as_tensor(c, dtype=torch.float64).to(self.device).contiguous()
        self.rho64 = torch.as_tensor(rho, dtype=torch.float64).to(self.device).contiguous()
        if self.c64.ndim != 2 or self.c64.shape != self.rho64.shape:
            raise ValueError("c and rho must be 2D arrays (ny, nx) of one shape.")
        if not bool(torch.all(self.rho64 > 0)):
            raise ValueError("Density must be positive.")
        self.ny, self.nx = (int(v) for v in self.c64.shape)
        self.phys_shape = (self.ny, self.nx)
        self.pml_cells = 0
        self.pitch = padded_width(self.nx)
        self.dx, self.dy, self.dt = float(dx), float(dy), float(dt)
        self.kappa = torch.zeros((self.ny, self.pitch), dtype=torch.float32, device=self.device)
        self.bx = torch.zeros((self.ny, self.pitch + 4), dtype=torch.float32, device=self.device)
        self.by = torch.zeros((self.ny + 1, self.pitch), dtype=torch.float32, device=self.device)
        self.mur = torch.zeros(2 * (2 * self.ny + 2 * self.nx + 8), dtype=torch.float32, device=self.device)
        self.prepare()

    def set_model(self, c=None, rho=None):
        if c is not None:
            self.c64.copy_(torch.as_tensor(c, dtype=torch.float64))
        if rho is not None:
            self.rho64.copy_(torch.as_tensor(rho, dtype=torch.float64))
        self.prepare()

    def prepare(self):
        _lib.check(_lib.load().fdtd_prepare_density(ptr(self.c64), ptr(self.rho64), self.ny, self.nx, self.pitch,
                                                    self.dt, self.dx, self.dy, ptr(self.kappa), ptr(self.bx),
                                                    ptr(self.by), ptr(self.mur), stream_handle(self.device)),
                   "prepare_density")

    def grid(self) -> _lib.Grid:
        return _lib.Grid(self.ny, self.nx, self.pitch, self.dx, self.dy, self.dt, ptr(self.kappa), ptr(self.mur), 0, 0)

    def density(self) -> _lib.Density:
        return _lib.Density(ptr(self.kappa), ptr(self.bx), ptr(self.by))

    def physical(self, field):
        return field[..., :self.ny, :self.nx]


def _tables(medium, receivers, sources, waveforms, n_steps):
    rows, cols, w = (np.asarray(a) for a in sources[:3])
    wave = sources[3] if len(sources) > 3 else np.zeros(np.shape(rows), dtype=np.int64)
    waves = torch.as_tensor(waveforms, dtype=torch.float32, device=medium.device).reshape(-1, np.shape(waveforms)[-1])
    return ProblemTables(medium, receivers, (rows, cols, w, wave), waves.contiguous(), n_steps)


def forward_density(medium: DensityMedium, receivers, sources, waveforms, n_steps):
    """Traces (shots, receivers, n_steps) float32 of every shot; ``sources`` as for
    the fused engine: (rows, cols, weights[, waveform index]), each (S, K)."""
    lib = _lib.load()
    t = _tables(medium, receivers, sources, waveforms, n_steps)
    prob = t.problem()
    nbytes = int(lib.fdtd_forward_plain_workspace(ctypes.byref(prob)))
    ws = torch.empty(nbytes, dtype=torch.uint8, device=medium.device)
    traces = torch.empty((t.n_shots, t.n_rx, t.n_steps), dtype=torch.float32, device=medium.device)
    dens = medium.density()
    _lib.check(lib.fdtd_forward_plain_density(ctypes.byref(prob), ctypes.byref(dens), ptr(traces), ptr(ws), nbytes,
                                              stream_handle(medium.device)), "forward_density")
    return traces


def gradient_density(medium: DensityMedium, receivers, sources, waveforms, n_steps, observed, mute, mask=None):
    """Misfit 0.5 sum(r^2) (float64) and the gradients with respect to slowness
    squared m = 1 / c^2 and density rho, float64 (ny, nx) device tensors, zero
    where ``mask`` is False; ``mute[s]`` is the channel left out of shot s's
    residual (None: none)."""
    lib = _lib.load()
    dev = medium.device
    t = _tables(medium, receivers, sources, waveforms, n_steps)
    prob = t.problem()
    nbytes = int(lib.fdtd_gradient_plain_workspace(ctypes.byref(prob)))
    ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    gk = torch.zeros((medium.ny, medium.pitch), dtype=torch.float64, device=dev)
    gbx = torch.zeros((medium.ny, medium.pitch + 4), dtype=torch.float64, device=dev)
    gby = torch.zeros((medium.ny + 1, medium.pitch), dtype=torch.float64, device=dev)
    misfit = torch.zeros(1, dtype=torch.float64, device=dev)
    mute_t = None if mute is None else torch.as_tensor(mute, dtype=torch.int32, device=dev)
    observed = torch.as_tensor(observed).to(device=dev, dtype=torch.float32).contiguous()
    dens = medium.density()
    stream = stream_handle(dev)
    _lib.check(lib.fdtd_gradient_plain_density(ctypes.byref(prob), ctypes.byref(dens), ptr(observed), ptr(mute_t),
                                               ptr(misfit), ptr(gk), ptr(gbx), ptr(gby), ptr(ws), nbytes, stream),
               "gradient_density")
    m = (1.0 / medium.c64 ** 2).contiguous()
    g_m = torch.empty_like(m)
    g_rho = torch.empty_like(m)
    mk = None if mask is None else torch.as_tensor(mask, device=dev).to(torch.uint8).contiguous()
    _lib.check(lib.fdtd_density_chain_rule(medium.ny, medium.nx, medium.pitch, ptr(m), ptr(medium.rho64), ptr(gk),
                                           ptr(gbx), ptr(gby), ptr(mk), ptr(g_m), ptr(g_rho), stream),
               "density_chain_rule")
    return float(misfit.item()), g_m, g_rho
