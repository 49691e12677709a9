"""Drop-in replacement for the reference's ``fdtd2d.torch_backend`` on GB300.

Same class names, constructor signatures, methods, return shapes and
``ValueError`` checks as fdtd2d/torch_backend.py, with the device work done by
the sm_103a kernels of ``libfdtd_gb300.so``:

* the per-step methods (``inject_and_step``, ``step_record``,
  ``adjoint_step_image`` ...) run the one-step kernels (``fdtd_step``,
  ``fdtd_gather``, ``fdtd_scatter``, ``fdtd_image``);
* ``simulate_shot`` / ``simulate_shots_batch`` run the whole time loop in the
  fused temporally blocked engine (``fdtd_forward``).

Fields propagate in float32 on a CUDA device; there is no CPU path. Field
tensors handed out (``solver.u``, ``batched.u_old`` ...) are ``(.., ny, nx)``
views of the engine's padded ``(.., ny, pitch)`` buffers.
"""

from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _lib
from .engine import DeviceMedium, FusedPlan, padded_width, ptr, require_cuda, stream_handle
from .waveforms import linear_chirp  # noqa: F401  (re-exported like the reference)

__all__ = [
    "resolve_device", "configure_runtime", "device_summary", "linear_chirp",
    "TorchScalarWave2D", "TorchFDTD2D", "TorchRingSampler", "TorchFDTD2DBatch",
    "simulate_shot", "simulate_shots_batch", "auto_batch_size", "set_engine_tuning",
    "engine_tuning",
]

_TUNING: dict = {}


def set_engine_tuning(**tuning):
    """Default launch shape of the fused engine (keys of ``fdtd_tuning``)."""
    _TUNING.clear()
    _TUNING.update({k: int(v) for k, v in tuning.items()})


def engine_tuning() -> dict:
    return dict(_TUNING)


def resolve_device(requested: str = "auto") -> torch.device:
    """auto/cuda/cuda:N -> a CUDA device (fdtd2d/torch_backend.py:17-46, CUDA only)."""
    requested = requested.lower()
    if requested == "auto":
        requested = "cuda"
    try:
        device = torch.device(requested)
    except (RuntimeError, ValueError) as exc:
        raise ValueError(f"Unknown device {requested!r}; use auto, cuda or cuda:N.") from exc
    if device.type != "cuda":
        raise ValueError("The GB300 engine supports CUDA devices only.")
    if not torch.cuda.is_available():
        raise ValueError("CUDA was requested, but PyTorch cannot access a CUDA GPU.")
    index = torch.cuda.current_device() if device.index is None else device.index
    if index < 0 or index >= torch.cuda.device_count():
        raise ValueError(f"CUDA device {index} is unavailable; found {torch.cuda.device_count()}.")
    return torch.device("cuda", index)


def configure_runtime(device: torch.device, cpu_threads: int = 0, allow_tf32: bool = False) -> None:
    """Host threads and current device (fdtd2d/torch_backend.py:49-63)."""
    if cpu_threads < 0:
        raise ValueError("cpu_threads must be zero (automatic) or positive.")
    if cpu_threads:
        torch.set_num_threads(cpu_threads)
    if torch.device(device).type == "cuda":
        torch.cuda.set_device(device)


def device_summary(device: torch.device) -> str:
    props = torch.cuda.get_device_properties(device)
    return (f"CUDA {torch.device(device).index or 0}: {props.name}; {props.multi_processor_count} SMs; "
            f"{props.total_memory / 1024 ** 3:.1f} GiB")


def _check_dtype(dtype):
    if dtype not in (None, torch.float32):
        raise ValueError("The GB300 engine propagates fields in float32 (dtype=torch.float32).")


class TorchScalarWave2D:
    """Sound-speed model on one CUDA device (fdtd2d/torch_backend.py:105-174)."""

    def __init__(self, c, dx: float, dy: float | None = None, *, device, dtype=torch.float32):
        _check_dtype(dtype)
        self.device = require_cuda(device)
        self.dtype = torch.float32
        c64 = torch.tensor(np.asarray(c.detach().cpu() if isinstance(c, torch.Tensor) else c,
                                      dtype=np.float64))
        if c64.ndim != 2:
            raise ValueError("Sound speed c must be a 2D array (ny, nx).")
        if not bool(torch.isfinite(c64).all()) or not bool((c64 > 0).all()):
            raise ValueError("Sound speed must contain finite positive values.")
        self._dx = float(dx)
        self._dy = float(dx if dy is None else dy)
        if self._dx <= 0.0 or self._dy <= 0.0:
            raise ValueError("Grid spacing must be positive.")
        self._c64 = c64.to(self.device)
        self._c = self._c64.to(torch.float32)
        self._c2 = self._c.square()
        self._c_max = float(c64.max())
        self.version = 0
        inv_dx2, inv_dy2 = 1.0 / self._dx ** 2, 1.0 / self._dy ** 2
        self.laplacian_kernel = torch.tensor(
            [[0.0, inv_dy2, 0.0], [inv_dx2, -2.0 * (inv_dx2 + inv_dy2), inv_dx2], [0.0, inv_dy2, 0.0]],
            device=self.device, dtype=torch.float32).reshape(1, 1, 3, 3)

    @property
    def shape(self):
        return tuple(self._c.shape)

    @property
    def dx(self):
        return self._dx

    @property
    def dy(self):
        return self._dy

    @property
    def c_max(self):
        return self._c_max

    @property
    def c(self):
        return self._c

    @property
    def c2(self):
        return self._c2

    def set_c(self, c):
        """Update the sound speed in place (fdtd2d/torch_backend.py:158-168).

        A tensor already on this CUDA device is taken without a host round trip.
        """
        if isinstance(c, torch.Tensor) and c.device == self.device:
            c64 = c.detach().to(torch.float64)
            if tuple(c64.shape) != self.shape:
                raise ValueError(f"Sound speed shape {tuple(c64.shape)} does not match {self.shape}.")
            if not bool(torch.isfinite(c64).all()) or not bool((c64 > 0).all()):
                raise ValueError("Sound speed must contain finite positive values.")
            self._c64.copy_(c64)
            self._c.copy_(c64)
            self._c2.copy_(self._c.square())
            self._c_max = float(c64.max())
            self.version += 1
            return
        src = c.detach().cpu().numpy() if isinstance(c, torch.Tensor) else c
        arr = np.ascontiguousarray(src, dtype=np.float64)
        if tuple(arr.shape) != self.shape:
            raise ValueError(f"Sound speed shape {tuple(arr.shape)} does not match {self.shape}.")
        if not bool(np.isfinite(arr).all()) or not bool((arr > 0).all()):
            raise ValueError("Sound speed must contain finite positive values.")
        # one host-to-device copy; the float32 and squared copies are made on the device
        self._c64.copy_(torch.from_numpy(arr))
        self._c.copy_(self._c64)
        self._c2.copy_(self._c.square())
        self._c_max = float(arr.max())
        self.version += 1

    def laplacian(self, field):
        """Zero-padded 5-point Laplacian of one field (a convenience; not an engine path)."""
        return torch.nn.functional.conv2d(field.to(torch.float32)[None, None],
                                          self.laplacian_kernel, padding=1)[0, 0]


class _Rotation:
    """Three padded field buffers rotated u_old <- u <- u_next (and, on a PML grid,
    two sets of face fields psi_x, psi_y swapped every step)."""

    def __init__(self, medium: DeviceMedium, n_shots=None):
        self.medium = medium
        shape = (3,) + ((medium.ny, medium.pitch) if n_shots is None else (n_shots, medium.ny, medium.pitch))
        self.buf = torch.zeros(shape, dtype=torch.float32, device=medium.device)
        self.io, self.ic, self.inx = 0, 1, 2
        self.psi = (torch.zeros((2, 2) + shape[1:], dtype=torch.float32, device=medium.device)
                    if medium.pml_cells else None)
        self.ps = 0

    def rotate(self):
        self.io, self.ic, self.inx = self.ic, self.inx, self.io
        self.ps ^= 1

    def view(self, i):
        return self.medium.physical(self.buf[i])

    def zero(self):
        self.buf.zero_()
        if self.psi is not None:
            self.psi.zero_()

    def step(self, lib, grid, n_shots, n_src, rows, cols, w, wave, value, dense, adjoint, stream):
        """One leapfrog step of the rotation's fields through the C ABI."""
        if self.psi is None:
            return lib.fdtd_step(ctypes.byref(grid), n_shots, ptr(self.buf[self.io]), ptr(self.buf[self.ic]),
                                 ptr(self.buf[self.inx]), n_src, ptr(rows), ptr(cols), ptr(w), ptr(wave),
                                 ptr(value), 1, 0, ptr(dense), int(adjoint), stream)
        if adjoint == 1:
            raise ValueError("a PML grid carries the adjoint as w = coef l (adjoint=2)")
        a, b = self.psi[self.ps], self.psi[self.ps ^ 1]
        return lib.fdtd_step_pml(ctypes.byref(grid), n_shots, ptr(self.buf[self.io]), ptr(self.buf[self.ic]),
                                 ptr(self.buf[self.inx]), ptr(a[0]), ptr(a[1]), ptr(b[0]), ptr(b[1]), n_src,
                                 ptr(rows), ptr(cols), ptr(w), ptr(wave), ptr(value), 1, 0, ptr(dense),
                                 int(adjoint), stream)


class TorchFDTD2D:
    """Single-shot leapfrog solver with Mur edges (fdtd2d/torch_backend.py:236-344)."""

    def __init__(self, model: TorchScalarWave2D, dt: float, compile_step=False, pml_cells=0, pml_reflection=1e-5):
        """``pml_cells`` > 0 replaces the Mur edges by a PML layer of that many cells
        padded outside the grid (an extension; the reference has Mur edges only).
        Fields, sources and receivers stay on the physical grid."""
        self.model = model
        self.dt = float(dt)
        self.dt2 = self.dt * self.dt
        if self.cfl >= 1.0:
            raise ValueError(f"Unstable time step: CFL = {self.cfl:.3f} >= 1.")
        self.medium = DeviceMedium(model._c64, model.dx, model.dy, self.dt, model.device, pml_cells=pml_cells,
                                   pml_reflection=pml_reflection)
        self._version = model.version
        self._rot = _Rotation(self.medium)
        self._dense = self.medium.new_field()
        self._value = torch.zeros(1, dtype=torch.float32, device=model.device)
        self._src = torch.zeros(2, dtype=torch.int32, device=model.device)
        self._src_w = torch.ones(1, dtype=torch.float32, device=model.device)
        self._src_wave = torch.zeros(1, dtype=torch.int32, device=model.device)
        self.source_row = 0
        self.source_col = 0
        # graph capture is what the fused engine does; the per-step API runs eagerly
        self.compiled = bool(compile_step)

    @property
    def cfl(self):
        return float(self.model.c_max * self.dt * math.sqrt(1.0 / self.model.dx ** 2 + 1.0 / self.model.dy ** 2))

    @property
    def u_old(self):
        return self._rot.view(self._rot.io)

    @property
    def u(self):
        return self._rot.view(self._rot.ic)

    def _sync_medium(self):
        if self.model.version != self._version:
            self.medium.set_c(self.model._c64)
            self._version = self.model.version

    def set_source(self, row: int, col: int):
        self.source_row = int(row)
        self.source_col = int(col)
        P = self.medium.pml_cells
        self._src.copy_(torch.tensor([self.source_row + P, self.source_col + P], dtype=torch.int32))

    def set_c(self, c):
        self.model.set_c(c)
        self._sync_medium()
        if self.cfl >= 1.0:
            raise ValueError(f"Updated medium is unstable: CFL = {self.cfl:.3f} >= 1.")

    def reset(self):
        self._rot.zero()

    def _step(self, value, source_field, source_mode, adjoint=False):
        self._sync_medium()
        lib = _lib.load()
        grid = self.medium.grid()
        n_src = 0
        dense = None
        if source_mode == 1:
            if isinstance(value, torch.Tensor):
                self._value.copy_(value.reshape(1))
            else:
                self._value.fill_(float(value))
            n_src = 1
        elif source_mode == 2:
            self.medium.physical(self._dense).copy_(torch.as_tensor(source_field, device=self.model.device))
            dense = self._dense
        r = self._rot
        if adjoint and self.medium.pml_cells:
            raise ValueError("the per-step adjoint runs on Mur grids; a PML grid's adjoint runs in the fused "
                             "gradient (TorchLeastSquaresFWI, fwi.WaveformMisfit)")
        _lib.check(r.step(lib, grid, 1, n_src, self._src, self._src[1:], self._src_w, self._src_wave, self._value,
                          dense, int(bool(adjoint)), stream_handle(self.model.device)), "step")
        r.rotate()
        return self.u

    def inject_and_step(self, value):
        return self._step(value, None, 1, adjoint=False)

    def step(self, zero=None):
        return self._step(zero, None, 0, adjoint=False)

    def inject_field_and_step(self, source_field, adjoint=True):
        source_field = torch.as_tensor(source_field, device=self.model.device, dtype=torch.float32)
        if tuple(source_field.shape) != self.model.shape:
            raise ValueError("Dense source field must match the FDTD grid shape.")
        return self._step(None, source_field, 2, adjoint=adjoint)


class TorchRingSampler:
    """Bilinear receivers on the device (fdtd2d/torch_backend.py:347-440)."""

    def __init__(self, ring_array, *, device, dtype=torch.float32):
        _check_dtype(dtype)
        self.device = require_cuda(device)
        self.n_elements = int(ring_array.n_elements)
        self.grid_shape = (ring_array._y_axis.size, ring_array._x_axis.size)
        row0, col0, w = (np.asarray(ring_array._row0), np.asarray(ring_array._col0),
                         np.stack([ring_array._w00, ring_array._w10, ring_array._w01, ring_array._w11], 1))
        self.row0 = row0.astype(np.int32)
        self.col0 = col0.astype(np.int32)
        self.weights = w.astype(np.float32)
        self._rc = torch.as_tensor(np.stack([self.row0, self.col0], 1), device=self.device).contiguous()
        self._w = torch.as_tensor(self.weights, device=self.device).contiguous()
        nodes, tw = _lib.tap_table(self.grid_shape[0], self.grid_shape[1], self.row0, self.col0, self.weights)
        self.n_tap_nodes = int(nodes.shape[0])
        self._tap_nodes = torch.as_tensor(nodes, device=self.device).contiguous()
        self._tap_w = torch.as_tensor(tw, device=self.device).contiguous()
        for name in ("_row0", "_row1", "_col0", "_col1"):
            setattr(self, name, torch.as_tensor(np.asarray(getattr(ring_array, name)), device=self.device,
                                                dtype=torch.long))
        for name in ("_w00", "_w10", "_w01", "_w11"):
            setattr(self, name, torch.as_tensor(np.asarray(getattr(ring_array, name)), device=self.device,
                                                dtype=torch.float32))
        self.receivers = (self._row0, self._row1, self._col0, self._col1,
                          self._w00, self._w10, self._w01, self._w11)

    def taps(self):
        """(row0, col0, weights (R, 4)) host arrays for engine plans."""
        return self.row0, self.col0, self.weights

    def _grid(self, pitch):
        return _lib.Grid(self.grid_shape[0], self.grid_shape[1], int(pitch), 1.0, 1.0, 1.0, 0, 0)

    def _gather(self, fields, n_shots):
        if fields.dtype != torch.float32 or fields.stride(-1) != 1 or fields.device != self.device:
            fields = fields.to(device=self.device, dtype=torch.float32).contiguous()
        pitch = fields.stride(-2)
        if fields.ndim == 3 and fields.stride(0) != self.grid_shape[0] * pitch:
            fields = fields.contiguous()
            pitch = fields.stride(-2)
        out = torch.empty((n_shots, self.n_elements), dtype=torch.float32, device=self.device)
        grid = self._grid(pitch)
        _lib.check(_lib.load().fdtd_gather(ctypes.byref(grid), n_shots, ptr(fields), self.n_elements,
                                           ptr(self._rc), ptr(self._w), ptr(out), self.n_elements, 1,
                                           stream_handle(self.device)), "gather")
        return out

    def record(self, field):
        if tuple(field.shape) != self.grid_shape:
            raise ValueError("Field must have shape (ny, nx) matching the grid.")
        return self._gather(field, 1)[0]

    def record_batch(self, fields):
        if fields.ndim != 3 or tuple(fields.shape[1:]) != self.grid_shape:
            raise ValueError("Batched fields must have shape (shots, ny, nx) matching the grid.")
        return self._gather(fields, int(fields.shape[0]))

    def _scatter(self, residual, out, n_shots):
        residual = residual.to(device=self.device, dtype=torch.float32).contiguous()
        if out is None:
            out = torch.zeros((n_shots,) + self.grid_shape, dtype=torch.float32, device=self.device)
        else:
            out.zero_()
        target = out if (out.dtype == torch.float32 and out.is_contiguous()) else \
            torch.zeros(out.shape, dtype=torch.float32, device=self.device)
        grid = self._grid(self.grid_shape[1])
        _lib.check(_lib.load().fdtd_scatter(ctypes.byref(grid), n_shots, self.n_tap_nodes, ptr(self._tap_nodes),
                                            ptr(self._tap_w), ptr(residual), self.n_elements, 1, ptr(target),
                                            stream_handle(self.device)), "scatter")
        if target is not out:
            out.copy_(target)
        return out

    def record_adjoint_batch(self, residual, out=None):
        if residual.ndim != 2 or residual.shape[1] != self.n_elements:
            raise ValueError("Batched residuals must have shape (shots, receivers).")
        return self._scatter(residual, out, int(residual.shape[0]))

    def record_adjoint(self, residual, out=None):
        residual = torch.as_tensor(residual, device=self.device, dtype=torch.float32)
        if tuple(residual.shape) != (self.n_elements,):
            raise ValueError(f"Residual shape {tuple(residual.shape)} does not match ({self.n_elements},).")
        res = self._scatter(residual[None], None if out is None else out[None], 1)
        return res[0]


def _source_values(solver, pulse, n_steps, source_values=None):
    if source_values is None:
        values = torch.zeros(n_steps, device=solver.model.device, dtype=torch.float32)
        p = torch.as_tensor(pulse, device=solver.model.device, dtype=torch.float32).reshape(-1)
        m = min(int(p.numel()), n_steps)
        values[:m].copy_(p[:m])
        if int(p.numel()) > n_steps:
            raise RuntimeError("pulse is longer than n_steps")
        return values
    values = torch.as_tensor(source_values, device=solver.model.device, dtype=torch.float32)
    if tuple(values.shape) != (n_steps,):
        raise ValueError("source_values must contain one value per time step.")
    return values


def _plan_for(owner, solver, sampler, rows, cols, n_steps, waveforms, weights=None, waves=None,
              for_gradient=False, tuning=None):
    """Cached fused plan keyed on everything that shapes it."""
    rows = np.asarray(rows, dtype=np.int64).reshape(len(rows), -1)
    cols = np.asarray(cols, dtype=np.int64).reshape(rows.shape)
    if weights is None:
        weights = np.ones(rows.shape)
    if waves is None:
        waves = np.zeros(rows.shape, dtype=np.int64)
    tuning = dict(_TUNING if tuning is None else tuning)
    key = (id(solver.medium), id(sampler), rows.tobytes(), cols.tobytes(),
           np.asarray(weights, np.float32).tobytes(), np.asarray(waves, np.int32).tobytes(),
           int(n_steps), tuple(waveforms.shape), bool(for_gradient), tuple(sorted(tuning.items())))
    cache = owner.__dict__.setdefault("_fused_plans", {})
    plan = cache.get(key)
    if plan is None:
        cache.clear()  # one live plan per owner keeps workspace memory bounded
        plan = FusedPlan(solver.medium, sampler.taps(), (rows, cols, weights, waves), waveforms, n_steps,
                         tuning=tuning, for_gradient=for_gradient)
        cache[key] = plan
    else:
        plan.set_waveforms(waveforms)
    return plan


def simulate_shot(solver: TorchFDTD2D, sampler: TorchRingSampler, pulse, source_row: int, source_col: int,
                  n_steps: int, snapshot_stride: int = 0):
    """One shot; returns traces (R, n_steps) and snapshots (fdtd2d/torch_backend.py:443-474)."""
    solver.reset()
    solver.set_source(source_row, source_col)
    solver._sync_medium()
    pulse_t = torch.as_tensor(pulse, device=solver.model.device, dtype=torch.float32).reshape(-1)
    if snapshot_stride:
        traces = torch.empty((sampler.n_elements, n_steps), device=solver.model.device, dtype=torch.float32)
        snapshots = []
        for step in range(n_steps):
            field = solver.inject_and_step(pulse_t[step]) if step < pulse_t.numel() else solver.step()
            traces[:, step] = sampler.record(field)
            if step % snapshot_stride == 0:
                snapshots.append((field.detach().cpu().numpy().copy(), step))
        return traces, snapshots
    values = torch.zeros(n_steps, device=solver.model.device, dtype=torch.float32)
    m = min(int(pulse_t.numel()), n_steps)
    values[:m].copy_(pulse_t[:m])
    plan = _plan_for(solver, solver, sampler, [source_row], [source_col], n_steps, values[None])
    r = solver._rot
    traces = plan.forward(u_prev_out=r.buf[r.io], u_out=r.buf[r.ic])
    return traces[0], []


def simulate_sources(solver: TorchFDTD2D, sampler: TorchRingSampler, source_rows, source_cols, source_values,
                     n_steps: int, snapshot_steps=()):
    """Every transmit element fires at once with its own waveform; the receivers record.

    The multi-element firing of 2DArcFDTD.py:203-228 (``simulate``) through the
    fused engine: ``source_values`` is ``(K, n_steps)``, one waveform per element
    at ``(source_rows[k], source_cols[k])``; elements that round to one grid node
    add up, like the reference's ``index_put_(..., accumulate=True)``. Returns
    traces ``(R, n_steps)`` on the device and a dict of host snapshots for
    ``snapshot_steps`` (those runs take the per-step form, as the reference does).
    """
    rows = np.asarray(source_rows, dtype=np.int64).reshape(-1)
    cols = np.asarray(source_cols, dtype=np.int64).reshape(-1)
    if rows.shape != cols.shape:
        raise ValueError("source_rows and source_cols must have the same length.")
    dev = solver.model.device
    values = torch.as_tensor(source_values, device=dev, dtype=torch.float32)
    if values.ndim != 2 or tuple(values.shape) != (rows.size, int(n_steps)):
        raise ValueError("source_values must be (n_sources, n_steps).")
    solver.reset()
    solver._sync_medium()
    snapshot_steps = set(int(s) for s in snapshot_steps)
    if snapshot_steps:
        rows_t = torch.as_tensor(rows, device=dev)
        cols_t = torch.as_tensor(cols, device=dev)
        source_field = torch.zeros(solver.model.shape, device=dev, dtype=torch.float32)
        traces = torch.empty((sampler.n_elements, int(n_steps)), device=dev, dtype=torch.float32)
        snapshots = {}
        for step in range(int(n_steps)):
            source_field.zero_()
            source_field.index_put_((rows_t, cols_t), values[:, step].contiguous(), accumulate=True)
            field = solver.inject_field_and_step(source_field, adjoint=False)
            traces[:, step] = sampler.record(field)
            if step in snapshot_steps:
                snapshots[step] = field.detach().cpu().numpy().copy()
        return traces, snapshots
    plan = _plan_for(solver, solver, sampler, rows[None], cols[None], int(n_steps), values.contiguous(),
                     waves=np.arange(rows.size, dtype=np.int64)[None])
    r = solver._rot
    traces = plan.forward(u_prev_out=r.buf[r.io], u_out=r.buf[r.ic])
    return traces[0], {}


class TorchFDTD2DBatch:
    """Independent shots advanced together (fdtd2d/torch_backend.py:601-733)."""

    def __init__(self, solver: TorchFDTD2D, n_shots: int):
        if n_shots < 1:
            raise ValueError("n_shots must be positive.")
        self.model = solver.model
        self._solver = solver
        self.dt2 = solver.dt2
        self.n_shots = int(n_shots)
        self._rot = _Rotation(solver.medium, self.n_shots)
        self.source_rows = torch.zeros(self.n_shots, device=self.model.device, dtype=torch.long)
        self.source_cols = torch.zeros(self.n_shots, device=self.model.device, dtype=torch.long)
        self._rows_h = np.zeros(self.n_shots, dtype=np.int64)
        self._cols_h = np.zeros(self.n_shots, dtype=np.int64)
        self._src_row = torch.zeros(self.n_shots, device=self.model.device, dtype=torch.int32)
        self._src_col = torch.zeros(self.n_shots, device=self.model.device, dtype=torch.int32)
        self._src_w = torch.ones(self.n_shots, device=self.model.device, dtype=torch.float32)
        self._src_wave = torch.zeros(self.n_shots, device=self.model.device, dtype=torch.int32)
        self._value = torch.zeros(1, device=self.model.device, dtype=torch.float32)
        self._dense = None
        self._fwd = None
        self._g64 = None
        self.compiled = solver.compiled

    @property
    def u_old(self):
        return self._rot.view(self._rot.io)

    @property
    def u(self):
        return self._rot.view(self._rot.ic)

    def reset(self):
        self._rot.zero()

    def set_sources(self, rows, cols):
        rows_h = np.asarray(torch.as_tensor(rows).cpu(), dtype=np.int64).reshape(-1)
        cols_h = np.asarray(torch.as_tensor(cols).cpu(), dtype=np.int64).reshape(-1)
        if rows_h.shape != (self.n_shots,) or cols_h.shape != (self.n_shots,):
            raise ValueError("One source row and column is required per batched shot.")
        self._rows_h, self._cols_h = rows_h, cols_h
        self.source_rows.copy_(torch.as_tensor(rows_h))
        self.source_cols.copy_(torch.as_tensor(cols_h))
        P = self._solver.medium.pml_cells
        self._src_row.copy_(torch.as_tensor(rows_h + P, dtype=torch.int32))
        self._src_col.copy_(torch.as_tensor(cols_h + P, dtype=torch.int32))

    def _launch(self, value=None, dense=None, adjoint=False):
        self._solver._sync_medium()
        n_src = 0
        if value is not None:
            if isinstance(value, torch.Tensor):
                self._value.copy_(value.reshape(1))
            else:
                self._value.fill_(float(value))
            n_src = 1
        r = self._rot
        grid = self._solver.medium.grid()
        if adjoint and self._solver.medium.pml_cells:
            raise ValueError("the per-step adjoint runs on Mur grids; a PML grid's adjoint runs in the fused "
                             "gradient (TorchLeastSquaresFWI, fwi.WaveformMisfit)")
        _lib.check(r.step(_lib.load(), grid, self.n_shots, n_src, self._src_row, self._src_col, self._src_w,
                          self._src_wave, self._value, dense, int(bool(adjoint)), stream_handle(self.model.device)),
                   "step")
        r.rotate()
        return self.u

    def _dense_buffer(self):
        if self._dense is None:
            self._dense = self._solver.medium.new_field(self.n_shots)
        return self._dense

    def step(self, source_value):
        return self._launch(value=source_value)

    def step_record(self, source_value, sampler):
        """Advance every shot one step and return its receiver samples."""
        u = self._launch(value=source_value)
        return u, sampler.record_batch(u)

    def _scatter_residual(self, residual, sampler):
        dense = self._dense_buffer()
        residual = residual.to(device=self.model.device, dtype=torch.float32).contiguous()
        if tuple(residual.shape) != (self.n_shots, sampler.n_elements):
            raise ValueError("Batched residuals must have shape (shots, receivers).")
        grid = self._solver.medium.grid()
        _lib.check(_lib.load().fdtd_scatter(ctypes.byref(grid), self.n_shots, sampler.n_tap_nodes,
                                            ptr(sampler._tap_nodes), ptr(sampler._tap_w), ptr(residual),
                                            sampler.n_elements, 1, ptr(dense), stream_handle(self.model.device)),
                   "scatter")
        return dense

    def adjoint_step_residual(self, residual, sampler):
        """Adjoint step driven by (shots, receivers) residual samples."""
        return self._launch(dense=self._scatter_residual(residual, sampler), adjoint=True)

    def adjoint_step_image(self, residual, sampler, forward_field, gradient, scale):
        """Adjoint step plus ``gradient + scale * sum(adjoint * L[forward_field])`` (returned)."""
        u = self.adjoint_step_residual(residual, sampler)
        medium = self._solver.medium
        if self._fwd is None:
            self._fwd = medium.new_field(self.n_shots)
            self._g64 = torch.zeros((medium.ny, medium.pitch), dtype=torch.float64, device=medium.device)
        self._fwd[..., :medium.nx].copy_(forward_field)
        self._g64[:, :medium.nx].copy_(gradient)
        r = self._rot
        grid = medium.grid()
        _lib.check(_lib.load().fdtd_image(ctypes.byref(grid), self.n_shots, ptr(r.buf[r.ic]), ptr(self._fwd),
                                          float(scale), ptr(self._g64), stream_handle(self.model.device)),
                   "image")
        del u
        return self._g64[:, :medium.nx].to(gradient.dtype if isinstance(gradient, torch.Tensor) else torch.float64)

    def adjoint_step(self, source_fields):
        dense = self._dense_buffer()
        dense[..., :self._solver.medium.nx].copy_(source_fields)
        return self._launch(dense=dense, adjoint=True)


def simulate_shots_batch(solver: TorchFDTD2D, sampler: TorchRingSampler, pulse, source_rows, source_cols,
                         n_steps: int, batched: TorchFDTD2DBatch | None = None, source_values=None, out=None):
    """All shots of a batch through the fused engine (fdtd2d/torch_backend.py:736-770).

    Returns traces ``(shots, receivers, n_steps)`` and the final field batch.
    ``out`` (optional, not in the reference's signature) receives the traces: a
    contiguous float32 tensor of that shape on the solver's device, or in pinned
    host memory, which the kernels then write directly over the host link (no copy
    after the run; synchronise the device before reading it, as after a
    non-blocking copy).
    """
    if batched is None:
        batched = TorchFDTD2DBatch(solver, len(source_rows))
    elif batched.n_shots != len(source_rows):
        raise ValueError("Batched solver size does not match the source batch.")
    if out is not None:
        shape = (len(source_rows), sampler.n_elements, int(n_steps))
        on_device = out.device == solver.medium.device
        if out.dtype != torch.float32 or not out.is_contiguous() or tuple(out.shape) != shape:
            raise ValueError(f"out must be a contiguous float32 tensor of shape {shape}.")
        if not on_device and not (out.device.type == "cpu" and out.is_pinned()):
            raise ValueError("out must live on the solver's device or in pinned host memory.")
    batched.set_sources(source_rows, source_cols)
    values = _source_values(solver, pulse, n_steps, source_values)
    solver._sync_medium()
    plan = _plan_for(batched, solver, sampler, batched._rows_h, batched._cols_h, n_steps, values[None])
    r = batched._rot
    r.io, r.ic, r.inx = 0, 1, 2
    traces = plan.forward(traces=out, u_prev_out=r.buf[0], u_out=r.buf[1])
    return traces, batched.u


def auto_batch_size(device, n_shots, bytes_per_shot, fallback=16, memory_fraction=0.75):
    """Shots per batch for ``n_shots`` shots of ``bytes_per_shot`` device bytes each.

    The contract of fdtd2d/torch_backend.py:773-789: the budget is
    ``memory_fraction`` of what the device can still hand out (free memory plus
    the caching allocator's reserved but unused bytes); the shots are split into
    the fewest batches whose size fits the budget, and the batches are made as
    equal as possible. Off CUDA the budget is ``fallback`` shots.
    """
    total = int(n_shots)
    device = torch.device(device)
    if device.type == "cuda":
        free, _ = torch.cuda.mem_get_info(device)
        idle = torch.cuda.memory_reserved(device) - torch.cuda.memory_allocated(device)
        fits = int((free + idle) * memory_fraction) // max(int(bytes_per_shot), 1)
    else:
        fits = int(fallback)
    fits = min(total, max(fits, 1))
    batches = math.ceil(total / fits)
    return math.ceil(total / batches)