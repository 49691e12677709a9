"""Device medium and fused-engine plans on top of the C ABI.

``DeviceMedium`` holds one grid's float32 update coefficients and Mur
coefficients in the padded device layout the kernels use. ``FusedPlan`` binds
one execution plan of the temporally blocked engine (fixed grid, receivers,
per-shot sources and step count) to a workspace owned by the PyTorch caching
allocator, and runs the batched forward and the checkpointed adjoint.

Layout: every field is float32 ``(shots, ny, pitch)`` with ``pitch`` the grid
width rounded up to a multiple of 4; the padding columns hold zeros.
"""

from __future__ import annotations

import ctypes
import warnings

import numpy as np
import torch

from . import _lib


def padded_width(nx: int) -> int:
    return (int(nx) + 3) // 4 * 4


def require_cuda(device) -> torch.device:
    device = torch.device(device)
    if device.type != "cuda":
        raise ValueError("The GB300 engine runs on CUDA devices only; got device "
                         f"{device!s}. There is no CPU fallback.")
    if not torch.cuda.is_available():
        raise RuntimeError("CUDA is not available; the GB300 engine needs a GPU.")
    if device.index is None:
        device = torch.device("cuda", torch.cuda.current_device())
    return device


def stream_handle(device=None) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def ptr(t) -> int:
    return 0 if t is None else t.data_ptr()


class DeviceMedium:
    """Float32 update coefficients (c dt / dy)^2 and Mur edge coefficients of one grid.

    With ``pml_cells`` > 0 the grid is padded by a PML layer of that many cells on
    every side (the medium extended with its edge values), which replaces the Mur
    edges; ``pml_reflection`` sets the damping profile's target reflection. The
    physical grid is then rows / columns ``[pml_cells, pml_cells + n)`` of the
    padded one: ``ny``, ``nx`` are the padded sizes, ``phys_shape`` the physical
    ones, and receivers / sources given on the physical grid are shifted by
    ``pml_cells`` (ProblemTables does that).
    """

    def __init__(self, c, dx, dy, dt, device, pml_cells=0, pml_reflection=1e-5):
        self.device = require_cuda(device)
        c64 = torch.as_tensor(c, dtype=torch.float64).to(self.device).contiguous()
        if c64.ndim != 2:
            raise ValueError("Sound speed c must be a 2D array (ny, nx).")
        self.pml_cells = int(pml_cells)
        self.pml_reflection = float(pml_reflection)
        if self.pml_cells < 0:
            raise ValueError("pml_cells must not be negative.")
        self.phys_shape = tuple(int(s) for s in c64.shape)
        P = self.pml_cells
        self.ny, self.nx = self.phys_shape[0] + 2 * P, self.phys_shape[1] + 2 * P
        self.pitch = padded_width(self.nx)
        self.dx, self.dy, self.dt = float(dx), float(dy), float(dt)
        self.c64 = torch.empty((self.ny, self.nx), dtype=torch.float64, device=self.device)
        self.coef = torch.zeros((self.ny, self.pitch), dtype=torch.float32, device=self.device)
        self.mur = torch.zeros(2 * (2 * self.ny + 2 * self.nx + 8), dtype=torch.float32, device=self.device)
        self.pml = (torch.zeros(4 * (self.nx + self.ny), dtype=torch.float32, device=self.device)
                    if P else None)
        self._load(c64)
        self.prepare()

    def _load(self, c64):
        P = self.pml_cells
        if P:
            c64 = torch.nn.functional.pad(c64[None, None], (P, P, P, P), mode="replicate")[0, 0]
        self.c64.copy_(c64)

    def set_c(self, c):
        c64 = torch.as_tensor(c, dtype=torch.float64).to(self.device)
        if tuple(c64.shape) != self.phys_shape:
            raise ValueError(f"Sound speed shape {tuple(c64.shape)} does not match {self.phys_shape}.")
        self._load(c64)
        self.prepare()

    def set_dt(self, dt):
        self.dt = float(dt)
        self.prepare()

    def prepare(self):
        lib = _lib.load()
        if self.pml_cells:
            _lib.check(lib.fdtd_prepare_medium_pml(ptr(self.c64), self.ny, self.nx, self.pitch, self.dt, self.dx,
                                                   self.dy, self.pml_cells, self.pml_reflection, ptr(self.coef),
                                                   ptr(self.mur), ptr(self.pml), stream_handle(self.device)),
                       "prepare_medium_pml")
            return
        _lib.check(lib.fdtd_prepare_medium(ptr(self.c64), self.ny, self.nx, self.pitch, self.dt,
                                           self.dx, self.dy, ptr(self.coef), ptr(self.mur),
                                           stream_handle(self.device)), "prepare_medium")

    def grid(self) -> _lib.Grid:
        return _lib.Grid(self.ny, self.nx, self.pitch, self.dx, self.dy, self.dt,
                         ptr(self.coef), ptr(self.mur), ptr(self.pml), self.pml_cells)

    def physical(self, field):
        """The physical-grid view of a padded (..., ny, pitch) field."""
        P = self.pml_cells
        return field[..., P:P + self.phys_shape[0], P:P + self.phys_shape[1]]

    def new_field(self, n_shots=None):
        shape = (self.ny, self.pitch) if n_shots is None else (int(n_shots), self.ny, self.pitch)
        return torch.zeros(shape, dtype=torch.float32, device=self.device)


class ProblemTables:
    """Host description of one acquisition for the C ABI (keeps the host arrays alive).

    receivers: (row0, col0, weights (R, 4)); sources: rows, cols, weights and
    waveform indices, each (S, K); waveforms: device float32 (n_waves, len).
    """

    def __init__(self, medium: DeviceMedium, receivers, sources, waveforms: torch.Tensor, n_steps: int):
        self.medium = medium
        row0, col0, w = receivers
        P = medium.pml_cells  # physical-grid indices into the padded grid
        self._rx_row0 = np.ascontiguousarray(np.asarray(row0) + P, dtype=np.int32)
        self._rx_col0 = np.ascontiguousarray(np.asarray(col0) + P, dtype=np.int32)
        self._rx_w = np.ascontiguousarray(w, dtype=np.float32).reshape(-1, 4)
        rows, cols, sw, wave = (np.ascontiguousarray(a) for a in sources)
        self._s_row = (rows.astype(np.int64) + P).astype(np.int32).reshape(rows.shape[0], -1)
        self._s_col = (cols.astype(np.int64) + P).astype(np.int32).reshape(self._s_row.shape)
        self._s_w = sw.astype(np.float32).reshape(self._s_row.shape)
        self._s_wave = wave.astype(np.int32).reshape(self._s_row.shape)
        if waveforms.dtype != torch.float32 or waveforms.device != medium.device or waveforms.ndim != 2:
            raise ValueError("waveforms must be a float32 (n_waves, length) tensor on the engine device")
        self.waveforms = waveforms.contiguous()
        self.n_shots = int(self._s_row.shape[0])
        self.n_rx = int(self._rx_row0.shape[0])
        self.n_steps = int(n_steps)

    def problem(self) -> _lib.Problem:
        m = self.medium
        rx = _lib.Receivers(self.n_rx, self._rx_row0.ctypes.data, self._rx_col0.ctypes.data,
                            self._rx_w.ctypes.data)
        src = _lib.Sources(int(self._s_row.shape[1]), self._s_row.ctypes.data, self._s_col.ctypes.data,
                           self._s_w.ctypes.data, self._s_wave.ctypes.data, ptr(self.waveforms),
                           int(self.waveforms.shape[0]), int(self.waveforms.shape[1]))
        return _lib.Problem(m.grid(), self.n_shots, self.n_steps, rx, src)


def forward_plain(tables: ProblemTables, traces=None):
    """The plain per-shot form: one step + one gather launch per step, shot after shot."""
    lib = _lib.load()
    prob = tables.problem()
    nbytes = int(lib.fdtd_forward_plain_workspace(ctypes.byref(prob)))
    ws = torch.empty(nbytes, dtype=torch.uint8, device=tables.medium.device)
    if traces is None:
        traces = torch.empty((tables.n_shots, tables.n_rx, tables.n_steps), dtype=torch.float32,
                             device=tables.medium.device)
    _lib.check(lib.fdtd_forward_plain(ctypes.byref(prob), ptr(traces), ptr(ws), nbytes,
                                      stream_handle(tables.medium.device)), "forward_plain")
    return traces


def gradient_plain(tables: ProblemTables, observed, mute, grad_c2=None, misfit=None):
    """The plain per-shot gradient (full float32 history, one launch per kernel per step)."""
    lib = _lib.load()
    prob = tables.problem()
    dev = tables.medium.device
    nbytes = int(lib.fdtd_gradient_plain_workspace(ctypes.byref(prob)))
    ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    if grad_c2 is None:
        grad_c2 = torch.zeros((tables.medium.ny, tables.medium.pitch), dtype=torch.float64, device=dev)
    if misfit is None:
        misfit = torch.zeros(1, dtype=torch.float64, device=dev)
    mute_t = None if mute is None else torch.as_tensor(mute, dtype=torch.int32, device=dev)
    observed = observed.to(device=dev, dtype=torch.float32).contiguous()
    _lib.check(lib.fdtd_gradient_plain(ctypes.byref(prob), ptr(observed), ptr(mute_t), ptr(misfit),
                                       ptr(grad_c2), ptr(ws), nbytes, stream_handle(dev)), "gradient_plain")
    return misfit, grad_c2


BF16_CHECKPOINT_WARNING = (
    "bfloat16 checkpoints (8-bit significand) give FWI gradients about 2e-3 rel-L2 from float64 at "
    "1024^2 x 6000 steps, outside the 1e-3 gradient budget; float16 checkpoints (11-bit significand, "
    "power-of-two scale per slot and shot) stay near 3e-4")


# Share of the free device memory a gradient plan spends on kept stencil streams
# (each kept checkpoint segment saves its recompute in every adjoint pass).
KEPT_MEMORY_FRACTION = 0.6


class FusedPlan(ProblemTables):
    """One bound plan of the temporally blocked engine over a ProblemTables acquisition.

    ``tuning`` takes the ``fdtd_tuning`` fields by name. A gradient plan whose tuning
    does not name ``kept_segments`` keeps the stencil stream of as many of its last
    checkpoint segments as KEPT_MEMORY_FRACTION of the free device memory holds
    (at least one); ``self.tuning`` reports the count in effect.
    """

    def __init__(self, medium: DeviceMedium, receivers, sources, waveforms: torch.Tensor,
                 n_steps: int, tuning: dict | None = None, for_gradient: bool = False):
        super().__init__(medium, receivers, sources, waveforms, n_steps)
        if for_gradient and int((tuning or {}).get("ckpt_store", 0)) == _lib.STORE_BF16:
            warnings.warn(BF16_CHECKPOINT_WARNING, UserWarning, stacklevel=2)
        self.lib = _lib.load()
        self.for_gradient = bool(for_gradient)
        self._problem_struct = self.problem()
        t = _lib.Tuning(**{k: int(v) for k, v in (tuning or {}).items()})
        self._plan = self._create(t)
        if self.for_gradient and "kept_segments" not in (tuning or {}):
            kept = self._kept_for_memory(medium)
            if kept > 1:
                self.close()
                t.kept_segments = kept
                self._plan = self._create(t)
        nbytes = ctypes.c_size_t()
        _lib.check(self.lib.fdtd_plan_workspace_bytes(self._plan, ctypes.byref(nbytes)))
        self.workspace_bytes = int(nbytes.value)
        self.workspace = torch.empty(self.workspace_bytes, dtype=torch.uint8, device=medium.device)
        _lib.check(self.lib.fdtd_plan_bind(self._plan, ptr(self.workspace), self.workspace_bytes,
                                           stream_handle(medium.device)), "bind")
        resolved = _lib.Tuning()
        _lib.check(self.lib.fdtd_plan_tuning(self._plan, ctypes.byref(resolved)))
        self.tuning = resolved.as_dict()

    def _create(self, t):
        handle = ctypes.c_void_p()
        _lib.check(self.lib.fdtd_plan_create(ctypes.byref(self._problem_struct), ctypes.byref(t),
                                             int(self.for_gradient), ctypes.byref(handle)), "plan")
        return handle

    def _kept_for_memory(self, medium) -> int:
        """Checkpoint segments whose stencil stream the forward keeps: as many as
        KEPT_MEMORY_FRACTION of the free device memory holds beside the plan's own
        workspace, at least 1 (grids with PML keep none)."""
        resolved = _lib.Tuning()
        _lib.check(self.lib.fdtd_plan_tuning(self._plan, ctypes.byref(resolved)))
        if resolved.kept_segments < 1:
            return 0
        nbytes = ctypes.c_size_t()
        _lib.check(self.lib.fdtd_plan_workspace_bytes(self._plan, ctypes.byref(nbytes)))
        every = int(resolved.ckpt_every)
        n_seg = -(-self.n_steps // every)
        seg_bytes = every * self.n_shots * medium.ny * medium.pitch * 4
        free, _ = torch.cuda.mem_get_info(medium.device)
        extra = int(max(0.0, KEPT_MEMORY_FRACTION * free - int(nbytes.value)) // seg_bytes)
        return min(n_seg, 1 + extra)

    def set_waveforms(self, waveforms: torch.Tensor):
        if tuple(waveforms.shape) != tuple(self.waveforms.shape):
            raise ValueError("waveform shape changed; build a new plan")
        self.waveforms.copy_(waveforms)

    def refresh_medium(self):
        """Re-point the plan at the medium's buffers (after DeviceMedium.prepare)."""
        _lib.check(self.lib.fdtd_plan_set_medium(self._plan, ptr(self.medium.coef), ptr(self.medium.mur),
                                                 ptr(self.waveforms)))

    def forward(self, traces=None, u_prev_out=None, u_out=None, save_checkpoints=False):
        """Run all shots for n_steps; returns traces (S, R, nt) float32."""
        if traces is None:
            traces = torch.empty((self.n_shots, self.n_rx, self.n_steps), dtype=torch.float32,
                                 device=self.medium.device)
        self.refresh_medium()
        _lib.check(self.lib.fdtd_forward(self._plan, ptr(traces), ptr(u_prev_out), ptr(u_out),
                                         int(bool(save_checkpoints)),
                                         stream_handle(self.medium.device)), "forward")
        return traces

    def adjoint(self, residual: torch.Tensor, grad_c2: torch.Tensor):
        """Add dt^2 sum_n adj^n lap(u^{n-1}) into grad_c2 (float64 (ny, pitch))."""
        if residual.dtype != torch.float32 or not residual.is_contiguous():
            raise ValueError("residual must be contiguous float32 (S, R, nt)")
        if grad_c2.dtype != torch.float64 or tuple(grad_c2.shape) != (self.medium.ny, self.medium.pitch):
            raise ValueError("grad_c2 must be float64 (ny, pitch)")
        _lib.check(self.lib.fdtd_adjoint(self._plan, ptr(residual), ptr(grad_c2),
                                         stream_handle(self.medium.device)), "adjoint")

    def close(self):
        if getattr(self, "_plan", None):
            self.lib.fdtd_plan_destroy(self._plan)
            self._plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PlanGroup:
    """Several FusedPlans (grids of different sizes and step counts, one launch
    shape) advanced together: each round of temporally blocked launches runs as
    one launch per kernel mode over the items of every plan."""

    def __init__(self, plans):
        self.plans = list(plans)
        if not self.plans:
            raise ValueError("a group needs at least one plan")
        dev = self.plans[0].medium.device
        if any(p.medium.device != dev for p in self.plans):
            raise ValueError("all plans of a group must live on one device")
        self.device = dev
        self.lib = _lib.load()
        self._handles = (ctypes.c_void_p * len(self.plans))(*[p._plan.value for p in self.plans])
        nbytes = int(self.lib.fdtd_group_workspace_bytes(self._handles, len(self.plans)))
        if nbytes == 0:
            raise ValueError("invalid plan group")
        self.workspace = torch.empty(nbytes, dtype=torch.uint8, device=dev)

    def _ptrs(self, tensors):
        return (ctypes.c_void_p * len(tensors))(*[ptr(t) for t in tensors])

    def forward(self, traces=None, save_checkpoints=False):
        """All plans' forward passes; returns the list of traces (S, R, nt) per plan."""
        if traces is None:
            traces = [torch.empty((p.n_shots, p.n_rx, p.n_steps), dtype=torch.float32, device=self.device)
                      for p in self.plans]
        for p in self.plans:
            p.refresh_medium()
        _lib.check(self.lib.fdtd_group_forward(self._handles, len(self.plans), self._ptrs(traces),
                                               int(bool(save_checkpoints)), ptr(self.workspace),
                                               self.workspace.numel(), stream_handle(self.device)), "group forward")
        return traces

    def adjoint(self, residuals, grads):
        """All plans' checkpointed adjoints; grads[i] float64 (ny, pitch) of plan i accumulate."""
        _lib.check(self.lib.fdtd_group_adjoint(self._handles, len(self.plans), self._ptrs(residuals),
                                               self._ptrs(grads), ptr(self.workspace), self.workspace.numel(),
                                               stream_handle(self.device)), "group adjoint")


def residual_misfit(traces, observed, mute, residual=None, misfit=None):
    """residual = traces - observed (muted channel per shot) and 0.5 * sum(residual^2) in float64."""
    lib = _lib.load()
    S, R, nt = (int(v) for v in traces.shape)
    if observed.shape[1:] != traces.shape[1:] or observed.stride(2) != 1 or observed.stride(1) != nt:
        raise ValueError("observed must be (shots, receivers, steps) with contiguous rows")
    if residual is None:
        residual = torch.empty_like(traces)
    if misfit is None:
        misfit = torch.zeros(1, dtype=torch.float64, device=traces.device)
    mute_t = None if mute is None else torch.as_tensor(mute, dtype=torch.int32, device=traces.device)
    _lib.check(lib.fdtd_residual_misfit(S, R, nt, ptr(traces), ptr(observed), observed.stride(0),
                                        ptr(mute_t), ptr(residual), ptr(misfit),
                                        stream_handle(traces.device)), "residual")
    return residual, misfit


def chain_rule(grad_c2, m, mask=None):
    """g_m = -g_{c^2} / m^2 on the mask (float64 device tensors of one shape)."""
    lib = _lib.load()
    out = torch.empty_like(m)
    mk = None if mask is None else mask.to(torch.uint8).contiguous()
    _lib.check(lib.fdtd_chain_rule(m.numel(), ptr(grad_c2.contiguous()), ptr(m.contiguous()), ptr(mk),
                                   ptr(out), stream_handle(m.device)), "chain_rule")
    return out
