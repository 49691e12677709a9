"""Least-squares FWI on the GB300 engine: a drop-in for the reference's gradient driver.

``TorchLeastSquaresFWI`` keeps the constructor, ``project`` / ``apply_medium``
/ ``misfit`` / ``misfit_and_grad`` / ``regularization`` of the reference
(invert_ring.py:483-701). Its device work runs in the fused engine:

1. the batched forward (``fdtd_forward``) records the traces and keeps
   checkpoints of (u_old, u) every ~sqrt(2 nt) steps instead of the full
   wavefield history;
2. ``fdtd_residual_misfit`` forms the residual with the transmitter channel
   zeroed and the misfit in float64;
3. ``fdtd_adjoint`` replays each checkpoint segment forward (storing the
   Laplacian of every step) and runs the reverse-time adjoint over it, imaging
   ``dt^2 * sum adj^n * lap(u^{n-1})`` into a float64 gradient;
4. ``fdtd_chain_rule`` maps g_{c^2} to g_m = -g_{c^2} / m^2 on the device.

The imaging uses every time step, so the gradient equals the reference's with
``store_every = 1``. ``store_every`` is accepted for signature compatibility
and only enters the memory estimate; ``wave_dtype`` float16 / bfloat16 selects
16-bit checkpoint storage: u and the leapfrog step u - u_old, each with one
power-of-two scale per shot.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .engine import FusedPlan, chain_rule, residual_misfit
from .medium import c_from_m, m_from_c, regularizers
from .optim import project_device, regularization_device
from .torch_backend import TorchFDTD2DBatch, auto_batch_size, engine_tuning

__all__ = ["TorchLeastSquaresFWI", "forward_store", "forward_store_batch", "stored_steps",
           "gradient_bytes_per_shot", "observed_bytes_per_shot", "WaveformMisfit", "simulate_traces"]


def forward_store(solver, sampler, array, pulse, tx, n_steps):
    """One shot with its whole wavefield history (invert_ring.py:395-419), one-step kernels."""
    row, col = array.inject_rows_cols(tx)
    solver.reset()
    solver.set_source(row, col)
    dev = solver.model.device
    traces = torch.empty((sampler.n_elements, n_steps), device=dev, dtype=torch.float32)
    wave = torch.empty((n_steps, *solver.model.shape), device=dev, dtype=torch.float32)
    pulse = torch.as_tensor(pulse, device=dev, dtype=torch.float32).reshape(-1)
    for step in range(n_steps):
        field = solver.inject_and_step(pulse[step]) if step < pulse.numel() else solver.step()
        traces[:, step] = sampler.record(field)
        wave[step].copy_(field)
    return traces, wave


def stored_steps(n_steps, store_every):
    """Snapshots kept when storing every k-th step (invert_ring.py:458-460)."""
    return -(-int(n_steps) // int(store_every))


def forward_store_batch(solver, sampler, array, source_values, sources, n_steps, batched,
                        store_every=1, wave_dtype=None):
    """Batched forward keeping every ``store_every``-th wavefield (invert_ring.py:422-455).

    Kept for callers of the reference API; the gradient path itself never stores
    the history.
    """
    rows_cols = [array.inject_rows_cols(int(tx)) for tx in sources]
    batched.set_sources([r for r, _ in rows_cols], [c for _, c in rows_cols])
    batched.reset()
    dev = solver.model.device
    S = len(sources)
    samples = torch.empty((n_steps, S, sampler.n_elements), device=dev, dtype=torch.float32)
    wave = torch.empty((stored_steps(n_steps, store_every), S, *solver.model.shape), device=dev,
                       dtype=torch.float32 if wave_dtype is None else wave_dtype)
    values = torch.as_tensor(source_values, device=dev, dtype=torch.float32)
    for step in range(n_steps):
        fields, s = batched.step_record(values[step], sampler)
        samples[step].copy_(s)
        if step % store_every == 0:
            wave[step // store_every].copy_(fields)
    return samples.permute(1, 2, 0).contiguous(), wave


def gradient_bytes_per_shot(n_steps, grid_shape, n_receivers, store_every=1, wave_dtype=None,
                            dtype=None, ckpt_every=None):
    """Device bytes one gradient shot needs in the fused engine.

    Eight live fields (forward and adjoint ping-pong), the checkpoints and the
    recompute segment buffer, plus traces, residual and observed data.
    """
    ny, nx = grid_shape
    field = ny * ((nx + 3) // 4 * 4) * 4
    c = ckpt_every or int(np.ceil(np.sqrt(2.0 * n_steps)))
    ck_bytes = 2 if wave_dtype in (torch.float16, torch.bfloat16) else 4
    n_ck = max(-(-int(n_steps) // c) - 1, 0)
    return (8 * field + n_ck * 2 * field // 4 * ck_bytes + c * field
            + 3 * n_steps * n_receivers * 4)


def observed_bytes_per_shot(n_steps, grid_shape, n_receivers, dtype=None):
    """Device bytes one forward-only shot needs (four fields plus traces)."""
    ny, nx = grid_shape
    return 4 * ny * ((nx + 3) // 4 * 4) * 4 + 2 * n_steps * n_receivers * 4


def _ckpt_store(wave_dtype):
    if wave_dtype is None or wave_dtype == torch.float32:
        return _lib.STORE_F32
    if wave_dtype == torch.float16:
        return _lib.STORE_F16
    if wave_dtype == torch.bfloat16:
        return _lib.STORE_BF16
    raise ValueError("wave_dtype must be float32, float16 or bfloat16")


class TorchLeastSquaresFWI:
    """Least-squares FWI with the fused forward / checkpointed adjoint (invert_ring.py:483-701)."""

    def __init__(self, solver, sampler, array, pulse, n_steps, n_shots, observed, mask, alpha=0.0,
                 tv=0.0, tv_eps=1.0e-9, c_min=1400.0, c_max=2000.0, c_background=1500.0, shot_seed=0,
                 parallel_shots=16, batched_solvers=None, store_every=1, wave_dtype=None,
                 ckpt_every=None, tuning=None):
        self.solver = solver
        self.model = solver.model
        self.sampler = sampler
        self.array = array
        self.pulse = pulse
        self.n_steps = int(n_steps)
        dev = self.model.device
        self.source_values = torch.zeros(self.n_steps, device=dev, dtype=torch.float32)
        p = torch.as_tensor(pulse, device=dev, dtype=torch.float32).reshape(-1)
        self.source_values[:min(p.numel(), self.n_steps)].copy_(p[:self.n_steps])
        self.n_shots = int(n_shots)
        if self.n_shots < 1 or self.n_shots > array.n_elements:
            raise ValueError("n_shots must be between 1 and the number of elements.")
        if not isinstance(observed, torch.Tensor):
            observed = torch.stack([torch.as_tensor(o) for o in observed])
        if observed.shape[0] != array.n_elements:
            raise ValueError("Observed data must contain one gather per transmitter.")
        self.observed = observed.to(device=dev, dtype=torch.float32).contiguous()
        self.store_every = int(store_every)
        if self.store_every < 1:
            raise ValueError("store_every must be positive.")
        self.wave_dtype = torch.float32 if wave_dtype is None else wave_dtype
        self._tuning = dict(engine_tuning() if tuning is None else tuning)
        self._tuning["ckpt_store"] = _ckpt_store(wave_dtype)
        if ckpt_every:
            self._tuning["ckpt_every"] = int(ckpt_every)
        if parallel_shots == "auto":
            parallel_shots = auto_batch_size(dev, self.n_shots, gradient_bytes_per_shot(
                self.n_steps, self.model.shape, sampler.n_elements, self.store_every, wave_dtype))
        self.parallel_shots = int(parallel_shots)
        if self.parallel_shots < 1:
            raise ValueError("parallel_shots must be positive.")
        self.parallel_shots = min(self.parallel_shots, self.n_shots)
        self._batched_solvers = {} if batched_solvers is None else batched_solvers
        self._shot_rng = np.random.default_rng(shot_seed)
        self.active_sources = None
        self.source_history = []
        self.mask = np.asarray(mask, dtype=bool)
        self._mask_dev = torch.as_tensor(self.mask, device=dev)
        self._mask_u8 = self._mask_dev.to(torch.uint8).contiguous()
        self.alpha = float(alpha)
        self.tv = float(tv)
        self.tv_eps = float(tv_eps)
        self.c_min = float(c_min)
        self.c_max = float(c_max)
        self.c_background = float(c_background)
        self._plans = {}

    # --- medium -----------------------------------------------------------------
    def project(self, m):
        m = np.asarray(m, dtype=float)
        out = np.clip(m, 1.0 / self.c_max ** 2, 1.0 / self.c_min ** 2).copy()
        out[~self.mask] = m_from_c(self.c_background)
        return out

    def apply_medium(self, m):
        m = self.project(m)
        self.solver.set_c(c_from_m(m))
        return m

    # --- shots ------------------------------------------------------------------
    @staticmethod
    def _residual(predicted, observed, tx):
        residual = (predicted - observed).clone()
        residual[tx].zero_()
        return residual

    def _mute(self, shot_batch):
        """Receiver channel zeroed per shot: the transmitter's own (invert_ring.py:603-609)."""
        return np.asarray(shot_batch)

    def _sample_sources(self):
        if self.n_shots == self.array.n_elements:
            selected = np.arange(self.array.n_elements, dtype=int)
        else:
            selected = np.sort(self._shot_rng.choice(self.array.n_elements, size=self.n_shots, replace=False))
        self.active_sources = selected
        self.source_history.append(selected.copy())
        return selected

    def _source_batches(self, sources):
        for start in range(0, len(sources), self.parallel_shots):
            yield sources[start:start + self.parallel_shots]

    def _batched_solver(self, batch_size):
        batched = self._batched_solvers.get(batch_size)
        if batched is None:
            batched = TorchFDTD2DBatch(self.solver, batch_size)
            self._batched_solvers[batch_size] = batched
        return batched

    def _plan(self, shot_batch, for_gradient):
        rows_cols = [self.array.inject_rows_cols(int(tx)) for tx in shot_batch]
        rows = np.array([[r] for r, _ in rows_cols])
        cols = np.array([[c] for _, c in rows_cols])
        key = (rows.tobytes(), cols.tobytes(), bool(for_gradient))
        plan = self._plans.get(key)
        if plan is None:
            if len(self._plans) >= 2:
                self._plans.clear()
            plan = FusedPlan(self.solver.medium, self.sampler.taps(),
                             (rows, cols, np.ones(rows.shape), np.zeros(rows.shape, dtype=np.int64)),
                             self.source_values[None], self.n_steps, tuning=self._tuning,
                             for_gradient=for_gradient)
            self._plans[key] = plan
        return plan

    # --- objective --------------------------------------------------------------
    def regularization(self, m):
        """Tikhonov + total-variation value and gradient of m (float64, host arrays),
        evaluated by the device kernel (invert_ring.py:662-666)."""
        if self.alpha <= 0.0 and self.tv <= 0.0:
            return 0.0, np.zeros(np.shape(m))
        return regularizers(m, self.mask, self.alpha, self.tv, self.tv_eps, device=self.model.device)

    def misfit(self, m):
        """Forward-only J(m) (invert_ring.py:611-632)."""
        m = self.apply_medium(m)
        sources = self.active_sources if self.active_sources is not None else self._sample_sources()
        self.solver._sync_medium()
        total = torch.zeros(1, dtype=torch.float64, device=self.model.device)
        for shot_batch in self._source_batches(sources):
            plan = self._plan(shot_batch, for_gradient=False)
            predicted = plan.forward()
            observed = self.observed[torch.as_tensor(shot_batch, device=self.model.device)]
            residual_misfit(predicted, observed, self._mute(shot_batch), residual=predicted, misfit=total)
        regularization, _ = self.regularization(m)
        return float(total.item()) + regularization

    def misfit_and_grad(self, m):
        """J(m) and g_m = dJ/dm (float64, zero outside the mask) (invert_ring.py:634-660)."""
        value, gradient = self.misfit_and_grad_device(torch.as_tensor(np.asarray(m, dtype=float)))
        return value, gradient.cpu().numpy()

    def misfit_and_grad_device(self, m):
        """``misfit_and_grad`` with m, the gradient and the regularisers on the device.

        ``m``: float64 (ny, nx) tensor (moved to the device if needed; not modified).
        Returns the float objective and g_m as a float64 device tensor, zero outside
        the mask. Only the objective is read back to the host.
        """
        dev = self.model.device
        medium = self.solver.medium
        m = torch.as_tensor(m, dtype=torch.float64).to(dev).contiguous().clone()
        project_device(m, self._mask_u8, self.c_min, self.c_max, self.c_background)
        self.solver.set_c(1.0 / torch.sqrt(m))
        sources = self._sample_sources()
        self.solver._sync_medium()
        total = torch.zeros(1, dtype=torch.float64, device=dev)
        g_c2 = torch.zeros((medium.ny, medium.pitch), dtype=torch.float64, device=dev)
        for shot_batch in self._source_batches(sources):
            plan = self._plan(shot_batch, for_gradient=True)
            predicted = plan.forward(save_checkpoints=True)
            observed = self.observed[torch.as_tensor(shot_batch, device=dev)]
            residual, _ = residual_misfit(predicted, observed, self._mute(shot_batch), residual=predicted,
                                          misfit=total)
            plan.adjoint(residual, g_c2)
        g_m = chain_rule(medium.physical(g_c2).contiguous(), m, self._mask_dev)
        regularization_device(m, self._mask_u8, self.alpha, self.tv, self.tv_eps, g_m, total)
        return float(total.item()), g_m

    def gradient_c2(self, m, sources):
        """Unmasked g_{c^2} and the data misfit for fixed transmitters (no projection, no sampling)."""
        self.solver.set_c(c_from_m(np.asarray(m, dtype=float)))
        self.solver._sync_medium()
        dev = self.model.device
        medium = self.solver.medium
        total = torch.zeros(1, dtype=torch.float64, device=dev)
        g_c2 = torch.zeros((medium.ny, medium.pitch), dtype=torch.float64, device=dev)
        sources = np.asarray(sources)
        for shot_batch in self._source_batches(sources):
            plan = self._plan(shot_batch, for_gradient=True)
            predicted = plan.forward(save_checkpoints=True)
            observed = self.observed[torch.as_tensor(shot_batch, device=dev)]
            residual, _ = residual_misfit(predicted, observed, self._mute(shot_batch), residual=predicted,
                                          misfit=total)
            plan.adjoint(residual, g_c2)
        return float(total.item()), medium.physical(g_c2).cpu().numpy()


class ArcLeastSquaresFWI(TorchLeastSquaresFWI):
    """FWI with separate transmit (``array``) and receive (``sampler``) arcs
    (invert_arc.py:294-307): no transmitter is also a receiver, so the full
    residual is kept (no muting)."""

    @staticmethod
    def _residual(predicted, observed, tx):
        return predicted - observed

    def _mute(self, shot_batch):
        return None


class WaveformMisfit(torch.autograd.Function):
    """traces = F(m) for slowness squared m, with the adjoint engine as its backward.

    forward(m, plan, solver) runs the fused forward with checkpoints and
    returns the traces (shots, receivers, steps); backward(grad_traces) injects
    grad_traces as the adjoint source, runs the checkpointed adjoint and
    returns dL/dm = -g_{c^2} / m^2. Any differentiable loss on the traces can
    sit on top (the least-squares misfit is 0.5 * sum((traces - d)^2)).
    """

    @staticmethod
    def forward(ctx, m, plan, solver):
        m64 = m.detach().to(torch.float64)
        solver.set_c((1.0 / torch.sqrt(m64)).cpu().numpy())
        solver._sync_medium()
        traces = plan.forward(save_checkpoints=True).clone()
        ctx.plan = plan
        ctx.m_dtype, ctx.m_device = m.dtype, m.device
        ctx.save_for_backward(m64)
        return traces

    @staticmethod
    def backward(ctx, grad_traces):
        (m64,) = ctx.saved_tensors
        plan = ctx.plan
        medium = plan.medium
        g_c2 = torch.zeros((medium.ny, medium.pitch), dtype=torch.float64, device=medium.device)
        plan.adjoint(grad_traces.detach().to(torch.float32).contiguous(), g_c2)
        g_m = chain_rule(medium.physical(g_c2).contiguous(), m64.to(medium.device), None)
        return g_m.to(device=ctx.m_device, dtype=ctx.m_dtype), None, None


def simulate_traces(m, solver, sampler, rows, cols, source_values, n_steps, tuning=None):
    """Differentiable batched forward: traces(m) through ``WaveformMisfit``."""
    rows = np.asarray(rows).reshape(len(rows), -1)
    cols = np.asarray(cols).reshape(rows.shape)
    values = torch.as_tensor(source_values, device=solver.model.device, dtype=torch.float32).reshape(1, -1)
    plan = FusedPlan(solver.medium, sampler.taps(), (rows, cols, np.ones(rows.shape),
                     np.zeros(rows.shape, dtype=np.int64)), values, n_steps,
                     tuning=tuning or engine_tuning(), for_gradient=True)
    return WaveformMisfit.apply(m, plan, solver)
