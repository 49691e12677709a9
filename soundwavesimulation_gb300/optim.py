"""Device-resident FWI iteration: regularisers, projection and projected Adam.

The reference runs every optimiser step on the host: ``misfit_and_grad`` copies
the float64 gradient off the device (invert_ring.py:655-659), the regularisers
are NumPy (fdtd2d/inversion/misfit.py:19-71) and Adam is NumPy
(invert_ring.py:817-861). Here the slowness squared ``m``, the moments and the
gradient stay on the GPU; each iteration reads back two scalars (misfit and
gradient norm). The kernels live in ``libfdtd_gb300.so`` (``fdtd_regularization``,
``fdtd_project``, ``fdtd_adam_step``) and keep NumPy's operation order, so the
iterates equal the host algorithm's to the last bit up to the order of the
misfit / norm reductions.
"""

from __future__ import annotations

import torch

from . import _lib
from .engine import ptr, require_cuda, stream_handle


def _mask_u8(mask, device):
    return torch.as_tensor(mask, device=device).to(torch.uint8).contiguous()


def regularization_device(m: torch.Tensor, mask_u8: torch.Tensor, alpha: float, tv: float, tv_eps: float,
                          grad: torch.Tensor, value: torch.Tensor) -> None:
    """grad += Tikhonov + TV gradients on the mask (0 outside); value += their values.

    ``m``, ``grad``: float64 (ny, nx) contiguous device tensors; ``value``: float64 (1,).
    """
    if m.dtype != torch.float64 or grad.dtype != torch.float64 or value.dtype != torch.float64:
        raise ValueError("m, grad and value must be float64")
    if m.shape != grad.shape or m.ndim != 2 or not (m.is_contiguous() and grad.is_contiguous()):
        raise ValueError("m and grad must be contiguous (ny, nx) tensors")
    ny, nx = (int(s) for s in m.shape)
    _lib.check(_lib.load().fdtd_regularization(ny, nx, ptr(m), ptr(mask_u8), float(alpha), float(tv),
                                               float(tv_eps), ptr(grad), ptr(value), stream_handle(m.device)),
               "regularization")


def project_device(m: torch.Tensor, mask_u8: torch.Tensor, c_min: float, c_max: float,
                   c_background: float) -> torch.Tensor:
    """In place: clip m to [1/c_max^2, 1/c_min^2] on the mask, 1/c_background^2 outside."""
    _lib.check(_lib.load().fdtd_project(m.numel(), ptr(m), ptr(mask_u8), 1.0 / c_max ** 2, 1.0 / c_min ** 2,
                                        1.0 / c_background ** 2, stream_handle(m.device)), "project")
    return m


class DeviceAdam:
    """Projected Adam state on the device (invert_ring.py:817-861)."""

    def __init__(self, shape, mask, device, learning_rate, beta1=0.9, beta2=0.999, epsilon=1e-30):
        self.device = require_cuda(device)
        self.mask = _mask_u8(mask, self.device)
        self.first = torch.zeros(shape, dtype=torch.float64, device=self.device)
        self.second = torch.zeros(shape, dtype=torch.float64, device=self.device)
        self.learning_rate = float(learning_rate)
        self.beta1, self.beta2, self.epsilon = float(beta1), float(beta2), float(epsilon)
        self.iteration = 0

    def step(self, m: torch.Tensor, grad: torch.Tensor, c_min: float, c_max: float, c_background: float):
        """m <- project(m - lr * m_hat / (sqrt(v_hat) + eps)), in place."""
        self.iteration += 1
        _lib.check(_lib.load().fdtd_adam_step(
            m.numel(), ptr(m), ptr(grad), ptr(self.mask), ptr(self.first), ptr(self.second),
            self.learning_rate, self.beta1, self.beta2, self.epsilon, self.iteration,
            1.0 / c_max ** 2, 1.0 / c_min ** 2, 1.0 / c_background ** 2, stream_handle(m.device)), "adam")
        return m


def adam_device(problem, m0, learning_rate, max_iter=15, beta1=0.9, beta2=0.999, epsilon=1e-30,
                verbose=True):
    """Projected Adam over ``problem.misfit_and_grad_device`` with everything on the GPU.

    The argument meaning and the returned ``(m, history)`` follow the reference's
    ``adam(m0, misfit_and_grad, project, mask, learning_rate, ...)``
    (invert_ring.py:817-861), with ``problem`` (a ``TorchLeastSquaresFWI``)
    supplying the objective, the projection bounds and the mask. ``m`` is
    returned as a float64 NumPy array.
    """
    dev = problem.model.device
    m = torch.as_tensor(m0, dtype=torch.float64).to(dev).contiguous().clone()
    mask = problem._mask_u8
    project_device(m, mask, problem.c_min, problem.c_max, problem.c_background)
    opt = DeviceAdam(m.shape, problem.mask, dev, learning_rate, beta1, beta2, epsilon)
    value, gradient = problem.misfit_and_grad_device(m)
    inside = problem._mask_dev
    history = {"misfit": [float(value)], "step_size": [0.0],
               "grad_norm": [float(torch.linalg.vector_norm(gradient[inside]))]}
    for iteration in range(1, max_iter + 1):
        opt.step(m, gradient, problem.c_min, problem.c_max, problem.c_background)
        value, gradient = problem.misfit_and_grad_device(m)
        grad_norm = float(torch.linalg.vector_norm(gradient[inside]))
        history["misfit"].append(float(value))
        history["step_size"].append(float(learning_rate))
        history["grad_norm"].append(grad_norm)
        if verbose:
            print(f"  Adam iter {iteration:3d}  J = {value:.6e}  lr = {learning_rate:.3e}  |g| = {grad_norm:.4e}")
    return m.cpu().numpy(), history
