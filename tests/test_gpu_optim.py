"""GPU parity of the device-resident FWI iteration: regularisers, projection, Adam.

The host restatements are ``medium.tikhonov`` / ``medium.total_variation``
(fdtd2d/inversion/misfit.py:19-71), ``TorchLeastSquaresFWI.project``
(invert_ring.py:559-565) and the Adam update of invert_ring.py:842-853 written
out below. Element values must match bit for bit (same operation order, float64);
reduced values (objective, norms) to 1e-12, and whole iterations (whose gradient
sums shots with float64 atomics in a run-dependent order) to 1e-13.
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mods():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from soundwavesimulation_gb300 import fwi, optim, torch_backend
    return torch_backend, fwi, optim


def _ring_mask(ny, nx, r):
    yy, xx = np.mgrid[:ny, :nx]
    return (yy - ny / 2) ** 2 + (xx - nx / 2) ** 2 < r * r


@pytest.mark.parametrize("alpha,tv", [(3.0e12, 0.0), (0.0, 2.0e5), (1.0e12, 5.0e4)])
def test_regularization_matches_host(mods, alpha, tv):
    _, _, optim = mods
    from soundwavesimulation_gb300.medium import tikhonov, total_variation
    rng = np.random.default_rng(4)
    ny, nx = 57, 73
    m = 1.0 / rng.uniform(1400.0, 1700.0, (ny, nx)) ** 2
    mask = _ring_mask(ny, nx, 24.0)
    eps = 1.0e-9
    g0 = rng.normal(size=(ny, nx)) * 1e-3
    v_t, g_t = tikhonov(m, mask, alpha)
    v_v, g_v = total_variation(m, mask, tv, eps)
    want = g0 + (g_t + g_v)
    want[~mask] = 0.0
    dm = torch.as_tensor(m, device="cuda")
    grad = torch.as_tensor(g0, device="cuda").clone()
    value = torch.zeros(1, dtype=torch.float64, device="cuda")
    optim.regularization_device(dm, torch.as_tensor(mask, device="cuda").to(torch.uint8), alpha, tv, eps,
                                grad, value)
    assert np.array_equal(grad.cpu().numpy(), want)
    assert float(value) == pytest.approx(v_t + v_v, rel=1e-12, abs=1e-300)


def test_adam_steps_match_numpy(mods):
    _, _, optim = mods
    rng = np.random.default_rng(8)
    shape = (40, 50)
    mask = _ring_mask(*shape, 18.0)
    c_min, c_max, c_bg = 1400.0, 2000.0, 1500.0
    m = 1.0 / rng.uniform(1380.0, 2050.0, shape) ** 2
    lr, b1, b2, eps = 2.0e-9, 0.9, 0.999, 1e-30
    opt = optim.DeviceAdam(shape, mask, "cuda", lr, b1, b2, eps)
    dm = torch.as_tensor(m, device="cuda").clone()
    first, second = np.zeros(shape), np.zeros(shape)
    for it in range(1, 4):
        g = rng.normal(size=shape) * 1e-2
        opt.step(dm, torch.as_tensor(g, device="cuda"), c_min, c_max, c_bg)
        # invert_ring.py:842-853
        first[mask] = b1 * first[mask] + (1.0 - b1) * g[mask]
        second[mask] = b2 * second[mask] + (1.0 - b2) * g[mask] ** 2
        first_hat = first[mask] / (1.0 - b1 ** it)
        second_hat = second[mask] / (1.0 - b2 ** it)
        update = np.zeros(shape)
        update[mask] = lr * first_hat / (np.sqrt(second_hat) + eps)
        m = np.clip(m - update, 1.0 / c_max ** 2, 1.0 / c_min ** 2)
        m[~mask] = 1.0 / c_bg ** 2
        assert np.array_equal(dm.cpu().numpy(), m), it


def test_adam_device_matches_host_loop(mods):
    """Two projected Adam iterations of a small ring FWI: device loop vs the
    reference's host loop over the same objective (all shots, deterministic)."""
    tb, fwi, optim = mods
    from soundwavesimulation_gb300 import RingArray, axis_centers, interior_mask, m_from_c, ricker, stable_dt
    from soundwavesimulation_gb300.phantoms import blurred_start, random_ellipses
    n, dx, nt, S = 64, 0.64e-3, 160, 6
    c_true, _ = random_ellipses(n, dx, 5, seed=2)
    dt = stable_dt(2000.0, dx, dx, cfl=0.3)
    x = axis_centers(n, dx)
    ring = RingArray(S, 0.38 * n * dx, x, x)
    wav = ricker(2.5e5, dt, nt)
    mask = interior_mask(x, x, 0.38 * n * dx, margin_m=3 * dx)
    model = tb.TorchScalarWave2D(c_true, dx, device="cuda")
    solver = tb.TorchFDTD2D(model, dt)
    sampler = tb.TorchRingSampler(ring, device="cuda")
    observed, _ = tb.simulate_shots_batch(solver, sampler, wav, ring.rows, ring.cols, nt)
    problem = fwi.TorchLeastSquaresFWI(solver, sampler, ring, wav, nt, S, observed.clone(), mask,
                                       alpha=1e10, tv=1e3, parallel_shots=S)
    m0 = m_from_c(blurred_start(c_true, 1.5, mask))
    lr = 5e-10
    m_dev, hist = optim.adam_device(problem, m0, lr, max_iter=2, verbose=False)

    # the reference's host loop (invert_ring.py:817-861) over problem.misfit_and_grad
    m = problem.project(m0)
    value, g = problem.misfit_and_grad(m)
    first, second = np.zeros_like(m), np.zeros_like(m)
    values = [value]
    for it in range(1, 3):
        first[mask] = 0.9 * first[mask] + (1.0 - 0.9) * g[mask]
        second[mask] = 0.999 * second[mask] + (1.0 - 0.999) * g[mask] ** 2
        update = np.zeros_like(m)
        update[mask] = lr * (first[mask] / (1.0 - 0.9 ** it)) / (
            np.sqrt(second[mask] / (1.0 - 0.999 ** it)) + 1e-30)
        m = problem.project(m - update)
        value, g = problem.misfit_and_grad(m)
        values.append(value)
    # the gradient's float64 atomics sum shots in a run-dependent order: last-bit differences
    assert np.allclose(m_dev, m, rtol=1e-13, atol=0.0)
    assert np.allclose(hist["misfit"], values, rtol=1e-12, atol=0.0)
    assert hist["misfit"][-1] < hist["misfit"][0]
