"""GPU parity of the device-resident FWI iteration: regularisers, projection, Adam.

Pinned on the reference's own outputs (tests/golden/optim.npz, made by running
fdtd2d/inversion/misfit.py:19-71 and invert_ring.py:817-861): the device
regularisers and the device Adam reproduce them. Against the oracle's
restatement (same operation order, float64) element values match bit for bit;
reduced values (objective, norms) to 1e-12, and whole iterations (whose gradient
sums shots with float64 atomics in a run-dependent order) to 1e-13.
"""

import numpy as np
import pytest
import torch

from oracle import fdtd_oracle as orc

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


def _device_reg(optim, m, mask, alpha, tv, eps, g0=None):
    dm = torch.as_tensor(m, device="cuda")
    grad = torch.zeros_like(dm) if g0 is None else torch.as_tensor(g0, device="cuda").clone()
    value = torch.zeros(1, dtype=torch.float64, device="cuda")
    optim.regularization_device(dm, torch.as_tensor(mask, device="cuda").to(torch.uint8), alpha, tv, eps,
                                grad, value)
    return float(value), grad.cpu().numpy()


def test_regularization_matches_reference_fixture(mods, golden):
    _, _, optim = mods
    g = golden("optim")
    v, gr = _device_reg(optim, g["m"], g["mask"], float(g["alpha"]), 0.0, 1.0)
    assert v == pytest.approx(float(g["tikhonov_value"]), rel=1e-12)
    np.testing.assert_allclose(gr, g["tikhonov_grad"], rtol=0, atol=1e-14 * np.abs(g["tikhonov_grad"]).max())
    v, gr = _device_reg(optim, g["m"], g["mask"], 0.0, float(g["tv"]), float(g["tv_eps"]))
    assert v == pytest.approx(float(g["tv_value"]), rel=1e-12)
    np.testing.assert_allclose(gr, g["tv_grad"], rtol=0, atol=1e-14 * np.abs(g["tv_grad"]).max())


@pytest.mark.parametrize("alpha,tv", [(3.0e12, 0.0), (0.0, 2.0e5), (1.0e12, 5.0e4)])
def test_regularization_matches_oracle_bitwise(mods, alpha, tv):
    _, _, optim = mods
    rng = np.random.default_rng(4)
    ny, nx = 57, 73
    m = 1.0 / rng.uniform(1400.0, 1700.0, (ny, nx)) ** 2
    mask = _ring_mask(ny, nx, 24.0)
    eps = 1.0e-9
    g0 = rng.normal(size=(ny, nx)) * 1e-3
    v_t, g_t = orc.tikhonov(m, mask, alpha)
    v_v, g_v = orc.total_variation(m, mask, tv, eps)
    want = g0 + (g_t + g_v)
    want[~mask] = 0.0
    v, grad = _device_reg(optim, m, mask, alpha, tv, eps, g0)
    assert np.array_equal(grad, want)
    assert v == pytest.approx(v_t + v_v, rel=1e-12, abs=1e-300)


def test_host_regularizer_api_runs_on_device(mods, golden):
    """medium.tikhonov / total_variation (the reference's names) give the fixture's values."""
    from soundwavesimulation_gb300 import tikhonov, total_variation
    g = golden("optim")
    v, gr = tikhonov(g["m"], g["mask"], float(g["alpha"]))
    assert v == pytest.approx(float(g["tikhonov_value"]), rel=1e-12)
    np.testing.assert_allclose(gr, g["tikhonov_grad"], rtol=0, atol=1e-14 * np.abs(g["tikhonov_grad"]).max())
    v, gr = total_variation(g["m"], g["mask"], float(g["tv"]), float(g["tv_eps"]))
    assert v == pytest.approx(float(g["tv_value"]), rel=1e-12)


def test_adam_matches_reference_fixture(mods, golden):
    """Three device Adam steps on the fixture's quadratic objective reproduce the
    reference adam's iterates."""
    _, _, optim = mods
    g = golden("optim")
    mask = g["mask"]
    c_min, c_max, c_bg = float(g["adam_c_min"]), float(g["adam_c_max"]), float(g["adam_c_background"])
    dm = torch.as_tensor(g["m"], device="cuda").clone()
    mk = torch.as_tensor(mask, device="cuda")
    target = torch.as_tensor(g["adam_target"], device="cuda")
    weight = torch.as_tensor(g["adam_weight"], device="cuda")
    optim.project_device(dm, mk.to(torch.uint8), c_min, c_max, c_bg)
    opt = optim.DeviceAdam(dm.shape, mask, "cuda", float(g["adam_lr"]))
    for k in range(3):
        grad = weight * torch.where(mk, dm - target, torch.zeros_like(dm))
        opt.step(dm, grad, c_min, c_max, c_bg)
        np.testing.assert_allclose(dm.cpu().numpy(), g["adam_iterates"][k], rtol=1e-14, atol=0,
                                   err_msg=f"iteration {k + 1}")


def test_adam_steps_match_oracle_bitwise(mods):
    _, _, optim = mods
    rng = np.random.default_rng(8)
    shape = (40, 50)
    mask = _ring_mask(*shape, 18.0)
    c_min, c_max, c_bg = 1400.0, 2000.0, 1500.0
    m = 1.0 / rng.uniform(1380.0, 2050.0, shape) ** 2
    lr = 2.0e-9
    grads = [rng.normal(size=shape) * 1e-2 for _ in range(4)]

    def project(mm):
        out = np.clip(mm, 1.0 / c_max ** 2, 1.0 / c_min ** 2)
        out[~mask] = 1.0 / c_bg ** 2
        return out

    calls = iter(range(4))

    def objective(mm):
        return 0.0, grads[next(calls)]

    want = orc.projected_adam(m, objective, project, mask, lr, 3)
    dm = torch.as_tensor(project(m), device="cuda").clone()
    opt = optim.DeviceAdam(shape, mask, "cuda", lr)
    for it in range(3):
        opt.step(dm, torch.as_tensor(grads[it], device="cuda"), c_min, c_max, c_bg)
        assert np.array_equal(dm.cpu().numpy(), want[it]), it + 1


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

    # the oracle's restatement of the reference's host loop (invert_ring.py:817-861)
    # over problem.misfit_and_grad
    values = []

    def objective(mm):
        value, g = problem.misfit_and_grad(mm)
        values.append(value)
        return value, g

    m = orc.projected_adam(m0, objective, problem.project, mask, lr, 2)[-1]
    # the gradient's float64 atomics sum shots in a run-dependent order: last-bit differences
    assert np.allclose(m_dev, m, rtol=1e-13, atol=0.0)
    assert np.allclose(hist["misfit"], values, rtol=1e-12, atol=0.0)
    assert hist["misfit"][-1] < hist["misfit"][0]
