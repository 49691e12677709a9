"""GPU parity of the variable-density engine (no 2-D reference counterpart: the
reference's planned conservative form, fdtd2d/wave.py:61-63, with 1/rho on the
faces as its 1-D solver has it, 1DWaveSimulation.py:116-143).

The checker is the float64 restatement in oracle/fdtd_oracle.py (at constant
density equal to the reference's fixture, and its gradients equal central
differences; tests/test_density_oracle.py). Budgets: traces rel-L2 <= 1e-5 and
gradients rel-L2 <= 1e-3 against float64, the chain-rule kernel to 1e-12.
"""

import numpy as np
import pytest
import torch

from oracle import fdtd_oracle as orc

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.fixture(scope="module")
def dens():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from soundwavesimulation_gb300 import density, engine
    return density, engine


def _problem(ny, nx, n_shots, nt, seed, rho_contrast=0.3):
    rng = np.random.default_rng(seed)
    dx = 0.25e-3
    c = 1480.0 + 150.0 * rng.random((ny, nx))
    c[ny // 3: ny // 2, nx // 4: nx // 2] = 1750.0
    rho = 1000.0 * (1.0 + rho_contrast * rng.random((ny, nx)))
    rho[ny // 2: 2 * ny // 3, nx // 2: 3 * nx // 4] = 1900.0
    dt = orc.stable_dt(c.max(), dx, dx, 0.3)
    x, y = orc.axis_centers(nx, dx), orc.axis_centers(ny, dx)
    geo = orc.ring_geometry(24, 0.4 * min(nx, ny) * dx, x, y)
    tx = np.arange(n_shots) * (24 // n_shots)
    taps = [orc.bilinear_source_taps(geo, t) for t in tx]
    rows, cols, w = (np.stack([t[i] for t in taps]) for i in range(3))
    fields = np.zeros((n_shots, ny, nx))
    for s in range(n_shots):
        np.add.at(fields[s], (rows[s], cols[s]), w[s])
    rx = (geo["row0"], geo["col0"], np.stack([geo[k] for k in ("w00", "w10", "w01", "w11")], axis=1))
    t = np.arange(nt) * dt
    f0 = 3.0e5
    a = (np.pi * f0 * (t - 1.5 / f0)) ** 2
    wav = (1 - 2 * a) * np.exp(-a)
    return dict(c=c, rho=rho, dx=dx, dt=dt, geo=geo, tx=tx, src=(rows, cols, w), fields=fields, rx=rx, wav=wav,
                nt=nt)


def _sources(p):
    rows, cols, w = p["src"]
    return rows, cols, w, np.zeros(rows.shape, dtype=np.int64)


@pytest.mark.parametrize("ny,nx", [(96, 110), (131, 77)])
def test_density_traces_vs_float64(dens, ny, nx):
    density, _ = dens
    p = _problem(ny, nx, 3, 300, seed=ny)
    medium = density.DensityMedium(p["c"], p["rho"], p["dx"], p["dx"], p["dt"], "cuda")
    traces = density.forward_density(medium, p["rx"], _sources(p), p["wav"][None], p["nt"])
    ref, _ = orc.simulate_density(p["c"], p["rho"], p["dx"], p["dx"], p["dt"], p["geo"], p["fields"], p["wav"],
                                  p["nt"])
    assert rel(traces.cpu().numpy(), ref) < 1e-5


def test_constant_density_matches_the_mur_engine(dens):
    density, engine = dens
    p = _problem(100, 90, 2, 250, seed=5)
    rho = np.full(p["c"].shape, 1020.0)
    medium = density.DensityMedium(p["c"], rho, p["dx"], p["dx"], p["dt"], "cuda")
    traces = density.forward_density(medium, p["rx"], _sources(p), p["wav"][None], p["nt"])
    plain = engine.DeviceMedium(p["c"], p["dx"], p["dx"], p["dt"], "cuda")
    tables = engine.ProblemTables(plain, p["rx"], _sources(p),
                                  torch.as_tensor(p["wav"][None], dtype=torch.float32, device="cuda"), p["nt"])
    ref = engine.forward_plain(tables)
    assert rel(traces.cpu().numpy(), ref.cpu().numpy()) < 2e-6


def test_density_gradients_vs_float64(dens):
    density, _ = dens
    p = _problem(90, 96, 2, 280, seed=11)
    obs, _ = orc.simulate_density(p["c"] * 1.01, p["rho"] * 1.04, p["dx"], p["dx"], p["dt"], p["geo"], p["fields"],
                                  p["wav"], p["nt"])
    mute = p["tx"]
    J_ref, gk, gbx, gby = orc.density_gradient(p["c"], p["rho"], p["dx"], p["dx"], p["dt"], p["geo"], p["fields"],
                                               p["wav"], p["nt"], obs, mute)
    m = 1.0 / p["c"] ** 2
    gm_ref, gr_ref = orc.density_chain_rule(m, p["rho"], gk, gbx, gby)
    medium = density.DensityMedium(p["c"], p["rho"], p["dx"], p["dx"], p["dt"], "cuda")
    J, g_m, g_rho = density.gradient_density(medium, p["rx"], _sources(p), p["wav"][None], p["nt"], obs, mute)
    assert abs(J - J_ref) / J_ref < 1e-5
    assert rel(g_m.cpu().numpy(), gm_ref) < 1e-3
    assert rel(g_rho.cpu().numpy(), gr_ref) < 1e-3
    # the mask zeroes the gradient outside it and leaves the rest unchanged
    mask = np.zeros(m.shape, dtype=bool)
    mask[20:70, 15:80] = True
    _, g_m2, g_rho2 = density.gradient_density(medium, p["rx"], _sources(p), p["wav"][None], p["nt"], obs, mute,
                                               mask=mask)
    mk = torch.as_tensor(mask, device="cuda")
    assert float(g_m2[~mk].abs().sum()) == 0.0 and float(g_rho2[~mk].abs().sum()) == 0.0
    assert rel(g_rho2[mk].cpu().numpy(), g_rho[mk].cpu().numpy()) < 1e-12
    assert rel(g_m2[mk].cpu().numpy(), g_m[mk].cpu().numpy()) < 1e-12


def test_density_chain_rule_kernel(dens):
    from soundwavesimulation_gb300 import _lib
    from soundwavesimulation_gb300.engine import padded_width, ptr, stream_handle
    rng = np.random.default_rng(2)
    ny, nx = 37, 53
    pitch = padded_width(nx)
    m = 1.0 / (1400.0 + 300.0 * rng.random((ny, nx))) ** 2
    rho = 900.0 + 800.0 * rng.random((ny, nx))
    gk = rng.standard_normal((ny, nx))
    gbx = rng.standard_normal((ny, nx + 1))
    gby = rng.standard_normal((ny + 1, nx))
    gm_ref, gr_ref = orc.density_chain_rule(m, rho, gk, gbx, gby)
    dev = "cuda"
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=dev)
    gk_d = torch.zeros((ny, pitch), dtype=torch.float64, device=dev)
    gk_d[:, :nx] = t(gk)
    gbx_d = torch.zeros((ny, pitch + 4), dtype=torch.float64, device=dev)
    gbx_d[:, :nx + 1] = t(gbx)
    gby_d = torch.zeros((ny + 1, pitch), dtype=torch.float64, device=dev)
    gby_d[:, :nx] = t(gby)
    m_d, rho_d = t(m), t(rho)
    g_m = torch.empty_like(m_d)
    g_rho = torch.empty_like(m_d)
    _lib.check(_lib.load().fdtd_density_chain_rule(ny, nx, pitch, ptr(m_d), ptr(rho_d), ptr(gk_d), ptr(gbx_d),
                                                   ptr(gby_d), None, ptr(g_m), ptr(g_rho), stream_handle(dev)),
               "density_chain_rule")
    assert rel(g_m.cpu().numpy(), gm_ref) < 1e-12
    assert rel(g_rho.cpu().numpy(), gr_ref) < 1e-12


def test_density_validation(dens):
    density, _ = dens
    p = _problem(40, 40, 1, 10, seed=1)
    with pytest.raises(ValueError):
        density.DensityMedium(p["c"], -p["rho"], p["dx"], p["dx"], p["dt"], "cuda")
    with pytest.raises(ValueError):
        density.DensityMedium(p["c"], p["rho"][:-1], p["dx"], p["dx"], p["dt"], "cuda")
