"""The float64 variable-density restatement (no reference counterpart in 2-D; the
conservative form of 1DWaveSimulation.py:116-143), on the CPU: at constant
density it is the reference's stencil, and its gradients with respect to slowness
squared and density equal central differences of the float64 objective where the
waves do not reach the Mur edges (there the reference's adjoint, which reuses the
forward Mur update, is exact)."""

import numpy as np

from oracle import fdtd_oracle as orc


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / np.linalg.norm(np.ravel(b)))


def test_constant_density_is_the_reference_stencil(golden):
    d = golden("ellipses64")
    geo = {k: d[k] for k in ("row0", "col0", "w00", "w10", "w01", "w11")}
    geo["row1"], geo["col1"] = geo["row0"] + 1, geo["col0"] + 1
    n = d["c"].shape[0]
    tx = d["tx"]
    src = orc.point_sources((n, n), d["rows"][tx], d["cols"][tx])
    nt = int(d["n_steps"])
    tr, _ = orc.simulate_density(d["c"], np.full((n, n), 1020.0), float(d["dx"]), float(d["dx"]), float(d["dt"]),
                                 geo, src, d["wavelet"], nt)
    assert rel(tr, d["traces_f64"]) < 1e-12


def test_density_gradients_against_central_differences():
    dx, nt = 1e-3, 60
    rng = np.random.default_rng(3)
    c = 1500 + 100 * rng.random((70, 66))
    ny, nx = c.shape
    dt = orc.stable_dt(c.max(), dx, dx, 0.3)
    geo = orc.ring_geometry(8, 0.008, orc.axis_centers(nx, dx), orc.axis_centers(ny, dx))
    wav = np.sin(np.arange(nt) * 0.5) * np.exp(-((np.arange(nt) - 12) / 5.0) ** 2)
    src = orc.point_sources((ny, nx), geo["rows"][[0, 3]], geo["cols"][[0, 3]])
    rho = 1000 + 150 * rng.random(c.shape)
    mute = np.array([0, 3])
    obs, _ = orc.simulate_density(c * 1.02, rho * 1.05, dx, dx, dt, geo, src, wav, nt)
    _, gk, gbx, gby = orc.density_gradient(c, rho, dx, dx, dt, geo, src, wav, nt, obs, mute)
    m = 1 / c ** 2
    gm, gr = orc.density_chain_rule(m, rho, gk, gbx, gby)

    def J(mm, rr):
        tr, _ = orc.simulate_density(1 / np.sqrt(mm), rr, dx, dx, dt, geo, src, wav, nt)
        return 0.5 * np.sum(orc.residual_batch(tr, obs, mute) ** 2)

    inner = np.zeros(c.shape, dtype=bool)
    inner[8:-8, 8:-8] = True  # Mur coefficients (edge cells) stay fixed
    for seed in range(2):
        r = np.random.default_rng(seed)
        d = np.where(inner, r.standard_normal(c.shape), 0.0)
        dm, dr = d * m * 1e-3, d * rho * 1e-3
        fd_m = (J(m + dm, rho) - J(m - dm, rho)) / 2
        fd_r = (J(m, rho + dr) - J(m, rho - dr)) / 2
        assert abs(fd_m - np.sum(gm * dm)) / abs(fd_m) < 1e-4
        assert abs(fd_r - np.sum(gr * dr)) / abs(fd_r) < 1e-4
