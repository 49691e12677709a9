"""Seeded synthetic media and acquisitions for the benchmark configurations.

No public dataset is involved: each configuration is generated from a NumPy
``default_rng`` seed with the shapes, sizes and value ranges of the
configurations it stands for. Ellipses use the mask convention of the
reference's phantom helper (fdtd2d/phantoms.py:27-35): a point is inside when
((x' / a)^2 + (y' / b)^2) <= 1 in the ellipse's rotated frame. Every grid spans
the same field of view L = 51.2 mm with the ring at radius 0.45 L; shots fire
on every other ring element with a Ricker wavelet, CFL 0.3.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .geometry import RingArray, axis_centers, stable_dt
from .waveforms import ricker

FIELD_OF_VIEW = 51.2e-3
WATER_C, WATER_RHO = 1500.0, 1000.0
CFL = 0.3


def _ellipse(xx, yy, x0, y0, a, b, phi):
    dx, dy = xx - x0, yy - y0
    xr = dx * np.cos(phi) + dy * np.sin(phi)
    yr = -dx * np.sin(phi) + dy * np.cos(phi)
    return (xr / a) ** 2 + (yr / b) ** 2 <= 1.0


def random_ellipses(n, dx, n_ellipses, seed, c_range=(1430.0, 1620.0), rho_range=(920.0, 1080.0)):
    """Water plus ``n_ellipses`` seeded ellipses inside the ring; returns (c, rho)."""
    rng = np.random.default_rng(seed)
    x = axis_centers(n, dx)
    xx, yy = np.meshgrid(x, x, indexing="xy")
    L = n * dx
    c = np.full((n, n), WATER_C)
    rho = np.full((n, n), WATER_RHO)
    for _ in range(n_ellipses):
        x0, y0 = rng.uniform(-0.22 * L, 0.22 * L, size=2)
        a, b = rng.uniform(0.03 * L, 0.11 * L, size=2)
        inside = _ellipse(xx, yy, x0, y0, a, b, rng.uniform(0.0, np.pi))
        c[inside] = rng.uniform(*c_range)
        rho[inside] = rng.uniform(*rho_range)
    return c, rho


def abdomen(n, dx, seed=2):
    """Abdomen-like phantom: 1540 m/s body, 1450 m/s fat rim, 8 organs at 1560-1640 m/s
    and a two-ellipse 2000 m/s inclusion; density 0.9-1.2 x water, rising with c."""
    rng = np.random.default_rng(seed)
    x = axis_centers(n, dx)
    xx, yy = np.meshgrid(x, x, indexing="xy")
    L = n * dx
    c = np.full((n, n), WATER_C)
    body_a, body_b = 0.36 * L, 0.28 * L
    c[_ellipse(xx, yy, 0.0, 0.0, body_a, body_b, 0.0)] = 1450.0          # fat rim
    c[_ellipse(xx, yy, 0.0, 0.0, body_a - 0.03 * L, body_b - 0.03 * L, 0.0)] = 1540.0
    for _ in range(8):
        while True:
            x0 = rng.uniform(-0.22 * L, 0.22 * L)
            y0 = rng.uniform(-0.15 * L, 0.15 * L)
            if (x0 / (body_a - 0.09 * L)) ** 2 + (y0 / (body_b - 0.09 * L)) ** 2 < 1.0:
                break
        a, b = rng.uniform(0.03 * L, 0.08 * L, size=2)
        c[_ellipse(xx, yy, x0, y0, a, b, rng.uniform(0.0, np.pi))] = rng.uniform(1560.0, 1640.0)
    y_spine = -(body_b - 0.08 * L)
    c[_ellipse(xx, yy, 0.0, y_spine, 0.035 * L, 0.03 * L, 0.0)] = 2000.0
    c[_ellipse(xx, yy, 0.0, y_spine + 0.045 * L, 0.015 * L, 0.02 * L, 0.0)] = 2000.0
    rho = WATER_RHO * np.clip(0.9 + 0.3 * (c - 1450.0) / 550.0, 0.9, 1.2)
    rho[c == WATER_C] = WATER_RHO
    return c, rho


def blurred_start(c, sigma_cells, mask, background=WATER_C):
    """Gaussian-blurred slowness^2 with the exterior reset (invert_ring.py:1179-1184)."""
    from scipy.ndimage import gaussian_filter
    m = gaussian_filter(1.0 / (c * c), sigma_cells, mode="nearest")
    m[~mask] = 1.0 / background ** 2
    return 1.0 / np.sqrt(m)


@dataclass
class Acquisition:
    """One grid of a configuration: medium, ring, shots and waveform."""
    name: str
    n: int
    dx: float
    c: np.ndarray
    rho: np.ndarray
    n_elements: int
    tx: np.ndarray
    f0: float
    n_steps: int
    source: str = "bilinear"   # "bilinear" (4 nodes) or "nearest"
    dt: float = 0.0
    x: np.ndarray = field(default=None, repr=False)
    ring: RingArray = field(default=None, repr=False)
    wavelet: np.ndarray = field(default=None, repr=False)

    def __post_init__(self):
        self.dt = stable_dt(float(self.c.max()), self.dx, self.dx, cfl=CFL)
        self.x = axis_centers(self.n, self.dx)
        self.ring = RingArray(self.n_elements, 0.45 * self.n * self.dx, self.x, self.x)
        self.wavelet = ricker(self.f0, self.dt, self.n_steps)

    @property
    def n_shots(self):
        return int(len(self.tx))

    @property
    def cell_updates(self):
        return float(self.n) ** 2 * self.n_shots * self.n_steps

    def source_tables(self):
        """Per-shot injection tables (rows, cols, weights, waveform index), each (S, K)."""
        if self.source == "nearest":
            rows = self.ring.rows[self.tx][:, None]
            cols = self.ring.cols[self.tx][:, None]
            w = np.ones(rows.shape)
        else:
            taps = [self.ring.bilinear_source(t) for t in self.tx]
            rows = np.stack([t[0] for t in taps])
            cols = np.stack([t[1] for t in taps])
            w = np.stack([t[2] for t in taps])
        return rows, cols, w, np.zeros(rows.shape, dtype=np.int64)

    def subset(self, n_shots=None, n_steps=None):
        """Same medium and ring with fewer shots and/or steps (for bounded CPU samples)."""
        return Acquisition(self.name + "-subset", self.n, self.dx, self.c, self.rho, self.n_elements,
                           self.tx[: n_shots or len(self.tx)], self.f0, n_steps or self.n_steps, self.source)


def config(k: int):
    """The benchmark configuration k (1..5) as a list of Acquisition objects (one per grid)."""
    if k == 1:
        c, rho = random_ellipses(256, 0.2e-3, 6, seed=1)
        return [Acquisition("c1-256", 256, 0.2e-3, c, rho, 128, np.array([0]), 0.5e6, 2000)]
    if k in (2, 3):
        c, rho = abdomen(512, 0.1e-3, seed=2)
        tx = np.arange(0, 256, 2) if k == 2 else np.arange(0, 256, 4)
        return [Acquisition(f"c{k}-512", 512, 0.1e-3, c, rho, 256, tx, 0.8e6, 4000)]
    if k == 4:
        out = []
        for i, (n, f0, shots, nt) in enumerate(((256, 0.3e6, 96, 2000), (384, 0.6e6, 96, 3000),
                                                (512, 1.0e6, 64, 4000))):
            dx = FIELD_OF_VIEW / n
            c, rho = random_ellipses(n, dx, 6, seed=40 + i)
            out.append(Acquisition(f"c4-{n}", n, dx, c, rho, 2 * shots, np.arange(0, 2 * shots, 2), f0, nt))
        return out
    if k == 5:
        c, rho = abdomen(1024, 0.05e-3, seed=2)
        return [Acquisition("c5-1024", 1024, 0.05e-3, c, rho, 512, np.arange(0, 512, 2), 1.0e6, 6000)]
    raise ValueError("configurations are numbered 1 to 5")
