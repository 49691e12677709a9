"""Grid axes, time step and ring / arc transducer geometry (host side).

Mirrors the reference's fdtd2d/experiment.py (axis_centers, stable_dt,
n_steps_for_crossing) and fdtd2d/array.py (RingArray, ArcArray) with the same
names, conventions and errors, so callers of the reference find the same API:
element i of a ring sits at angle 2*pi*i/N; its source node is the nearest grid
node and its receiver samples the four surrounding nodes bilinearly.
"""

from __future__ import annotations

import numpy as np


def axis_centers(n, spacing):
    """Cell-centre coordinates of ``n`` cells centred on 0 (fdtd2d/experiment.py:6-8)."""
    return (np.arange(n, dtype=float) - (n - 1) / 2.0) * float(spacing)


def stable_dt(c_max, dx, dy, cfl=0.45):
    """dt = cfl / (c_max * sqrt(1/dx^2 + 1/dy^2))  (fdtd2d/experiment.py:11-13)."""
    return float(cfl) / (float(c_max) * np.sqrt(dx ** -2.0 + dy ** -2.0))


def n_steps_for_crossing(radius_m, c_min, dt, extras=1.6):
    """Steps for a wave to cross the ring diameter, with margin (fdtd2d/experiment.py:16-18)."""
    return int(np.ceil(extras * 2.0 * float(radius_m) / float(c_min) / float(dt)))


class _ElementGeometry:
    """Shared index and weight computation of ring-like arrays."""

    def _place(self, theta, x_m, y_m):
        self.theta = np.asarray(theta, dtype=float)
        self.x = self.center[0] + self.radius_m * np.cos(self.theta)
        self.y = self.center[1] + self.radius_m * np.sin(self.theta)
        self._x_axis = np.asarray(x_m, dtype=float)
        self._y_axis = np.asarray(y_m, dtype=float)
        hx = self._x_axis[1] - self._x_axis[0]
        hy = self._y_axis[1] - self._y_axis[0]
        fcol = (self.x - self._x_axis[0]) / hx   # fractional grid positions
        frow = (self.y - self._y_axis[0]) / hy
        self.cols = np.rint(fcol).astype(np.intp)
        self.rows = np.rint(frow).astype(np.intp)
        self._check_inside()
        self._col0 = np.floor(fcol).astype(np.intp)
        self._row0 = np.floor(frow).astype(np.intp)
        self._col1 = self._col0 + 1
        self._row1 = self._row0 + 1
        ax = fcol - self._col0
        ay = frow - self._row0
        self._w00 = (1.0 - ax) * (1.0 - ay)
        self._w10 = ax * (1.0 - ay)
        self._w01 = (1.0 - ax) * ay
        self._w11 = ax * ay

    def _check_bounds(self, what):
        nx, ny = self._x_axis.size, self._y_axis.size
        if self.cols.min() < 1 or self.cols.max() > nx - 2:
            raise ValueError(f"{what} extends too close to the x boundaries.")
        if self.rows.min() < 1 or self.rows.max() > ny - 2:
            raise ValueError(f"{what} extends too close to the y boundaries.")

    def transmitter_index(self, tx):
        tx = int(tx)
        if not 0 <= tx < self.n_elements:
            raise ValueError(f"Transmitter index {tx} is out of range.")
        return tx

    def inject_rows_cols(self, tx):
        tx = self.transmitter_index(tx)
        return self.rows[tx], self.cols[tx]

    # bilinear taps in the receiver order (w00, w10, w01, w11)
    def receiver_taps(self):
        """(row0, col0, weights (N, 4)) of the bilinear receivers."""
        w = np.stack([self._w00, self._w10, self._w01, self._w11], axis=1)
        return self._row0.copy(), self._col0.copy(), w

    def bilinear_source(self, tx):
        """Rows, columns and weights of the 4-node bilinear source of element ``tx``
        (desmond/src/phase2_numerics.py:107-118)."""
        tx = self.transmitter_index(tx)
        r0, c0 = self._row0[tx], self._col0[tx]
        rows = np.array([r0, r0, r0 + 1, r0 + 1])
        cols = np.array([c0, c0 + 1, c0, c0 + 1])
        w = np.array([self._w00[tx], self._w10[tx], self._w01[tx], self._w11[tx]])
        return rows, cols, w

    def record(self, field):
        """Bilinear sample of a (ny, nx) field at every element (fdtd2d/array.py:78-85)."""
        return (field[self._row0, self._col0] * self._w00 + field[self._row0, self._col1] * self._w10
                + field[self._row1, self._col0] * self._w01 + field[self._row1, self._col1] * self._w11)

    def record_adjoint(self, residual, out=None):
        """Transpose of ``record`` (fdtd2d/array.py:87-105)."""
        residual = np.asarray(residual, dtype=float)
        if residual.shape != (self.n_elements,):
            raise ValueError(f"Residual shape {residual.shape} does not match ({self.n_elements},).")
        shape = (self._y_axis.size, self._x_axis.size)
        if out is None:
            out = np.zeros(shape)
        else:
            out.fill(0.0)
        for rows, cols, w in ((self._row0, self._col0, self._w00), (self._row0, self._col1, self._w10),
                              (self._row1, self._col0, self._w01), (self._row1, self._col1, self._w11)):
            np.add.at(out, (rows, cols), residual * w)
        return out


class RingArray(_ElementGeometry):
    """N point elements equally spaced on a circle (fdtd2d/array.py:6-105)."""

    def __init__(self, n_elements, radius_m, x_m, y_m, center=(0.0, 0.0)):
        if n_elements < 2:
            raise ValueError("Need at least 2 ring elements.")
        self.n_elements = int(n_elements)
        self.radius_m = float(radius_m)
        self.center = (float(center[0]), float(center[1]))
        self._place(2.0 * np.pi * np.arange(self.n_elements) / self.n_elements, x_m, y_m)

    def _check_inside(self):
        self._check_bounds("Ring radius")
        pitch = 2.0 * np.pi * self.radius_m / self.n_elements
        dx = abs(self._x_axis[1] - self._x_axis[0])
        if pitch < dx:
            raise ValueError(
                f"Element spacing {pitch:.4g} m is smaller than dx = {dx:.4g} m; "
                "two elements would share a pixel. Reduce N or refine the grid.")


class ArcArray(_ElementGeometry):
    """N elements equally spaced along a circular arc (fdtd2d/array.py:108-167)."""

    def __init__(self, n_elements, radius_m, span_deg, center_deg, x_m, y_m,
                 center=(0.0, 0.0), allow_shared_pixels=False):
        if n_elements < 2:
            raise ValueError("Need at least 2 arc elements.")
        if not 0.0 < span_deg < 360.0:
            raise ValueError("Arc span must be between 0 and 360 degrees.")
        self.n_elements = int(n_elements)
        self.radius_m = float(radius_m)
        self.span_deg = float(span_deg)
        self.center_deg = float(center_deg)
        self.center = (float(center[0]), float(center[1]))
        self.allow_shared_pixels = bool(allow_shared_pixels)
        half = np.deg2rad(self.span_deg) / 2.0
        self._place(np.deg2rad(self.center_deg) + np.linspace(-half, half, self.n_elements), x_m, y_m)

    @property
    def pitch_m(self):
        return self.radius_m * np.deg2rad(self.span_deg) / (self.n_elements - 1)

    def _check_inside(self):
        self._check_bounds("Arc")
        dx = abs(self._x_axis[1] - self._x_axis[0])
        if self.pitch_m < dx and not self.allow_shared_pixels:
            max_elements = int(self.radius_m * np.deg2rad(self.span_deg) / dx) + 1
            raise ValueError(
                f"Element pitch {self.pitch_m:.4g} m is smaller than dx = {dx:.4g} m; "
                f"two elements would share a pixel. At most {max_elements} elements fit.")
