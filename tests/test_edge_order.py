"""The order of the GPU kernel's compact edge update equals the reference's Mur order.

The reference (fdtd2d/torch_backend.py:477-490, restated as ``oracle.apply_mur``)
updates the left/right columns on rows 1..ny-2, the bottom/top rows on columns
1..nx-2, then each corner as the average of an x- and a y-direction Mur from the
updated edge neighbours. The kernel's compact edge loop instead updates the
edge rows on whole 4-cell lane rows and the edge columns on every band row,
padding cells included, then writes the corners. This test restates that order
in float64 NumPy on a padded region (zero padding cells, zero Mur coefficients
there, as the kernel's shared-memory table holds them) and checks that it gives
the reference's field bit for bit and keeps the padding at zero.
"""

import numpy as np
import pytest

from oracle import fdtd_oracle as orc

_CORNERS = ((0, 0, 1, 1), (0, -1, 1, -2), (-1, 0, -2, 1), (-1, -1, -2, -2))


def compact_order(u, u_next, k, pad_rows, pad_cols):
    """Rows on all columns, columns on all rows, corners last, on a padded region."""
    ny, nx = u.shape[0] - pad_rows, u.shape[1] - pad_cols
    u = u.copy()
    un = u_next.copy()

    def table(edge, n, pad):
        # per-position k of the kernel's table: the reference's k inside, an
        # arbitrary finite value at the corner positions, zero in the padding
        v = np.zeros(n + pad)
        v[1:n - 1] = edge
        v[0], v[n - 1] = 0.37, -0.41
        return v

    kb = table(k["bottom"], nx, pad_cols)
    kt = table(k["top"], nx, pad_cols)
    kl = table(k["left"], ny, pad_rows)
    kr = table(k["right"], ny, pad_rows)
    # Mur rows: every column of the region
    un[0, :] = u[1, :] + kb * (un[1, :] - u[0, :])
    un[ny - 1, :] = u[ny - 2, :] + kt * (un[ny - 2, :] - u[ny - 1, :])
    # Mur columns: every row of the region
    un[:, 0] = u[:, 1] + kl * (un[:, 1] - u[:, 0])
    un[:, nx - 1] = u[:, nx - 2] + kr * (un[:, nx - 2] - u[:, nx - 1])
    # corners from their updated neighbours
    for i, (r, c, ri, ci) in enumerate(_CORNERS):
        r, c = r % ny, c % nx
        ri, ci = ri % ny, ci % nx
        cu = u[r, c]
        fx = u[r, ci] + k["corner_kx"][i] * (un[r, ci] - cu)
        fy = u[ri, c] + k["corner_ky"][i] * (un[ri, c] - cu)
        un[r, c] = 0.5 * (fx + fy)
    return un


@pytest.mark.parametrize("ny,nx,pad_rows,pad_cols", [(9, 7, 0, 1), (16, 12, 5, 0), (31, 29, 3, 3), (8, 8, 0, 0)])
def test_compact_edge_order_matches_reference(ny, nx, pad_rows, pad_cols):
    rng = np.random.default_rng(ny * 100 + nx)
    c = rng.uniform(1400.0, 1700.0, size=(ny, nx))
    dx, dy = 0.5e-3, 0.6e-3
    dt = orc.stable_dt(1700.0, dx, dy, cfl=0.4)
    k = orc.mur_coefficients(c, dt, dx, dy)
    u = np.zeros((ny + pad_rows, nx + pad_cols))
    un = np.zeros_like(u)
    u[:ny, :nx] = rng.standard_normal((ny, nx))
    un[:ny, :nx] = rng.standard_normal((ny, nx))
    want = orc.apply_mur(u[:ny, :nx].copy(), un[:ny, :nx].copy(), k)
    got = compact_order(u, un, k, pad_rows, pad_cols)
    assert np.array_equal(got[:ny, :nx], want)
    assert not np.any(got[ny:, :]) and not np.any(got[:, nx:])
