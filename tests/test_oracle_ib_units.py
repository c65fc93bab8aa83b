"""The reference's manufactured-solution checks of the Eulerian-Lagrangian transfer, on the oracle.

After tests/test_numeric/test_immersed_boundary_ops/test_eulerian_lagrangian_grid_communicator_{2,3}d.py:
markers on grid nodes give their node index and offsets k dx (k = -1..2);
interpolating a field of ones with weights 0..4^dim - 1 gives their sum times
dx^dim; spreading 2 with unit weights puts n_lag * 2 * 4^dim on the grid;
with offsets 0 along x and dx along the other axes both delta kernels weigh
every support cell the same, 2 (0.25/dx)^dim (a factor 2 along x, 1 along the
others).  Tolerance: 1e3 eps, as in the reference.
"""

from __future__ import annotations

import numpy as np
import pytest
from conftest import real_t_of, ref_tol

from oracle import ib

N = 16
W = 2
N_LAG = 3


def _setup(precision, dim):
    rt = real_t_of(precision)
    dx = rt(1.0 / N)
    shift = rt(0.5 * dx)
    nearest = np.stack([np.arange(N // 3, N // 3 + N_LAG)] * dim)
    positions = (nearest * dx + shift).astype(np.float64)
    return rt, dx, shift, nearest, positions


@pytest.mark.parametrize("dim", [2, 3])
def test_support_of_markers_on_nodes(precision, dim):
    rt, dx, shift, nearest, positions = _setup(precision, dim)
    got_nearest, support, _ = ib.nearest_index_and_support(positions, dx, shift, W)
    np.testing.assert_array_equal(got_nearest, nearest)
    k = np.arange(-W + 1, W + 1).reshape(1, -1, 1)
    np.testing.assert_allclose(support, np.broadcast_to(k * dx, support.shape), atol=ref_tol(precision))


@pytest.mark.parametrize("dim", [2, 3])
def test_interpolation_with_synthetic_weights(precision, dim):
    rt, dx, _, nearest, _ = _setup(precision, dim)
    cells = (2 * W) ** dim
    weights = np.tile(np.arange(cells, dtype=rt).reshape(*(2 * W,) * dim, 1), (1,) * dim + (N_LAG,))
    field = np.ones((dim, *(N,) * dim), dtype=rt)
    out = ib.interpolate(field, weights, nearest, dx, W)
    np.testing.assert_allclose(out, cells * (cells - 1) / 2 * dx ** dim, atol=ref_tol(precision))


@pytest.mark.parametrize("dim", [2, 3])
def test_spreading_integral(precision, dim):
    rt, _, _, nearest, _ = _setup(precision, dim)
    cells = (2 * W) ** dim
    weights = np.ones((*(2 * W,) * dim, N_LAG), dtype=rt)
    lag = np.full((dim, N_LAG), 2.0, dtype=rt)
    field = np.zeros((dim, *(N,) * dim), dtype=rt)
    ib.spread(field, lag, weights, nearest, W)
    for c in range(dim):
        np.testing.assert_allclose(field[c].sum(), N_LAG * 2.0 * cells, atol=ref_tol(precision))


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("kernel", ["cosine", "peskin"])
def test_weights_on_nodes(precision, dim, kernel):
    rt, dx, _, _, _ = _setup(precision, dim)
    support = np.full((dim, 2 * W, N_LAG), dx, dtype=rt)
    support[0] = 0.0  # x offsets 0, the others dx
    fn = ib.cosine_weights if kernel == "cosine" else ib.peskin_weights
    w = fn(support, dx, rt)
    expected = rt(2 * (0.25 / dx) ** dim)
    np.testing.assert_allclose(w, np.full(w.shape, expected), rtol=ref_tol(precision))
