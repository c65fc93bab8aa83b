"""Precision helpers and the base forcing grid, after the reference's own tests
(tests/test_utils/test_precision.py, tests/test_simulator/test_immersed_body/test_immersed_body_forcing_grid.py).
"""

from __future__ import annotations

import logging

import numpy as np
import pytest

import sopht_gb300.simulator as sps
import sopht_gb300.utils as spu


@pytest.mark.parametrize("precision", ["half", "single", "double"])
def test_get_real_t(precision):
    if precision == "half":
        with pytest.raises(ValueError, match="Precision argument must be single or double"):
            spu.get_real_t(precision)
    else:
        assert spu.get_real_t(precision) == {"single": np.float32, "double": np.float64}[precision]


@pytest.mark.parametrize("precision,real_t", [("single", np.float32), ("double", np.float64)])
def test_get_test_tol(precision, real_t):
    assert spu.get_test_tol(precision) == real_t(1e3 * np.finfo(real_t).eps)


def test_vector_field_axes():
    assert (spu.VectorField.x_axis_idx(), spu.VectorField.y_axis_idx(), spu.VectorField.z_axis_idx()) == (0, 1, 2)


@pytest.mark.parametrize("grid_dim", [2, 3])
@pytest.mark.parametrize("num_lag_nodes", [8, 16])
def test_base_forcing_grid(caplog, grid_dim, num_lag_nodes):
    with caplog.at_level(logging.WARNING, logger="sopht_gb300"):
        grid = sps.ImmersedBodyForcingGrid(grid_dim=grid_dim, num_lag_nodes=num_lag_nodes)
    assert (grid.grid_dim, grid.num_lag_nodes) == (grid_dim, num_lag_nodes)
    np.testing.assert_array_equal(grid.position_field, np.zeros((grid_dim, num_lag_nodes)))
    np.testing.assert_array_equal(grid.velocity_field, np.zeros((grid_dim, num_lag_nodes)))
    warned = [r for r in caplog.records if r.levelno == logging.WARNING and "XY plane" in r.getMessage()]
    assert bool(warned) == (grid_dim == 2)
