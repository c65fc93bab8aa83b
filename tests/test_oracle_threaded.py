"""The slab-threaded 3D oracle step (used for the timed CPU baseline) is bitwise the serial oracle.

Several forced steps with free stream and penalisation on grids whose z extent
does not divide evenly among the threads; the stable dt, vorticity, velocity
and stream function must be identical to the serial ``NavierStokes3DOracle``.
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle.flow import NavierStokes3DOracle
from oracle.threaded import ThreadedNavierStokes3DOracle


@pytest.mark.parametrize("grid,threads", [((13, 10, 12), 3), ((16, 12, 8), 5), ((8, 8, 8), 16)])
@pytest.mark.parametrize("real_t", [np.float32, np.float64])
def test_threaded_step_is_bitwise_serial(grid, threads, real_t):
    kw = dict(grid_size=grid, x_range=1.0, kinematic_viscosity=3e-3, real_t=real_t, with_forcing=True,
              with_free_stream_flow=True)
    serial, threaded = NavierStokes3DOracle(**kw), ThreadedNavierStokes3DOracle(**kw, threads=threads)
    rng = np.random.default_rng(5)
    w0 = (0.1 * rng.standard_normal((3, *grid))).astype(real_t)
    serial.vorticity_field[...] = w0
    threaded.vorticity_field[...] = w0
    for _ in range(3):
        f = (0.1 * rng.standard_normal((3, *grid))).astype(real_t)
        serial.eul_grid_forcing_field[...] = f
        threaded.eul_grid_forcing_field[...] = f
        dt = serial.compute_stable_timestep()
        assert threaded.compute_stable_timestep() == dt
        serial.time_step(dt, np.array([1.0, 0.2, 0.0]))
        threaded.time_step(dt, np.array([1.0, 0.2, 0.0]))
        for name in ("vorticity_field", "velocity_field", "stream_func_field", "eul_grid_forcing_field"):
            np.testing.assert_array_equal(getattr(threaded, name), getattr(serial, name), err_msg=name)


@pytest.mark.parametrize("ftype,grid,threads", [("scalar", (13, 11, 12), 3), ("vector", (17, 10, 9), 4),
                                                ("vector", (6, 8, 8), 8)])
@pytest.mark.parametrize("real_t", [np.float32, np.float64])
def test_threaded_passive_transport_is_bitwise_serial(ftype, grid, threads, real_t):
    from oracle.flow import PassiveTransportOracle
    from oracle.threaded import ThreadedPassiveTransportOracle
    kw = dict(kinematic_viscosity=2e-3, grid_dim=3, grid_size=grid, x_range=1.0, real_t=real_t, field_type=ftype)
    serial, threaded = PassiveTransportOracle(**kw), ThreadedPassiveTransportOracle(**kw, threads=threads)
    rng = np.random.default_rng(9)
    f0 = rng.standard_normal(serial.primary_field.shape).astype(real_t)
    u = rng.standard_normal((3, *grid)).astype(real_t)
    for o in (serial, threaded):
        o.primary_field[...] = f0
        o.velocity_field[...] = u
    for _ in range(3):
        dt = serial.compute_stable_timestep()
        serial.time_step(dt)
        threaded.time_step(dt)
        np.testing.assert_array_equal(threaded.primary_field, serial.primary_field)
