"""Immersed-boundary transfer and virtual-boundary forcing (oracle only).

Restates ``immersed_boundary_ops/EulerianLagrangianGridCommunicator{2,3}D.py``
and ``immersed_boundary_ops/VirtualBoundaryForcing.py:20-283``.  Marker
positions and body velocities are float64 (as the reference's forcing grids
hold them); the Lagrangian buffers are ``real_t``.
"""

from __future__ import annotations

import numpy as np


def nearest_index_and_support(positions, dx, shift, kernel_width=2):
    """n_d = floor((X_d - shift)/dx); r = (n + k) dx + shift - X for k in [-w+1, w].

    EulerianLagrangianGridCommunicator2D.py:68-131 / ...3D.py:68-138.  The
    support is returned per axis as an array ``(dim, 2w, n_lag)`` of offsets
    along that axis (the reference stores the full tensor-product grid; every
    entry of it is one of these per-axis values).
    """
    dim = positions.shape[0]
    nearest = ((positions - shift) // dx).astype(np.int64)
    k = np.arange(-kernel_width + 1, kernel_width + 1).reshape(1, -1, 1)
    support = (nearest[:, None, :] + k) * dx + shift - positions[:, None, :]
    return nearest, support, dim


def cosine_weights(support, dx, real_t):
    """phi = (0.25/dx)^dim prod_d (1 + cos(pi r_d / (2 dx))).

    EulerianLagrangianGridCommunicator2D.py:377-408 / ...3D.py:387-412.
    Returns the tensor-product weights, axis order (z,)y,x then marker.
    """
    dim = support.shape[0]
    r = support.astype(real_t) / dx
    one_d = real_t(1.0) + np.cos(real_t(0.5 * np.pi) * r)
    pref = real_t((0.25 / dx) ** dim)
    # reference evaluation order: pref * phi_x * phi_y (* phi_z)
    if dim == 2:
        return pref * one_d[0][None, :, :] * one_d[1][:, None, :]
    return pref * one_d[0][None, None, :, :] * one_d[1][None, :, None, :] * one_d[2][:, None, None, :]


def peskin_weights(support, dx, real_t):
    """Peskin (2002, eq. 6.27) 4-point delta.  ...Communicator2D.py:411-494."""
    dim = support.shape[0]
    r = np.fabs(support.astype(real_t)) / dx

    def phi(a):
        inner = (3.0 - 2 * a + np.sqrt(np.fabs(1 + 4 * a - 4 * a**2)))
        outer = (5.0 - 2 * a - np.sqrt(np.fabs(-7 + 12 * a - 4 * a**2)))
        return (a < 1.0) * inner + (a >= 1.0) * (a < 2.0) * outer

    one_d = phi(r)
    pref = (0.125 / dx) ** dim
    if dim == 2:
        w = pref * one_d[0][None, :, :] * one_d[1][:, None, :]
    else:
        w = pref * one_d[0][None, None, :, :] * one_d[1][None, :, None, :] * one_d[2][:, None, None, :]
    return w.astype(real_t)


def _window(nearest, i, kernel_width=2):
    dim = nearest.shape[0]
    lo = [nearest[d, i] - kernel_width + 1 for d in range(dim)]
    # array axis order is reversed: (z,) y, x
    return tuple(slice(lo[d], lo[d] + 2 * kernel_width) for d in reversed(range(dim)))


def interpolate(eul_field, weights, nearest, dx, kernel_width=2):
    """U_d(X_i) = dx^dim * sum_window u_d * phi.  ...Communicator2D.py:167-264."""
    dim = nearest.shape[0]
    n_lag = nearest.shape[1]
    out = np.zeros((dim, n_lag), dtype=eul_field.dtype)
    for i in range(n_lag):
        win = _window(nearest, i, kernel_width)
        for c in range(dim):
            out[c, i] = np.sum(eul_field[(c, *win)] * weights[..., i]) * (dx ** dim)
    return out


def spread(eul_field, lag_field, weights, nearest, kernel_width=2):
    """f_d(window_i) += F_d(i) * phi_i, markers in index order, in place.

    ...Communicator2D.py:267-374 / ...3D.py:302-384.
    """
    dim = nearest.shape[0]
    for i in range(nearest.shape[1]):
        win = _window(nearest, i, kernel_width)
        for c in range(dim):
            eul_field[(c, *win)] += lag_field[c, i] * weights[..., i]


class VirtualBoundaryForcingOracle:
    """VirtualBoundaryForcing.py:20-283 (feedback F = K xi + C dU)."""

    def __init__(self, stiffness, damping, grid_dim, dx, num_lag_nodes, real_t,
                 eul_grid_coord_shift=None, interp_kernel_width=2,
                 enable_eul_grid_forcing_reset=False, kernel="cosine", start_time=0.0):
        self.K, self.C = stiffness, damping
        self.dim, self.dx, self.real_t = grid_dim, dx, real_t
        self.shift = real_t(dx / 2) if eul_grid_coord_shift is None else eul_grid_coord_shift
        self.width = interp_kernel_width
        self.reset = enable_eul_grid_forcing_reset
        self.kernel = kernel
        self.time = start_time
        z = np.zeros((grid_dim, num_lag_nodes), dtype=real_t)
        self.lag_grid_flow_velocity_field = z.copy()
        self.lag_grid_position_mismatch_field = z.copy()
        self.lag_grid_velocity_mismatch_field = z.copy()
        self.lag_grid_forcing_field = z.copy()
        self.nearest = None
        self.weights = None

    def compute_interaction_force_on_lag_grid(self, eul_velocity, lag_position, lag_velocity):
        """VirtualBoundaryForcing.py:187-230"""
        nearest, support, _ = nearest_index_and_support(lag_position, self.dx, self.shift, self.width)
        wfn = cosine_weights if self.kernel == "cosine" else peskin_weights
        self.nearest = nearest
        self.weights = wfn(support, self.dx, self.real_t)
        self.lag_grid_flow_velocity_field[...] = interpolate(
            eul_velocity, self.weights, nearest, self.dx, self.width)
        self.lag_grid_velocity_mismatch_field[...] = self.lag_grid_flow_velocity_field - lag_velocity
        self.lag_grid_forcing_field[...] = (
            self.K * self.lag_grid_position_mismatch_field
            + self.C * self.lag_grid_velocity_mismatch_field)

    def compute_interaction_forcing(self, eul_forcing, eul_velocity, lag_position, lag_velocity):
        """VirtualBoundaryForcing.py:232-274 (optional reset, then spread)."""
        if self.reset:
            eul_forcing[...] = 0
        self.compute_interaction_force_on_lag_grid(eul_velocity, lag_position, lag_velocity)
        spread(eul_forcing, self.lag_grid_forcing_field, self.weights, self.nearest, self.width)

    def time_step(self, dt):
        """VirtualBoundaryForcing.py:276-283: xi += dt * dU."""
        self.lag_grid_position_mismatch_field[...] = (
            self.lag_grid_position_mismatch_field + dt * self.lag_grid_velocity_mismatch_field)
        self.time += dt
