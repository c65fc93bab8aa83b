"""The small contracts of the coupling API, after the reference's own tests.

``FlowForces.apply_forces`` adds the interactor's loads to a system
(tests/test_simulator/test_immersed_body/test_flow_forces.py), the
interaction's grid-resolution log (warning when the Lagrangian spacing is
above 2 dx or below dx / 2, info otherwise) and
``get_grid_deviation_error_l2_norm`` = ||xi|| / sqrt(n)
(test_immersed_body_flow_interaction.py).
"""

from __future__ import annotations

import logging

import numpy as np
import pytest

import sopht_gb300.simulator as sps


class _Interactor:
    def __init__(self) -> None:
        self.body_flow_forces = 0.0
        self.body_flow_torques = 0.0

    def compute_flow_forces_and_torques(self) -> None:
        self.body_flow_forces = 1.0
        self.body_flow_torques = 2.0


class _System:
    def __init__(self) -> None:
        self.external_forces = 3.0
        self.external_torques = 4.0


def test_flow_forces_adds_the_interactor_loads():
    interactor = _Interactor()
    forcing = sps.FlowForces(body_flow_interactor=interactor)
    assert forcing.body_flow_interactor is interactor
    system = _System()
    forcing.apply_forces(system=system)
    assert (system.external_forces, system.external_torques) == (4.0, 6.0)


def _cylinder_interactor(num_forcing_points):
    import torch
    grid = (16, 16)
    u = torch.from_numpy(np.random.default_rng(0).random((2, *grid))).cuda()
    f = torch.zeros_like(u)
    cyl = sps.Cylinder([0.5, 0.5, 0.0], base_radius=0.1, base_length=0.5)
    dx = 0.5 / 4.0  # the cylinder lies within the 16 x 16 grid
    inter = sps.RigidBodyFlowInteraction(
        rigid_body=cyl, eul_grid_forcing_field=f, eul_grid_velocity_field=u, virtual_boundary_stiffness_coeff=1.0,
        virtual_boundary_damping_coeff=1.0, dx=dx, grid_dim=2, real_t=np.float64,
        forcing_grid_cls=sps.CircularCylinderForcingGrid, num_forcing_points=num_forcing_points)
    return inter, dx


@pytest.mark.gpu
@pytest.mark.parametrize("num_forcing_points,level,words", [(1, logging.WARNING, "too coarse"),
                                                             (64, logging.WARNING, "redundant"),
                                                             (6, logging.INFO, "resolved")])
def test_grid_resolution_log(caplog, num_forcing_points, level, words):
    with caplog.at_level(logging.INFO, logger="sopht_gb300"):
        inter, dx = _cylinder_interactor(num_forcing_points)
    spacing = inter.forcing_grid.get_maximum_lagrangian_grid_spacing()
    assert spacing == pytest.approx(0.1 * 2 * np.pi / num_forcing_points)
    hits = [r for r in caplog.records if "CircularCylinderForcingGrid" in r.getMessage()]
    assert hits and hits[-1].levelno == level and words in hits[-1].getMessage()


@pytest.mark.gpu
def test_grid_deviation_error_l2_norm():
    inter, _ = _cylinder_interactor(16)
    inter.lag_grid_position_mismatch_field[...] = 2.0
    assert inter.get_grid_deviation_error_l2_norm() == pytest.approx(2.0 * np.sqrt(2))


def test_feedback_law_helpers_in_place():
    """VirtualBoundaryForcing's static helpers (VirtualBoundaryForcing.py:132-185) on host arrays."""
    from sopht_gb300.numeric.immersed_boundary_ops import VirtualBoundaryForcing as vbf
    rng = np.random.default_rng(4)
    u_flow, u_body, xi = (rng.standard_normal((3, 7)).astype(np.float32) for _ in range(3))
    du = np.empty_like(u_flow)
    vbf.compute_lag_grid_velocity_mismatch_field(du, u_flow, u_body)
    np.testing.assert_array_equal(du, u_flow - u_body)
    xi0 = xi.copy()
    vbf.update_lag_grid_position_mismatch_field_via_euler_forward(xi, du, 0.25)
    np.testing.assert_array_equal(xi, xi0 + np.float32(0.25) * du)
    f = np.empty_like(xi)
    vbf.compute_lag_grid_forcing_field(f, xi, du, -3.0, -0.5)
    np.testing.assert_array_equal(f, np.float32(-3.0) * xi + np.float32(-0.5) * du)
