"""Simulator-level oracle: the 2D/3D Navier-Stokes steps and body coupling.

Restates ``simulator/flow/navier_stokes_flow_simulators.py`` (step order and
prefactors), ``simulator/flow/flow_simulators.py:50-95`` (cell-centred grid),
``simulator/flow/passive_transport_flow_simulators.py:139-155`` (stable dt) and
the forcing grids / interaction of ``simulator/immersed_body``.  Test
infrastructure only.
"""

from __future__ import annotations

import numpy as np

from . import stencils as st
from .ib import VirtualBoundaryForcingOracle
from .poisson import UnboundedPoisson2D, UnboundedPoisson3D


def stable_timestep(velocity, grid_dim, dx, cfl, nu, real_t, dt_prefac=1.0):
    """passive_transport_flow_simulators.py:139-155 (times ``dt_prefac``)."""
    tol = 10 * np.finfo(real_t).eps
    umax = np.amax(np.sum(np.fabs(velocity), axis=0))
    dt = min(cfl * dx / (umax + tol), 0.9 * dx**2 / (2 * grid_dim) / nu + tol)
    return dt * dt_prefac


def position_field(grid_size, x_range, real_t):
    """flow_simulators.py:50-81: cell-centred coordinates, component 0 = x."""
    nx = grid_size[-1]
    dx = real_t(x_range / nx)
    shift = dx / 2.0
    axes = []
    for n in grid_size:
        extent = x_range * n / nx
        axes.append(np.linspace(shift, extent - shift, n).astype(real_t))
    return dx, np.flipud(np.array(np.meshgrid(*axes, indexing="ij")))


class NavierStokes2DOracle:
    """UnboundedNavierStokesFlowSimulator2D (navier_stokes_flow_simulators.py:24-223)."""

    def __init__(self, grid_size, x_range, kinematic_viscosity, cfl=0.1, real_t=np.float32,
                 time=0.0, with_forcing=False, with_free_stream_flow=False, flow_density=1.0,
                 penalty_zone_width=2, greens_dtype=None):
        self.grid_size = tuple(grid_size)
        self.x_range = x_range
        self.nu = kinematic_viscosity
        self.cfl = cfl
        self.real_t = real_t
        self.time = time
        self.with_forcing = with_forcing
        self.with_free_stream_flow = with_free_stream_flow
        self.rho = flow_density
        self.width = penalty_zone_width
        self.dx, self.position_field = position_field(self.grid_size, x_range, real_t)
        self.vorticity_field = np.zeros(self.grid_size, dtype=real_t)
        self.velocity_field = np.zeros((2, *self.grid_size), dtype=real_t)
        self.stream_func_field = np.zeros_like(self.vorticity_field)
        self.eul_grid_forcing_field = np.zeros_like(self.velocity_field)
        self.poisson = UnboundedPoisson2D(*self.grid_size, x_range=x_range, real_t=real_t,
                                          greens_dtype=greens_dtype)

    def compute_stable_timestep(self, dt_prefac=1.0):
        return stable_timestep(self.velocity_field, 2, self.dx, self.cfl, self.nu, self.real_t,
                               dt_prefac)

    def _ns_step(self, dt, free_stream_velocity):
        """navier_stokes_flow_simulators.py:171-198"""
        rt, dx = self.real_t, self.dx
        w = self.vorticity_field
        st.advection_step_2d(w, self.velocity_field, rt(dt / dx))
        st.diffusion_step_2d(w, rt(self.nu * dt / dx / dx))
        st.penalise_2d(w, self.width, dx, self.position_field[0], self.position_field[1])
        self.stream_func_field[...] = self.poisson.solve(w)
        st.outplane_curl_2d(self.stream_func_field, rt(0.5 / dx), out=self.velocity_field)
        if self.with_free_stream_flow:
            fs = np.asarray(free_stream_velocity)
            for c in range(2):
                self.velocity_field[c] = self.velocity_field[c] + fs[c]

    def time_step(self, dt, free_stream_velocity=(0.0, 0.0)):
        """navier_stokes_flow_simulators.py:200-209 plus flow_simulators.py:130-133."""
        if self.with_forcing:
            st.forcing_curl_update_2d(self.vorticity_field, self.eul_grid_forcing_field,
                                      self.real_t(dt / (2 * self.dx * self.rho)))
        self._ns_step(dt, free_stream_velocity)
        if self.with_forcing:
            self.eul_grid_forcing_field[...] = 0
        self.time += dt


class NavierStokes3DOracle:
    """UnboundedNavierStokesFlowSimulator3D (navier_stokes_flow_simulators.py:226-522)."""

    def __init__(self, grid_size, x_range, kinematic_viscosity, cfl=0.1, real_t=np.float32,
                 time=0.0, with_forcing=False, with_free_stream_flow=False, flow_density=1.0,
                 penalty_zone_width=2, filter_vorticity=False, filter_setting_dict=None,
                 greens_dtype=None):
        self.grid_size = tuple(grid_size)
        self.x_range = x_range
        self.nu = kinematic_viscosity
        self.cfl = cfl
        self.real_t = real_t
        self.time = time
        self.with_forcing = with_forcing
        self.with_free_stream_flow = with_free_stream_flow
        self.rho = flow_density
        self.width = penalty_zone_width
        self.filter = None
        if filter_vorticity:
            self.filter = filter_setting_dict or {"order": 2, "type": "multiplicative"}
        self.dx, self.position_field = position_field(self.grid_size, x_range, real_t)
        self.vorticity_field = np.zeros((3, *self.grid_size), dtype=real_t)
        self.velocity_field = np.zeros_like(self.vorticity_field)
        self.stream_func_field = np.zeros_like(self.vorticity_field)
        self.eul_grid_forcing_field = np.zeros_like(self.vorticity_field)
        self.poisson = UnboundedPoisson3D(*self.grid_size, x_range=x_range, real_t=real_t,
                                          greens_dtype=greens_dtype)

    def compute_stable_timestep(self, dt_prefac=1.0):
        return stable_timestep(self.velocity_field, 3, self.dx, self.cfl, self.nu, self.real_t,
                               dt_prefac)

    def get_vorticity_divergence_l2_norm(self):
        """navier_stokes_flow_simulators.py:514-522"""
        div = st.divergence_3d(self.vorticity_field, 1.0 / self.dx)
        return np.linalg.norm(div) * self.dx ** (3 / 2.0)

    def _ns_step(self, dt, free_stream_velocity):
        """navier_stokes_flow_simulators.py:449-485"""
        rt, dx = self.real_t, self.dx
        w = self.vorticity_field
        c = st.cross_3d(self.velocity_field, w)
        st.forcing_curl_update_3d(w, c, rt(dt / (2 * dx)))
        st.diffusion_step_3d(w, rt(self.nu * dt / dx / dx))
        if self.filter is not None:
            st.laplacian_filter_3d(w, self.filter["order"], self.filter["type"])
        p = self.position_field
        for comp in range(3):
            st.penalise_3d(w[comp], self.width, dx, p[0], p[1], p[2])
        self.stream_func_field[...] = self.poisson.vector_solve(w)
        st.curl_3d(self.stream_func_field, rt(0.5 / dx), out=self.velocity_field)
        if self.with_free_stream_flow:
            fs = np.asarray(free_stream_velocity)
            for comp in range(3):
                self.velocity_field[comp] = self.velocity_field[comp] + fs[comp]

    def time_step(self, dt, free_stream_velocity=(0.0, 0.0, 0.0)):
        """navier_stokes_flow_simulators.py:487-498"""
        if self.with_forcing:
            st.forcing_curl_update_3d(self.vorticity_field, self.eul_grid_forcing_field,
                                      self.real_t(dt / (2 * self.dx * self.rho)))
        self._ns_step(dt, free_stream_velocity)
        if self.with_forcing:
            self.eul_grid_forcing_field[...] = 0
        self.time += dt


class PassiveTransportOracle:
    """PassiveTransportFlowSimulator (passive_transport_flow_simulators.py:14-136).

    One step is the ENO3 advection step then the diffusion step of the primary
    field (:104-118); a 3D vector field is advected and diffused component by
    component.  The stable dt is passive_transport_flow_simulators.py:139-155.
    """

    def __init__(self, kinematic_viscosity, grid_dim, grid_size, x_range, cfl=0.1, real_t=np.float32,
                 time=0.0, field_type="scalar"):
        if field_type not in ("scalar", "vector"):
            raise ValueError("Invalid field type. Supported values include 'scalar' and 'vector'")
        if grid_dim == 2 and field_type == "vector":
            raise ValueError("Passive transport of vector 2D fields not supported yet.")
        self.nu = kinematic_viscosity
        self.grid_dim = grid_dim
        self.grid_size = tuple(grid_size)
        self.cfl = cfl
        self.real_t = real_t
        self.time = time
        self.field_type = field_type
        self.dx, self.position_field = position_field(self.grid_size, x_range, real_t)
        shape = self.grid_size if field_type == "scalar" else (grid_dim, *self.grid_size)
        self.primary_field = np.zeros(shape, dtype=real_t)
        self.velocity_field = np.zeros((grid_dim, *self.grid_size), dtype=real_t)

    def compute_stable_timestep(self, dt_prefac=1.0):
        return stable_timestep(self.velocity_field, self.grid_dim, self.dx, self.cfl, self.nu, self.real_t,
                               dt_prefac)

    def time_step(self, dt):
        rt, dx = self.real_t, self.dx
        dt_by_dx = rt(dt / dx)
        k = rt(self.nu * dt / dx / dx)
        if self.grid_dim == 2:
            st.advection_step_2d(self.primary_field, self.velocity_field, dt_by_dx)
            st.diffusion_step_2d(self.primary_field, k)
        else:
            comps = self.primary_field[None] if self.field_type == "scalar" else self.primary_field
            for c in range(comps.shape[0]):
                st.advection_step_3d(comps[c], self.velocity_field, dt_by_dx)
            st.diffusion_step_3d(comps, k)
        self.time += dt


# ---------------------------------------------------------------------------
# forcing grids and the interaction wrapper
# ---------------------------------------------------------------------------


class CircularCylinderOracle:
    """rigid_body/rigid_body_forcing_grids.py:11-105 for a cylinder in the XY plane."""

    def __init__(self, centre, radius, num_forcing_points, director=None, velocity=None,
                 omega_z=0.0):
        self.grid_dim = 2
        self.num_lag_nodes = num_forcing_points
        self.centre = np.asarray(centre, dtype=np.float64)
        self.radius = radius
        self.director = np.eye(3) if director is None else np.asarray(director)
        self.body_velocity = np.zeros(3) if velocity is None else np.asarray(velocity)
        self.omega_z = omega_z
        dtheta = 2.0 * np.pi / num_forcing_points
        theta = np.linspace(dtheta / 2.0, 2.0 * np.pi - dtheta / 2.0, num_forcing_points)
        self.local_rel = np.stack([radius * np.cos(theta), radius * np.sin(theta)])
        self.global_rel = np.zeros_like(self.local_rel)
        self.position_field = np.zeros((2, num_forcing_points))
        self.velocity_field = np.zeros_like(self.position_field)
        self.compute_lag_grid_position_field()
        self.compute_lag_grid_velocity_field()

    def compute_lag_grid_position_field(self):
        self.global_rel[...] = np.dot(self.director[:2, :2].T, self.local_rel)
        self.position_field[...] = self.centre[:2].reshape(2, 1) + self.global_rel

    def compute_lag_grid_velocity_field(self):
        wz = self.director[2, 2] * self.omega_z
        self.velocity_field[0] = self.body_velocity[0] - wz * self.global_rel[1]
        self.velocity_field[1] = self.body_velocity[1] + wz * self.global_rel[0]

    def transfer_forcing_from_grid_to_body(self, forces, torques, lag_forcing):
        forces[:2] = -np.sum(lag_forcing, axis=1).reshape(-1, 1)
        torques[2] = self.director[2, 2] * np.sum(
            -self.global_rel[0] * lag_forcing[1] + self.global_rel[1] * lag_forcing[0])

    def get_maximum_lagrangian_grid_spacing(self):
        return self.radius * (2.0 * np.pi / self.num_lag_nodes)


class RodNodalGridOracle:
    """cosserat_rod/cosserat_rod_forcing_grids.py:10-79 (markers at rod nodes)."""

    def __init__(self, rod, grid_dim=3):
        self.rod = rod
        self.grid_dim = grid_dim
        self.num_lag_nodes = rod.n_elems + 1
        self.position_field = np.zeros((grid_dim, self.num_lag_nodes))
        self.velocity_field = np.zeros_like(self.position_field)
        self.moment_arm = np.zeros((3, rod.n_elems))
        self.compute_lag_grid_position_field()
        self.compute_lag_grid_velocity_field()

    def compute_lag_grid_position_field(self):
        self.position_field[...] = self.rod.position_collection[: self.grid_dim]

    def compute_lag_grid_velocity_field(self):
        self.velocity_field[...] = self.rod.velocity_collection[: self.grid_dim]

    def transfer_forcing_from_grid_to_body(self, forces, torques, lag_forcing):
        forces[: self.grid_dim] = -lag_forcing
        pos = self.rod.position_collection
        self.moment_arm[...] = (pos[..., 1:] - pos[..., :-1]) / 2.0
        torques[...] = np.cross(self.moment_arm, (forces[..., 1:] - forces[..., :-1]) / 2.0, axis=0)
        torques[..., -1] += np.cross(self.moment_arm[..., -1], forces[..., -1]) / 2.0
        torques[..., 0] -= np.cross(self.moment_arm[..., 0], forces[..., 0]) / 2.0
        torques[...] = np.einsum("ijk,jk->ik", self.rod.director_collection, torques)

    def get_maximum_lagrangian_grid_spacing(self):
        return np.amax(self.rod.lengths)


class RodElementCentricGridOracle:
    """cosserat_rod/cosserat_rod_forcing_grids.py:82-130 (markers at element centres)."""

    def __init__(self, rod, grid_dim=3):
        self.rod = rod
        self.grid_dim = grid_dim
        self.num_lag_nodes = rod.n_elems
        self.position_field = np.zeros((grid_dim, self.num_lag_nodes))
        self.velocity_field = np.zeros_like(self.position_field)
        self.compute_lag_grid_position_field()
        self.compute_lag_grid_velocity_field()

    def compute_lag_grid_position_field(self):
        p = self.rod.position_collection
        self.position_field[...] = (p[: self.grid_dim, 1:] + p[: self.grid_dim, :-1]) / 2.0

    def compute_lag_grid_velocity_field(self):
        m, v = self.rod.mass, self.rod.velocity_collection
        # pyelastica _node_to_element_velocity: mass-weighted mean of the two nodes
        self.velocity_field[...] = ((m[1:] * v[:, 1:] + m[:-1] * v[:, :-1]) / (m[1:] + m[:-1]))[
            : self.grid_dim]

    def transfer_forcing_from_grid_to_body(self, forces, torques, lag_forcing):
        forces[...] = 0.0
        forces[: self.grid_dim, 1:] -= 0.5 * lag_forcing
        forces[: self.grid_dim, :-1] -= 0.5 * lag_forcing

    def get_maximum_lagrangian_grid_spacing(self):
        return np.amax(self.rod.lengths)


class ImmersedBodyInteractionOracle(VirtualBoundaryForcingOracle):
    """immersed_body_flow_interaction.py:15-141 (coefficient rescale, call order)."""

    def __init__(self, eul_grid_forcing_field, eul_grid_velocity_field, body_forces, body_torques,
                 forcing_grid, stiffness, damping, dx, grid_dim, real_t=np.float64,
                 enable_eul_grid_forcing_reset=False, kernel="cosine"):
        self.forcing_grid = forcing_grid
        self.eul_grid_forcing_field = eul_grid_forcing_field
        self.eul_grid_velocity_field = eul_grid_velocity_field
        self.body_flow_forces = body_forces
        self.body_flow_torques = body_torques
        h = forcing_grid.get_maximum_lagrangian_grid_spacing()
        stiffness *= h ** (grid_dim - 1)
        damping *= h ** (grid_dim - 1)
        super().__init__(stiffness, damping, grid_dim, dx, forcing_grid.num_lag_nodes, real_t,
                         enable_eul_grid_forcing_reset=enable_eul_grid_forcing_reset,
                         kernel=kernel)

    def __call__(self):
        self.forcing_grid.compute_lag_grid_position_field()
        self.forcing_grid.compute_lag_grid_velocity_field()
        self.compute_interaction_forcing(self.eul_grid_forcing_field, self.eul_grid_velocity_field,
                                         self.forcing_grid.position_field,
                                         self.forcing_grid.velocity_field)

    def compute_flow_forces_and_torques(self):
        self.forcing_grid.compute_lag_grid_position_field()
        self.forcing_grid.compute_lag_grid_velocity_field()
        self.compute_interaction_force_on_lag_grid(self.eul_grid_velocity_field,
                                                   self.forcing_grid.position_field,
                                                   self.forcing_grid.velocity_field)
        self.forcing_grid.transfer_forcing_from_grid_to_body(
            self.body_flow_forces, self.body_flow_torques, self.lag_grid_forcing_field)

    def get_grid_deviation_error_l2_norm(self):
        return np.linalg.norm(self.lag_grid_position_mismatch_field) / np.sqrt(
            self.forcing_grid.num_lag_nodes)
