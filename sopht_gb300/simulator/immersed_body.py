"""Immersed body - flow interaction (mirrors sopht/simulator/immersed_body).

The forcing grids stay on the host in float64 numpy, exactly as the reference
keeps them (they are pyelastica geometry); every interaction call uploads the
marker positions and velocities through pinned memory and runs the
GPU virtual-boundary forcing.  Body forces and torques come back to the host
for pyelastica (``compute_flow_forces_and_torques``).

``Cylinder`` and ``Sphere`` are small stand-ins carrying the attributes the
forcing grids read, for users without pyelastica; a real ``elastica.Cylinder``
/ ``elastica.Sphere`` works unchanged, and so does any rod object with
pyelastica's ``CosseratRod`` attributes (``position_collection``,
``velocity_collection``, ``omega_collection``, ``director_collection``,
``mass``, ``radius``, ``lengths``, ``tangents``, ``n_elems``).
"""

from __future__ import annotations

import logging
from abc import abstractmethod

import numpy as np
import torch

from .. import _lib
from ..numeric.immersed_boundary_ops import VirtualBoundaryForcing, _IBBinding
from ..utils import ptr, stream_ptr

logger = logging.getLogger(__name__)


# ------------------------------------------------------------ forcing grids


class ImmersedBodyForcingGrid:
    """immersed_body_forcing_grid.py:9-54."""

    def __init__(self, grid_dim: int, num_lag_nodes: int) -> None:
        self.grid_dim = grid_dim
        self.num_lag_nodes = num_lag_nodes
        self.position_field = np.zeros((self.grid_dim, self.num_lag_nodes))
        self.velocity_field = np.zeros_like(self.position_field)
        if grid_dim == 2:
            logger.warning("2D body forcing grid generated, this assumes the body moves in XY plane!")

    @abstractmethod
    def compute_lag_grid_position_field(self) -> None: ...

    @abstractmethod
    def compute_lag_grid_velocity_field(self) -> None: ...

    @abstractmethod
    def transfer_forcing_from_grid_to_body(self, body_flow_forces, body_flow_torques, lag_grid_forcing_field): ...

    @abstractmethod
    def get_maximum_lagrangian_grid_spacing(self) -> float: ...


class Cylinder:
    """Rigid cylinder with the attributes the forcing grids read (pyelastica layout).

    Stand-in for ``elastica.Cylinder`` when pyelastica is absent: position
    (3, 1), directors (3, 3, 1) with rows d1, d2, d3, velocity (3, 1), angular
    velocity in the local frame (3, 1) and radius.  ``direction`` is d3 and
    ``normal`` is d1, as pyelastica defines them.
    """

    def __init__(self, start, direction=(0.0, 0.0, 1.0), normal=(1.0, 0.0, 0.0), base_length=1.0,
                 base_radius=0.1, density=1.0):
        d3 = np.asarray(direction, dtype=np.float64)
        d1 = np.asarray(normal, dtype=np.float64)
        d2 = np.cross(d3, d1)
        self.position_collection = np.asarray(start, dtype=np.float64).reshape(3, 1).copy()
        self.director_collection = np.stack([d1, d2, d3]).reshape(3, 3, 1)
        self.velocity_collection = np.zeros((3, 1))
        self.omega_collection = np.zeros((3, 1))
        self.radius = base_radius
        self.length = base_length
        self.density = density


class TwoDimensionalCylinderForcingGrid(ImmersedBodyForcingGrid):
    """rigid_body_forcing_grids.py:11-79: markers on a cylinder in the XY plane."""

    def __init__(self, grid_dim: int, num_lag_nodes: int, rigid_body) -> None:
        if grid_dim != 2:
            raise ValueError("Invalid grid dimensions. 2D cylinder forcing grid is only defined for grid_dim=2")
        self.cylinder = rigid_body
        super().__init__(grid_dim, num_lag_nodes)
        self.local_frame_relative_position_field = np.zeros_like(self.position_field)
        self.global_frame_relative_position_field = np.zeros_like(self.position_field)

    def compute_lag_grid_position_field(self) -> None:
        q = self.cylinder.director_collection[: self.grid_dim, : self.grid_dim, 0]
        self.global_frame_relative_position_field[...] = q.T @ self.local_frame_relative_position_field
        self.position_field[...] = (self.cylinder.position_collection[: self.grid_dim]
                                    + self.global_frame_relative_position_field)

    def compute_lag_grid_velocity_field(self) -> None:
        # the angular velocity lies along d3 (global Z): v = V + omega_z e_z x r
        omega_z = (self.cylinder.director_collection[self.grid_dim, self.grid_dim, 0]
                   * self.cylinder.omega_collection[self.grid_dim, 0])
        rel = self.global_frame_relative_position_field
        self.velocity_field[0] = self.cylinder.velocity_collection[0] - omega_z * rel[1]
        self.velocity_field[1] = self.cylinder.velocity_collection[1] + omega_z * rel[0]

    def transfer_forcing_from_grid_to_body(self, body_flow_forces, body_flow_torques, lag_grid_forcing_field):
        f = np.asarray(lag_grid_forcing_field, dtype=np.float64)
        body_flow_forces[: self.grid_dim] = -np.sum(f, axis=1).reshape(-1, 1)
        rel = self.global_frame_relative_position_field
        body_flow_torques[self.grid_dim] = self.cylinder.director_collection[self.grid_dim, self.grid_dim, 0] * np.sum(
            -rel[0] * f[1] + rel[1] * f[0])

    def get_maximum_lagrangian_grid_spacing(self) -> float:
        raise NotImplementedError


class CircularCylinderForcingGrid(TwoDimensionalCylinderForcingGrid):
    """rigid_body_forcing_grids.py:82-105: markers at theta_k = (k + 1/2) 2 pi / N."""

    def __init__(self, grid_dim: int, rigid_body, num_forcing_points: int) -> None:
        super().__init__(grid_dim=grid_dim, num_lag_nodes=num_forcing_points, rigid_body=rigid_body)
        dtheta = 2.0 * np.pi / self.num_lag_nodes
        theta = np.linspace(dtheta / 2.0, 2.0 * np.pi - dtheta / 2.0, self.num_lag_nodes)
        self.local_frame_relative_position_field[0, :] = self.cylinder.radius * np.cos(theta)
        self.local_frame_relative_position_field[1, :] = self.cylinder.radius * np.sin(theta)
        self.compute_lag_grid_position_field()
        self.compute_lag_grid_velocity_field()

    def get_maximum_lagrangian_grid_spacing(self) -> float:
        return self.cylinder.radius * (2.0 * np.pi / self.num_lag_nodes)


class Sphere:
    """Rigid sphere with the attributes the forcing grids read (pyelastica layout).

    Stand-in for ``elastica.Sphere`` when pyelastica is absent: centre (3, 1),
    identity directors (3, 3, 1), velocity and local-frame angular velocity
    (3, 1), radius."""

    def __init__(self, center, base_radius, density=1.0):
        self.position_collection = np.asarray(center, dtype=np.float64).reshape(3, 1).copy()
        self.director_collection = np.eye(3).reshape(3, 3, 1)
        self.velocity_collection = np.zeros((3, 1))
        self.omega_collection = np.zeros((3, 1))
        self.radius = base_radius
        self.density = density


try:  # the plane is a pyelastica rigid body when pyelastica is installed
    from elastica import RigidBodyBase as _RigidBodyBase  # type: ignore
except Exception:  # pragma: no cover - pyelastica absent
    class _RigidBodyBase:  # minimal stand-in of elastica.RigidBodyBase
        def __init__(self) -> None:
            pass


class RectangularPlane(_RigidBodyBase):
    """rigid_body/derived_rigid_bodies.py:12-63: a rigid rectangle for imposed motions.

    Directors (rows): d1 the unit tangent along the length, d2 the unit
    normal x tangent, d3 the unit normal.  One element, centred at ``origin``,
    at rest.  Pyelastica cannot integrate its dynamics; move it by setting its
    position, director, velocity and omega collections."""

    def __init__(self, origin, plane_normal, plane_tangent_along_length, plane_length, plane_breadth) -> None:
        super().__init__()
        logger.warning("Initialising a rectangular plane: pyelastica cannot track its dynamics, so do not add "
                       "the plane to a pyelastica simulator (it supports imposed motions only).")
        self.n_elems = 1
        self.length = plane_length
        self.breadth = plane_breadth
        normal = np.asarray(plane_normal, dtype=np.float64).reshape(3)
        tangent = np.asarray(plane_tangent_along_length, dtype=np.float64).reshape(3)
        binormal = np.cross(normal, tangent)
        self.director_collection = np.zeros((3, 3, 1))
        for row, v in enumerate((tangent, binormal, normal)):
            self.director_collection[row, :, 0] = v / np.linalg.norm(v)
        self.position_collection = np.asarray(origin, dtype=np.float64).reshape(3, 1).copy()
        self.velocity_collection = np.zeros((3, 1))
        self.omega_collection = np.zeros((3, 1))


class ThreeDimensionalRigidBodyForcingGrid(ImmersedBodyForcingGrid):
    """rigid_body_forcing_grids.py:108-178: markers fixed in a 3D rigid body's frame.

    With Q the body's directors (rows d1, d2, d3) and l_k a marker's offset in
    the body frame: position x + Q^T l_k, velocity V + (Q^T omega) x (Q^T l_k);
    the body takes the force -sum F_k and the body-frame torque
    -Q sum_k (Q^T l_k) x F_k (Newton's third law)."""

    def __init__(self, grid_dim: int, num_lag_nodes: int, rigid_body) -> None:
        if grid_dim != 3:
            raise ValueError("Invalid grid dimensions. 3D Rigid body forcing grid is only defined for grid_dim=3")
        self.rigid_body = rigid_body
        super().__init__(grid_dim, num_lag_nodes)
        self.local_frame_relative_position_field = np.zeros_like(self.position_field)
        self.global_frame_relative_position_field = np.zeros_like(self.position_field)

    def compute_lag_grid_position_field(self) -> None:
        q = self.rigid_body.director_collection[:, :, 0]
        self.global_frame_relative_position_field[...] = q.T @ self.local_frame_relative_position_field
        self.position_field[...] = self.rigid_body.position_collection + self.global_frame_relative_position_field

    def compute_lag_grid_velocity_field(self) -> None:
        omega = self.rigid_body.director_collection[:, :, 0].T @ self.rigid_body.omega_collection
        self.velocity_field[...] = self.rigid_body.velocity_collection + np.cross(
            omega, self.global_frame_relative_position_field, axis=0)

    def transfer_forcing_from_grid_to_body(self, body_flow_forces, body_flow_torques, lag_grid_forcing_field):
        f = np.asarray(lag_grid_forcing_field, dtype=np.float64)
        body_flow_forces[...] = -np.sum(f, axis=1).reshape(-1, 1)
        arm_sum = np.sum(np.cross(self.global_frame_relative_position_field, f, axis=0), axis=1)
        body_flow_torques[...] = -(self.rigid_body.director_collection[:, :, 0] @ arm_sum).reshape(-1, 1)

    def get_maximum_lagrangian_grid_spacing(self) -> float:
        raise NotImplementedError


class OpenEndCircularCylinderForcingGrid(ThreeDimensionalRigidBodyForcingGrid):
    """rigid_body_forcing_grids.py:181-238: a 3D cylinder's side wall, no end caps.

    ``num_forcing_points_along_length`` rings, evenly spaced from -L/2 to L/2
    along d3, each with ceil(n_length * 2 pi R / L) markers at
    theta_j = (j + 1/2) 2 pi / n (the same marker density around as along)."""

    def __init__(self, grid_dim: int, rigid_body, num_forcing_points_along_length: int) -> None:
        self.num_forcing_points_along_length = n_len = num_forcing_points_along_length
        circumference = 2 * np.pi * rigid_body.radius
        self.num_forcing_points_along_circumference = n_circ = int(
            np.ceil(n_len * circumference / rigid_body.length))
        super().__init__(grid_dim=grid_dim, num_lag_nodes=n_len * n_circ, rigid_body=rigid_body)
        dtheta = 2.0 * np.pi / n_circ
        theta = np.linspace(dtheta / 2.0, 2.0 * np.pi - dtheta / 2.0, n_circ)
        along = np.linspace(-0.5 * rigid_body.length, 0.5 * rigid_body.length, n_len)
        local = self.local_frame_relative_position_field  # ring after ring
        local[0] = np.tile(rigid_body.radius * np.cos(theta), n_len)
        local[1] = np.tile(rigid_body.radius * np.sin(theta), n_len)
        local[2] = np.repeat(along, n_circ)
        self.compute_lag_grid_position_field()
        self.compute_lag_grid_velocity_field()

    def get_maximum_lagrangian_grid_spacing(self) -> float:
        return max(self.rigid_body.radius * (2.0 * np.pi / self.num_forcing_points_along_circumference),
                   self.rigid_body.length / self.num_forcing_points_along_length)


class SphereForcingGrid(ThreeDimensionalRigidBodyForcingGrid):
    """rigid_body_forcing_grids.py:241-304: latitude rings on a sphere.

    n_eq // 2 polar angles evenly from 0 to pi; the ring at polar angle phi
    holds rint(n_eq sin phi) + 1 markers at azimuths evenly from 0 (the poles
    hold one).  The offsets are laid out in the global frame directly (a
    sphere's rotation does not move its surface)."""

    def __init__(self, grid_dim: int, rigid_body, num_forcing_points_along_equator: int) -> None:
        self.num_forcing_points_along_equator = n_eq = num_forcing_points_along_equator
        polar = np.linspace(0, np.pi, n_eq // 2)
        ring = np.rint(n_eq * np.sin(polar)).astype(int) + 1
        super().__init__(grid_dim=grid_dim, num_lag_nodes=int(ring.sum()), rigid_body=rigid_body)
        phi = np.repeat(polar, ring)
        azimuth = np.concatenate([np.linspace(0.0, 2 * np.pi, k, endpoint=False) for k in ring] or [np.empty(0)])
        r = rigid_body.radius
        rel = self.global_frame_relative_position_field
        rel[0] = r * np.sin(phi) * np.cos(azimuth)
        rel[1] = r * np.sin(phi) * np.sin(azimuth)
        rel[2] = r * np.cos(phi)
        self.compute_lag_grid_position_field()
        self.compute_lag_grid_velocity_field()

    def compute_lag_grid_position_field(self) -> None:
        self.position_field[...] = self.rigid_body.position_collection + self.global_frame_relative_position_field

    def get_maximum_lagrangian_grid_spacing(self) -> float:
        return self.rigid_body.radius * (2 * np.pi / self.num_forcing_points_along_equator)


class RectangularPlaneForcingGrid(ThreeDimensionalRigidBodyForcingGrid):
    """rigid_body_forcing_grids.py:307-349: a lattice on a rectangular plane.

    n_length points evenly from -L/2 to L/2 along d1 by int(n_length B / L)
    from -B/2 to B/2 along d2 (length index fastest), in the plane d3 = 0."""

    def __init__(self, grid_dim: int, rigid_body, num_forcing_points_along_length: int) -> None:
        self.num_forcing_points_along_length = n_len = num_forcing_points_along_length
        self.num_forcing_points_along_breadth = n_br = int(n_len * rigid_body.breadth / rigid_body.length)
        self.grid_spacing = rigid_body.length / n_len
        super().__init__(grid_dim=grid_dim, num_lag_nodes=n_len * n_br, rigid_body=rigid_body)
        along_length = np.linspace(-0.5 * rigid_body.length, 0.5 * rigid_body.length, n_len)
        along_breadth = np.linspace(-0.5 * rigid_body.breadth, 0.5 * rigid_body.breadth, n_br)
        local = self.local_frame_relative_position_field
        local[0] = np.tile(along_length, n_br)
        local[1] = np.repeat(along_breadth, n_len)
        local[2] = 0.0
        self.compute_lag_grid_position_field()
        self.compute_lag_grid_velocity_field()

    def get_maximum_lagrangian_grid_spacing(self) -> float:
        return self.grid_spacing


def _node_to_element_velocity(mass, node_velocity):
    """Element velocity as the mass-weighted mean of its two nodes (pyelastica)."""
    return (mass[1:] * node_velocity[:, 1:] + mass[:-1] * node_velocity[:, :-1]) / (mass[1:] + mass[:-1])


class CosseratRodNodalForcingGrid(ImmersedBodyForcingGrid):
    """cosserat_rod_forcing_grids.py:10-79: markers at the rod nodes."""

    def __init__(self, grid_dim: int, cosserat_rod) -> None:
        super().__init__(grid_dim, cosserat_rod.n_elems + 1)
        self.cosserat_rod = cosserat_rod
        self.moment_arm = np.zeros((3, cosserat_rod.n_elems))
        self.compute_lag_grid_position_field()
        self.compute_lag_grid_velocity_field()

    def compute_lag_grid_position_field(self) -> None:
        self.position_field[...] = self.cosserat_rod.position_collection[: self.grid_dim]

    def compute_lag_grid_velocity_field(self) -> None:
        self.velocity_field[...] = self.cosserat_rod.velocity_collection[: self.grid_dim]

    def transfer_forcing_from_grid_to_body(self, body_flow_forces, body_flow_torques, lag_grid_forcing_field):
        body_flow_forces[: self.grid_dim] = -np.asarray(lag_grid_forcing_field, dtype=np.float64)
        pos = self.cosserat_rod.position_collection
        self.moment_arm[...] = (pos[..., 1:] - pos[..., :-1]) / 2.0
        body_flow_torques[...] = np.cross(self.moment_arm, (body_flow_forces[..., 1:] - body_flow_forces[..., :-1])
                                          / 2.0, axis=0)
        body_flow_torques[..., -1] += np.cross(self.moment_arm[..., -1], body_flow_forces[..., -1]) / 2.0
        body_flow_torques[..., 0] -= np.cross(self.moment_arm[..., 0], body_flow_forces[..., 0]) / 2.0
        body_flow_torques[...] = np.einsum("ijk,jk->ik", self.cosserat_rod.director_collection, body_flow_torques)

    def get_maximum_lagrangian_grid_spacing(self) -> float:
        return np.amax(self.cosserat_rod.lengths)


class CosseratRodElementCentricForcingGrid(ImmersedBodyForcingGrid):
    """cosserat_rod_forcing_grids.py:82-130: markers at element centres."""

    def __init__(self, grid_dim: int, cosserat_rod) -> None:
        super().__init__(grid_dim, cosserat_rod.n_elems)
        self.cosserat_rod = cosserat_rod
        self.compute_lag_grid_position_field()
        self.compute_lag_grid_velocity_field()

    def compute_lag_grid_position_field(self) -> None:
        p = self.cosserat_rod.position_collection
        self.position_field[...] = (p[: self.grid_dim, 1:] + p[: self.grid_dim, :-1]) / 2.0

    def compute_lag_grid_velocity_field(self) -> None:
        self.velocity_field[...] = _node_to_element_velocity(self.cosserat_rod.mass,
                                                             self.cosserat_rod.velocity_collection)[: self.grid_dim]

    def transfer_forcing_from_grid_to_body(self, body_flow_forces, body_flow_torques, lag_grid_forcing_field):
        f = np.asarray(lag_grid_forcing_field, dtype=np.float64)
        body_flow_forces[...] = 0.0
        body_flow_forces[: self.grid_dim, 1:] -= 0.5 * f
        body_flow_forces[: self.grid_dim, :-1] -= 0.5 * f

    def get_maximum_lagrangian_grid_spacing(self) -> float:
        return np.amax(self.cosserat_rod.lengths)


def _global_frame(directors, local_vectors):
    """Q^T v per element (directors (3, 3, n), rows d1, d2, d3; vectors (3, n))."""
    return np.einsum("jik,jk->ik", directors, local_vectors)


def _local_frame(directors, global_vectors):
    """Q v per element."""
    return np.einsum("ijk,jk->ik", directors, global_vectors)


def _elements_to_nodes(element_vectors, node_vectors) -> None:
    """Half of each element's vector to each of its two nodes, in place (pyelastica's
    ``_elements_to_nodes_inplace``: node k receives element k-1's half, then element k's)."""
    half = 0.5 * element_vectors
    node_vectors[..., 1:] += half
    node_vectors[..., :-1] += half


class CosseratRodEdgeForcingGrid(ImmersedBodyForcingGrid):
    """cosserat_rod_forcing_grids.py:134-283: element centres plus two edge points (2D).

    For tapered or thick rods in the XY plane: markers at the n element
    centres, then the n left edges x_e + r n_e, then the n right edges
    x_e - r n_e, with n_e = e_z x t_e (t_e the element tangent, r its radius).
    The edge velocities add (Q^T omega) x (+/- r n_e).  The centre forcing
    goes half to each node; the edge forcing gives the element torque
    (+/- r n_e) x (-F) and is then split half to each node; torques are
    returned in the element frames."""

    def __init__(self, grid_dim: int, cosserat_rod) -> None:
        if grid_dim != 2:
            raise ValueError("Invalid grid dimensions. Cosserat rod edge forcing grid is only defined for grid_dim=2")
        self.cosserat_rod = cosserat_rod
        n = cosserat_rod.n_elems
        super().__init__(grid_dim, 3 * n)
        self.z_vector = np.repeat(np.array([0.0, 0.0, 1.0]).reshape(3, 1), n, axis=-1)
        self.moment_arm = np.zeros((3, n))
        self.start_idx_elems, self.end_idx_elems = 0, n
        self.start_idx_left_edge_nodes, self.end_idx_left_edge_nodes = n, 2 * n
        self.start_idx_right_edge_nodes, self.end_idx_right_edge_nodes = 2 * n, 3 * n
        self.element_forces_left_edge_nodes = np.zeros((3, n))
        self.element_forces_right_edge_nodes = np.zeros((3, n))
        self.compute_lag_grid_position_field()
        self.compute_lag_grid_velocity_field()

    def compute_lag_grid_position_field(self) -> None:
        rod, n, d = self.cosserat_rod, self.cosserat_rod.n_elems, self.grid_dim
        p = rod.position_collection
        centre = 0.5 * (p[..., 1:] + p[..., :-1])
        self.moment_arm[...] = np.cross(self.z_vector, rod.tangents, axis=0) * rod.radius
        self.position_field[:, :n] = centre[:d]
        self.position_field[:, n:2 * n] = (centre + self.moment_arm)[:d]
        self.position_field[:, 2 * n:] = (centre - self.moment_arm)[:d]

    def compute_lag_grid_velocity_field(self) -> None:
        rod, n, d = self.cosserat_rod, self.cosserat_rod.n_elems, self.grid_dim
        v = _node_to_element_velocity(rod.mass, rod.velocity_collection)
        swirl = np.cross(_global_frame(rod.director_collection, rod.omega_collection), self.moment_arm, axis=0)
        self.velocity_field[:, :n] = v[:d]
        self.velocity_field[:, n:2 * n] = (v + swirl)[:d]
        self.velocity_field[:, 2 * n:] = (v - swirl)[:d]

    def transfer_forcing_from_grid_to_body(self, body_flow_forces, body_flow_torques, lag_grid_forcing_field):
        f = np.asarray(lag_grid_forcing_field, dtype=np.float64)
        n, d = self.cosserat_rod.n_elems, self.grid_dim
        body_flow_forces[...] = 0.0
        body_flow_forces[:d, 1:] -= 0.5 * f[:, :n]
        body_flow_forces[:d, :-1] -= 0.5 * f[:, :n]
        left, right = self.element_forces_left_edge_nodes, self.element_forces_right_edge_nodes
        left[:d] = -f[:, n:2 * n]
        right[:d] = -f[:, 2 * n:]
        torque = np.cross(self.moment_arm, left, axis=0) + np.cross(-self.moment_arm, right, axis=0)
        _elements_to_nodes(left + right, body_flow_forces)
        body_flow_torques[...] = _local_frame(self.cosserat_rod.director_collection, torque)

    def get_maximum_lagrangian_grid_spacing(self) -> float:
        return np.amax(self.cosserat_rod.lengths)


class CosseratRodSurfaceForcingGrid(ImmersedBodyForcingGrid):
    """cosserat_rod_forcing_grids.py:286-589: rings of markers on a 3D rod's surface.

    Element i carries rint(r_i / r_max * density) markers on its surface
    circle at angles evenly from 0 in its (d1, d2) plane, or a single marker
    at its centre when that count is below 3.  With ``with_cap`` each end
    element (if it has a ring) also gets concentric inner rings: k =
    max(int(r // (r 2 pi / n)), 1) rings at radii j r / k (j < k) holding
    int(1 + j (n - 1) / k) markers (numpy's linspace(1, n, k) truncated), placed
    after the outer ring in that element's slice.  Each marker is x_e + m,
    m = rho Q_e^T (cos a, sin a, 0); it moves with v_e + (Q_e^T omega_e) x m.
    An element's forcing goes half to each node; its torque Q_e sum m x (-F)
    is returned in the element frame."""

    def __init__(self, grid_dim: int, cosserat_rod, surface_grid_density_for_largest_element: int,
                 with_cap: bool = False) -> None:
        if grid_dim != 3:
            raise ValueError("Invalid grid dimensions. Cosserat rod surface forcing grid is only defined for "
                             "grid_dim=3")
        self.cosserat_rod = cosserat_rod
        self.n_elems = n = cosserat_rod.n_elems
        self.surface_grid_density_for_largest_element = density = surface_grid_density_for_largest_element
        self.with_cap = with_cap
        radius = np.asarray(cosserat_rod.radius, dtype=np.float64)
        counts = np.rint(radius / np.max(radius) * density).astype(int)
        counts[counts < 3] = 1
        ratios = [np.ones(c) for c in counts]
        angles = [np.linspace(0, 2 * np.pi, c, endpoint=False) if c > 1 else np.array([]) for c in counts]
        if with_cap:
            for end in (0, n - 1):  # the two ends in turn (the same element twice for a one-element rod)
                c, r = int(counts[end]), radius[end]
                rings = max(int(r // (r * (2.0 * np.pi / c))), 1) if c > 1 else 0
                ring_points = np.linspace(1, c, rings, endpoint=False).astype(int)
                ring_ratio = np.linspace(0, r, rings, endpoint=False) / r
                counts[end] = c + ring_points.sum()
                ratios[end] = np.concatenate([ratios[end], np.repeat(ring_ratio, ring_points)])
                if counts[end] > 1:
                    angles[end] = np.concatenate([np.linspace(0, 2 * np.pi, c, endpoint=False)]
                                                 + [np.linspace(0, 2 * np.pi, k, endpoint=False)
                                                    for k in ring_points])
        self.surface_grid_points = counts
        self.surface_point_rotation_angle_list = angles
        self.grid_point_radius_ratio = np.concatenate(ratios)
        super().__init__(grid_dim, int(counts.sum()))
        self.end_idx = np.cumsum(counts)
        self.start_idx = self.end_idx - counts
        self._point_element = np.repeat(np.arange(n), counts)
        self.moment_arm = np.zeros_like(self.position_field)
        self.local_frame_surface_points = np.zeros_like(self.position_field)
        for i, a in enumerate(angles):
            if a.size:
                self.local_frame_surface_points[0, self.start_idx[i]:self.end_idx[i]] = np.cos(a)
                self.local_frame_surface_points[1, self.start_idx[i]:self.end_idx[i]] = np.sin(a)
        self.rod_director_collection_transpose = np.zeros_like(cosserat_rod.director_collection)
        self.rod_element_position = np.zeros((self.grid_dim, n))
        self.rod_element_velocity = np.zeros_like(self.rod_element_position)
        self.rod_element_global_frame_omega = np.zeros_like(self.rod_element_position)
        self.grid_point_director_transpose = np.zeros((3, 3, self.num_lag_nodes))
        self.grid_point_radius = np.zeros(self.num_lag_nodes)
        self.grid_point_omega = np.zeros_like(self.position_field)
        self.lag_grid_torque_field = np.zeros_like(self.position_field)
        self.compute_lag_grid_position_field()
        self.compute_lag_grid_velocity_field()

    def compute_lag_grid_position_field(self) -> None:
        rod, e = self.cosserat_rod, self._point_element
        p = rod.position_collection
        self.rod_element_position[...] = 0.5 * (p[..., 1:] + p[..., :-1])
        self.rod_director_collection_transpose[...] = np.transpose(rod.director_collection, (1, 0, 2))
        self.grid_point_director_transpose[...] = self.rod_director_collection_transpose[:, :, e]
        self.grid_point_radius[...] = np.asarray(rod.radius)[e] * self.grid_point_radius_ratio
        self.moment_arm[...] = self.grid_point_radius * np.einsum(
            "ijk,jk->ik", self.grid_point_director_transpose, self.local_frame_surface_points)
        self.position_field[...] = self.rod_element_position[:, e] + self.moment_arm

    def compute_lag_grid_velocity_field(self) -> None:
        rod, e = self.cosserat_rod, self._point_element
        self.rod_element_velocity[...] = _node_to_element_velocity(rod.mass, rod.velocity_collection)
        self.rod_element_global_frame_omega[...] = np.einsum(
            "ijk,jk->ik", self.rod_director_collection_transpose, rod.omega_collection)
        self.grid_point_omega[...] = self.rod_element_global_frame_omega[:, e]
        self.velocity_field[...] = self.rod_element_velocity[:, e] + np.cross(
            self.grid_point_omega, self.moment_arm, axis=0)

    def transfer_forcing_from_grid_to_body(self, body_flow_forces, body_flow_torques, lag_grid_forcing_field):
        f = np.asarray(lag_grid_forcing_field, dtype=np.float64)
        per_element = np.add.reduceat(f, self.start_idx, axis=1)
        body_flow_forces[...] = 0.0
        body_flow_forces[:, 1:] -= 0.5 * per_element
        body_flow_forces[:, :-1] -= 0.5 * per_element
        self.lag_grid_torque_field[...] = np.cross(self.moment_arm, -f, axis=0)
        body_flow_torques[...] = _local_frame(self.cosserat_rod.director_collection,
                                              np.add.reduceat(self.lag_grid_torque_field, self.start_idx, axis=1))

    def get_maximum_lagrangian_grid_spacing(self) -> float:
        grid_angular_spacing = 2 * np.pi / self.surface_grid_density_for_largest_element
        return np.amax([self.cosserat_rod.lengths, self.cosserat_rod.radius * grid_angular_spacing])


# ----------------------------------------------------------------- interaction


class ImmersedBodyFlowInteraction(VirtualBoundaryForcing):
    """immersed_body_flow_interaction.py:15-141."""

    def __init__(self, eul_grid_forcing_field, eul_grid_velocity_field, body_flow_forces, body_flow_torques,
                 forcing_grid_cls, virtual_boundary_stiffness_coeff, virtual_boundary_damping_coeff, dx, grid_dim,
                 real_t=np.float64, eul_grid_coord_shift=None, interp_kernel_width=None,
                 enable_eul_grid_forcing_reset=False, num_threads=False, start_time=0.0, **forcing_grid_kwargs):
        self.body_flow_forces = body_flow_forces
        self.body_flow_torques = body_flow_torques
        interp_kernel_type = forcing_grid_kwargs.pop("interp_kernel_type", "cosine")
        self.forcing_grid = forcing_grid_cls(grid_dim=grid_dim, **forcing_grid_kwargs)
        if not isinstance(eul_grid_forcing_field, torch.Tensor) or not eul_grid_forcing_field.is_cuda:
            raise ValueError("eul_grid_forcing_field must be the simulator's CUDA tensor")
        self.eul_grid_forcing_field = eul_grid_forcing_field
        self.eul_grid_velocity_field = eul_grid_velocity_field
        max_lag_grid_dx = self.forcing_grid.get_maximum_lagrangian_grid_spacing()
        grid_type = type(self.forcing_grid).__name__
        if max_lag_grid_dx > 2 * dx:
            logger.warning("For %s: max Lagrangian grid spacing %s > 2 * dx (%s); the Lagrangian grid is too "
                           "coarse relative to the Eulerian grid.", grid_type, max_lag_grid_dx, dx)
        elif max_lag_grid_dx < 0.5 * dx:
            logger.warning("For %s: max Lagrangian grid spacing %s < 0.5 * dx (%s); redundant forcing points.",
                           grid_type, max_lag_grid_dx, dx)
        else:
            logger.info("For %s: Lagrangian grid is resolved almost the same as the Eulerian grid (dx = %s).",
                        grid_type, dx)
        # immersed_body_flow_interaction.py:83-86
        virtual_boundary_stiffness_coeff *= max_lag_grid_dx ** (grid_dim - 1)
        virtual_boundary_damping_coeff *= max_lag_grid_dx ** (grid_dim - 1)
        super().__init__(virtual_boundary_stiffness_coeff, virtual_boundary_damping_coeff, grid_dim, dx,
                         self.forcing_grid.num_lag_nodes, real_t, eul_grid_coord_shift, interp_kernel_width,
                         enable_eul_grid_forcing_reset, num_threads, start_time,
                         interp_kernel_type=interp_kernel_type, device=eul_grid_forcing_field.device)
        self._host_forcing = torch.empty(self.lag_grid_forcing_field.shape, dtype=self.lag_grid_forcing_field.dtype,
                                         pin_memory=True)
        # early copy of the Lagrangian forcing, taken right after the interaction of ``__call__`` once a
        # caller has read it: a later read waits for that copy only, not for the rest of the step
        self._snapshot_wanted = False
        self._snapshot_key = None
        self._snapshot_src = None
        self._snapshot_event = torch.cuda.Event()
        self._binding = None
        self._rod_args_cache = None

    def compute_interaction_on_lag_grid(self) -> None:
        self.forcing_grid.compute_lag_grid_position_field()
        self.forcing_grid.compute_lag_grid_velocity_field()
        self.compute_interaction_force_on_lag_grid(self.eul_grid_velocity_field, self.forcing_grid.position_field,
                                                   self.forcing_grid.velocity_field)

    def __call__(self) -> None:
        fg = self.forcing_grid
        b = self._bound(fg)
        rod = self._rod_kinematics_args(fg) if b is not None else None
        if rod is None:
            fg.compute_lag_grid_position_field()
            fg.compute_lag_grid_velocity_field()
        if b is None:
            self.compute_interaction_forcing(eul_grid_forcing_field=self.eul_grid_forcing_field,
                                             eul_grid_velocity_field=self.eul_grid_velocity_field,
                                             lag_grid_position_field=fg.position_field,
                                             lag_grid_velocity_field=fg.velocity_field)
            if self._snapshot_wanted:
                self._host_forcing.copy_(self.lag_grid_forcing_field, non_blocking=True)
                if torch.cuda.current_device() == self.device.index:
                    self._snapshot_event.record()
                else:  # the copy ran on the forcing field's device
                    self._snapshot_event.record(torch.cuda.current_stream(self.device))
                self._snapshot_key = (self._n_interactions, self.lag_grid_forcing_field._version)
                self._snapshot_src = None
            return
        # one native call: kinematics upload, interaction (with a deferred time_step), spreading, and the
        # early copy of the Lagrangian forcing once a caller reads it
        if rod is None:
            slot = b.stage(fg.position_field, fg.velocity_field)
        else:  # the grid's kinematics computed natively, into its arrays and the staging slot at once
            slot = b.next_slot()
            _lib.call("sg_rod_element_kinematics", *rod, b.kin_ptr[slot])
        pending = self._pending_xi_dt
        self._pending_xi_dt = None
        self._n_interactions += 1
        snap = self._snapshot_wanted
        _lib.call("sg_ib_bound_step", b.handle, slot, ptr(self.eul_grid_velocity_field),
                  ptr(self.eul_grid_forcing_field), 1 if self.enable_eul_grid_forcing_reset else 0,
                  float(self.virtual_boundary_stiffness_coeff), float(self.virtual_boundary_damping_coeff),
                  0 if pending is None else 1, 0.0 if pending is None else pending, 1 if snap else 0,
                  stream_ptr(self.device))
        if snap:
            self._snapshot_key = (self._n_interactions, self.lag_grid_forcing_field._version)
            self._snapshot_src = b

    def _rod_kinematics_args(self, fg):
        """Arguments of ``sg_rod_element_kinematics`` for an element-centric rod grid (exactly that
        class, so overridden kinematics keep running), or None where numpy computes them.  Cached by
        array identity: pyelastica updates the rod arrays in place."""
        if type(fg) is not CosseratRodElementCentricForcingGrid:
            return None
        rod = fg.cosserat_rod
        arrays = (rod.position_collection, rod.velocity_collection, rod.mass, fg.position_field, fg.velocity_field)
        c = self._rod_args_cache
        if c is not None and all(x is y for x, y in zip(c[0], arrays)):
            return c[1]
        self._rod_args_cache = None
        p, v, m, po, vo = arrays
        n = fg.num_lag_nodes
        dim = fg.grid_dim
        if not all(isinstance(a, np.ndarray) and a.dtype == np.float64 for a in arrays):
            return None
        if (p.shape != (3, n + 1) or v.shape != (3, n + 1) or m.shape != (n + 1,) or po.shape != (dim, n)
                or vo.shape != (dim, n)):
            return None
        if not (p.strides[1] == 8 and v.strides[1] == 8 and p.strides[0] % 8 == 0 and v.strides[0] % 8 == 0
                and p.strides[0] >= 8 * (n + 1) and v.strides[0] >= 8 * (n + 1)
                and m.flags.c_contiguous and po.flags.c_contiguous and vo.flags.c_contiguous):
            return None
        args = (dim, n, p.ctypes.data, p.strides[0] // 8, v.ctypes.data, v.strides[0] // 8, m.ctypes.data,
                po.ctypes.data, vo.ctypes.data)
        self._rod_args_cache = (arrays, args)
        return args

    def _bound(self, fg):
        """The native binding of this interactor's buffers, or None where the generic path applies
        (kinematics that are not host arrays, an Eulerian field of another dtype or layout)."""
        if not (isinstance(fg.position_field, np.ndarray) and isinstance(fg.velocity_field, np.ndarray)):
            return None
        u, f = self.eul_grid_velocity_field, self.eul_grid_forcing_field
        key = (self.nearest_eul_grid_index_to_lag_grid, self.interp_weights, self.lag_grid_flow_velocity_field,
               self._du, self._xi, self.lag_grid_forcing_field, self._status, u, f)
        b = self._binding
        if b is not None and all(x is y for x, y in zip(b.key, key)):
            return b
        self._binding = None
        tdt = self.lag_grid_forcing_field.dtype
        for t in (u, f):
            if not isinstance(t, torch.Tensor) or t.dtype != tdt or t.device != self.device or not t.is_contiguous():
                return None
        if u.shape != f.shape:
            return None
        self._binding = b = _IBBinding(self, key, u)
        return b

    def device_call(self, dev_scalars: int) -> None:
        """``time_step(dt)`` then ``__call__()`` with dt read on the GPU (one kernel pair).

        For captured time loops: the marker kinematics are taken from the
        device copies already uploaded (static bodies or bodies whose
        kinematics the caller refreshes with ``upload_kinematics``)."""
        self._interaction(self.eul_grid_velocity_field, self._pos_stage.dev, self._vel_stage.dev, xi_step=True,
                          dev_scalars=dev_scalars)
        self._spread(self.eul_grid_forcing_field, reset=self.enable_eul_grid_forcing_reset)

    def upload_kinematics(self) -> None:
        """Refresh the device copies of the marker positions and velocities."""
        self.forcing_grid.compute_lag_grid_position_field()
        self.forcing_grid.compute_lag_grid_velocity_field()
        self._kin_stage.upload(self.forcing_grid.position_field, self.forcing_grid.velocity_field)

    def lag_grid_forcing_host(self) -> np.ndarray:
        """A host copy of the Lagrangian forcing (waits for the GPU work that produces it).

        When the forcing still holds what the last ``__call__`` computed, the
        pinned copy queued right after that interaction is returned (the wait
        ends there, not at the end of the flow step queued after it); otherwise
        the field is copied now."""
        self._snapshot_wanted = True
        if self._snapshot_key is not None and self._snapshot_key == (self._n_interactions,
                                                                     self.lag_grid_forcing_field._version):
            src = self._snapshot_src
            if src is not None:
                src.wait(2)
                return src.forcing.copy()
            self._snapshot_event.synchronize()
        else:
            self._host_forcing.copy_(self.lag_grid_forcing_field)
            self._snapshot_key = None
        return self._host_forcing.numpy().copy()

    def compute_flow_forces_and_torques(self) -> None:
        """immersed_body_flow_interaction.py:124-131 (one device->host read)."""
        self.compute_interaction_on_lag_grid()
        self.forcing_grid.transfer_forcing_from_grid_to_body(
            body_flow_forces=self.body_flow_forces, body_flow_torques=self.body_flow_torques,
            lag_grid_forcing_field=self.lag_grid_forcing_host())

    def get_grid_deviation_error_l2_norm(self) -> float:
        """immersed_body_flow_interaction.py:133-141."""
        xi = self.lag_grid_position_mismatch_field.double()
        return float(torch.linalg.vector_norm(xi).item()) / np.sqrt(self.forcing_grid.num_lag_nodes)


class RigidBodyFlowInteraction(ImmersedBodyFlowInteraction):
    """rigid_body/rigid_body_flow_interaction.py:9-54."""

    def __init__(self, rigid_body, eul_grid_forcing_field, eul_grid_velocity_field,
                 virtual_boundary_stiffness_coeff, virtual_boundary_damping_coeff, dx, grid_dim, forcing_grid_cls,
                 real_t=np.float64, eul_grid_coord_shift=None, interp_kernel_width=None,
                 enable_eul_grid_forcing_reset=False, num_threads=False, start_time=0.0, **forcing_grid_kwargs):
        forcing_grid_kwargs["rigid_body"] = rigid_body
        super().__init__(eul_grid_forcing_field, eul_grid_velocity_field, np.zeros((3, 1)), np.zeros((3, 1)),
                         forcing_grid_cls, virtual_boundary_stiffness_coeff, virtual_boundary_damping_coeff, dx,
                         grid_dim, real_t, eul_grid_coord_shift, interp_kernel_width, enable_eul_grid_forcing_reset,
                         num_threads, start_time, **forcing_grid_kwargs)


class CosseratRodFlowInteraction(ImmersedBodyFlowInteraction):
    """cosserat_rod/cosserat_rod_flow_interaction.py:9-58."""

    def __init__(self, cosserat_rod, eul_grid_forcing_field, eul_grid_velocity_field,
                 virtual_boundary_stiffness_coeff, virtual_boundary_damping_coeff, dx, grid_dim, forcing_grid_cls,
                 real_t=np.float64, eul_grid_coord_shift=None, interp_kernel_width=None,
                 enable_eul_grid_forcing_reset=False, num_threads=False, start_time=0.0, **forcing_grid_kwargs):
        forcing_grid_kwargs["cosserat_rod"] = cosserat_rod
        super().__init__(eul_grid_forcing_field, eul_grid_velocity_field, np.zeros((3, cosserat_rod.n_elems + 1)),
                         np.zeros((3, cosserat_rod.n_elems)), forcing_grid_cls, virtual_boundary_stiffness_coeff,
                         virtual_boundary_damping_coeff, dx, grid_dim, real_t, eul_grid_coord_shift,
                         interp_kernel_width, enable_eul_grid_forcing_reset, num_threads, start_time,
                         **forcing_grid_kwargs)


try:  # FlowForces plugs into pyelastica's forcing interface when it is installed
    from elastica import NoForces as _NoForces  # type: ignore
except Exception:  # pragma: no cover - pyelastica absent
    class _NoForces:  # minimal stand-in of elastica.NoForces
        def __init__(self) -> None:
            pass


class FlowForces(_NoForces):
    """flow_forces.py:12-25: adds the flow forces/torques to a pyelastica system."""

    def __init__(self, body_flow_interactor) -> None:
        super().__init__()
        self.body_flow_interactor = body_flow_interactor

    def apply_forces(self, system, time: float = 0.0) -> None:
        self.body_flow_interactor.compute_flow_forces_and_torques()
        system.external_forces += self.body_flow_interactor.body_flow_forces
        system.external_torques += self.body_flow_interactor.body_flow_torques
