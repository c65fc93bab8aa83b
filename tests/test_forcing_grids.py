"""The host-side forcing grids of the 3D rigid bodies and the tapered rods.

Geometry, kinematics, force/torque transfer and grid spacing of
``SphereForcingGrid``, ``OpenEndCircularCylinderForcingGrid``,
``RectangularPlaneForcingGrid`` (with the ``RectangularPlane`` body),
``CosseratRodEdgeForcingGrid`` and ``CosseratRodSurfaceForcingGrid`` against
fixtures made by running the reference classes on moving bodies and random
forcing (``golden_grids_*``), plus the reference tests' analytic checks
(markers on the body surface, uniform loads giving zero torque, the error on a
wrong grid dimension).  These run on the host in float64, so they run on CPU;
the ``gpu`` tests couple a sphere and a capped surface rod to a 3D flow, and a
tapered edge-grid rod to a 2D flow, through the virtual-boundary kernels and
compare with the reference interaction.
"""

from __future__ import annotations

import types

import numpy as np
import pytest
from conftest import load_golden, real_t_of, ref_tol

import sopht_gb300.simulator as sps

RTOL = 1e-12
ATOL = 1e-14


@pytest.fixture(scope="module")
def g():
    return load_golden("grids", "double")


def close(a, b):
    np.testing.assert_allclose(a, b, rtol=RTOL, atol=ATOL)


def _body(g, tag, **extra):
    return types.SimpleNamespace(
        position_collection=g[f"{tag}/body_position"].copy(), director_collection=g[f"{tag}/body_directors"].copy(),
        velocity_collection=g[f"{tag}/body_velocity"].copy(), omega_collection=g[f"{tag}/body_omega"].copy(),
        radius=float(g[f"{tag}/body_radius"]), length=float(g[f"{tag}/body_length"]), **extra)


def _rod(g, tag):
    names = ("position_collection", "velocity_collection", "omega_collection", "director_collection", "mass",
             "radius", "lengths", "tangents")
    rod = types.SimpleNamespace(**{n: g[f"{tag}/rod_{n}"].copy() for n in names})
    rod.n_elems = rod.lengths.shape[0]
    return rod


def _check_grid(g, tag, grid, n_forces, n_torques):
    assert grid.num_lag_nodes == int(g[f"{tag}/num_lag_nodes"])
    close(grid.position_field, g[f"{tag}/position"])
    close(grid.velocity_field, g[f"{tag}/velocity"])
    close(grid.get_maximum_lagrangian_grid_spacing(), g[f"{tag}/spacing"])
    forces, torques = np.full((3, n_forces), 9.0), np.full((3, n_torques), 9.0)
    grid.transfer_forcing_from_grid_to_body(body_flow_forces=forces, body_flow_torques=torques,
                                            lag_grid_forcing_field=g[f"{tag}/lag_forcing_in"])
    close(forces, g[f"{tag}/body_forces"])
    close(torques, g[f"{tag}/body_torques"])


@pytest.mark.parametrize("tag,n_eq", [("sphere16", 16), ("sphere7", 7)])
def test_sphere_grid_vs_reference(g, tag, n_eq):
    body = _body(g, tag)
    grid = sps.SphereForcingGrid(grid_dim=3, rigid_body=body, num_forcing_points_along_equator=n_eq)
    _check_grid(g, tag, grid, 1, 1)
    # every marker on the surface; the poles hold one marker each
    r = np.linalg.norm(grid.position_field - body.position_collection, axis=0)
    close(r, np.full_like(r, body.radius))
    assert grid.num_lag_nodes == sum(int(np.rint(n_eq * np.sin(p))) + 1 for p in np.linspace(0, np.pi, n_eq // 2))


def test_open_end_cylinder_grid_vs_reference(g):
    body = _body(g, "open_cylinder")
    grid = sps.OpenEndCircularCylinderForcingGrid(grid_dim=3, rigid_body=body, num_forcing_points_along_length=8)
    _check_grid(g, "open_cylinder", grid, 1, 1)
    n_circ = grid.num_forcing_points_along_circumference
    assert n_circ == int(np.ceil(8 * 2 * np.pi * body.radius / body.length))
    # distance from the axis d3 is the radius; the rings span the length
    rel = grid.position_field - body.position_collection
    d3 = body.director_collection[2, :, 0]
    along = d3 @ rel
    radial = rel - np.outer(d3, along)
    close(np.linalg.norm(radial, axis=0), np.full(grid.num_lag_nodes, body.radius))
    close(along.reshape(8, n_circ)[:, 0], np.linspace(-body.length / 2, body.length / 2, 8))


def test_rectangular_plane_body_and_grid_vs_reference(g):
    plane = sps.RectangularPlane(origin=np.array([0.5, 0.4, 0.6]), plane_normal=np.array([0.2, 0.1, 1.0]),
                                 plane_tangent_along_length=np.array([1.0, 0.0, -0.2]), plane_length=0.4,
                                 plane_breadth=0.25)
    close(plane.director_collection, g["plane/directors_as_built"])
    assert plane.n_elems == 1 and plane.position_collection.shape == (3, 1)
    assert not plane.velocity_collection.any() and not plane.omega_collection.any()
    body = _body(g, "plane", breadth=0.25)
    grid = sps.RectangularPlaneForcingGrid(grid_dim=3, rigid_body=body, num_forcing_points_along_length=10)
    _check_grid(g, "plane", grid, 1, 1)
    assert grid.num_forcing_points_along_breadth == int(10 * 0.25 / 0.4)
    # every marker in the plane through the origin with normal d3
    d3 = body.director_collection[2, :, 0]
    close(d3 @ (grid.position_field - body.position_collection), np.zeros(grid.num_lag_nodes))


def test_sphere_uniform_forcing_force_and_torque(g):
    body = _body(g, "sphere16")
    body.director_collection = np.eye(3).reshape(3, 3, 1)
    grid = sps.SphereForcingGrid(grid_dim=3, rigid_body=body, num_forcing_points_along_equator=16)
    f = np.zeros((3, grid.num_lag_nodes))
    f[...] = np.array([1.0, 2.0, 3.0]).reshape(3, 1)
    forces, torques = np.zeros((3, 1)), np.zeros((3, 1))
    grid.transfer_forcing_from_grid_to_body(forces, torques, f)
    close(forces[:, 0], -grid.num_lag_nodes * np.array([1.0, 2.0, 3.0]))
    # with identity directors the torque is -(sum of the arms) x F
    arm_sum = np.sum(grid.global_frame_relative_position_field, axis=1)
    close(torques[:, 0], -np.cross(arm_sum, np.array([1.0, 2.0, 3.0])))


def test_edge_grid_vs_reference(g):
    rod = _rod(g, "edge")
    grid = sps.CosseratRodEdgeForcingGrid(grid_dim=2, cosserat_rod=rod)
    close(grid.moment_arm, g["edge/moment_arm"])
    _check_grid(g, "edge", grid, rod.n_elems + 1, rod.n_elems)
    n = rod.n_elems
    assert (grid.start_idx_left_edge_nodes, grid.end_idx_right_edge_nodes) == (n, 3 * n)
    # the edges sit at +/- r (e_z x t) about the centres
    gap = grid.position_field[:, n:2 * n] - grid.position_field[:, :n]
    close(gap, grid.moment_arm[:2])
    close(grid.position_field[:, :n] - gap, grid.position_field[:, 2 * n:])
    t = rod.tangents
    close(grid.moment_arm, rod.radius * np.stack([-t[1], t[0], np.zeros(n)]))


@pytest.mark.parametrize("tag,density,cap", [("surface_cap", 12, True), ("surface_nocap", 8, False),
                                             ("surface_one", 16, True)])
def test_surface_grid_vs_reference(g, tag, density, cap):
    rod = _rod(g, tag)
    grid = sps.CosseratRodSurfaceForcingGrid(grid_dim=3, cosserat_rod=rod,
                                             surface_grid_density_for_largest_element=density, with_cap=cap)
    np.testing.assert_array_equal(grid.surface_grid_points, g[f"{tag}/surface_grid_points"])
    np.testing.assert_array_equal(grid.start_idx, g[f"{tag}/start_idx"])
    np.testing.assert_array_equal(grid.end_idx, g[f"{tag}/end_idx"])
    close(grid.grid_point_radius_ratio, g[f"{tag}/grid_point_radius_ratio"])
    close(grid.local_frame_surface_points, g[f"{tag}/local_frame_surface_points"])
    for i in range(rod.n_elems):
        close(grid.surface_point_rotation_angle_list[i], g[f"{tag}/surface_point_rotation_angle_list/{i}"])
    close(grid.moment_arm, g[f"{tag}/moment_arm"])
    _check_grid(g, tag, grid, rod.n_elems + 1, rod.n_elems)


def test_surface_grid_uniform_load_and_caps(g):
    rod = _rod(g, "surface_cap")
    grid = sps.CosseratRodSurfaceForcingGrid(grid_dim=3, cosserat_rod=rod,
                                             surface_grid_density_for_largest_element=12, with_cap=True)
    plain = sps.CosseratRodSurfaceForcingGrid(grid_dim=3, cosserat_rod=rod,
                                              surface_grid_density_for_largest_element=12)
    # caps add inner rings to the two end elements only
    extra = grid.surface_grid_points - plain.surface_grid_points
    assert extra[0] > 0 and extra[-1] >= 0 and not extra[1:-1].any()
    # a uniform load: half of each element's total to each node, and no torque when every ring is whole
    f = np.zeros((3, grid.num_lag_nodes))
    f[...] = np.array([1.0, 2.0, 3.0]).reshape(3, 1)
    forces, torques = np.zeros((3, rod.n_elems + 1)), np.zeros((3, rod.n_elems))
    grid.transfer_forcing_from_grid_to_body(forces, torques, f)
    per = np.outer([1.0, 2.0, 3.0], grid.surface_grid_points)
    ref = np.zeros_like(forces)
    ref[:, :-1] -= 0.5 * per
    ref[:, 1:] -= 0.5 * per
    close(forces, ref)
    np.testing.assert_allclose(torques, 0.0, atol=1e-13)


@pytest.mark.parametrize("cls,kw,dim", [
    (sps.SphereForcingGrid, {"num_forcing_points_along_equator": 8}, 2),
    (sps.OpenEndCircularCylinderForcingGrid, {"num_forcing_points_along_length": 4}, 2),
    (sps.RectangularPlaneForcingGrid, {"num_forcing_points_along_length": 4}, 4),
])
def test_rigid_grid_invalid_dim(cls, kw, dim):
    body = types.SimpleNamespace(radius=0.1, length=0.4, breadth=0.2)
    with pytest.raises(ValueError, match="3D Rigid body forcing grid is only defined for grid_dim=3"):
        cls(grid_dim=dim, rigid_body=body, **kw)


def test_rod_grid_invalid_dim(g):
    rod = _rod(g, "surface_cap")
    with pytest.raises(ValueError, match="edge forcing grid is only defined for grid_dim=2"):
        sps.CosseratRodEdgeForcingGrid(grid_dim=3, cosserat_rod=rod)
    with pytest.raises(ValueError, match="surface forcing grid is only defined for grid_dim=3"):
        sps.CosseratRodSurfaceForcingGrid(grid_dim=2, cosserat_rod=rod, surface_grid_density_for_largest_element=4)


# ------------------------------------------------------------------- on the GPU


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.gpu
@pytest.mark.parametrize("tag", ["sphere_inter", "surface_inter", "edge_inter"])
def test_interaction_through_grids_vs_reference(precision, tag):
    import torch

    from sopht_gb300 import _lib
    from sopht_gb300.build import build
    build()
    _lib.load()
    gg = load_golden("grids", precision)
    rt = real_t_of(precision)
    tdt = torch.float32 if rt == np.float32 else torch.float64
    if tag == "edge_inter":
        force = torch.zeros((2, 32, 48), dtype=tdt, device="cuda")
        common = dict(eul_grid_forcing_field=force, eul_grid_velocity_field=_dev(gg[f"{tag}/eul_velocity"]),
                      virtual_boundary_stiffness_coeff=-5e4, virtual_boundary_damping_coeff=-20.0, dx=rt(1.0 / 48),
                      grid_dim=2, real_t=rt)
    else:
        force = torch.zeros((3, 16, 16, 16), dtype=tdt, device="cuda")
        common = dict(eul_grid_forcing_field=force, eul_grid_velocity_field=_dev(gg["eul_velocity"]),
                      virtual_boundary_stiffness_coeff=-2e4, virtual_boundary_damping_coeff=-1e2, dx=rt(1.0 / 16),
                      grid_dim=3, real_t=rt)
    if tag == "edge_inter":
        inter = sps.CosseratRodFlowInteraction(cosserat_rod=_rod(gg, tag),
                                               forcing_grid_cls=sps.CosseratRodEdgeForcingGrid, **common)
    elif tag == "sphere_inter":
        names = ("position_collection", "velocity_collection", "omega_collection", "director_collection")
        body = types.SimpleNamespace(**{n: gg[f"{tag}/body_{n}"].copy() for n in names},
                                     radius=float(gg[f"{tag}/body_radius"]))
        inter = sps.RigidBodyFlowInteraction(rigid_body=body, forcing_grid_cls=sps.SphereForcingGrid,
                                             num_forcing_points_along_equator=20, **common)
    else:
        rod = _rod(gg, tag)
        inter = sps.CosseratRodFlowInteraction(cosserat_rod=rod, forcing_grid_cls=sps.CosseratRodSurfaceForcingGrid,
                                               surface_grid_density_for_largest_element=6, with_cap=True, **common)
    inter.time_step(dt=1e-3)
    inter()
    tol = ref_tol(precision)
    torch.cuda.synchronize()
    np.testing.assert_allclose(inter.lag_grid_forcing_field.cpu().numpy(), gg[f"{tag}/lag_forcing"], rtol=tol,
                               atol=tol)
    # the spread forcing peaks at several hundred here: 1e3 eps of its largest value (FP32 sums of the
    # overlapping marker supports round differently from the reference's loop)
    ref = gg[f"{tag}/eul_forcing_out"]
    np.testing.assert_allclose(force.cpu().numpy(), ref, rtol=tol, atol=tol * max(1.0, float(np.abs(ref).max())))
    inter.compute_flow_forces_and_torques()
    np.testing.assert_allclose(inter.body_flow_forces, gg[f"{tag}/body_forces"], rtol=tol, atol=tol)
    np.testing.assert_allclose(inter.body_flow_torques, gg[f"{tag}/body_torques"], rtol=tol, atol=tol)


# ------------------------------------------------------- randomised cases


@pytest.fixture(scope="module")
def gr():
    return load_golden("gridsrandom", "double")


@pytest.mark.parametrize("kind", ["sphere", "open_cylinder", "plane"])
@pytest.mark.parametrize("i", range(12))
def test_rigid_grids_random_cases_vs_reference(gr, kind, i):
    tag = f"{kind}/{i}"
    radius, length, breadth, count = gr[f"{tag}/params"]
    body = types.SimpleNamespace(**{n: gr[f"{tag}/body_{n}"].copy() for n in
                                    ("position_collection", "director_collection", "velocity_collection",
                                     "omega_collection")}, radius=radius, length=length, breadth=breadth)
    cls, key = {"sphere": (sps.SphereForcingGrid, "num_forcing_points_along_equator"),
                "open_cylinder": (sps.OpenEndCircularCylinderForcingGrid, "num_forcing_points_along_length"),
                "plane": (sps.RectangularPlaneForcingGrid, "num_forcing_points_along_length")}[kind]
    _check_grid(gr, tag, cls(grid_dim=3, rigid_body=body, **{key: int(count)}), 1, 1)


@pytest.mark.parametrize("kind", ["edge", "surface", "surface_wide"])
@pytest.mark.parametrize("i", range(12))
def test_rod_grids_random_cases_vs_reference(gr, kind, i):
    tag = f"{kind}/{i}"
    rod = _rod(gr, tag)
    if kind == "edge":
        grid = sps.CosseratRodEdgeForcingGrid(grid_dim=2, cosserat_rod=rod)
    else:
        density, cap = gr[f"{tag}/params"]
        grid = sps.CosseratRodSurfaceForcingGrid(grid_dim=3, cosserat_rod=rod,
                                                 surface_grid_density_for_largest_element=int(density),
                                                 with_cap=bool(cap))
        np.testing.assert_array_equal(grid.surface_grid_points, gr[f"{tag}/surface_grid_points"])
    _check_grid(gr, tag, grid, rod.n_elems + 1, rod.n_elems)
