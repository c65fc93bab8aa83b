"""The oracle against golden fixtures generated by running the reference code.

Every fixture in ``tests/golden`` was produced by ``make_golden.py`` from the
reference implementation itself; these tests pin the numpy oracle to them at
the reference tests' tolerance (1e3 eps absolute) or, where a different FFT
rounding path is involved, a stated relative-L2 bound.
"""

from __future__ import annotations

import numpy as np
import pytest
from conftest import load_golden, real_t_of, ref_tol, rel_l2

from oracle import stencils as st
from oracle.flow import (
    CircularCylinderOracle,
    ImmersedBodyInteractionOracle,
    NavierStokes2DOracle,
    NavierStokes3DOracle,
    RodElementCentricGridOracle,
    RodNodalGridOracle,
)
from oracle.ib import VirtualBoundaryForcingOracle
from oracle.poisson import UnboundedPoisson2D, UnboundedPoisson3D


@pytest.mark.parametrize("tag", ["sq", "rect"])
def test_stencils_2d(precision, tag):
    g = load_golden("stencils2d", precision)
    rt = real_t_of(precision)
    tol = ref_tol(precision)
    f, v, fo = g[f"{tag}/field"], g[f"{tag}/velocity"], g[f"{tag}/forcing"]
    np.testing.assert_allclose(st.eno3_flux_2d(f, v, rt(0.1)), g[f"{tag}/eno3_flux"], atol=tol)
    out = f.copy()
    st.advection_step_2d(out, v, rt(0.3))
    np.testing.assert_allclose(out, g[f"{tag}/advection_step"], atol=tol)
    np.testing.assert_allclose(st.diffusion_flux_2d(f, rt(0.1)), g[f"{tag}/diffusion_flux"], atol=tol)
    out = f.copy()
    st.diffusion_step_2d(out, rt(0.2))
    np.testing.assert_allclose(out, g[f"{tag}/diffusion_step"], atol=tol)
    np.testing.assert_allclose(st.outplane_curl_2d(f, rt(0.7)), g[f"{tag}/outplane_curl"], atol=tol)
    out = f.copy()
    st.forcing_curl_update_2d(out, fo, rt(0.4))
    np.testing.assert_allclose(out, g[f"{tag}/forcing_curl_update"], atol=tol)
    pos = g[f"{tag}/position"]
    dx = rt(1.0 / f.shape[1])
    for width in (0, 2, 3):
        out = f.copy()
        st.penalise_2d(out, width, dx, pos[0], pos[1])
        np.testing.assert_allclose(out, g[f"{tag}/penalise_w{width}"], atol=tol)


@pytest.mark.parametrize("tag", ["sq", "rect", "r3"])
def test_poisson_2d(precision, tag):
    g = load_golden("poisson2d", precision)
    ny, nx, x_range = g[f"{tag}/meta"]
    solver = UnboundedPoisson2D(int(ny), int(nx), float(x_range), real_t_of(precision))
    np.testing.assert_allclose(solver.solve(g[f"{tag}/rhs"]), g[f"{tag}/solution"],
                               atol=ref_tol(precision))


@pytest.mark.parametrize("tag", ["a", "b", "c"])
def test_ns_step_2d(precision, tag):
    g = load_golden("ns2d", precision)
    rt = real_t_of(precision)
    ny, nx, x_range, nu, fs, rho, width, dt, ux, uy = g[f"{tag}/meta"]
    sim = NavierStokes2DOracle((int(ny), int(nx)), float(x_range), float(nu), real_t=rt, time=0.5,
                               with_forcing=True, with_free_stream_flow=bool(fs),
                               flow_density=float(rho), penalty_zone_width=int(width))
    sim.vorticity_field[...] = g[f"{tag}/vorticity_in"]
    sim.velocity_field[...] = g[f"{tag}/velocity_in"]
    sim.eul_grid_forcing_field[...] = g[f"{tag}/forcing_in"]
    assert sim.compute_stable_timestep() == g[f"{tag}/stable_dt"]
    assert sim.compute_stable_timestep(0.25) == g[f"{tag}/stable_dt_prefac"]
    sim.time_step(float(dt), np.array([ux, uy]))
    tol = ref_tol(precision)
    np.testing.assert_allclose(sim.vorticity_field, g[f"{tag}/vorticity_out"], atol=tol)
    np.testing.assert_allclose(sim.velocity_field, g[f"{tag}/velocity_out"], atol=tol)
    np.testing.assert_allclose(sim.stream_func_field, g[f"{tag}/stream_func_out"], atol=tol)
    assert np.all(sim.eul_grid_forcing_field == 0)
    assert sim.time == pytest.approx(float(g[f"{tag}/time_out"]))
    # without forcing
    sim2 = NavierStokes2DOracle((int(ny), int(nx)), float(x_range), float(nu), real_t=rt,
                                with_free_stream_flow=bool(fs), penalty_zone_width=int(width))
    sim2.vorticity_field[...] = g[f"{tag}/vorticity_in"]
    sim2.velocity_field[...] = g[f"{tag}/velocity_in"]
    sim2.time_step(float(dt), np.array([ux, uy]))
    np.testing.assert_allclose(sim2.vorticity_field, g[f"{tag}/noforce_vorticity_out"], atol=tol)
    np.testing.assert_allclose(sim2.velocity_field, g[f"{tag}/noforce_velocity_out"], atol=tol)


@pytest.mark.parametrize("tag", ["cube", "rect"])
def test_stencils_3d(precision, tag):
    g = load_golden("stencils3d", precision)
    rt = real_t_of(precision)
    tol = ref_tol(precision)
    f, f2 = g[f"{tag}/field"], g[f"{tag}/field2"]
    np.testing.assert_allclose(st.curl_3d(f, rt(0.6)), g[f"{tag}/curl"], atol=tol)
    out = f.copy()
    st.forcing_curl_update_3d(out, f2, rt(0.3))
    np.testing.assert_allclose(out, g[f"{tag}/forcing_curl_update"], atol=tol)
    np.testing.assert_allclose(st.cross_3d(f, f2), g[f"{tag}/cross"], atol=tol)
    out = f.copy()
    st.diffusion_step_3d(out, rt(0.1))
    np.testing.assert_allclose(out, g[f"{tag}/diffusion_step"], atol=tol)
    np.testing.assert_allclose(st.divergence_3d(f, rt(3.0)), g[f"{tag}/divergence"], atol=tol)
    pos = g[f"{tag}/position"]
    dx = rt(1.0 / f.shape[-1])
    for width in (0, 2):
        out = f.copy()
        for c in range(3):
            st.penalise_3d(out[c], width, dx, pos[0], pos[1], pos[2])
        np.testing.assert_allclose(out, g[f"{tag}/penalise_w{width}"], atol=tol)
    for ftype, order in (("multiplicative", 2), ("convolution", 1), ("convolution", 3)):
        out = f.copy()
        st.laplacian_filter_3d(out, order, ftype)
        np.testing.assert_allclose(out, g[f"{tag}/filter_{ftype}_{order}"], atol=tol)


@pytest.mark.parametrize("tag", ["cube", "rect"])
def test_poisson_3d(precision, tag):
    g = load_golden("poisson3d", precision)
    nz, ny, nx, x_range = g[f"{tag}/meta"]
    solver = UnboundedPoisson3D(int(nz), int(ny), int(nx), float(x_range), real_t_of(precision))
    np.testing.assert_allclose(solver.vector_solve(g[f"{tag}/rhs"]), g[f"{tag}/solution"],
                               atol=ref_tol(precision))


@pytest.mark.parametrize("tag", ["a", "b", "c", "d"])
def test_ns_step_3d(precision, tag):
    g = load_golden("ns3d", precision)
    rt = real_t_of(precision)
    m = g[f"{tag}/meta"]
    grid = tuple(int(v) for v in m[:3])
    x_range, nu, fs, rho, dt = (float(v) for v in m[3:8])
    u_inf = m[8:11]
    order, ftype = int(m[11]), int(m[12])
    filt = None if ftype == 0 else {"order": order,
                                    "type": "multiplicative" if ftype == 1 else "convolution"}
    sim = NavierStokes3DOracle(grid, x_range, nu, real_t=rt, with_forcing=True,
                               with_free_stream_flow=bool(fs), flow_density=rho,
                               filter_vorticity=filt is not None, filter_setting_dict=filt)
    sim.vorticity_field[...] = g[f"{tag}/vorticity_in"]
    sim.velocity_field[...] = g[f"{tag}/velocity_in"]
    sim.eul_grid_forcing_field[...] = g[f"{tag}/forcing_in"]
    np.testing.assert_allclose(sim.get_vorticity_divergence_l2_norm(), g[f"{tag}/divergence_l2"],
                               rtol=1e-6 if rt == np.float32 else 1e-12)
    assert sim.compute_stable_timestep() == g[f"{tag}/stable_dt"]
    sim.time_step(dt, u_inf)
    tol = ref_tol(precision)
    np.testing.assert_allclose(sim.vorticity_field, g[f"{tag}/vorticity_out"], atol=tol)
    np.testing.assert_allclose(sim.velocity_field, g[f"{tag}/velocity_out"], atol=tol)


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("kernel", ["cosine", "peskin"])
def test_virtual_boundary_forcing(precision, dim, kernel):
    g = load_golden("ib", precision)
    rt = real_t_of(precision)
    tag = f"d{dim}_{kernel}"
    meta = g[f"{tag}/meta"]
    grid = tuple(int(v) for v in meta[1: 1 + dim])
    n_lag = int(meta[1 + dim])
    K, C, dt = (float(v) for v in meta[2 + dim:])
    dx = rt(1.0 / grid[-1])
    vbf = VirtualBoundaryForcingOracle(K, C, dim, dx, n_lag, rt, kernel=kernel)
    vbf.lag_grid_position_mismatch_field[...] = g[f"{tag}/position_mismatch_in"]
    force = g[f"{tag}/eul_forcing_in"].copy()
    vbf.compute_interaction_forcing(force, g[f"{tag}/eul_velocity"], g[f"{tag}/position"],
                                    g[f"{tag}/lag_velocity"])
    np.testing.assert_array_equal(vbf.nearest, g[f"{tag}/nearest_index"])
    tol = ref_tol(precision)
    np.testing.assert_allclose(vbf.weights, g[f"{tag}/weights"], rtol=tol, atol=tol * 1e-3)
    np.testing.assert_allclose(vbf.lag_grid_flow_velocity_field, g[f"{tag}/lag_flow_velocity"], atol=tol)
    np.testing.assert_allclose(vbf.lag_grid_forcing_field, g[f"{tag}/lag_forcing"],
                               rtol=tol, atol=tol)
    np.testing.assert_allclose(force, g[f"{tag}/eul_forcing_out"], rtol=tol, atol=tol)
    vbf.time_step(dt)
    np.testing.assert_allclose(vbf.lag_grid_position_mismatch_field,
                               g[f"{tag}/position_mismatch_out"], atol=tol)


def test_cylinder_coupled_steps(precision):
    """Four steps of the flow-past-cylinder loop, each against the reference run."""
    g = load_golden("cylinder2d", precision)
    rt = real_t_of(precision)
    ny, nx, x_range, nu, radius, n_mk, cx, cy, K, C = g["meta"]
    sim = NavierStokes2DOracle((int(ny), int(nx)), float(x_range), float(nu), real_t=rt,
                               with_forcing=True, with_free_stream_flow=True)
    sim.vorticity_field[...] = g["vorticity_init"]
    grid = CircularCylinderOracle([cx, cy, 0.0], float(radius), int(n_mk))
    np.testing.assert_allclose(grid.position_field, g["marker_position"], rtol=1e-15)
    inter = ImmersedBodyInteractionOracle(
        sim.eul_grid_forcing_field, sim.velocity_field, np.zeros((3, 1)), np.zeros((3, 1)),
        grid, float(K), float(C), sim.dx, 2, real_t=rt)
    for step in range(4):
        dt = sim.compute_stable_timestep()
        # the dt sequence is replayed; our own dt must agree to rounding
        assert dt == pytest.approx(g["dt"][step], rel=1e-6 if rt == np.float32 else 1e-14)
        dt = g["dt"][step]
        inter.time_step(dt)
        inter()
        sim.time_step(dt, np.array([1.0, 0.0]))
        scale = np.abs(g[f"step{step}/vorticity"]).max()
        bound = 1e-5 if rt == np.float32 else 1e-12
        assert rel_l2(sim.vorticity_field, g[f"step{step}/vorticity"]) < bound, scale
        assert rel_l2(sim.velocity_field, g[f"step{step}/velocity"]) < bound
        assert rel_l2(inter.lag_grid_forcing_field, g[f"step{step}/lag_forcing"]) < bound
    inter.compute_flow_forces_and_torques()
    # the lift and torque are sums of nearly cancelling marker forces, so the
    # bound is absolute, scaled by the drag magnitude
    scale = np.abs(g["body_forces"]).max()
    atol = scale * (1e-5 if rt == np.float32 else 1e-12)
    np.testing.assert_allclose(inter.body_flow_forces, g["body_forces"], atol=atol, rtol=0)
    np.testing.assert_allclose(inter.body_flow_torques, g["body_torques"], atol=atol, rtol=0)


class _Rod:
    def __init__(self, g, name):
        self.position_collection = g[f"{name}/rod_position"]
        self.velocity_collection = g[f"{name}/rod_velocity"]
        self.mass = g[f"{name}/rod_mass"]
        self.director_collection = g[f"{name}/rod_directors"]
        self.n_elems = self.position_collection.shape[1] - 1
        self.lengths = np.linalg.norm(np.diff(self.position_collection, axis=1), axis=0)


@pytest.mark.parametrize("name", ["nodal", "element"])
def test_rod_forcing_grids(precision, name):
    g = load_golden("rod3d", precision)
    rt = real_t_of(precision)
    rod = _Rod(g, name)
    cls = RodNodalGridOracle if name == "nodal" else RodElementCentricGridOracle
    grid = cls(rod)
    force = np.zeros((3, 16, 16, 16), dtype=rt)
    eul_vel = g["eul_velocity"]
    inter = ImmersedBodyInteractionOracle(
        force, eul_vel, np.zeros((3, rod.n_elems + 1)), np.zeros((3, rod.n_elems)), grid,
        -2e4, -1e2, rt(1.0 / 16), 3, real_t=rt)
    inter.time_step(1e-3)
    inter()
    tol = ref_tol(precision)
    np.testing.assert_allclose(inter.lag_grid_forcing_field, g[f"{name}/lag_forcing"], rtol=tol, atol=tol)
    np.testing.assert_allclose(force, g[f"{name}/eul_forcing_out"], rtol=tol, atol=tol)
    inter.lag_grid_position_mismatch_field[...] = g[f"{name}/position_mismatch_in"]
    inter.compute_flow_forces_and_torques()
    np.testing.assert_allclose(inter.body_flow_forces, g[f"{name}/body_forces"], rtol=tol, atol=tol)
    np.testing.assert_allclose(inter.body_flow_torques, g[f"{name}/body_torques"], rtol=tol, atol=tol)


# ------------------------------------------------------------- passive transport


@pytest.mark.parametrize("tag", ["cube", "rect"])
def test_eno3_advection_3d(precision, tag):
    """advection_flux_3d.py (accumulating into its buffer) and advection_timestep_3d.py, scalar and vector."""
    g = load_golden("passive", precision)
    rt = real_t_of(precision)
    tol = ref_tol(precision)
    f, v, vec = g[f"{tag}/field"], g[f"{tag}/velocity"], g[f"{tag}/vector_field"]
    flux = g[f"{tag}/flux_in"] + st.eno3_flux_3d(f, v, rt(0.7))
    np.testing.assert_allclose(flux, g[f"{tag}/flux_out"], atol=tol)
    out = f.copy()
    st.advection_step_3d(out, v, rt(0.3))
    np.testing.assert_allclose(out, g[f"{tag}/advection_step"], atol=tol)
    out = vec.copy()
    for c in range(3):
        st.advection_step_3d(out[c], v, rt(0.3))
    np.testing.assert_allclose(out, g[f"{tag}/advection_step_vector"], atol=tol)


@pytest.mark.parametrize("tag,dim,grid,ftype", [("s2d", 2, (12, 16), "scalar"), ("s3d", 3, (8, 10, 12), "scalar"),
                                                ("v3d", 3, (8, 8, 10), "vector")])
def test_passive_transport_steps(precision, tag, dim, grid, ftype):
    """Three steps of PassiveTransportFlowSimulator (stable dt with dt_prefac 0.8, advection, diffusion)."""
    from oracle.flow import PassiveTransportOracle
    g = load_golden("passive", precision)
    rt = real_t_of(precision)
    sim = PassiveTransportOracle(1e-2, dim, grid, 1.0, cfl=0.2, real_t=rt, time=0.5, field_type=ftype)
    sim.velocity_field[...] = g[f"sim_{tag}/velocity"]
    sim.primary_field[...] = g[f"sim_{tag}/primary_in"]
    for step in range(3):
        dt = sim.compute_stable_timestep(dt_prefac=0.8)
        assert dt == g[f"sim_{tag}/dt"][step]
        sim.time_step(dt)
        np.testing.assert_allclose(sim.primary_field, g[f"sim_{tag}/primary_step{step}"], atol=ref_tol(precision))
    assert sim.time == g[f"sim_{tag}/time_out"]


def test_passive_transport_rejects_2d_vector():
    from oracle.flow import PassiveTransportOracle
    with pytest.raises(ValueError):
        PassiveTransportOracle(1e-2, 2, (8, 8), 1.0, field_type="vector")
    with pytest.raises(ValueError):
        PassiveTransportOracle(1e-2, 3, (8, 8, 8), 1.0, field_type="tensor")
