"""Generate the golden fixtures in this directory by running the reference SophT code.

Run where a checkout of the reference is available (read only), giving its path::

    python tests/golden/make_golden.py /path/to/reference [group ...]

The reference is imported through the test-only stand-ins in ``ref_shims.py``
(pystencils kernels evaluated with numpy, pyfftw replaced by scipy.fft, numba's
``njit`` as identity, pyelastica helper functions restated).  Every case uses a
``numpy.random.default_rng`` with a fixed seed, and writes inputs and the
reference outputs to ``golden_<group>_<precision>.npz``.  The fixtures are small
(grids of at most a few thousand cells) so the CPU test suite loads them in
milliseconds.  Nothing at test time reads the reference checkout.
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))

import ref_shims  # noqa: E402


def _import_reference(ref_root: str):
    ref_shims.install()
    sys.path.insert(0, ref_root)
    import sopht.numeric.eulerian_grid_ops as spne
    import sopht.numeric.immersed_boundary_ops as spib
    import sopht.simulator as sps
    return spne, spib, sps


PRECISIONS = {"single": np.float32, "double": np.float64}


class _Recorder:
    def __init__(self) -> None:
        self.data: dict[str, np.ndarray] = {}

    def put(self, key: str, value) -> None:
        self.data[key] = np.array(value, copy=True)


# ----------------------------------------------------------------------------
# 2D stencil operators
# ----------------------------------------------------------------------------


def stencils_2d(spne, real_t, rec: _Recorder, seed: int) -> None:
    rng = np.random.default_rng(seed)
    for tag, shape in (("sq", (16, 16)), ("rect", (12, 20))):
        ny, nx = shape
        field = rng.standard_normal(shape).astype(real_t)
        vel = rng.standard_normal((2, *shape)).astype(real_t)
        forcing = rng.standard_normal((2, *shape)).astype(real_t)
        rec.put(f"{tag}/field", field)
        rec.put(f"{tag}/velocity", vel)
        rec.put(f"{tag}/forcing", forcing)
        # ENO3 flux (advection_flux_2d.py:12-165)
        flux = np.zeros_like(field)
        k = spne.gen_advection_flux_conservative_eno3_pyst_kernel_2d(real_t=real_t)
        k(advection_flux=flux, field=field, velocity=vel, inv_dx=real_t(0.1))
        rec.put(f"{tag}/eno3_flux", flux)
        # advection timestep (advection_timestep_2d.py:10-55)
        out = field.copy()
        buf = rng.standard_normal(shape).astype(real_t)  # garbage buffer: must be reset
        k = spne.gen_advection_timestep_euler_forward_conservative_eno3_pyst_kernel_2d(real_t=real_t)
        k(field=out, advection_flux=buf, velocity=vel, dt_by_dx=real_t(0.3))
        rec.put(f"{tag}/advection_step", out)
        # diffusion flux / timestep (diffusion_flux_2d.py, diffusion_timestep_2d.py)
        dflux = rng.standard_normal(shape).astype(real_t)
        k = spne.gen_diffusion_flux_pyst_kernel_2d(real_t=real_t)
        k(diffusion_flux=dflux, field=field, prefactor=real_t(0.1))
        rec.put(f"{tag}/diffusion_flux", dflux)
        out = field.copy()
        k = spne.gen_diffusion_timestep_euler_forward_pyst_kernel_2d(real_t=real_t)
        k(field=out, diffusion_flux=np.zeros_like(field), nu_dt_by_dx2=real_t(0.2))
        rec.put(f"{tag}/diffusion_step", out)
        # outplane curl (outplane_field_curl_2d.py)
        curl = rng.standard_normal((2, *shape)).astype(real_t)
        k = spne.gen_outplane_field_curl_pyst_kernel_2d(real_t=real_t)
        k(curl=curl, field=field, prefactor=real_t(0.7))
        rec.put(f"{tag}/outplane_curl", curl)
        # forcing curl update (update_vorticity_from_velocity_forcing_2d.py:12-71)
        out = field.copy()
        k = spne.gen_update_vorticity_from_velocity_forcing_pyst_kernel_2d(real_t=real_t)
        k(vorticity_field=out, velocity_forcing_field=forcing, prefactor=real_t(0.4))
        rec.put(f"{tag}/forcing_curl_update", out)
        # penalise (penalise_field_boundary_2d.py:12-142) at widths 0, 2, 3
        dx = real_t(1.0 / nx)
        x = np.linspace(dx / 2, 1.0 - dx / 2, nx).astype(real_t)
        y_range = 1.0 * ny / nx
        y = np.linspace(dx / 2, y_range - dx / 2, ny).astype(real_t)
        pos = np.flipud(np.array(np.meshgrid(y, x, indexing="ij")))
        rec.put(f"{tag}/position", pos)
        for width in (0, 2, 3):
            out = field.copy()
            k = spne.gen_penalise_field_boundary_pyst_kernel_2d(
                width=width, dx=dx, x_grid_field=pos[0], y_grid_field=pos[1], real_t=real_t)
            k(field=out)
            rec.put(f"{tag}/penalise_w{width}", out)
        # elementwise: add fixed value (vector), set fixed value (vector)
        out = vel.copy()
        k = spne.gen_add_fixed_val_pyst_kernel_2d(real_t=real_t, field_type="vector")
        k(sum_field=out, vector_field=out, fixed_vals=[1.5, -0.25])
        rec.put(f"{tag}/add_fixed_val", out)


def poisson_2d(spne, real_t, rec: _Recorder, seed: int) -> None:
    rng = np.random.default_rng(seed)
    for tag, (ny, nx, x_range) in (("sq", (16, 16, 1.0)), ("rect", (12, 24, 2.0)), ("r3", (6, 12, 1.0))):
        rhs = rng.standard_normal((ny, nx)).astype(real_t)
        solver = spne.UnboundedPoissonSolverPYFFTW2D(
            grid_size_y=ny, grid_size_x=nx, x_range=x_range, real_t=real_t)
        sol = np.zeros_like(rhs)
        solver.solve(solution_field=sol, rhs_field=rhs)
        rec.put(f"{tag}/rhs", rhs)
        rec.put(f"{tag}/solution", sol)
        rec.put(f"{tag}/meta", [ny, nx, x_range])
        rec.put(f"{tag}/greens_hat_dx2", solver.fourier_greens_function_times_dx_squared)


def ns_2d(sps, real_t, rec: _Recorder, seed: int) -> None:
    """One full with-forcing step of the 2D simulator (navier_stokes_flow_simulators.py:200-209)."""
    rng = np.random.default_rng(seed)
    cases = (
        ("a", (16, 16), 1.0, 1e-2, True, 1.0, 2),
        ("b", (12, 24), 1.0, 1e-3, True, 0.1, 2),
        ("c", (16, 32), 2.0, 5e-3, False, 1.0, 3),
    )
    for tag, grid, x_range, nu, free_stream, rho, width in cases:
        sim = sps.UnboundedNavierStokesFlowSimulator2D(
            grid_size=grid, x_range=x_range, kinematic_viscosity=nu, real_t=real_t,
            time=0.5, with_forcing=True, with_free_stream_flow=free_stream,
            flow_density=rho, penalty_zone_width=width)
        sim.vorticity_field[...] = rng.standard_normal(grid).astype(real_t)
        sim.velocity_field[...] = rng.standard_normal((2, *grid)).astype(real_t)
        sim.eul_grid_forcing_field[...] = rng.standard_normal((2, *grid)).astype(real_t)
        rec.put(f"{tag}/vorticity_in", sim.vorticity_field)
        rec.put(f"{tag}/velocity_in", sim.velocity_field)
        rec.put(f"{tag}/forcing_in", sim.eul_grid_forcing_field)
        dt = sim.compute_stable_timestep()
        rec.put(f"{tag}/stable_dt", dt)
        rec.put(f"{tag}/stable_dt_prefac", sim.compute_stable_timestep(dt_prefac=0.25))
        dt = 0.5 * dt
        u_inf = np.array([0.7, -0.2])
        sim.time_step(dt=dt, free_stream_velocity=u_inf)
        rec.put(f"{tag}/meta", [grid[0], grid[1], x_range, nu, float(free_stream), rho, width, dt,
                                u_inf[0], u_inf[1]])
        rec.put(f"{tag}/vorticity_out", sim.vorticity_field)
        rec.put(f"{tag}/velocity_out", sim.velocity_field)
        rec.put(f"{tag}/stream_func_out", sim.stream_func_field)
        rec.put(f"{tag}/forcing_out", sim.eul_grid_forcing_field)
        rec.put(f"{tag}/time_out", sim.time)
        # the no-forcing variant (navier_stokes_flow_simulators.py:171-198)
        sim2 = sps.UnboundedNavierStokesFlowSimulator2D(
            grid_size=grid, x_range=x_range, kinematic_viscosity=nu, real_t=real_t,
            with_forcing=False, with_free_stream_flow=free_stream, penalty_zone_width=width)
        sim2.vorticity_field[...] = rec.data[f"{tag}/vorticity_in"]
        sim2.velocity_field[...] = rec.data[f"{tag}/velocity_in"]
        sim2.time_step(dt=dt, free_stream_velocity=u_inf)
        rec.put(f"{tag}/noforce_vorticity_out", sim2.vorticity_field)
        rec.put(f"{tag}/noforce_velocity_out", sim2.velocity_field)


# ----------------------------------------------------------------------------
# 3D operators
# ----------------------------------------------------------------------------


def stencils_3d(spne, real_t, rec: _Recorder, seed: int) -> None:
    rng = np.random.default_rng(seed)
    for tag, shape in (("cube", (10, 10, 10)), ("rect", (8, 10, 12))):
        nz, ny, nx = shape
        vec = rng.standard_normal((3, *shape)).astype(real_t)
        vec2 = rng.standard_normal((3, *shape)).astype(real_t)
        rec.put(f"{tag}/field", vec)
        rec.put(f"{tag}/field2", vec2)
        out = rng.standard_normal((3, *shape)).astype(real_t)
        spne.gen_curl_pyst_kernel_3d(real_t=real_t)(curl=out, field=vec, prefactor=real_t(0.6))
        rec.put(f"{tag}/curl", out)
        out = vec.copy()
        spne.gen_update_vorticity_from_velocity_forcing_pyst_kernel_3d(real_t=real_t)(
            vorticity_field=out, velocity_forcing_field=vec2, prefactor=real_t(0.3))
        rec.put(f"{tag}/forcing_curl_update", out)
        out = np.zeros_like(vec)
        spne.gen_elementwise_cross_product_pyst_kernel_3d(real_t=real_t)(
            result_field=out, field_1=vec, field_2=vec2)
        rec.put(f"{tag}/cross", out)
        out = vec.copy()
        spne.gen_diffusion_timestep_euler_forward_pyst_kernel_3d(real_t=real_t, field_type="vector")(
            vector_field=out, diffusion_flux=np.zeros(shape, real_t), nu_dt_by_dx2=real_t(0.1))
        rec.put(f"{tag}/diffusion_step", out)
        div = np.zeros(shape, real_t)
        spne.gen_divergence_pyst_kernel_3d(real_t=real_t)(divergence=div, field=vec, inv_dx=real_t(3.0))
        rec.put(f"{tag}/divergence", div)
        dx = real_t(1.0 / nx)
        x = np.linspace(dx / 2, 1.0 - dx / 2, nx).astype(real_t)
        y = np.linspace(dx / 2, ny / nx - dx / 2, ny).astype(real_t)
        z = np.linspace(dx / 2, nz / nx - dx / 2, nz).astype(real_t)
        pos = np.flipud(np.array(np.meshgrid(z, y, x, indexing="ij")))
        rec.put(f"{tag}/position", pos)
        for width in (0, 2):
            out = vec.copy()
            spne.gen_penalise_field_boundary_pyst_kernel_3d(
                width=width, dx=dx, x_grid_field=pos[0], y_grid_field=pos[1],
                z_grid_field=pos[2], real_t=real_t, field_type="vector")(vector_field=out)
            rec.put(f"{tag}/penalise_w{width}", out)
        for ftype, order in (("multiplicative", 2), ("convolution", 1), ("convolution", 3)):
            out = vec.copy()
            flux_buf = rng.standard_normal(shape).astype(real_t)
            field_buf = rng.standard_normal(shape).astype(real_t)
            spne.gen_laplacian_filter_kernel_3d(
                filter_order=order, filter_flux_buffer=flux_buf, field_buffer=field_buf,
                real_t=real_t, field_type="vector", filter_type=ftype)(vector_field=out)
            rec.put(f"{tag}/filter_{ftype}_{order}", out)


def poisson_3d(spne, real_t, rec: _Recorder, seed: int) -> None:
    rng = np.random.default_rng(seed)
    for tag, (nz, ny, nx, x_range) in (("cube", (8, 8, 8, 1.0)), ("rect", (6, 8, 12, 1.5))):
        rhs = rng.standard_normal((3, nz, ny, nx)).astype(real_t)
        solver = spne.UnboundedPoissonSolverPYFFTW3D(
            grid_size_z=nz, grid_size_y=ny, grid_size_x=nx, x_range=x_range, real_t=real_t)
        sol = np.zeros_like(rhs)
        solver.vector_field_solve(solution_vector_field=sol, rhs_vector_field=rhs)
        rec.put(f"{tag}/rhs", rhs)
        rec.put(f"{tag}/solution", sol)
        rec.put(f"{tag}/meta", [nz, ny, nx, x_range])


def ns_3d(sps, real_t, rec: _Recorder, seed: int) -> None:
    """One full step of the 3D simulator (navier_stokes_flow_simulators.py:449-498)."""
    rng = np.random.default_rng(seed)
    cases = (
        ("a", (10, 10, 10), 1.0, 1e-2, True, 1.0, None),
        ("b", (8, 10, 12), 1.0, 2e-3, True, 0.5, None),
        ("c", (8, 8, 12), 1.5, 1e-2, False, 1.0, {"order": 2, "type": "multiplicative"}),
        ("d", (10, 10, 10), 1.0, 1e-2, True, 1.0, {"order": 3, "type": "convolution"}),
    )
    for tag, grid, x_range, nu, free_stream, rho, filt in cases:
        kwargs = {}
        if filt is not None:
            kwargs = {"filter_vorticity": True, "filter_setting_dict": filt}
        sim = sps.UnboundedNavierStokesFlowSimulator3D(
            grid_size=grid, x_range=x_range, kinematic_viscosity=nu, real_t=real_t,
            with_forcing=True, with_free_stream_flow=free_stream, flow_density=rho, **kwargs)
        sim.vorticity_field[...] = rng.standard_normal((3, *grid)).astype(real_t)
        sim.velocity_field[...] = rng.standard_normal((3, *grid)).astype(real_t)
        sim.eul_grid_forcing_field[...] = rng.standard_normal((3, *grid)).astype(real_t)
        rec.put(f"{tag}/vorticity_in", sim.vorticity_field)
        rec.put(f"{tag}/velocity_in", sim.velocity_field)
        rec.put(f"{tag}/forcing_in", sim.eul_grid_forcing_field)
        rec.put(f"{tag}/divergence_l2", sim.get_vorticity_divergence_l2_norm())
        dt = sim.compute_stable_timestep()
        rec.put(f"{tag}/stable_dt", dt)
        dt = 0.5 * dt
        u_inf = np.array([0.6, -0.1, 0.3])
        sim.time_step(dt=dt, free_stream_velocity=u_inf)
        order = -1 if filt is None else filt["order"]
        ftype = 0 if filt is None else (1 if filt["type"] == "multiplicative" else 2)
        rec.put(f"{tag}/meta", [*grid, x_range, nu, float(free_stream), rho, dt, *u_inf, order, ftype])
        rec.put(f"{tag}/vorticity_out", sim.vorticity_field)
        rec.put(f"{tag}/velocity_out", sim.velocity_field)
        rec.put(f"{tag}/stream_func_out", sim.stream_func_field)


# ----------------------------------------------------------------------------
# immersed boundary
# ----------------------------------------------------------------------------


def ib_ops(spib, real_t, rec: _Recorder, seed: int) -> None:
    """VirtualBoundaryForcing on random markers (VirtualBoundaryForcing.py:20-283)."""
    rng = np.random.default_rng(seed)
    for dim, grid in ((2, (16, 20)), (3, (12, 12, 14))):
        nx = grid[-1]
        dx = real_t(1.0 / nx)
        n_lag = 7
        extent = np.array([g * dx for g in grid[::-1]])  # (x, y[, z]) extents
        for kernel in ("cosine", "peskin"):
            tag = f"d{dim}_{kernel}"
            vbf = spib.VirtualBoundaryForcing(
                virtual_boundary_stiffness_coeff=-3.0e2, virtual_boundary_damping_coeff=-1.5,
                grid_dim=dim, dx=dx, num_lag_nodes=n_lag, real_t=real_t,
                enable_eul_grid_forcing_reset=False)
            if kernel == "peskin":
                comm = vbf.eul_lag_grid_communicator
                mod = sys.modules[type(comm).__module__]
                gen = getattr(mod, f"generate_peskin_interpolation_weights_kernel_{dim}d")
                comm.interpolation_weights_kernel = gen(dx=dx, interp_kernel_width=2, real_t=real_t)
            pos = (0.3 + 0.4 * rng.random((dim, n_lag))) * extent.reshape(dim, 1)
            pos[:, 0] = (np.array([5, 6, 5][:dim]) + 0.5) * dx  # exactly on a node
            lag_vel = rng.standard_normal((dim, n_lag))
            eul_vel = rng.standard_normal((dim, *grid)).astype(real_t)
            eul_force = rng.standard_normal((dim, *grid)).astype(real_t)
            vbf.lag_grid_position_mismatch_field[...] = rng.standard_normal((dim, n_lag))
            rec.put(f"{tag}/position", pos)
            rec.put(f"{tag}/lag_velocity", lag_vel)
            rec.put(f"{tag}/eul_velocity", eul_vel)
            rec.put(f"{tag}/eul_forcing_in", eul_force)
            rec.put(f"{tag}/position_mismatch_in", vbf.lag_grid_position_mismatch_field)
            vbf.compute_interaction_forcing(
                eul_grid_forcing_field=eul_force, eul_grid_velocity_field=eul_vel,
                lag_grid_position_field=pos, lag_grid_velocity_field=lag_vel)
            rec.put(f"{tag}/nearest_index", vbf.nearest_eul_grid_index_to_lag_grid)
            rec.put(f"{tag}/weights", vbf.interp_weights)
            rec.put(f"{tag}/lag_flow_velocity", vbf.lag_grid_flow_velocity_field)
            rec.put(f"{tag}/velocity_mismatch", vbf.lag_grid_velocity_mismatch_field)
            rec.put(f"{tag}/lag_forcing", vbf.lag_grid_forcing_field)
            rec.put(f"{tag}/eul_forcing_out", eul_force)
            vbf.time_step(dt=0.01)
            rec.put(f"{tag}/position_mismatch_out", vbf.lag_grid_position_mismatch_field)
            rec.put(f"{tag}/meta", [dim, *grid, n_lag, -3.0e2, -1.5, 0.01])


class _FakeCylinder:
    """Fixed cylinder with the attributes the reference forcing grid reads."""

    def __init__(self, centre, radius) -> None:
        self.position_collection = np.array(centre, dtype=float).reshape(3, 1)
        self.director_collection = np.eye(3).reshape(3, 3, 1)
        self.velocity_collection = np.zeros((3, 1))
        self.omega_collection = np.zeros((3, 1))
        self.radius = radius


def cylinder_2d(sps, real_t, rec: _Recorder, seed: int) -> None:
    """A few coupled steps of the flow-past-cylinder loop (flow_past_cylinder.py:129-136)."""
    rng = np.random.default_rng(seed)
    grid = (32, 64)
    x_range = 1.0
    radius = 0.08
    nu = 2.0 * radius * 1.0 / 200.0
    sim = sps.UnboundedNavierStokesFlowSimulator2D(
        grid_size=grid, x_range=x_range, kinematic_viscosity=nu, real_t=real_t,
        with_forcing=True, with_free_stream_flow=True)
    sim.vorticity_field[...] = (1e-3 * rng.standard_normal(grid)).astype(real_t)
    cyl = _FakeCylinder([0.25, 0.25, 0.0], radius)
    n_markers = 24
    inter = sps.RigidBodyFlowInteraction(
        rigid_body=cyl, eul_grid_forcing_field=sim.eul_grid_forcing_field,
        eul_grid_velocity_field=sim.velocity_field, virtual_boundary_stiffness_coeff=-5e4,
        virtual_boundary_damping_coeff=-20.0, dx=sim.dx, grid_dim=2, real_t=real_t,
        forcing_grid_cls=sps.CircularCylinderForcingGrid, num_forcing_points=n_markers)
    rec.put("vorticity_init", sim.vorticity_field)
    rec.put("marker_position", inter.forcing_grid.position_field)
    u_inf = np.array([1.0, 0.0])
    dts, drags = [], []
    for step in range(4):
        dt = sim.compute_stable_timestep()
        inter.time_step(dt=dt)
        inter()
        sim.time_step(dt=dt, free_stream_velocity=u_inf)
        dts.append(dt)
        drags.append(np.sum(inter.lag_grid_forcing_field[0]))
        rec.put(f"step{step}/vorticity", sim.vorticity_field)
        rec.put(f"step{step}/velocity", sim.velocity_field)
        rec.put(f"step{step}/lag_forcing", inter.lag_grid_forcing_field)
        rec.put(f"step{step}/position_mismatch", inter.lag_grid_position_mismatch_field)
    rec.put("dt", dts)
    rec.put("drag", drags)
    rec.put("grid_deviation", inter.get_grid_deviation_error_l2_norm())
    inter.compute_flow_forces_and_torques()
    rec.put("body_forces", inter.body_flow_forces)
    rec.put("body_torques", inter.body_flow_torques)
    rec.put("meta", [grid[0], grid[1], x_range, nu, radius, n_markers, 0.25, 0.25, -5e4, -20.0])


class _FakeRod:
    """Straight rod with the attributes the reference rod forcing grids read."""

    def __init__(self, rng, n_elems: int) -> None:
        self.n_elems = n_elems
        s = np.linspace(0.0, 0.3, n_elems + 1)
        self.position_collection = np.stack(
            [0.35 + 0.01 * np.sin(7 * s), 0.5 + 0.0 * s, 0.35 + s])
        self.position_collection += 1e-3 * rng.standard_normal(self.position_collection.shape)
        self.velocity_collection = 0.1 * rng.standard_normal((3, n_elems + 1))
        self.mass = 1.0 + 0.1 * rng.random(n_elems + 1)
        self.lengths = np.linalg.norm(np.diff(self.position_collection, axis=1), axis=0)
        th = 0.2 * rng.standard_normal(n_elems)
        d = np.zeros((3, 3, n_elems))
        d[0, 0] = np.cos(th)
        d[0, 1] = np.sin(th)
        d[1, 0] = -np.sin(th)
        d[1, 1] = np.cos(th)
        d[2, 2] = 1.0
        self.director_collection = d


def rod_3d(sps, real_t, rec: _Recorder, seed: int) -> None:
    """Rod forcing grids (cosserat_rod_forcing_grids.py:10-130) on a random 3D flow."""
    rng = np.random.default_rng(seed)
    grid = (16, 16, 16)
    dx = real_t(1.0 / 16)
    eul_vel = rng.standard_normal((3, *grid)).astype(real_t)
    rec.put("eul_velocity", eul_vel)
    for name, cls in (("nodal", sps.CosseratRodNodalForcingGrid),
                      ("element", sps.CosseratRodElementCentricForcingGrid)):
        rod = _FakeRod(rng, 10)
        force = np.zeros((3, *grid), dtype=real_t)
        inter = sps.CosseratRodFlowInteraction(
            cosserat_rod=rod, eul_grid_forcing_field=force, eul_grid_velocity_field=eul_vel,
            virtual_boundary_stiffness_coeff=-2e4, virtual_boundary_damping_coeff=-1e2, dx=dx,
            grid_dim=3, real_t=real_t, forcing_grid_cls=cls)
        rec.put(f"{name}/rod_position", rod.position_collection)
        rec.put(f"{name}/rod_velocity", rod.velocity_collection)
        rec.put(f"{name}/rod_mass", rod.mass)
        rec.put(f"{name}/rod_directors", rod.director_collection)
        inter.time_step(dt=1e-3)
        inter()
        rec.put(f"{name}/eul_forcing_out", force)
        rec.put(f"{name}/lag_forcing", inter.lag_grid_forcing_field)
        inter.lag_grid_position_mismatch_field[...] = 1e-3 * rng.standard_normal(
            inter.lag_grid_position_mismatch_field.shape)
        rec.put(f"{name}/position_mismatch_in", inter.lag_grid_position_mismatch_field)
        inter.compute_flow_forces_and_torques()
        rec.put(f"{name}/body_forces", inter.body_flow_forces)
        rec.put(f"{name}/body_torques", inter.body_flow_torques)
        rec.put(f"{name}/lag_forcing_after", inter.lag_grid_forcing_field)


def passive(sps, real_t, rec: _Recorder, seed: int) -> None:
    """3D ENO3 advection (advection_flux_3d.py, advection_timestep_3d.py) and steps of the passive
    transport simulator (passive_transport_flow_simulators.py:14-155)."""
    import sopht.numeric.eulerian_grid_ops as spne
    rng = np.random.default_rng(seed)
    for tag, shape in (("cube", (10, 10, 10)), ("rect", (8, 10, 12))):
        field = rng.standard_normal(shape).astype(real_t)
        vel = rng.standard_normal((3, *shape)).astype(real_t)
        vec = rng.standard_normal((3, *shape)).astype(real_t)
        flux_in = rng.standard_normal(shape).astype(real_t)  # the flux kernel accumulates into its buffer
        rec.put(f"{tag}/field", field)
        rec.put(f"{tag}/velocity", vel)
        rec.put(f"{tag}/vector_field", vec)
        rec.put(f"{tag}/flux_in", flux_in)
        out = flux_in.copy()
        spne.gen_advection_flux_conservative_eno3_pyst_kernel_3d(real_t=real_t)(
            advection_flux=out, field=field, velocity=vel, inv_dx=real_t(0.7))
        rec.put(f"{tag}/flux_out", out)
        out = field.copy()
        spne.gen_advection_timestep_euler_forward_conservative_eno3_pyst_kernel_3d(real_t=real_t)(
            out, advection_flux=rng.standard_normal(shape).astype(real_t), velocity=vel, dt_by_dx=real_t(0.3))
        rec.put(f"{tag}/advection_step", out)
        out = vec.copy()
        spne.gen_advection_timestep_euler_forward_conservative_eno3_pyst_kernel_3d(
            real_t=real_t, field_type="vector")(
            out, advection_flux=np.zeros(shape, real_t), velocity=vel, dt_by_dx=real_t(0.3))
        rec.put(f"{tag}/advection_step_vector", out)
    for tag, dim, grid, ftype in (("s2d", 2, (12, 16), "scalar"), ("s3d", 3, (8, 10, 12), "scalar"),
                                  ("v3d", 3, (8, 8, 10), "vector")):
        sim = sps.PassiveTransportFlowSimulator(kinematic_viscosity=1e-2, grid_dim=dim, grid_size=grid,
                                                x_range=1.0, cfl=0.2, real_t=real_t, time=0.5, field_type=ftype)
        sim.velocity_field[...] = rng.standard_normal(sim.velocity_field.shape).astype(real_t)
        sim.primary_field[...] = rng.random(sim.primary_field.shape).astype(real_t)
        rec.put(f"sim_{tag}/velocity", sim.velocity_field)
        rec.put(f"sim_{tag}/primary_in", sim.primary_field)
        dts = []
        for step in range(3):
            dt = sim.compute_stable_timestep(dt_prefac=0.8)
            sim.time_step(dt=dt)
            dts.append(dt)
            rec.put(f"sim_{tag}/primary_step{step}", sim.primary_field)
        rec.put(f"sim_{tag}/dt", np.array(dts))
        rec.put(f"sim_{tag}/time_out", sim.time)


def _random_directors(rng) -> np.ndarray:
    """Rows d1, d2, d3 of a random proper rotation, shaped (3, 3, 1)."""
    q, _ = np.linalg.qr(rng.standard_normal((3, 3)))
    if np.linalg.det(q) < 0:
        q[2] *= -1.0
    return q.reshape(3, 3, 1)


class _FakeRigid3D:
    """Moving 3D rigid body with the attributes the reference forcing grids read."""

    def __init__(self, rng, radius: float, length: float = 0.0) -> None:
        self.position_collection = (0.5 + 0.01 * rng.standard_normal(3)).reshape(3, 1)
        self.director_collection = _random_directors(rng)
        self.velocity_collection = 0.1 * rng.standard_normal((3, 1))
        self.omega_collection = rng.standard_normal((3, 1))
        self.radius = radius
        self.length = length


class _FakeTaperedRod(_FakeRod):
    """``_FakeRod`` with a tapered radius, unit tangents and angular velocities."""

    def __init__(self, rng, n_elems: int, taper: float) -> None:
        super().__init__(rng, n_elems)
        self.radius = 0.02 * np.linspace(1.0, 1.0 / taper, n_elems)
        diff = np.diff(self.position_collection, axis=1)
        self.tangents = diff / np.linalg.norm(diff, axis=0)
        self.omega_collection = rng.standard_normal((3, n_elems))
        self.director_collection = np.concatenate(
            [_random_directors(rng) for _ in range(n_elems)], axis=2)


def _record_grid(rec: _Recorder, tag: str, grid, rng, n_forces: int, n_torques: int, extra=()) -> None:
    rec.put(f"{tag}/num_lag_nodes", grid.num_lag_nodes)
    rec.put(f"{tag}/position", grid.position_field)
    rec.put(f"{tag}/velocity", grid.velocity_field)
    rec.put(f"{tag}/spacing", grid.get_maximum_lagrangian_grid_spacing())
    for name in extra:
        value = getattr(grid, name)
        if isinstance(value, list):
            for i, v in enumerate(value):
                rec.put(f"{tag}/{name}/{i}", v)
        else:
            rec.put(f"{tag}/{name}", value)
    f = rng.standard_normal(grid.position_field.shape)
    forces, torques = np.zeros((3, n_forces)), np.zeros((3, n_torques))
    grid.transfer_forcing_from_grid_to_body(body_flow_forces=forces, body_flow_torques=torques,
                                            lag_grid_forcing_field=f)
    rec.put(f"{tag}/lag_forcing_in", f)
    rec.put(f"{tag}/body_forces", forces)
    rec.put(f"{tag}/body_torques", torques)


def forcing_grids(sps, real_t, rec: _Recorder, seed: int) -> None:
    """The 3D rigid-body grids (rigid_body_forcing_grids.py:108-349), the plane body
    (derived_rigid_bodies.py:12-63), the rod edge and surface grids
    (cosserat_rod_forcing_grids.py:134-589), and two 3D interactions using them."""
    rng = np.random.default_rng(seed)
    bodies = {}
    for tag, cls, make, kw in (
            ("sphere16", sps.SphereForcingGrid, lambda: _FakeRigid3D(rng, 0.15),
             {"num_forcing_points_along_equator": 16}),
            ("sphere7", sps.SphereForcingGrid, lambda: _FakeRigid3D(rng, 0.1),
             {"num_forcing_points_along_equator": 7}),
            ("open_cylinder", sps.OpenEndCircularCylinderForcingGrid, lambda: _FakeRigid3D(rng, 0.1, 0.4),
             {"num_forcing_points_along_length": 8}),
            ("plane", sps.RectangularPlaneForcingGrid,
             lambda: sps.RectangularPlane(origin=np.array([0.5, 0.4, 0.6]), plane_normal=np.array([0.2, 0.1, 1.0]),
                                          plane_tangent_along_length=np.array([1.0, 0.0, -0.2]),
                                          plane_length=0.4, plane_breadth=0.25),
             {"num_forcing_points_along_length": 10})):
        body = make()
        if tag == "plane":
            rec.put("plane/directors_as_built", body.director_collection)
            body.velocity_collection[...] = 0.1 * rng.standard_normal((3, 1))
            body.omega_collection[...] = rng.standard_normal((3, 1))
        grid = cls(grid_dim=3, rigid_body=body, **kw)
        # the grid follows the body: move it and recompute
        body.position_collection += 0.01
        body.velocity_collection *= -1.5
        grid.compute_lag_grid_position_field()
        grid.compute_lag_grid_velocity_field()
        bodies[tag] = body
        rec.put(f"{tag}/body_position", body.position_collection)
        rec.put(f"{tag}/body_directors", body.director_collection)
        rec.put(f"{tag}/body_velocity", body.velocity_collection)
        rec.put(f"{tag}/body_omega", body.omega_collection)
        rec.put(f"{tag}/body_radius", getattr(body, "radius", 0.0))
        rec.put(f"{tag}/body_length", getattr(body, "length", 0.0))
        _record_grid(rec, tag, grid, rng, 1, 1)
    rod_cases = (("edge", 2, 10, 2.0, {}),
                 ("surface_cap", 3, 8, 3.0, {"surface_grid_density_for_largest_element": 12, "with_cap": True}),
                 ("surface_nocap", 3, 8, 5.0, {"surface_grid_density_for_largest_element": 8, "with_cap": False}),
                 ("surface_one", 3, 1, 1.0, {"surface_grid_density_for_largest_element": 16, "with_cap": True}))
    for tag, dim, n_elems, taper, kw in rod_cases:
        rod = _FakeTaperedRod(rng, n_elems, taper)
        if tag == "edge":
            grid = sps.CosseratRodEdgeForcingGrid(grid_dim=dim, cosserat_rod=rod)
            extra = ("moment_arm",)
        else:
            grid = sps.CosseratRodSurfaceForcingGrid(grid_dim=dim, cosserat_rod=rod, **kw)
            extra = ("surface_grid_points", "start_idx", "end_idx", "grid_point_radius_ratio",
                     "local_frame_surface_points", "moment_arm", "surface_point_rotation_angle_list")
        for name in ("position_collection", "velocity_collection", "omega_collection", "director_collection",
                     "mass", "radius", "lengths", "tangents"):
            rec.put(f"{tag}/rod_{name}", getattr(rod, name))
        _record_grid(rec, tag, grid, rng, n_elems + 1, n_elems, extra)
    # 3D interactions through the grids (immersed_body_flow_interaction.py:15-141)
    grid_shape = (16, 16, 16)
    dx = real_t(1.0 / 16)
    eul_vel = rng.standard_normal((3, *grid_shape)).astype(real_t)
    rec.put("eul_velocity", eul_vel)
    sphere = _FakeRigid3D(rng, 0.2)
    rod = _FakeTaperedRod(rng, 6, 2.0)
    rod.radius = 0.06 * np.linspace(1.0, 0.5, 6)
    for tag, make in (
            ("sphere_inter", lambda force: sps.RigidBodyFlowInteraction(
                rigid_body=sphere, eul_grid_forcing_field=force, eul_grid_velocity_field=eul_vel,
                virtual_boundary_stiffness_coeff=-2e4, virtual_boundary_damping_coeff=-1e2, dx=dx, grid_dim=3,
                real_t=real_t, forcing_grid_cls=sps.SphereForcingGrid, num_forcing_points_along_equator=20)),
            ("surface_inter", lambda force: sps.CosseratRodFlowInteraction(
                cosserat_rod=rod, eul_grid_forcing_field=force, eul_grid_velocity_field=eul_vel,
                virtual_boundary_stiffness_coeff=-2e4, virtual_boundary_damping_coeff=-1e2, dx=dx, grid_dim=3,
                real_t=real_t, forcing_grid_cls=sps.CosseratRodSurfaceForcingGrid,
                surface_grid_density_for_largest_element=6, with_cap=True))):
        force = np.zeros((3, *grid_shape), dtype=real_t)
        inter = make(force)
        inter.time_step(dt=1e-3)
        inter()
        rec.put(f"{tag}/eul_forcing_out", force)
        rec.put(f"{tag}/lag_forcing", inter.lag_grid_forcing_field)
        inter.compute_flow_forces_and_torques()
        rec.put(f"{tag}/body_forces", inter.body_flow_forces)
        rec.put(f"{tag}/body_torques", inter.body_flow_torques)
    for name in ("position_collection", "velocity_collection", "omega_collection", "director_collection"):
        rec.put(f"sphere_inter/body_{name}", getattr(sphere, name))
        rec.put(f"surface_inter/rod_{name}", getattr(rod, name))
    for name in ("mass", "radius", "lengths", "tangents"):
        rec.put(f"surface_inter/rod_{name}", getattr(rod, name))
    rec.put("sphere_inter/body_radius", sphere.radius)
    # a 2D interaction through the edge grid: a tapered rod lying in the XY plane
    grid_2d = (32, 48)
    dx = real_t(1.0 / 48)
    eul_vel_2d = rng.standard_normal((2, *grid_2d)).astype(real_t)
    rod = _FakeTaperedRod(rng, 12, 2.0)
    s = np.linspace(0.0, 0.4, 13)
    rod.position_collection = np.stack([0.3 + s, 0.33 + 0.02 * np.sin(9 * s), 0.0 * s])
    diff = np.diff(rod.position_collection, axis=1)
    rod.lengths = np.linalg.norm(diff, axis=0)
    rod.tangents = diff / rod.lengths
    rod.radius = 0.03 * np.linspace(1.0, 0.5, 12)
    force = np.zeros((2, *grid_2d), dtype=real_t)
    inter = sps.CosseratRodFlowInteraction(
        cosserat_rod=rod, eul_grid_forcing_field=force, eul_grid_velocity_field=eul_vel_2d,
        virtual_boundary_stiffness_coeff=-5e4, virtual_boundary_damping_coeff=-20.0, dx=dx, grid_dim=2,
        real_t=real_t, forcing_grid_cls=sps.CosseratRodEdgeForcingGrid)
    inter.time_step(dt=1e-3)
    inter()
    rec.put("edge_inter/eul_velocity", eul_vel_2d)
    rec.put("edge_inter/eul_forcing_out", force)
    rec.put("edge_inter/lag_forcing", inter.lag_grid_forcing_field)
    inter.compute_flow_forces_and_torques()
    rec.put("edge_inter/body_forces", inter.body_flow_forces)
    rec.put("edge_inter/body_torques", inter.body_flow_torques)
    for name in ("position_collection", "velocity_collection", "omega_collection", "director_collection",
                 "mass", "radius", "lengths", "tangents"):
        rec.put(f"edge_inter/rod_{name}", getattr(rod, name))


def forcing_grids_random(sps, real_t, rec: _Recorder, seed: int) -> None:
    """Randomised cases of every 3D rigid-body and tapered-rod forcing grid: sizes, marker
    counts, tapers, cap flags and body states drawn at random (including one-element rods,
    one-point rings and densities below 3), with the reference's geometry, kinematics and
    force/torque transfer for a random forcing."""
    rng = np.random.default_rng(seed)
    body_names = ("position_collection", "director_collection", "velocity_collection", "omega_collection")
    rod_names = ("position_collection", "velocity_collection", "omega_collection", "director_collection",
                 "mass", "radius", "lengths", "tangents")
    for i in range(12):
        radius, length, breadth = rng.uniform(0.01, 0.3), rng.uniform(0.05, 1.0), rng.uniform(0.05, 1.0)
        for kind, cls, key, hi in (("sphere", sps.SphereForcingGrid, "num_forcing_points_along_equator", 40),
                                   ("open_cylinder", sps.OpenEndCircularCylinderForcingGrid,
                                    "num_forcing_points_along_length", 24),
                                   ("plane", sps.RectangularPlaneForcingGrid, "num_forcing_points_along_length", 24)):
            body = _FakeRigid3D(rng, radius, length)
            body.breadth = breadth
            count = int(rng.integers(1, hi))
            grid = cls(grid_dim=3, rigid_body=body, **{key: count})
            tag = f"{kind}/{i}"
            for name in body_names:
                rec.put(f"{tag}/body_{name}", getattr(body, name))
            rec.put(f"{tag}/params", [radius, length, breadth, count])
            _record_grid(rec, tag, grid, rng, 1, 1)
        n_elems, taper = int(rng.integers(1, 13)), float(rng.uniform(1.0, 12.0))
        rod = _FakeTaperedRod(rng, n_elems, taper)
        grid = sps.CosseratRodEdgeForcingGrid(grid_dim=2, cosserat_rod=rod)
        for name in rod_names:
            rec.put(f"edge/{i}/rod_{name}", getattr(rod, name))
        _record_grid(rec, f"edge/{i}", grid, rng, n_elems + 1, n_elems)
        for kind, scale in (("surface", 1.0), ("surface_wide", 20.0)):  # wide: caps with several rings
            rod = _FakeTaperedRod(rng, n_elems, taper)
            rod.radius = rod.radius * scale
            density, cap = int(rng.integers(1, 24)), bool(rng.integers(0, 2))
            grid = sps.CosseratRodSurfaceForcingGrid(grid_dim=3, cosserat_rod=rod,
                                                     surface_grid_density_for_largest_element=density, with_cap=cap)
            tag = f"{kind}/{i}"
            for name in rod_names:
                rec.put(f"{tag}/rod_{name}", getattr(rod, name))
            rec.put(f"{tag}/params", [density, int(cap)])
            _record_grid(rec, tag, grid, rng, n_elems + 1, n_elems, ("surface_grid_points",))


def field_io(sps, real_t, rec: _Recorder, seed: int) -> None:
    """The HDF5 + XDMF field IO (sopht/utils/io.py:13-694) through the in-memory h5py
    stand-in: the saved tree (datasets, attributes) and the XDMF text of three cases."""
    import os
    import tempfile

    import memory_h5
    import sopht.utils.io as ref_io
    ref_io.h5py = memory_h5
    rng = np.random.default_rng(seed)
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as tmp:
        os.chdir(tmp)
        try:
            # 3D: scalar and vector Eulerian fields, a named and an unnamed (connected) Lagrangian grid
            grid = np.array([8, 10, 12])
            io = ref_io.IO(dim=3, real_dtype=real_t)
            origin, dx = np.array([0.1, 0.2, 0.3]), np.array([0.05, 0.05, 0.05])
            io.define_eulerian_grid(origin=origin, dx=dx, grid_size=grid)
            eul = {"vorticity_mag": rng.standard_normal(tuple(grid)).astype(real_t),
                   "velocity": rng.standard_normal((3, *grid)).astype(real_t)}
            io.add_as_eulerian_fields_for_io(**eul)
            lag = {"sphere_grid": rng.standard_normal((3, 20)), "radius_field": rng.standard_normal(20),
                   "forcing": rng.standard_normal((3, 20)), "rod_grid": rng.standard_normal((3, 7)),
                   "rod_velocity": rng.standard_normal((3, 7))}
            io.add_as_lagrangian_fields_for_io(lagrangian_grid=lag["sphere_grid"], lagrangian_grid_name="sphere",
                                               radius_field=lag["radius_field"], forcing=lag["forcing"])
            io.add_as_lagrangian_fields_for_io(lagrangian_grid=lag["rod_grid"], lagrangian_grid_connect=True,
                                               rod_velocity=lag["rod_velocity"])
            io.save(h5_file_name="sopht_0003.h5", time=0.125)
            for k, v in {**eul, **lag}.items():
                rec.put(f"eul3d/in/{k}", v)
            for k, v in memory_h5.dump("sopht_0003.h5").items():
                rec.put(f"eul3d/h5/{k}", v)
            for name in ("eulerian", "sphere", "Lagrangian_grid_0"):
                rec.put(f"eul3d/xmf/{name}", Path(f"sopht_0003_{name}.xmf").read_text())
            # 2D, from a simulator-style position field
            ny, nx = 6, 10
            h = 1.0 / nx
            axes = [np.linspace(h / 2, n * h - h / 2, n).astype(real_t) for n in (ny, nx)]
            position = np.flipud(np.array(np.meshgrid(*axes, indexing="ij")))
            fields = {"vorticity": rng.standard_normal((ny, nx)).astype(real_t),
                      "velocity": rng.standard_normal((2, ny, nx)).astype(real_t)}
            io = ref_io.EulerianFieldIO(position_field=position, eulerian_fields_dict=fields)
            io.save(h5_file_name="flow_0001.h5", time=2.5)
            rec.put("eul2d/in/position", position)
            for k, v in fields.items():
                rec.put(f"eul2d/in/{k}", v)
            for k, v in memory_h5.dump("flow_0001.h5").items():
                rec.put(f"eul2d/h5/{k}", v)
            rec.put("eul2d/xmf/eulerian", Path("flow_0001_eulerian.xmf").read_text())
            # a rod
            rod = _FakeTaperedRod(rng, 9, 2.0)
            io = ref_io.CosseratRodIO(cosserat_rod=rod, dim=3, real_dtype=real_t)
            rod.position_collection += 0.01  # save reads the rod as it is then
            io.save(h5_file_name="rod_0007.h5", time=1.0)
            rec.put("rod/in/position_collection", rod.position_collection)
            rec.put("rod/in/radius", rod.radius)
            for k, v in memory_h5.dump("rod_0007.h5").items():
                rec.put(f"rod/h5/{k}", v)
            rec.put("rod/xmf/rod", Path("rod_0007_rod.xmf").read_text())
        finally:
            os.chdir(cwd)


GROUPS = {
    "stencils2d": ("spne", stencils_2d, 11),
    "poisson2d": ("spne", poisson_2d, 12),
    "ns2d": ("sps", ns_2d, 13),
    "stencils3d": ("spne", stencils_3d, 21),
    "poisson3d": ("spne", poisson_3d, 22),
    "ns3d": ("sps", ns_3d, 23),
    "ib": ("spib", ib_ops, 31),
    "cylinder2d": ("sps", cylinder_2d, 32),
    "rod3d": ("sps", rod_3d, 33),
    "passive": ("sps", passive, 41),
    "grids": ("sps", forcing_grids, 42),
    "io": ("sps", field_io, 43),
    "gridsrandom": ("sps", forcing_grids_random, 44),
}
HOST_ONLY = {"gridsrandom"}


def _load_test_restatements(ref_root: str, rel: str, ns: dict | None = None) -> dict:
    """Load the numpy restatement functions from one reference test file.

    Only top-level ``def``s that are not ``test_*`` are executed, with numpy,
    scipy.fft and the reference's precision helpers in scope; the pytest
    fixtures and sopht imports of the file are skipped.  Passing the namespace
    of an earlier file lets this file's restatements call that file's.
    """
    import ast

    from scipy.fft import irfftn, rfftn

    src = (Path(ref_root) / "tests" / rel).read_text()
    if ns is None:
        ns = {"np": np, "rfftn": rfftn, "irfftn": irfftn}
    for node in ast.parse(src).body:
        if isinstance(node, ast.FunctionDef) and not node.name.startswith("test_"):
            exec(compile(ast.Module([node], []), rel, "exec"), ns)
    return ns


def validate_shims(ref_root: str, spne) -> None:
    """Check the stand-ins against the reference tests' own numpy restatements.

    Each reference kernel run through ``ref_shims`` must agree with the
    restatement in the corresponding reference test file to the tolerance those
    tests use (1e3 machine epsilons, absolute).
    """
    t2 = "test_numeric/test_eulerian_grid_ops/test_stencil_ops_2d/"
    t3 = "test_numeric/test_eulerian_grid_ops/test_stencil_ops_3d/"
    rng = np.random.default_rng(42)
    checked = 0
    for real_t in (np.float32, np.float64):
        tol = real_t(1e3) * np.finfo(real_t).eps
        n = 16
        f = rng.standard_normal((n, n)).astype(real_t)
        v = rng.standard_normal((2, n, n)).astype(real_t)

        def close(a, b):
            nonlocal checked
            np.testing.assert_allclose(a, b, atol=tol)
            checked += 1

        ns = _load_test_restatements(ref_root, t2 + "test_advection_flux_2d.py")
        out = np.zeros_like(f)
        spne.gen_advection_flux_conservative_eno3_pyst_kernel_2d(real_t=real_t)(
            advection_flux=out, field=f, velocity=v, inv_dx=real_t(0.1))
        close(out, ns["advection_flux_conservative_eno_ord3_reference"](f, v[0], v[1], real_t(0.1), real_t))
        ns = _load_test_restatements(ref_root, t2 + "test_diffusion_timestep_2d.py")
        ns.update(_load_test_restatements(ref_root, t2 + "test_diffusion_flux_2d.py"))
        out = f.copy()
        spne.gen_diffusion_timestep_euler_forward_pyst_kernel_2d(real_t=real_t)(
            field=out, diffusion_flux=np.zeros_like(f), nu_dt_by_dx2=real_t(0.1))
        close(out, ns["diffusion_timestep_euler_forward_reference"](f, real_t(0.1), real_t))
        ns = _load_test_restatements(ref_root, t2 + "test_outplane_field_curl_2d.py")
        out = np.zeros_like(v)
        spne.gen_outplane_field_curl_pyst_kernel_2d(real_t=real_t)(curl=out, field=f, prefactor=real_t(0.3))
        close(out, ns["outplane_curl_reference"](f, real_t(0.3), real_t))
        ns = _load_test_restatements(ref_root, t2 + "test_update_vorticity_from_velocity_forcing_2d.py")
        out = f.copy()
        spne.gen_update_vorticity_from_velocity_forcing_pyst_kernel_2d(real_t=real_t)(
            vorticity_field=out, velocity_forcing_field=v, prefactor=real_t(0.2))
        close(out[1:-1, 1:-1], ns["update_vorticity_from_velocity_forcing_reference"](f, v, real_t(0.2))[1:-1, 1:-1])
        ns = _load_test_restatements(ref_root, t2 + "test_penalise_field_boundary_2d.py")
        dx = real_t(1.0 / n)
        x = np.linspace(dx / 2, 1 - dx / 2, n).astype(real_t)
        pos = np.flipud(np.array(np.meshgrid(x, x, indexing="ij")))
        for width in (2, 3):
            out = f.copy()
            spne.gen_penalise_field_boundary_pyst_kernel_2d(
                width=width, dx=dx, x_grid_field=pos[0], y_grid_field=pos[1], real_t=real_t)(field=out)
            ref = f.copy()
            ns["penalise_field_boundary_reference"](ref, f, pos[0], pos[1], width, dx)
            close(out, ref)
        # 3D
        m = 8
        w3 = rng.standard_normal((3, m, m, m)).astype(real_t)
        g3 = rng.standard_normal((3, m, m, m)).astype(real_t)
        ns = _load_test_restatements(ref_root, t3 + "test_curl_3d.py")
        out = np.zeros_like(w3)
        spne.gen_curl_pyst_kernel_3d(real_t=real_t)(curl=out, field=w3, prefactor=real_t(0.5))
        close(out, np.stack(ns["curl_reference"](w3[0], w3[1], w3[2], real_t(0.5))))
        ns = _load_test_restatements(ref_root, t3 + "test_diffusion_timestep_3d.py")
        out = w3.copy()
        spne.gen_diffusion_timestep_euler_forward_pyst_kernel_3d(real_t=real_t, field_type="vector")(
            vector_field=out, diffusion_flux=np.zeros_like(w3[0]), nu_dt_by_dx2=real_t(0.1))
        close(out, np.stack([ns["diffusion_timestep_euler_forward_reference"](c, real_t(0.1), real_t) for c in w3]))
        ns = _load_test_restatements(ref_root, t3 + "test_advection_flux_3d.py")
        out = np.zeros_like(w3[0])
        spne.gen_advection_flux_conservative_eno3_pyst_kernel_3d(real_t=real_t)(
            advection_flux=out, field=w3[0], velocity=g3, inv_dx=real_t(0.1))
        close(out, ns["advection_flux_conservative_eno3_reference"](w3[0], g3[0], g3[1], g3[2], real_t(0.1),
                                                                    real_t))
        ns = _load_test_restatements(ref_root, t3 + "test_advection_timestep_3d.py", ns)
        out = w3[1].copy()
        spne.gen_advection_timestep_euler_forward_conservative_eno3_pyst_kernel_3d(real_t=real_t)(
            out, advection_flux=np.zeros_like(out), velocity=g3, dt_by_dx=real_t(0.02))
        close(out, ns["advection_timestep_conservative_eno3_euler_forward_reference"](
            w3[1], g3[0], g3[1], g3[2], real_t(0.2), real_t(0.1), real_t))
        ns = _load_test_restatements(ref_root, t3 + "test_divergence_3d.py")
        out = np.zeros_like(w3[0])
        spne.gen_divergence_pyst_kernel_3d(real_t=real_t)(divergence=out, field=w3, inv_dx=real_t(2.0))
        close(out, ns["divergence_reference"](w3, real_t(2.0)))
        ns = _load_test_restatements(ref_root, t3 + "test_update_vorticity_from_velocity_forcing_3d.py")
        out = w3.copy()
        spne.gen_update_vorticity_from_velocity_forcing_pyst_kernel_3d(real_t=real_t)(
            vorticity_field=out, velocity_forcing_field=g3, prefactor=real_t(0.2))
        ref = ns["update_vorticity_from_velocity_forcing_reference_3d"](w3, g3, real_t(0.2))
        close(out[:, 1:-1, 1:-1, 1:-1], ref[:, 1:-1, 1:-1, 1:-1])
        ns = _load_test_restatements(ref_root, t3 + "test_penalise_field_boundary_3d.py")
        dx = real_t(1.0 / m)
        x = np.linspace(dx / 2, 1 - dx / 2, m).astype(real_t)
        pos3 = np.flipud(np.array(np.meshgrid(x, x, x, indexing="ij")))
        out = w3[0].copy()
        spne.gen_penalise_field_boundary_pyst_kernel_3d(
            width=2, dx=dx, x_grid_field=pos3[0], y_grid_field=pos3[1], z_grid_field=pos3[2],
            real_t=real_t)(field=out)
        ref = w3[0].copy()
        ns["penalise_field_boundary_reference_3d"](ref, w3[0], pos3[0], pos3[1], pos3[2], 2, dx)
        close(out, ref)
        ns = _load_test_restatements(ref_root, t3 + "test_laplacian_filter_3d.py")
        for ftype, order in (("multiplicative", 2), ("convolution", 3)):
            out = w3.copy()
            spne.gen_laplacian_filter_kernel_3d(
                filter_order=order, filter_flux_buffer=np.zeros_like(w3[0]),
                field_buffer=np.zeros_like(w3[0]), real_t=real_t, field_type="vector",
                filter_type=ftype)(vector_field=out)
            ref = w3.copy()
            ns["vector_laplacian_filter"](ref, order, ftype)
            close(out, ref)
        # Poisson 2D: the reference test's scipy restatement
        ns = _load_test_restatements(
            ref_root, "test_numeric/test_eulerian_grid_ops/test_poisson_solver_2d/test_unbounded_poisson_solver_2d.py")
        rhs = rng.standard_normal((8, 16)).astype(real_t)
        solver = spne.UnboundedPoissonSolverPYFFTW2D(grid_size_y=8, grid_size_x=16, x_range=1.0, real_t=real_t)
        out = np.zeros_like(rhs)
        solver.solve(solution_field=out, rhs_field=rhs)
        from scipy.fft import irfftn, rfftn
        dx = real_t(1.0 / 16)
        xd = np.linspace(0, 2 - dx, 32).astype(real_t)
        yd = np.linspace(0, 1 - dx, 16).astype(real_t)
        xg, yg = np.meshgrid(xd, yd)
        r = np.sqrt(np.minimum(xg, 2 - xg) ** 2 + np.minimum(yg, 1 - yg) ** 2)
        with np.errstate(divide="ignore"):
            g = -np.log(r) / (2 * np.pi)
        g[0, 0] = -(2 * np.log(dx / np.sqrt(np.pi)) - 1) / (4 * np.pi)
        big = np.zeros((16, 32), real_t)
        big[:8, :16] = rhs
        ref = irfftn(rfftn(big) * rfftn(g) * dx**2)[:8, :16]
        close(out, ref)
    print(f"shim validation: {checked} reference-test restatements agree")


SIGNATURE_MODULES = ("sopht.simulator", "sopht.numeric.eulerian_grid_ops", "sopht.numeric.immersed_boundary_ops",
                     "sopht.utils")


def _params(sig):
    import inspect
    params = []
    for p in sig.parameters.values():
        if p.name == "self" or p.kind in (p.VAR_POSITIONAL, p.VAR_KEYWORD):
            continue
        params.append([p.name, None if p.default is inspect.Parameter.empty else repr(p.default)])
    return params


def write_signatures() -> None:
    """The parameter names and defaults of every public callable of the reference's API modules
    (classes: their constructors and public methods), as ``reference_signatures.json``."""
    import importlib
    import inspect
    import json
    out = {}
    for modname in SIGNATURE_MODULES:
        mod = importlib.import_module(modname)
        for name in sorted(getattr(mod, "__all__", [])):
            obj = getattr(mod, name)
            if not callable(obj):
                continue
            try:
                sig = inspect.signature(obj.__init__ if inspect.isclass(obj) else obj)
            except (TypeError, ValueError):
                continue
            out[f"{modname}.{name}"] = _params(sig)
            if inspect.isclass(obj):  # and the public methods the class defines or inherits
                for meth_name, meth in inspect.getmembers(obj, inspect.isfunction):
                    if meth_name.startswith("_"):
                        continue
                    try:
                        out[f"{modname}.{name}.{meth_name}"] = _params(inspect.signature(meth))
                    except (TypeError, ValueError):
                        continue
    path = HERE / "reference_signatures.json"
    path.write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
    print(f"{path.name}: {len(out)} callables")


def main(ref_root: str, *groups: str) -> None:
    """Validate the stand-ins, then write every group's fixtures (or only the named ``groups``)."""
    spne, spib, sps = _import_reference(ref_root)
    if not groups or "signatures" in groups:
        write_signatures()
    validate_shims(ref_root, spne)
    mods = {"spne": spne, "spib": spib, "sps": sps}
    for group, (modname, fn, seed) in GROUPS.items():
        if groups and group not in groups:
            continue
        for prec, real_t in PRECISIONS.items():
            if group in HOST_ONLY and prec != "double":
                continue  # float64 host geometry: one file serves both precisions
            rec = _Recorder()
            fn(mods[modname], real_t, rec, seed)
            out = HERE / f"golden_{group}_{prec}.npz"
            np.savez_compressed(out, **rec.data)
            print(f"{out.name}: {len(rec.data)} arrays, {out.stat().st_size / 1024:.1f} KiB")


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: make_golden.py /path/to/reference [group ...]")
    main(*sys.argv[1:])
