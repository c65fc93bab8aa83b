"""GPU parity: the sm_103a path against the reference fixtures and the oracle.

Every call goes through the C ABI of ``libsopht_gb300.so`` (via the package's
drop-in classes).  Tolerances:
  * single operators vs the reference fixtures: the reference tests' own bound,
    1e3 machine epsilons absolute (1.2e-4 in FP32, 2.2e-13 in FP64);
  * anything through the FFT Poisson solve: relative L2 <= 1e-5 in FP32 and
    <= 1e-12 in FP64 against the same-precision reference, plus the
    1e3-eps absolute bound on the small fixtures;
  * determinism: two runs from the same state are bitwise equal.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch
from conftest import load_golden, real_t_of, ref_tol, rel_l2

pytestmark = pytest.mark.gpu

RTOL_L2 = {"single": 1e-5, "double": 1e-12}


@pytest.fixture(scope="module", autouse=True)
def _built():
    from sopht_gb300 import _lib
    from sopht_gb300.build import build
    build()
    _lib.load()
    assert torch.cuda.is_available()


def dev(a, precision=None):
    t = torch.from_numpy(np.ascontiguousarray(a))
    if precision is not None:
        t = t.to(torch.float32 if precision == "single" else torch.float64)
    return t.cuda()


def host(t):
    torch.cuda.synchronize()
    return t.detach().cpu().numpy()


# ------------------------------------------------------------------ Poisson


@pytest.mark.parametrize("tag", ["sq", "rect", "r3"])
def test_poisson_2d_vs_reference(precision, tag):
    from sopht_gb300.numeric import UnboundedPoissonSolverPYFFTW2D
    g = load_golden("poisson2d", precision)
    ny, nx, xr = g[f"{tag}/meta"]
    solver = UnboundedPoissonSolverPYFFTW2D(int(ny), int(nx), float(xr), real_t=real_t_of(precision))
    rhs = dev(g[f"{tag}/rhs"])
    sol = torch.zeros_like(rhs)
    solver.solve(sol, rhs)
    out = host(sol)
    np.testing.assert_allclose(out, g[f"{tag}/solution"], atol=ref_tol(precision))
    assert rel_l2(out, g[f"{tag}/solution"]) < RTOL_L2[precision]


@pytest.mark.parametrize("tag", ["cube", "rect"])
def test_poisson_3d_vs_reference(precision, tag):
    from sopht_gb300.numeric import UnboundedPoissonSolverPYFFTW3D
    g = load_golden("poisson3d", precision)
    nz, ny, nx, xr = g[f"{tag}/meta"]
    solver = UnboundedPoissonSolverPYFFTW3D(int(nz), int(ny), int(nx), float(xr), real_t=real_t_of(precision))
    rhs = dev(g[f"{tag}/rhs"])
    sol = torch.zeros_like(rhs)
    solver.vector_field_solve(sol, rhs)
    out = host(sol)
    np.testing.assert_allclose(out, g[f"{tag}/solution"], atol=ref_tol(precision))
    assert rel_l2(out, g[f"{tag}/solution"]) < RTOL_L2[precision]


@pytest.mark.parametrize("shape", [(64, 128), (96, 192), (48, 96), (128, 64), (81, 162), (50, 100), (35, 70),
                                   (32, 64), (128, 256), (192, 384), (256, 512), (384, 768), (512, 1024)])
def test_poisson_2d_vs_oracle_sizes(precision, shape):
    """Generic (radix 2, 3, 5, 7) and size-specialised FFT lengths against the FP64 oracle.

    Size-specialised lengths: 64, 128, 192, 256, 384, 512, 768, 1024 (rows use
    M = nx, columns 2 ny); the others take the generic kernels."""
    from oracle.poisson import UnboundedPoisson2D
    from sopht_gb300.numeric import UnboundedPoissonSolver2D as GPUPoisson
    ny, nx = shape
    rt = real_t_of(precision)
    rhs = np.random.default_rng(7).standard_normal(shape).astype(rt)
    ref = UnboundedPoisson2D(ny, nx, 1.0, np.float64, greens_dtype=np.float64).solve(rhs.astype(np.float64))
    solver = GPUPoisson(ny, nx, 1.0, real_t=rt)
    sol = torch.zeros(shape, dtype=torch.float32 if rt == np.float32 else torch.float64, device="cuda")
    solver.solve(sol, dev(rhs))
    assert rel_l2(host(sol), ref) < (2e-6 if rt == np.float32 else 1e-13)


@pytest.mark.parametrize("shape", [(32, 48, 64), (24, 24, 24), (16, 32, 48), (64, 64, 64), (32, 64, 128),
                                   (128, 128, 128), (256, 64, 64), (64, 256, 64), (128, 256, 32), (64, 64, 256)])
def test_poisson_3d_vs_oracle_sizes(precision, shape):
    """Doubled lengths 256 and 512 along y and z take the register line kernels in fp32 (shared-memory
    kernels in fp64); the others the shared-memory kernels."""
    from oracle.poisson import UnboundedPoisson3D
    from sopht_gb300.numeric import UnboundedPoissonSolver3D as GPUPoisson
    rt = real_t_of(precision)
    rhs = np.random.default_rng(8).standard_normal((3, *shape)).astype(rt)
    ref = UnboundedPoisson3D(*shape, 1.0, np.float64, greens_dtype=np.float64).vector_solve(rhs.astype(np.float64))
    solver = GPUPoisson(*shape, 1.0, real_t=rt)
    sol = torch.zeros_like(dev(rhs))
    solver.vector_field_solve(sol, dev(rhs))
    assert rel_l2(host(sol), ref) < (2e-6 if rt == np.float32 else 1e-13)


def test_poisson_3d_256_cube_vs_oracle():
    """The 256^3 vector solve (512-point y and z line passes, the configuration of the 16-rod carpet)
    against the FP64 oracle."""
    from oracle.poisson import UnboundedPoisson3D
    from sopht_gb300.numeric import UnboundedPoissonSolver3D as GPUPoisson
    shape = (256, 256, 256)
    rhs = np.random.default_rng(9).standard_normal((3, *shape)).astype(np.float32)
    ora = UnboundedPoisson3D(*shape, 1.0, np.float64, greens_dtype=np.float64)
    solver = GPUPoisson(*shape, 1.0, real_t=np.float32)
    sol = torch.zeros_like(dev(rhs))
    solver.vector_field_solve(sol, dev(rhs))
    out = host(sol)
    for c in range(3):
        assert rel_l2(out[c], ora.solve(rhs[c].astype(np.float64))) < 2e-6, c


# ---------------------------------------------------------- single operators


@pytest.mark.parametrize("tag", ["sq", "rect"])
def test_stencils_2d_vs_reference(precision, tag):
    import sopht_gb300.numeric.eulerian_grid_ops as ops
    g = load_golden("stencils2d", precision)
    rt = real_t_of(precision)
    tol = ref_tol(precision)
    f, v, fo = dev(g[f"{tag}/field"]), dev(g[f"{tag}/velocity"]), dev(g[f"{tag}/forcing"])
    out = f.clone()
    ops.gen_advection_timestep_euler_forward_conservative_eno3_pyst_kernel_2d(rt)(
        field=out, advection_flux=torch.empty_like(f), velocity=v, dt_by_dx=rt(0.3))
    np.testing.assert_allclose(host(out), g[f"{tag}/advection_step"], atol=tol)
    out = f.clone()
    ops.gen_diffusion_timestep_euler_forward_pyst_kernel_2d(rt)(
        field=out, diffusion_flux=torch.empty_like(f), nu_dt_by_dx2=rt(0.2))
    np.testing.assert_allclose(host(out), g[f"{tag}/diffusion_step"], atol=tol)
    curl = torch.empty_like(v)
    ops.gen_outplane_field_curl_pyst_kernel_2d(rt)(curl=curl, field=f, prefactor=rt(0.7))
    np.testing.assert_allclose(host(curl), g[f"{tag}/outplane_curl"], atol=tol)
    out = f.clone()
    ops.gen_update_vorticity_from_velocity_forcing_pyst_kernel_2d(rt)(
        vorticity_field=out, velocity_forcing_field=fo, prefactor=rt(0.4))
    np.testing.assert_allclose(host(out), g[f"{tag}/forcing_curl_update"], atol=tol)
    pos = g[f"{tag}/position"]
    dx = rt(1.0 / g[f"{tag}/field"].shape[1])
    for width in (0, 2, 3):
        out = f.clone()
        ops.gen_penalise_field_boundary_pyst_kernel_2d(width, dx, pos[0], pos[1], rt)(field=out)
        np.testing.assert_allclose(host(out), g[f"{tag}/penalise_w{width}"], atol=tol)


@pytest.mark.parametrize("tag", ["cube", "rect"])
def test_stencils_3d_vs_reference(precision, tag):
    import sopht_gb300.numeric.eulerian_grid_ops as ops
    g = load_golden("stencils3d", precision)
    rt = real_t_of(precision)
    tol = ref_tol(precision)
    f, f2 = dev(g[f"{tag}/field"]), dev(g[f"{tag}/field2"])
    out = torch.empty_like(f)
    ops.gen_curl_pyst_kernel_3d(rt)(curl=out, field=f, prefactor=rt(0.6))
    np.testing.assert_allclose(host(out), g[f"{tag}/curl"], atol=tol)
    out = f.clone()
    ops.gen_update_vorticity_from_velocity_forcing_pyst_kernel_3d(rt)(
        vorticity_field=out, velocity_forcing_field=f2, prefactor=rt(0.3))
    np.testing.assert_allclose(host(out), g[f"{tag}/forcing_curl_update"], atol=tol)
    out = torch.empty_like(f)
    ops.gen_elementwise_cross_product_pyst_kernel_3d(rt)(result_field=out, field_1=f, field_2=f2)
    np.testing.assert_allclose(host(out), g[f"{tag}/cross"], atol=tol)
    out = f.clone()
    ops.gen_diffusion_timestep_euler_forward_pyst_kernel_3d(rt, field_type="vector")(
        vector_field=out, diffusion_flux=None, nu_dt_by_dx2=rt(0.1))
    np.testing.assert_allclose(host(out), g[f"{tag}/diffusion_step"], atol=tol)
    div = torch.empty_like(f[0])
    ops.gen_divergence_pyst_kernel_3d(rt)(divergence=div, field=f, inv_dx=rt(3.0))
    np.testing.assert_allclose(host(div), g[f"{tag}/divergence"], atol=tol)
    pos = g[f"{tag}/position"]
    dx = rt(1.0 / g[f"{tag}/field"].shape[-1])
    for width in (0, 2):
        out = f.clone()
        ops.gen_penalise_field_boundary_pyst_kernel_3d(width, dx, pos[0], pos[1], pos[2], rt,
                                                       field_type="vector")(vector_field=out)
        np.testing.assert_allclose(host(out), g[f"{tag}/penalise_w{width}"], atol=tol)
    for ftype, order in (("multiplicative", 2), ("convolution", 1), ("convolution", 3)):
        out = f.clone()
        a, b = torch.empty_like(f[0]), torch.empty_like(f[0])
        ops.gen_laplacian_filter_kernel_3d(order, a, b, rt, field_type="vector", filter_type=ftype)(
            vector_field=out)
        np.testing.assert_allclose(host(out), g[f"{tag}/filter_{ftype}_{order}"], atol=tol)


# ------------------------------------------------------------ full flow step


def _check_step(out, ref, precision):
    np.testing.assert_allclose(out, ref, atol=ref_tol(precision))
    assert rel_l2(out, ref) < RTOL_L2[precision]


@pytest.mark.parametrize("tag", ["a", "b", "c"])
def test_ns_step_2d_vs_reference(precision, tag):
    import sopht_gb300.simulator as sps
    g = load_golden("ns2d", precision)
    rt = real_t_of(precision)
    ny, nx, xr, nu, fs, rho, width, dt, ux, uy = g[f"{tag}/meta"]
    sim = sps.UnboundedNavierStokesFlowSimulator2D(
        grid_size=(int(ny), int(nx)), x_range=float(xr), kinematic_viscosity=float(nu), real_t=rt, time=0.5,
        with_forcing=True, with_free_stream_flow=bool(fs), flow_density=float(rho), penalty_zone_width=int(width))
    sim.vorticity_field.copy_(dev(g[f"{tag}/vorticity_in"]))
    sim.velocity_field.copy_(dev(g[f"{tag}/velocity_in"]))
    sim.eul_grid_forcing_field.copy_(dev(g[f"{tag}/forcing_in"]))
    assert sim.compute_stable_timestep() == g[f"{tag}/stable_dt"]
    assert sim.compute_stable_timestep(dt_prefac=0.25) == g[f"{tag}/stable_dt_prefac"]
    sim.time_step(dt=float(dt), free_stream_velocity=np.array([ux, uy]))
    _check_step(host(sim.vorticity_field), g[f"{tag}/vorticity_out"], precision)
    _check_step(host(sim.velocity_field), g[f"{tag}/velocity_out"], precision)
    _check_step(host(sim.stream_func_field), g[f"{tag}/stream_func_out"], precision)
    assert torch.count_nonzero(sim.eul_grid_forcing_field).item() == 0
    assert sim.time == pytest.approx(float(g[f"{tag}/time_out"]))
    sim2 = sps.UnboundedNavierStokesFlowSimulator2D(
        grid_size=(int(ny), int(nx)), x_range=float(xr), kinematic_viscosity=float(nu), real_t=rt,
        with_forcing=False, with_free_stream_flow=bool(fs), penalty_zone_width=int(width))
    sim2.vorticity_field.copy_(dev(g[f"{tag}/vorticity_in"]))
    sim2.velocity_field.copy_(dev(g[f"{tag}/velocity_in"]))
    sim2.time_step(dt=float(dt), free_stream_velocity=np.array([ux, uy]))
    _check_step(host(sim2.vorticity_field), g[f"{tag}/noforce_vorticity_out"], precision)
    _check_step(host(sim2.velocity_field), g[f"{tag}/noforce_velocity_out"], precision)


@pytest.mark.parametrize("tag", ["a", "b", "c", "d"])
def test_ns_step_3d_vs_reference(precision, tag):
    import sopht_gb300.simulator as sps
    g = load_golden("ns3d", precision)
    rt = real_t_of(precision)
    m = g[f"{tag}/meta"]
    grid = tuple(int(v) for v in m[:3])
    xr, nu, fs, rho, dt = (float(v) for v in m[3:8])
    order, ftype = int(m[11]), int(m[12])
    kw = {}
    if ftype:
        kw = {"filter_vorticity": True,
              "filter_setting_dict": {"order": order, "type": "multiplicative" if ftype == 1 else "convolution"}}
    sim = sps.UnboundedNavierStokesFlowSimulator3D(
        grid_size=grid, x_range=xr, kinematic_viscosity=nu, real_t=rt, with_forcing=True,
        with_free_stream_flow=bool(fs), flow_density=rho, **kw)
    sim.vorticity_field.copy_(dev(g[f"{tag}/vorticity_in"]))
    sim.velocity_field.copy_(dev(g[f"{tag}/velocity_in"]))
    sim.eul_grid_forcing_field.copy_(dev(g[f"{tag}/forcing_in"]))
    np.testing.assert_allclose(sim.get_vorticity_divergence_l2_norm(), g[f"{tag}/divergence_l2"],
                               rtol=1e-5 if rt == np.float32 else 1e-12)
    assert sim.compute_stable_timestep() == g[f"{tag}/stable_dt"]
    sim.time_step(dt=dt, free_stream_velocity=m[8:11])
    _check_step(host(sim.vorticity_field), g[f"{tag}/vorticity_out"], precision)
    _check_step(host(sim.velocity_field), g[f"{tag}/velocity_out"], precision)
    _check_step(host(sim.stream_func_field), g[f"{tag}/stream_func_out"], precision)
    assert torch.count_nonzero(sim.eul_grid_forcing_field).item() == 0


@pytest.mark.parametrize("dim,grid", [(2, (64, 128)), (2, (96, 192)), (3, (24, 30, 40)), (3, (32, 32, 64))])
def test_multi_step_vs_oracle_and_determinism(precision, dim, grid):
    """Ten forced steps on a larger grid against the oracle; two runs bitwise equal."""
    import sopht_gb300.simulator as sps
    from oracle.flow import NavierStokes2DOracle, NavierStokes3DOracle
    rt = real_t_of(precision)
    rng = np.random.default_rng(3)
    kw = dict(grid_size=grid, x_range=1.0, kinematic_viscosity=2e-3, real_t=rt, with_forcing=True,
              with_free_stream_flow=True)
    w0 = rng.standard_normal((grid if dim == 2 else (3, *grid))).astype(rt)
    u0 = (0.3 * rng.standard_normal((dim, *grid))).astype(rt)
    fs = np.array([1.0, 0.2, -0.1][:dim])
    forcings = [(0.5 * rng.standard_normal((dim, *grid))).astype(rt) for _ in range(10)]
    Sim = sps.UnboundedNavierStokesFlowSimulator2D if dim == 2 else sps.UnboundedNavierStokesFlowSimulator3D
    Ora = NavierStokes2DOracle if dim == 2 else NavierStokes3DOracle
    runs = []
    for _ in range(2):
        sim = Sim(**kw)
        sim.vorticity_field.copy_(dev(w0))
        sim.velocity_field.copy_(dev(u0))
        for k in range(10):
            sim.eul_grid_forcing_field.copy_(dev(forcings[k]))
            sim.time_step(dt=sim.compute_stable_timestep(), free_stream_velocity=fs)
        runs.append((host(sim.vorticity_field), host(sim.velocity_field)))
    np.testing.assert_array_equal(runs[0][0], runs[1][0])
    np.testing.assert_array_equal(runs[0][1], runs[1][1])
    ora = Ora(**kw)
    ora.vorticity_field[...] = w0
    ora.velocity_field[...] = u0
    for k in range(10):
        ora.eul_grid_forcing_field[...] = forcings[k]
        ora.time_step(ora.compute_stable_timestep(), fs)
    bound = 1e-5 if rt == np.float32 else 1e-11
    assert rel_l2(runs[0][0], ora.vorticity_field) < bound
    assert rel_l2(runs[0][1], ora.velocity_field) < bound


def test_device_dt_matches_host_path(precision):
    """Device-resident dt/prefactors give the same dt and a bitwise-equal step."""
    import sopht_gb300.simulator as sps
    rt = real_t_of(precision)
    rng = np.random.default_rng(11)
    grid = (48, 96)
    kw = dict(grid_size=grid, x_range=1.0, kinematic_viscosity=5e-4, real_t=rt, with_forcing=True,
              with_free_stream_flow=True)
    w0 = rng.standard_normal(grid).astype(rt)
    u0 = rng.standard_normal((2, *grid)).astype(rt)
    f0 = rng.standard_normal((2, *grid)).astype(rt)
    fs = np.array([1.0, 0.0])
    a, b = sps.UnboundedNavierStokesFlowSimulator2D(**kw), sps.UnboundedNavierStokesFlowSimulator2D(**kw)
    for s in (a, b):
        s.vorticity_field.copy_(dev(w0))
        s.velocity_field.copy_(dev(u0))
        s.eul_grid_forcing_field.copy_(dev(f0))
    for step in range(3):
        dt = a.compute_stable_timestep(dt_prefac=0.5)
        a.time_step(dt=dt, free_stream_velocity=fs)
        if step == 0:
            b.prime_velocity_max()
        dsc = b.device_stable_timestep(dt_prefac=0.5, free_stream_velocity=fs, recompute_max=False)
        b.time_step_device(dsc)
        np.testing.assert_array_equal(host(a.vorticity_field), host(b.vorticity_field))
        np.testing.assert_array_equal(host(a.velocity_field), host(b.velocity_field))


# --------------------------------------------------------- immersed boundary


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("kernel", ["cosine", "peskin"])
def test_virtual_boundary_forcing_vs_reference(precision, dim, kernel):
    from sopht_gb300.numeric import VirtualBoundaryForcing
    g = load_golden("ib", precision)
    rt = real_t_of(precision)
    tag = f"d{dim}_{kernel}"
    meta = g[f"{tag}/meta"]
    grid = tuple(int(v) for v in meta[1: 1 + dim])
    n_lag = int(meta[1 + dim])
    K, C, dt = (float(v) for v in meta[2 + dim:])
    dx = rt(1.0 / grid[-1])
    vbf = VirtualBoundaryForcing(K, C, dim, dx, n_lag, rt, enable_eul_grid_forcing_reset=False,
                                 interp_kernel_type=kernel)
    vbf.lag_grid_position_mismatch_field.copy_(dev(g[f"{tag}/position_mismatch_in"]))
    force = dev(g[f"{tag}/eul_forcing_in"])
    vbf.compute_interaction_forcing(force, dev(g[f"{tag}/eul_velocity"]), g[f"{tag}/position"],
                                    g[f"{tag}/lag_velocity"])
    vbf.check_markers_in_domain()
    np.testing.assert_array_equal(host(vbf.nearest_eul_grid_index_to_lag_grid), g[f"{tag}/nearest_index"])
    tol = ref_tol(precision)
    w_ref = g[f"{tag}/weights"].reshape(-1, n_lag)
    np.testing.assert_allclose(host(vbf.interp_weights), w_ref, rtol=tol, atol=tol * np.abs(w_ref).max())
    np.testing.assert_allclose(host(vbf.lag_grid_flow_velocity_field), g[f"{tag}/lag_flow_velocity"], atol=tol)
    np.testing.assert_allclose(host(vbf.lag_grid_forcing_field), g[f"{tag}/lag_forcing"], rtol=tol, atol=tol)
    # spreading sums up to 4^dim marker contributions per cell: allow a few
    # roundings of those partial sums on top of the reference tests' bound
    np.testing.assert_allclose(host(force), g[f"{tag}/eul_forcing_out"], rtol=4 * tol, atol=4 * tol)
    vbf.time_step(dt)
    np.testing.assert_allclose(host(vbf.lag_grid_position_mismatch_field), g[f"{tag}/position_mismatch_out"],
                               atol=tol)


def test_force_conservation_and_spread_determinism():
    """sum_cells f dx^dim == sum_markers F (VirtualBoundaryForcing tests); reruns are bitwise equal."""
    from sopht_gb300.numeric import VirtualBoundaryForcing
    rng = np.random.default_rng(2)
    n = 96
    grid = (64, 128)
    dx = 1.0 / 128
    theta = np.linspace(0, 2 * np.pi, n, endpoint=False)
    pos = np.stack([0.25 + 0.05 * np.cos(theta), 0.25 + 0.05 * np.sin(theta)])
    xi = dev(1e-4 * rng.standard_normal((2, n)))
    u = dev(rng.standard_normal((2, *grid)))
    outs = []
    for _ in range(2):
        vbf = VirtualBoundaryForcing(-5e4, -20.0, 2, dx, n, np.float64, enable_eul_grid_forcing_reset=True)
        vbf.lag_grid_position_mismatch_field.copy_(xi)
        f = torch.full_like(u, 7.0)  # reset variant must clear this
        vbf.compute_interaction_forcing(f, u, pos, np.zeros((2, n)))
        outs.append(host(f))
        total = outs[-1].reshape(2, -1).sum(axis=1) * dx**2
        np.testing.assert_allclose(total, host(vbf.lag_grid_forcing_field).sum(axis=1), rtol=1e-10)
    np.testing.assert_array_equal(outs[0], outs[1])


def test_out_of_domain_marker_is_reported():
    from sopht_gb300.numeric import VirtualBoundaryForcing
    vbf = VirtualBoundaryForcing(-1.0, -1.0, 2, 1.0 / 32, 2, np.float32)
    pos = np.array([[0.5, 0.01], [0.5, 0.5]])
    u = torch.zeros((2, 32, 32), device="cuda")
    vbf.compute_interaction_force_on_lag_grid(u, pos, np.zeros((2, 2)))
    with pytest.raises(ValueError, match="outside"):
        vbf.check_markers_in_domain()


def test_cylinder_coupled_steps_vs_reference(precision):
    import sopht_gb300.simulator as sps
    g = load_golden("cylinder2d", precision)
    rt = real_t_of(precision)
    ny, nx, xr, nu, radius, n_mk, cx, cy, K, C = g["meta"]
    sim = sps.UnboundedNavierStokesFlowSimulator2D(
        grid_size=(int(ny), int(nx)), x_range=float(xr), kinematic_viscosity=float(nu), real_t=rt,
        with_forcing=True, with_free_stream_flow=True)
    sim.vorticity_field.copy_(dev(g["vorticity_init"]))
    cyl = sps.Cylinder([cx, cy, 0.0], base_radius=float(radius))
    inter = sps.RigidBodyFlowInteraction(
        rigid_body=cyl, eul_grid_forcing_field=sim.eul_grid_forcing_field, eul_grid_velocity_field=sim.velocity_field,
        virtual_boundary_stiffness_coeff=float(K), virtual_boundary_damping_coeff=float(C), dx=sim.dx, grid_dim=2,
        real_t=rt, forcing_grid_cls=sps.CircularCylinderForcingGrid, num_forcing_points=int(n_mk))
    np.testing.assert_allclose(inter.forcing_grid.position_field, g["marker_position"], rtol=1e-15)
    bound = 1e-5 if rt == np.float32 else 1e-11
    for step in range(4):
        dt = sim.compute_stable_timestep()
        assert dt == pytest.approx(g["dt"][step], rel=1e-6 if rt == np.float32 else 1e-13)
        dt = g["dt"][step]
        inter.time_step(dt=dt)
        inter()
        sim.time_step(dt=dt, free_stream_velocity=np.array([1.0, 0.0]))
        assert rel_l2(host(sim.vorticity_field), g[f"step{step}/vorticity"]) < bound
        assert rel_l2(host(sim.velocity_field), g[f"step{step}/velocity"]) < bound
        assert rel_l2(host(inter.lag_grid_forcing_field), g[f"step{step}/lag_forcing"]) < bound
        assert rel_l2(host(inter.lag_grid_position_mismatch_field), g[f"step{step}/position_mismatch"]) < bound
    # immersed_body_flow_interaction.py:133-141
    assert inter.get_grid_deviation_error_l2_norm() == pytest.approx(float(g["grid_deviation"]), rel=bound)
    inter.compute_flow_forces_and_torques()
    scale = np.abs(g["body_forces"]).max()
    atol = scale * (1e-5 if rt == np.float32 else 1e-11)
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
def test_rod_coupling_vs_reference(precision, name):
    import sopht_gb300.simulator as sps
    g = load_golden("rod3d", precision)
    rt = real_t_of(precision)
    rod = _Rod(g, name)
    cls = sps.CosseratRodNodalForcingGrid if name == "nodal" else sps.CosseratRodElementCentricForcingGrid
    force = torch.zeros((3, 16, 16, 16), dtype=torch.float32 if rt == np.float32 else torch.float64,
                        device="cuda")
    inter = sps.CosseratRodFlowInteraction(
        cosserat_rod=rod, eul_grid_forcing_field=force, eul_grid_velocity_field=dev(g["eul_velocity"]),
        virtual_boundary_stiffness_coeff=-2e4, virtual_boundary_damping_coeff=-1e2, dx=rt(1.0 / 16), grid_dim=3,
        real_t=rt, forcing_grid_cls=cls)
    inter.time_step(dt=1e-3)
    inter()
    tol = ref_tol(precision)
    np.testing.assert_allclose(host(inter.lag_grid_forcing_field), g[f"{name}/lag_forcing"], rtol=tol, atol=tol)
    np.testing.assert_allclose(host(force), g[f"{name}/eul_forcing_out"], rtol=tol, atol=tol)
    inter.lag_grid_position_mismatch_field.copy_(dev(g[f"{name}/position_mismatch_in"]))
    inter.compute_flow_forces_and_torques()
    np.testing.assert_allclose(inter.body_flow_forces, g[f"{name}/body_forces"], rtol=tol, atol=tol)
    np.testing.assert_allclose(inter.body_flow_torques, g[f"{name}/body_torques"], rtol=tol, atol=tol)


@pytest.mark.parametrize("dim,grid,steps", [(3, (128, 128, 128), 2), (2, (512, 1024), 5)])
def test_full_size_steps_vs_oracle(precision, dim, grid, steps):
    """Forced steps at the benchmark sizes: the 128^3 rod-flow grid (256^3 doubled FFT, radix-16
    line passes) and the largest batched 2D grid (1024-point rows) against the oracle."""
    import sopht_gb300.simulator as sps
    from oracle.flow import NavierStokes2DOracle, NavierStokes3DOracle
    rt = real_t_of(precision)
    rng = np.random.default_rng(29)
    kw = dict(grid_size=grid, x_range=1.0, kinematic_viscosity=3e-3, real_t=rt, with_forcing=True,
              with_free_stream_flow=True)
    w0 = (1e-2 * rng.standard_normal((grid if dim == 2 else (3, *grid)))).astype(rt)
    fs = np.array([1.0, 0.0, 0.0][:dim])
    f0 = (0.1 * rng.standard_normal((dim, *grid))).astype(rt)
    Sim = sps.UnboundedNavierStokesFlowSimulator2D if dim == 2 else sps.UnboundedNavierStokesFlowSimulator3D
    Ora = NavierStokes2DOracle if dim == 2 else NavierStokes3DOracle
    sim, ora = Sim(**kw), Ora(**kw)
    sim.vorticity_field.copy_(dev(w0))
    ora.vorticity_field[...] = w0
    for _ in range(steps):
        sim.eul_grid_forcing_field.copy_(dev(f0))
        ora.eul_grid_forcing_field[...] = f0
        dt = ora.compute_stable_timestep()  # both driven by the same dt sequence
        sim.time_step(dt=dt, free_stream_velocity=fs)
        ora.time_step(dt, fs)
    bound = 1e-5 if rt == np.float32 else 1e-12
    assert rel_l2(host(sim.vorticity_field), ora.vorticity_field) < bound
    assert rel_l2(host(sim.velocity_field), ora.velocity_field) < bound
