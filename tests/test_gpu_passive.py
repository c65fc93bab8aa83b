"""GPU parity of passive transport: 3D ENO3 advection and PassiveTransportFlowSimulator.

Against the fixtures generated by running the reference (``golden_passive_*``)
at the reference tests' bound (1e3 machine epsilons, absolute), against the
oracle at larger grids (relative L2 <= 1e-12 in FP64, <= 1e-5 in FP32), the
reference test's exact stable-dt check, and bitwise determinism.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch
from conftest import load_golden, real_t_of, ref_tol, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from sopht_gb300 import _lib
    from sopht_gb300.build import build
    build()
    _lib.load()
    assert torch.cuda.is_available()


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("tag", ["cube", "rect"])
def test_eno3_3d_vs_reference(precision, tag):
    from sopht_gb300.numeric import eulerian_grid_ops as ops
    g = load_golden("passive", precision)
    rt = real_t_of(precision)
    tol = ref_tol(precision)
    f, v, vec = dev(g[f"{tag}/field"]), dev(g[f"{tag}/velocity"]), dev(g[f"{tag}/vector_field"])
    flux = dev(g[f"{tag}/flux_in"])
    ops.gen_advection_flux_conservative_eno3_pyst_kernel_3d(real_t=rt)(
        advection_flux=flux, field=f, velocity=v, inv_dx=rt(0.7))
    np.testing.assert_allclose(host(flux), g[f"{tag}/flux_out"], atol=tol)
    out = f.clone()
    ops.gen_advection_timestep_euler_forward_conservative_eno3_pyst_kernel_3d(real_t=rt)(
        out, advection_flux=torch.empty_like(out), velocity=v, dt_by_dx=rt(0.3))
    np.testing.assert_allclose(host(out), g[f"{tag}/advection_step"], atol=tol)
    out = vec.clone()
    ops.gen_advection_timestep_euler_forward_conservative_eno3_pyst_kernel_3d(real_t=rt, field_type="vector")(
        out, advection_flux=torch.empty_like(out[0]), velocity=v, dt_by_dx=rt(0.3))
    np.testing.assert_allclose(host(out), g[f"{tag}/advection_step_vector"], atol=tol)


@pytest.mark.parametrize("tag,dim,grid,ftype", [("s2d", 2, (12, 16), "scalar"), ("s3d", 3, (8, 10, 12), "scalar"),
                                                ("v3d", 3, (8, 8, 10), "vector")])
def test_passive_simulator_vs_reference(precision, tag, dim, grid, ftype):
    import sopht_gb300.simulator as sps
    g = load_golden("passive", precision)
    rt = real_t_of(precision)
    sim = sps.PassiveTransportFlowSimulator(kinematic_viscosity=1e-2, grid_dim=dim, grid_size=grid, x_range=1.0,
                                            cfl=0.2, real_t=rt, time=0.5, field_type=ftype)
    sim.velocity_field.copy_(dev(g[f"sim_{tag}/velocity"]))
    sim.primary_field.copy_(dev(g[f"sim_{tag}/primary_in"]))
    for step in range(3):
        dt = sim.compute_stable_timestep(dt_prefac=0.8)
        assert dt == g[f"sim_{tag}/dt"][step]
        sim.time_step(dt=dt)
        np.testing.assert_allclose(host(sim.primary_field), g[f"sim_{tag}/primary_step{step}"],
                                   atol=ref_tol(precision))
    assert sim.time == g[f"sim_{tag}/time_out"]


@pytest.mark.parametrize("dim,grid,ftype", [(2, (96, 160), "scalar"), (3, (40, 48, 64), "scalar"),
                                            (3, (24, 32, 40), "vector")])
def test_passive_simulator_vs_oracle(precision, dim, grid, ftype):
    """Ten steps at grids the fixtures do not reach, against the oracle from the same state."""
    import sopht_gb300.simulator as sps
    from oracle.flow import PassiveTransportOracle
    rt = real_t_of(precision)
    rng = np.random.default_rng(17)
    sim = sps.PassiveTransportFlowSimulator(kinematic_viscosity=2e-3, grid_dim=dim, grid_size=grid, x_range=1.0,
                                            real_t=rt, field_type=ftype)
    ora = PassiveTransportOracle(2e-3, dim, grid, 1.0, real_t=rt, field_type=ftype)
    vel = rng.standard_normal(ora.velocity_field.shape).astype(rt)
    prim = rng.random(ora.primary_field.shape).astype(rt)
    ora.velocity_field[...] = vel
    ora.primary_field[...] = prim
    sim.velocity_field.copy_(dev(vel))
    sim.primary_field.copy_(dev(prim))
    bound = 1e-12 if rt == np.float64 else 1e-5
    for _ in range(10):
        dt = ora.compute_stable_timestep()
        assert sim.compute_stable_timestep() == dt
        ora.time_step(dt)
        sim.time_step(dt=dt)
    assert rel_l2(host(sim.primary_field), ora.primary_field) < bound


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("n", [4, 8])
def test_passive_small_grids_and_dt(precision, dim, n):
    """The reference test's cases: grids of 4 and 8 cells per side (the ENO3 interior of a 4-cell side
    is empty) and the exact stable dt for a uniform velocity of 2 (cfl 0.2, dt_prefac 0.5)."""
    import sopht_gb300.simulator as sps
    from oracle.flow import PassiveTransportOracle
    rt = real_t_of(precision)
    grid = (n,) * dim
    rng = np.random.default_rng(n + dim)
    for ftype in (("scalar",) if dim == 2 else ("scalar", "vector")):
        sim = sps.PassiveTransportFlowSimulator(kinematic_viscosity=1e-2, grid_dim=dim, grid_size=grid, x_range=1.0,
                                                real_t=rt, time=1.0, field_type=ftype)
        ora = PassiveTransportOracle(1e-2, dim, grid, 1.0, real_t=rt, time=1.0, field_type=ftype)
        vel = rng.random(ora.velocity_field.shape).astype(rt)
        prim = rng.random(ora.primary_field.shape).astype(rt)
        ora.velocity_field[...] = vel
        ora.primary_field[...] = prim
        sim.velocity_field.copy_(dev(vel))
        sim.primary_field.copy_(dev(prim))
        sim.time_step(dt=2.0)
        ora.time_step(2.0)
        assert sim.time == 3.0
        np.testing.assert_allclose(host(sim.primary_field), ora.primary_field, atol=ref_tol(precision))
    sim = sps.PassiveTransportFlowSimulator(kinematic_viscosity=1e-2, cfl=0.2, grid_dim=dim, grid_size=grid,
                                            x_range=1.0, real_t=rt)
    sim.velocity_field.fill_(2.0)
    dx = rt(1.0 / n)
    tol = 10 * np.finfo(rt).eps
    ref_dt = 0.5 * min(0.2 * dx / (dim * 2.0 + tol), 0.9 * dx**2 / (2 * dim) / 1e-2)
    assert sim.compute_stable_timestep(dt_prefac=0.5) == ref_dt


def test_passive_step_is_deterministic():
    import sopht_gb300.simulator as sps
    grid = (48, 40, 56)
    outs = []
    for _ in range(2):
        sim = sps.PassiveTransportFlowSimulator(kinematic_viscosity=1e-3, grid_dim=3, grid_size=grid, x_range=1.0,
                                                real_t=np.float32, field_type="vector")
        r = np.random.default_rng(5)
        sim.velocity_field.copy_(dev(r.standard_normal((3, *grid)).astype(np.float32)))
        sim.primary_field.copy_(dev(r.random((3, *grid)).astype(np.float32)))
        for _ in range(5):
            sim.time_step(dt=sim.compute_stable_timestep())
        outs.append(host(sim.primary_field))
    np.testing.assert_array_equal(outs[0], outs[1])


def test_passive_simulator_argument_errors():
    import sopht_gb300.simulator as sps
    with pytest.raises(ValueError):
        sps.PassiveTransportFlowSimulator(kinematic_viscosity=1e-2, grid_dim=2, grid_size=(8, 8), x_range=1.0,
                                          field_type="vector")
    with pytest.raises(ValueError):
        sps.PassiveTransportFlowSimulator(kinematic_viscosity=1e-2, grid_dim=3, grid_size=(8, 8, 8), x_range=1.0,
                                          field_type="tensor")
    sim = sps.PassiveTransportFlowSimulator(kinematic_viscosity=1e-2, grid_dim=3, grid_size=(8, 8, 8), x_range=1.0)
    sim.primary_field = sim.primary_field.double()
    with pytest.raises(ValueError):
        sim.time_step(dt=1e-3)


@pytest.mark.parametrize("rt", [np.float32, np.float64])
def test_vector_threads_equal_per_component_launches(rt):
    """ncomp = 3 (one thread advects all three components) against three single-component launches."""
    from sopht_gb300 import _lib
    from sopht_gb300.utils import ptr, sg_dtype, stream_ptr
    rng = np.random.default_rng(8)
    grid = (20, 36, 44)
    f = dev(rng.standard_normal((3, *grid)).astype(rt))
    u = dev(rng.standard_normal((3, *grid)).astype(rt))
    out3 = torch.empty_like(f)
    out1 = torch.empty_like(f)
    s = stream_ptr(f.device)
    _lib.call("sg_advection_eno3_step_3d", sg_dtype(rt), *grid, 3, ptr(f), ptr(out3), ptr(u), 0.05, s)
    for c in range(3):
        _lib.call("sg_advection_eno3_step_3d", sg_dtype(rt), *grid, 1, ptr(f[c]), ptr(out1[c]), ptr(u), 0.05, s)
    np.testing.assert_array_equal(host(out3), host(out1))


@pytest.mark.parametrize("grid", [(83, 256, 256), (163, 256, 256)])
def test_large_grids_vs_oracle(grid):
    """Large grids with odd plane counts: the vector step and the scalar flux form in FP64 against the
    oracle, and the planes outside the interior copied unchanged."""
    from oracle import stencils as st
    from sopht_gb300 import _lib
    from sopht_gb300.utils import ptr, sg_dtype, stream_ptr
    rt = np.float64
    rng = np.random.default_rng(grid[0])
    f = rng.standard_normal((3, *grid)).astype(rt)
    u = rng.standard_normal((3, *grid)).astype(rt)
    fd, ud = dev(f), dev(u)
    out = torch.empty_like(fd)
    s = stream_ptr(fd.device)
    _lib.call("sg_advection_eno3_step_3d", sg_dtype(rt), *grid, 3, ptr(fd), ptr(out), ptr(ud), 0.05, s)
    got = host(out)
    for c in range(3):
        ref = f[c].copy()
        st.advection_step_3d(ref, u, rt(0.05))
        assert rel_l2(got[c], ref) < 1e-13
        np.testing.assert_array_equal(got[c][:2], f[c][:2])  # planes outside the interior are copied
        np.testing.assert_array_equal(got[c][-2:], f[c][-2:])
    base = rng.standard_normal(grid).astype(rt)
    flux = dev(base)
    _lib.call("sg_advection_eno3_flux_3d", sg_dtype(rt), *grid, ptr(fd[1]), ptr(flux), ptr(ud), 0.7, s)
    ref = base + st.eno3_flux_3d(f[1], u, rt(0.7))
    assert rel_l2(host(flux), ref) < 1e-13


@pytest.mark.parametrize("rt", [np.float32, np.float64])
@pytest.mark.parametrize("dim", [2, 3])
def test_module_stable_timestep_function(rt, dim):
    """compute_advection_diffusion_stable_timestep (passive_transport_flow_simulators.py:139-155): the dt
    equals the oracle's, and the magnitude field holds sum_d |u_d|."""
    from oracle.flow import stable_timestep
    from sopht_gb300.simulator.flow import compute_advection_diffusion_stable_timestep
    rng = np.random.default_rng(dim)
    grid = (24, 40) if dim == 2 else (12, 16, 20)
    u = rng.standard_normal((dim, *grid)).astype(rt)
    mag = torch.zeros(grid, dtype=torch.float32 if rt == np.float32 else torch.float64, device="cuda")
    dx = rt(1.0 / grid[-1])
    dt = compute_advection_diffusion_stable_timestep(dev(u), mag, dim, dx, 0.1, 1e-3, real_t=rt)
    assert dt == stable_timestep(u, dim, dx, 0.1, 1e-3, rt)
    np.testing.assert_allclose(host(mag), np.sum(np.fabs(u), axis=0), rtol=1e-6 if rt == np.float32 else 1e-14)
