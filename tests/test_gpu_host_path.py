"""The public-API host path: deferred time_step, early forcing copies, host dt.

``VirtualBoundaryForcing.time_step`` is folded into the next interaction
launch, ``lag_grid_forcing_host`` returns a copy queued right after the
interaction, and ``compute_stable_timestep`` reads the max through the plan's
pinned word.  Each must give bitwise the results of the explicit form it
replaces.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from sopht_gb300 import _lib
    from sopht_gb300.build import build
    build()
    _lib.load()
    assert torch.cuda.is_available()


def host(t):
    torch.cuda.synchronize()
    return t.detach().cpu().numpy()


def _cylinder_case(rt, seed=3):
    import sopht_gb300.simulator as sps
    grid = (64, 128)
    sim = sps.UnboundedNavierStokesFlowSimulator2D(grid_size=grid, x_range=1.0, kinematic_viscosity=5e-4,
                                                   real_t=rt, with_forcing=True, with_free_stream_flow=True)
    rng = np.random.default_rng(seed)
    sim.vorticity_field.copy_(torch.from_numpy(1e-2 * rng.standard_normal(grid).astype(rt)).cuda())
    cyl = sps.Cylinder([0.25, 0.125, 0.0], base_radius=0.05)
    inter = sps.RigidBodyFlowInteraction(
        rigid_body=cyl, eul_grid_forcing_field=sim.eul_grid_forcing_field, eul_grid_velocity_field=sim.velocity_field,
        virtual_boundary_stiffness_coeff=-5e4, virtual_boundary_damping_coeff=-20.0, dx=sim.dx, grid_dim=2,
        real_t=rt, forcing_grid_cls=sps.CircularCylinderForcingGrid, num_forcing_points=48)
    return sim, inter


@pytest.mark.parametrize("rt", [np.float32, np.float64])
def test_deferred_time_step_is_bitwise_the_explicit_update(rt):
    """time_step folded into the interaction == its own kernel first; reads in between see the update."""
    sim_a, a = _cylinder_case(rt)
    sim_b, b = _cylinder_case(rt)
    fs = np.array([1.0, 0.0])
    for step in range(5):
        dt = sim_a.compute_stable_timestep()
        assert dt == sim_b.compute_stable_timestep()
        a.time_step(dt=dt)
        b.time_step(dt=dt)
        b._flush_time_step()  # the standalone mismatch-step kernel
        assert b._pending_xi_dt is None
        if step == 1:  # a read between time_step and the call applies the pending update first
            np.testing.assert_array_equal(host(a.lag_grid_position_mismatch_field),
                                          host(b.lag_grid_position_mismatch_field))
            assert a._pending_xi_dt is None
        if step == 2:  # two time_steps before one call
            a.time_step(dt=0.5 * dt)
            b.time_step(dt=0.5 * dt)
            b._flush_time_step()
        a()
        b()
        sim_a.time_step(dt=dt, free_stream_velocity=fs)
        sim_b.time_step(dt=dt, free_stream_velocity=fs)
        for name in ("lag_grid_position_mismatch_field", "lag_grid_velocity_mismatch_field",
                     "lag_grid_forcing_field"):
            np.testing.assert_array_equal(host(getattr(a, name)), host(getattr(b, name)), err_msg=name)
        np.testing.assert_array_equal(host(sim_a.vorticity_field), host(sim_b.vorticity_field))
    # time_step with no call after it: the read applies it
    a.time_step(dt=1e-4)
    b.time_step(dt=1e-4)
    b._flush_time_step()
    np.testing.assert_array_equal(host(a.lag_grid_position_mismatch_field), host(b.lag_grid_position_mismatch_field))


def test_forcing_snapshot_matches_the_field():
    rt = np.float32
    sim, inter = _cylinder_case(rt)
    fs = np.array([1.0, 0.0])
    for _ in range(4):
        dt = sim.compute_stable_timestep()
        inter.time_step(dt=dt)
        inter()
        sim.time_step(dt=dt, free_stream_velocity=fs)
        f = inter.lag_grid_forcing_host()
        np.testing.assert_array_equal(f, host(inter.lag_grid_forcing_field))
    assert inter._snapshot_key is not None  # the early copy was taken and used
    first = inter.lag_grid_forcing_host()
    first_again = inter.lag_grid_forcing_host()
    np.testing.assert_array_equal(first, first_again)
    # a torch write to the field after the interaction: the read copies the field now
    inter.lag_grid_forcing_field.mul_(2.0)
    np.testing.assert_array_equal(inter.lag_grid_forcing_host(), 2.0 * first)
    # an interaction outside __call__ (no early copy): the read copies the new forcing
    inter.compute_interaction_on_lag_grid()
    np.testing.assert_array_equal(inter.lag_grid_forcing_host(), host(inter.lag_grid_forcing_field))
    # the returned array is the caller's: a later step does not overwrite it
    kept = inter.lag_grid_forcing_host()
    ref = kept.copy()
    inter()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(kept, ref)


@pytest.mark.parametrize("rt", [np.float32, np.float64])
@pytest.mark.parametrize("dim", [2, 3])
def test_host_max_matches_the_reduction(rt, dim):
    import ctypes

    import sopht_gb300.simulator as sps
    from sopht_gb300 import _lib
    from sopht_gb300.utils import ptr, sg_dtype, stream_ptr
    rng = np.random.default_rng(5)
    if dim == 2:
        grid = (40, 72)
        sim = sps.UnboundedNavierStokesFlowSimulator2D(grid_size=grid, x_range=1.0, kinematic_viscosity=1e-3,
                                                       real_t=rt)
    else:
        grid = (24, 32, 40)
        sim = sps.UnboundedNavierStokesFlowSimulator3D(grid_size=grid, x_range=1.0, kinematic_viscosity=1e-3,
                                                       real_t=rt)
    sim.velocity_field.copy_(torch.from_numpy(rng.standard_normal((dim, *grid)).astype(rt)).cuda())
    dt = sim.compute_stable_timestep()
    slot = torch.zeros(1, dtype=torch.float64, device="cuda")
    _lib.call("sg_max_abs_sum", sg_dtype(rt), dim, int(np.prod(grid)), ptr(sim.velocity_field), ptr(slot),
              stream_ptr(sim.device))
    umax = float(slot.item())
    assert sim._host_max.value == umax
    u = host(sim.velocity_field)
    s = np.abs(u[0])
    for d in range(1, dim):
        s = s + np.abs(u[d])
    assert umax == float(s.max())
    umax_rt = rt(umax)
    tol = 10 * np.finfo(rt).eps
    expect = min(sim.cfl * sim.dx / (umax_rt + tol), 0.9 * sim.dx**2 / (2 * dim) / sim.kinematic_viscosity + tol)
    assert dt == expect
    assert isinstance(sim._host_max, ctypes.c_double)


def _arm_direct(sim):
    """Arm timing events on the plan: the next step runs as direct launches (no graph).  The caller
    keeps the returned events alive until that step has run."""
    import ctypes

    from sopht_gb300 import _lib
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(8)]
    for e in evs:
        e.record()
    arr = (ctypes.c_void_p * 8)(*[e.cuda_event for e in evs])
    _lib.call("sg_flow_set_timing_events", sim._plan, 8 if sim.grid_dim == 3 else 6, arr)
    return evs


@pytest.mark.parametrize("rt", [np.float32, np.float64])
@pytest.mark.parametrize("dim", [2, 3])
def test_graph_replayed_step_is_bitwise_the_direct_step(rt, dim):
    """The host-scalar step replays a captured graph; it equals the direct launches bitwise, also after
    the fields move (re-capture) and with and without a free stream."""
    import sopht_gb300.simulator as sps
    rng = np.random.default_rng(9)
    if dim == 2:
        grid = (48, 96)
        cls, extra = sps.UnboundedNavierStokesFlowSimulator2D, {}
    else:
        grid = (20, 24, 32)
        cls, extra = sps.UnboundedNavierStokesFlowSimulator3D, {"filter_vorticity": True,
                                                                 "filter_setting_dict": {"order": 2, "type": "multiplicative"}}
    kw = dict(grid_size=grid, x_range=1.0, kinematic_viscosity=1e-3, real_t=rt, with_forcing=True,
              with_free_stream_flow=True, **extra)
    a, b = cls(**kw), cls(**kw)
    ncomp = 1 if dim == 2 else 3
    w0 = rng.standard_normal((ncomp, *grid) if dim == 3 else grid).astype(rt)
    for s in (a, b):
        s.vorticity_field.copy_(torch.from_numpy(w0).cuda())
    for step in range(6):
        f = torch.from_numpy(rng.standard_normal((dim, *grid)).astype(rt)).cuda()
        a.eul_grid_forcing_field.copy_(f)
        b.eul_grid_forcing_field.copy_(f)
        if step == 3:  # move a field: the graph is captured again for the new pointer
            for s in (a, b):
                s.stream_func_field = torch.zeros_like(s.stream_func_field)
        fs = np.zeros(dim) if step % 2 else np.array([1.0, 0.25, 0.0][:dim])
        dt = a.compute_stable_timestep()
        assert dt == b.compute_stable_timestep()
        a.time_step(dt=dt, free_stream_velocity=fs)
        events = _arm_direct(b)  # held until the step has run: the plan records them
        b.time_step(dt=dt, free_stream_velocity=fs)
        torch.cuda.synchronize()
        del events
        np.testing.assert_array_equal(host(a.vorticity_field), host(b.vorticity_field))
        np.testing.assert_array_equal(host(a.velocity_field), host(b.velocity_field))
        np.testing.assert_array_equal(host(a.stream_func_field), host(b.stream_func_field))


@pytest.mark.parametrize("rt", [np.float32, np.float64])
def test_bound_interactor_call_is_bitwise_the_generic_path(rt):
    """``inter()`` (one native call: staging, interaction, spreading, forcing copy) against the generic
    per-operator path on the same kinematics, over steps with a moving body."""
    sim_a, a = _cylinder_case(rt)
    sim_b, b = _cylinder_case(rt)
    fs = np.array([1.0, 0.0])
    for step in range(5):
        for inter in (a, b):  # a moving body: kinematics change every step
            inter.forcing_grid.cylinder.velocity_collection[:2, 0] = [0.1 * step, -0.05 * step]
            inter.forcing_grid.cylinder.position_collection[:2, 0] += [1e-3, 5e-4]
        dt = sim_a.compute_stable_timestep()
        a.time_step(dt=dt)
        b.time_step(dt=dt)
        a()
        fg = b.forcing_grid
        fg.compute_lag_grid_position_field()
        fg.compute_lag_grid_velocity_field()
        b.compute_interaction_forcing(eul_grid_forcing_field=b.eul_grid_forcing_field,
                                      eul_grid_velocity_field=b.eul_grid_velocity_field,
                                      lag_grid_position_field=fg.position_field,
                                      lag_grid_velocity_field=fg.velocity_field)
        assert a._binding is not None
        for name in ("lag_grid_position_mismatch_field", "lag_grid_velocity_mismatch_field",
                     "lag_grid_forcing_field", "lag_grid_flow_velocity_field", "interp_weights",
                     "nearest_eul_grid_index_to_lag_grid"):
            np.testing.assert_array_equal(host(getattr(a, name)), host(getattr(b, name)), err_msg=name)
        np.testing.assert_array_equal(host(a.eul_grid_forcing_field), host(b.eul_grid_forcing_field))
        np.testing.assert_array_equal(a.lag_grid_forcing_host(), b.lag_grid_forcing_host())
        sim_a.time_step(dt=dt, free_stream_velocity=fs)
        sim_b.time_step(dt=dt, free_stream_velocity=fs)
    np.testing.assert_array_equal(host(sim_a.vorticity_field), host(sim_b.vorticity_field))
    # a replaced buffer re-binds
    old = a._binding
    a.lag_grid_forcing_field = torch.zeros_like(a.lag_grid_forcing_field)
    a()
    assert a._binding is not old
    np.testing.assert_array_equal(a.lag_grid_forcing_host(), host(a.lag_grid_forcing_field))


def test_bound_call_reports_markers_outside_the_grid():
    """The one-call interactor path shares the status word: a body moved off the grid is reported,
    and after the report a body back inside runs clean."""
    sim, inter = _cylinder_case(np.float32)
    inter()
    inter.check_markers_in_domain()  # inside: no error
    assert inter._binding is not None
    inter.forcing_grid.cylinder.position_collection[1, 0] = 0.02  # the support now crosses y = 0
    inter()
    with pytest.raises(ValueError, match="outside"):
        inter.check_markers_in_domain()
    inter.forcing_grid.cylinder.position_collection[1, 0] = 0.125
    inter()
    inter.check_markers_in_domain()


def test_graph_cache_gives_up_on_moving_fields_and_stays_exact():
    """Fields replaced before every step: after a few captures the plan stops capturing and launches
    directly, and every step still equals the direct-launch step bitwise."""
    import sopht_gb300.simulator as sps
    grid = (40, 72)
    kw = dict(grid_size=grid, x_range=1.0, kinematic_viscosity=1e-3, real_t=np.float32, with_forcing=True,
              with_free_stream_flow=True)
    a, b = sps.UnboundedNavierStokesFlowSimulator2D(**kw), sps.UnboundedNavierStokesFlowSimulator2D(**kw)
    rng = np.random.default_rng(4)
    w0 = torch.from_numpy(rng.standard_normal(grid).astype(np.float32)).cuda()
    a.vorticity_field.copy_(w0)
    b.vorticity_field.copy_(w0)
    keep = []
    for step in range(12):
        for s in (a, b):  # a new stream-function tensor every step (kept alive: new addresses)
            s.stream_func_field = torch.zeros_like(s.stream_func_field)
            keep.append(s.stream_func_field)
        dt = a.compute_stable_timestep()
        a.time_step(dt=dt, free_stream_velocity=np.array([1.0, 0.0]))
        events = _arm_direct(b)
        b.time_step(dt=dt, free_stream_velocity=np.array([1.0, 0.0]))
        torch.cuda.synchronize()
        del events
        np.testing.assert_array_equal(host(a.vorticity_field), host(b.vorticity_field))
        np.testing.assert_array_equal(host(a.velocity_field), host(b.velocity_field))


class _MovingRod:
    """A rod with the attributes the forcing grids read (pyelastica layout)."""

    def __init__(self, n, rng):
        s = np.linspace(0.0, 0.3, n + 1)
        self.position_collection = np.stack([0.5 + 0.0 * s, 0.5 + 0.05 * np.sin(3 * s), 0.35 + s])
        self.velocity_collection = 0.1 * rng.standard_normal((3, n + 1))
        self.mass = 0.5 + rng.random(n + 1)
        self.director_collection = np.tile(np.eye(3)[:, :, None], (1, 1, n))
        self.n_elems = n
        self.lengths = np.linalg.norm(np.diff(self.position_collection, axis=1), axis=0)


def test_native_rod_kinematics_path_is_bitwise_the_numpy_path():
    """An element-centric rod interactor computes its marker kinematics natively; a subclass of the
    grid (the numpy path) gives bitwise the same grid arrays, forcing and flow over moving steps."""
    import sopht_gb300.simulator as sps

    class _NumpyGrid(sps.CosseratRodElementCentricForcingGrid):
        pass

    grid = (32, 32, 32)
    sims, inters = [], []
    for cls in (sps.CosseratRodElementCentricForcingGrid, _NumpyGrid):
        sim = sps.UnboundedNavierStokesFlowSimulator3D(grid_size=grid, x_range=1.0, kinematic_viscosity=3e-3,
                                                       real_t=np.float32, with_forcing=True,
                                                       with_free_stream_flow=True)
        rod = _MovingRod(24, np.random.default_rng(2))
        inter = sps.CosseratRodFlowInteraction(
            cosserat_rod=rod, eul_grid_forcing_field=sim.eul_grid_forcing_field,
            eul_grid_velocity_field=sim.velocity_field, virtual_boundary_stiffness_coeff=-2e4,
            virtual_boundary_damping_coeff=-1e2, dx=sim.dx, grid_dim=3, real_t=np.float32, forcing_grid_cls=cls)
        sims.append(sim)
        inters.append(inter)
    fs = np.array([1.0, 0.0, 0.0])
    for step in range(4):
        for inter in inters:  # move the rods in place, as pyelastica does
            rod = inter.forcing_grid.cosserat_rod
            rod.position_collection[0] += 1e-3 * (step + 1)
            rod.velocity_collection[1] = 0.05 * step
        dt = sims[0].compute_stable_timestep()
        for sim, inter in zip(sims, inters, strict=True):
            inter.time_step(dt=dt)
            inter()
            sim.time_step(dt=dt, free_stream_velocity=fs)
        assert inters[0]._rod_args_cache is not None and inters[1]._rod_args_cache is None
        a, b = inters
        np.testing.assert_array_equal(a.forcing_grid.position_field, b.forcing_grid.position_field)
        np.testing.assert_array_equal(a.forcing_grid.velocity_field, b.forcing_grid.velocity_field)
        np.testing.assert_array_equal(a.lag_grid_forcing_host(), b.lag_grid_forcing_host())
        np.testing.assert_array_equal(host(sims[0].vorticity_field), host(sims[1].vorticity_field))
