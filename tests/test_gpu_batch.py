"""Batched 2D instances against the same instances stepped one by one.

The batched step runs the same arithmetic per element as the single-instance
device-dt step (the FFT line counts per block differ, the per-line butterflies
do not), so after several steps every instance's fields must be bitwise equal
to its individually stepped twin, for every autotuner launch shape.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SIZES = [(128, 256), (256, 512), (384, 768), (512, 1024), (128, 256)]


def _make(i, ny, nx):
    import sopht_gb300.simulator as sps
    rng = np.random.default_rng(100 + i)
    re = 50 + 350 * rng.random()
    nu = 0.1 / re
    sim = sps.UnboundedNavierStokesFlowSimulator2D(grid_size=(ny, nx), x_range=1.0, kinematic_viscosity=nu,
                                                   real_t=np.float32, with_forcing=True,
                                                   with_free_stream_flow=True)
    sim.vorticity_field.copy_(torch.from_numpy((1e-3 * rng.standard_normal((ny, nx))).astype(np.float32)).cuda())
    y_range = ny / nx
    centre = (0.25 + 0.04 * (rng.random() - 0.5), 0.5 * y_range + 0.04 * (rng.random() - 0.5), 0.0)
    cyl = sps.Cylinder(centre, base_radius=0.05)
    inter = sps.RigidBodyFlowInteraction(
        rigid_body=cyl, eul_grid_forcing_field=sim.eul_grid_forcing_field, eul_grid_velocity_field=sim.velocity_field,
        virtual_boundary_stiffness_coeff=-5e4, virtual_boundary_damping_coeff=-20.0, dx=sim.dx, grid_dim=2,
        real_t=np.float32, forcing_grid_cls=sps.CircularCylinderForcingGrid, num_forcing_points=96)
    return sim, inter


@pytest.mark.parametrize("tuning", [(16, 8, 256), (8, 0, 256), (16, 2, 512), (8, 8, 512)])
def test_batched_equals_individual(tuning):
    from sopht_gb300.build import build
    from sopht_gb300.simulator import BatchedFlowSimulator2D
    build()
    fs = np.array([1.0, 0.0])
    batch_members = [_make(i, *s) for i, s in enumerate(SIZES)]
    single_members = [_make(i, *s) for i, s in enumerate(SIZES)]
    batch = BatchedFlowSimulator2D([m[0] for m in batch_members], [m[1] for m in batch_members],
                                   free_stream_velocities=[fs] * len(SIZES))
    batch.set_tuning(*tuning)
    for sim, inter in single_members:
        inter.upload_kinematics()
        sim.prime_velocity_max()
    steps = 4
    for _ in range(steps):
        batch.step()
        for sim, inter in single_members:
            dsc = sim.device_stable_timestep(free_stream_velocity=fs, recompute_max=False)
            inter.device_call(dsc)
            sim.time_step_device(dsc)
    torch.cuda.synchronize()
    for (bs, bi), (ss, si) in zip(batch_members, single_members, strict=True):
        assert torch.equal(bs.vorticity_field, ss.vorticity_field)
        assert torch.equal(bs.velocity_field, ss.velocity_field)
        assert torch.equal(bi.lag_grid_forcing_field, si.lag_grid_forcing_field)
        assert bs.device_time() == ss.device_time()


def test_batched_follows_host_dt_path():
    """The batch tracks the plain drop-in loop (host dt) to FP32 rounding."""
    from sopht_gb300.simulator import BatchedFlowSimulator2D
    fs = np.array([1.0, 0.0])
    sizes = SIZES[:2]
    bm = [_make(i, *s) for i, s in enumerate(sizes)]
    pm = [_make(i, *s) for i, s in enumerate(sizes)]
    batch = BatchedFlowSimulator2D([m[0] for m in bm], [m[1] for m in bm], free_stream_velocities=[fs] * 2)
    for _ in range(3):
        batch.step()
        for sim, inter in pm:
            dt = sim.compute_stable_timestep()
            inter.time_step(dt=dt)
            inter()
            sim.time_step(dt=dt, free_stream_velocity=fs)
    torch.cuda.synchronize()
    for (bs, _), (ps, _) in zip(bm, pm, strict=True):
        num = torch.linalg.vector_norm((bs.vorticity_field - ps.vorticity_field).double())
        den = torch.linalg.vector_norm(ps.vorticity_field.double())
        assert float(num / den) < 1e-6
        assert abs(bs.device_time() - ps.time) < 1e-9 * max(1.0, ps.time)


def test_autotune_picks_a_candidate():
    from sopht_gb300.simulator import BatchedFlowSimulator2D
    members = [_make(i, *s) for i, s in enumerate(SIZES[:3])]
    batch = BatchedFlowSimulator2D([m[0] for m in members], [m[1] for m in members])
    best = batch.autotune(steps=2, candidates=[(16, 0, 256), (8, 4, 512)])
    assert best in [(16, 0, 256), (8, 4, 512)]
    assert batch.tuning == best
