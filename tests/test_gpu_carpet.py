"""The benchmarked 256^3 carpet (16 driven Cosserat rods in a 512^3-doubled unbounded flow) against
the oracle, step for step.

Two coupled steps of the workload ``bench.py`` times (its own construction: 16 rods of 100 elements
on the GPU, one batch interactor, the 256^3 fp32 flow) run beside the oracle's restatement of the
reference loop (the slab-threaded numpy flow step, the numpy rod model with its forces at every
half step, one interactor per rod as the reference example builds them), both driven by the
oracle's dt.  The flow starts from the workload's vorticity with the free stream as its velocity,
so each step takes about 30 rod sub-steps.  Checked in FP32: vorticity and velocity within 1e-5
relative L2 of the oracle after each step, the rod state within 2e-5 of scale.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_carpet_256_coupled_steps_vs_oracle():
    import bench
    from sopht_gb300.build import build
    build()
    wl = bench.make_workload("carpet256")
    dev = torch.device("cuda", torch.cuda.current_device())
    sim, (inter,) = bench.make_gpu_case(wl, np.float32, dev)
    osim, ointers = bench.make_cpu_case(wl, np.float32)
    u0 = np.zeros((3, *wl.grid), np.float32)
    u0[0] = 1.0
    sim.velocity_field.copy_(torch.from_numpy(u0).to(dev))
    osim.velocity_field[...] = u0
    t = 0.0
    for step in range(2):
        dt = float(osim.compute_stable_timestep(dt_prefac=wl.dt_prefac))
        n_sub = inter.advance_rods(dt, wl.rod_dt, flow_time=t)
        assert n_sub >= 10
        inter()
        sim.time_step(dt=dt, free_stream_velocity=wl.u_inf)
        bench.cpu_step(wl, osim, ointers, dt=dt, t=t)
        t += dt
        torch.cuda.synchronize()
        inter.check_markers_in_domain()
        w = sim.vorticity_field.double().cpu().numpy()
        u = sim.velocity_field.double().cpu().numpy()
        assert _rel(w, osim.vorticity_field) < 1e-5, (step, _rel(w, osim.vorticity_field))
        assert _rel(u, osim.velocity_field) < 1e-5, (step, _rel(u, osim.velocity_field))
    for i, rod in enumerate(osim.rods):
        for name, ref in (("position_collection", rod.position), ("velocity_collection", rod.velocity),
                          ("director_collection", rod.directors)):
            got = inter.rod_batch.arrays[name][i].cpu().numpy()
            scale = max(np.abs(ref).max(), 1e-30)
            assert np.abs(got - ref).max() <= 2e-5 * scale, (i, name)
