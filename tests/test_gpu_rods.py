"""GPU checks of the batched rod kernels and of the divergence without a ring reset.

* the batched rod kernel against the numpy rod model: three rods (clamped and
  free, bent, twisted, loaded) in one ``CosseratRodBatch``, 300 sub-steps in
  one launch and again one launch per sub-step with damping, compared with
  ``oracle.rod.CosseratRod`` at 1e-10 of scale (FP64; the host run of the same
  passes agrees to 8e-14);
* the batch's element-centric markers and reaction loads on the device,
  bitwise the forcing grid's numpy formulas;
* ``gen_divergence_pyst_kernel_3d(reset_ghost_zone=False)`` keeps the output's
  ring and writes the same interior as the default.
"""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("per_call,damping", [(300, 0.0), (1, 3.0)])
def test_rod_batch_on_gpu_matches_the_rod_model(per_call, damping):
    import torch

    import sopht_gb300.simulator as sps
    from sopht_gb300 import _lib
    from sopht_gb300.build import build
    from test_rod_batch_host import _PyelasticaNamed, _rods
    build()
    _lib.load()
    rods = _rods()
    batch = sps.CosseratRodBatch([_PyelasticaNamed(r) for r in rods], clamped=[r.clamped is not None for r in rods])
    dt, steps = 2e-5, 300
    for _ in range(steps // per_call):
        batch.step(dt, n_substeps=per_call, damping_rate=damping)
    torch.cuda.synchronize()
    for i, rod in enumerate(rods):
        rod.damping_rate = damping
        for _ in range(steps):
            rod.step(dt)
        for name, ref in (("position_collection", rod.position), ("velocity_collection", rod.velocity),
                          ("director_collection", rod.directors), ("omega_collection", rod.omega)):
            got = batch.arrays[name][i].cpu().numpy()
            assert np.abs(got - ref).max() <= 1e-10 * max(np.abs(ref).max(), 1e-30), (i, name)


def test_divergence_keeps_the_ring_without_reset():
    import torch

    import sopht_gb300.numeric.eulerian_grid_ops as ops
    from sopht_gb300 import _lib
    from sopht_gb300.build import build
    build()
    _lib.load()
    field = torch.from_numpy(np.random.default_rng(1).standard_normal((3, 9, 10, 11))).cuda()
    reset = torch.empty((9, 10, 11), dtype=torch.float64, device="cuda")
    ops.gen_divergence_pyst_kernel_3d(np.float64)(divergence=reset, field=field, inv_dx=2.0)
    kept = torch.full((9, 10, 11), 7.0, dtype=torch.float64, device="cuda")
    ops.gen_divergence_pyst_kernel_3d(np.float64, reset_ghost_zone=False)(divergence=kept, field=field, inv_dx=2.0)
    torch.cuda.synchronize()
    r, k = reset.cpu().numpy(), kept.cpu().numpy()
    np.testing.assert_array_equal(k[1:-1, 1:-1, 1:-1], r[1:-1, 1:-1, 1:-1])
    ring = np.ones_like(k, dtype=bool)
    ring[1:-1, 1:-1, 1:-1] = False
    assert (k[ring] == 7.0).all() and (r[ring] == 0.0).all()


@pytest.mark.parametrize("dim,dtype", [(3, "float64"), (2, "float32")])
def test_rod_batch_element_markers_and_loads_on_gpu(dim, dtype):
    import torch

    import sopht_gb300.simulator as sps
    from sopht_gb300 import _lib
    from sopht_gb300.build import build
    from sopht_gb300.simulator.immersed_body import _node_to_element_velocity
    from test_rod_batch_host import N, _PyelasticaNamed, _rods
    build()
    _lib.load()
    rods = _rods()
    batch = sps.CosseratRodBatch([_PyelasticaNamed(r) for r in rods])
    m = len(rods) * N
    pos = torch.zeros((dim, m), dtype=torch.float64, device="cuda")
    vel = torch.zeros_like(pos)
    batch.element_markers(pos, vel, dim=dim)
    forcing = torch.from_numpy(np.random.default_rng(7).standard_normal((dim, m)).astype(dtype)).cuda()
    batch.set_element_loads(forcing, dim=dim)
    torch.cuda.synchronize()
    f_host = forcing.cpu().numpy().astype(np.float64)
    for r, rod in enumerate(rods):
        p = rod.position
        np.testing.assert_array_equal(pos.cpu().numpy()[:, r * N:(r + 1) * N], (p[:dim, 1:] + p[:dim, :-1]) / 2.0)
        np.testing.assert_array_equal(vel.cpu().numpy()[:, r * N:(r + 1) * N],
                                      _node_to_element_velocity(rod.mass, rod.velocity)[:dim])
        ref = np.zeros((3, N + 1))
        ref[:dim, 1:] -= 0.5 * f_host[:, r * N:(r + 1) * N]
        ref[:dim, :-1] -= 0.5 * f_host[:, r * N:(r + 1) * N]
        np.testing.assert_array_equal(batch.arrays["external_forces"][r].cpu().numpy(), ref)
        assert not batch.arrays["external_torques"][r].cpu().numpy().any()


def _flow_velocity(shape, dtype):
    """A smooth 3D velocity on the grid: a uniform stream plus a few seeded Fourier modes."""
    nz, ny, nx = shape
    z, y, x = np.meshgrid(*(np.arange(n) / n for n in shape), indexing="ij")
    rng = np.random.default_rng(11)
    u = np.zeros((3, nz, ny, nx))
    u[0] = 1.0
    for d in range(3):
        for _ in range(3):
            k = rng.integers(1, 4, 3)
            a = 0.2 * rng.standard_normal()
            u[d] += a * np.sin(2 * np.pi * (k[0] * x + k[1] * y + k[2] * z) + rng.uniform(0, 2 * np.pi))
    return u.astype(dtype)


@pytest.mark.parametrize("real_t", [np.float64, np.float32])
def test_coupled_rod_substeps_match_the_reference_loop(real_t):
    """``CosseratRodBatchFlowInteraction.advance_rods`` (one launch of sg_rod_batch_coupled_substeps)
    against the reference's rod loop restated on the oracle: every sub-step a position-Verlet step
    with the flow forces of the element-centric markers at the half step, then xi += dt dU; two flow
    steps of 5 sub-steps each, three rods (two clamped with turning bases, one free), then the
    interaction and spreading of the final configuration.  FP64: 1e-10 of scale; FP32 Lagrangian
    fields: 2e-5 of scale (the interpolation sums in another order)."""
    import torch

    import sopht_gb300.simulator as sps
    from oracle.flow import ImmersedBodyInteractionOracle, RodElementCentricGridOracle
    from oracle.rod import CosseratRod, coupled_rod_loop, element_centric_view
    from sopht_gb300 import _lib
    from sopht_gb300.build import build
    from test_rod_batch_host import _PyelasticaNamed
    build()
    _lib.load()
    shape, dx, n = (32, 32, 32), 1.0 / 32, 12
    rods = []
    for i in range(3):
        rod = CosseratRod(n, start=[0.3 + 0.2 * i, 0.5, 0.25], direction=[0.0, 0.0, 1.0], normal=[1.0, 0.0, 0.0],
                          length=0.3, radius=0.01, density=1.0, youngs_modulus=1e4, shear_modulus=1e4 / 1.5)
        if i != 1:
            rod.clamp_start()
        rods.append(rod)
    # the base drive turns every clamped rod (here rods 0 and 2, with phases 0 and 0.7)
    drive = (0.2, 1.0, 0.7, np.array([0.0, 1.0, 0.0]))
    rods[0].drive = (drive[0], drive[1], 0.0, drive[3])
    rods[2].drive = drive
    u_np = _flow_velocity(shape, real_t)
    dev = torch.device("cuda")
    u = torch.from_numpy(u_np).to(dev)
    f = torch.zeros_like(u)
    batch = sps.CosseratRodBatch([_PyelasticaNamed(r) for r in rods], clamped=[r.clamped is not None for r in rods])
    inter = sps.CosseratRodBatchFlowInteraction(batch, f, u, virtual_boundary_stiffness_coeff=-2e4,
                                                virtual_boundary_damping_coeff=-1e2, dx=dx, real_t=real_t)
    phases = np.array([0.0, 0.0, drive[2]])
    inter.set_base_drive(drive[0], drive[1], phases, axis=drive[3])
    inters = [ImmersedBodyInteractionOracle(np.zeros_like(u_np), u_np, np.zeros((3, n + 1)), np.zeros((3, n)),
                                            RodElementCentricGridOracle(element_centric_view(r)), -2e4, -1e2, dx, 3,
                                            real_t=real_t) for r in rods]
    flow_dt, rod_dt, t = 5e-4, 1e-4, 0.0
    for _ in range(2):
        for r in rods:
            r.time = t
        assert coupled_rod_loop(rods, inters, flow_dt, rod_dt) == 5
        assert inter.advance_rods(flow_dt, rod_dt, flow_time=t) == 5
        t += flow_dt
    f_ora = np.zeros_like(u_np)
    for o in inters:
        o.eul_grid_forcing_field = f_ora
        o()
    inter()
    torch.cuda.synchronize()
    inter.check_markers_in_domain()
    tol = 1e-10 if real_t == np.float64 else 2e-5
    for i, rod in enumerate(rods):
        for name, ref in (("position_collection", rod.position), ("velocity_collection", rod.velocity),
                          ("director_collection", rod.directors), ("omega_collection", rod.omega)):
            got = batch.arrays[name][i].cpu().numpy()
            scale = max(np.abs(ref).max(), 1e-30)
            assert np.abs(got - ref).max() <= tol * scale, (i, name, np.abs(got - ref).max() / scale)
    lag = {"lag_grid_forcing_field": "lag_grid_forcing_field",
           "lag_grid_position_mismatch_field": "lag_grid_position_mismatch_field",
           "lag_grid_velocity_mismatch_field": "lag_grid_velocity_mismatch_field"}
    for name, oname in lag.items():
        got = getattr(inter, name).cpu().numpy().astype(np.float64)
        ref = np.concatenate([getattr(o, oname) for o in inters], axis=1).astype(np.float64)
        assert np.abs(got - ref).max() <= tol * max(np.abs(ref).max(), 1e-30), name
    got_f = f.cpu().numpy().astype(np.float64)
    assert np.abs(got_f - f_ora).max() <= tol * np.abs(f_ora).max()
    # the driven base turned: element 0's director d3 leans by theta(t) in the x-z plane
    theta = drive[0] * np.sin(2 * np.pi * drive[1] * t + drive[2])
    d3 = batch.arrays["director_collection"][2, 2, :, 0].cpu().numpy()
    np.testing.assert_allclose(d3, [np.sin(theta), 0.0, np.cos(theta)], atol=1e-12)
