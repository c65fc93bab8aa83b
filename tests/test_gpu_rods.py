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
