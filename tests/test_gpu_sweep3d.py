"""The 3D step's stencil chain equals the single-operator entry points, bitwise.

One 3D step writes back Pen(w3) with w3 = diffusion(rotational update(forcing
curl(w))).  Here the same chain runs through the single-operator entry points
(forcing curl, cross product, a second curl update with the advection prefactor,
diffusion, penalisation) and the vorticity must agree to the bit.  Ragged
extents (FFT lengths with factors 2, 3, 5, 7 only) cover partial tiles and
partial z blocks.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from sopht_gb300.build import build
    build()


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


@pytest.mark.parametrize("precision", ["single", "double"])
@pytest.mark.parametrize("shape,forcing,width", [((20, 36, 42), True, 2), ((35, 21, 70), True, 3),
                                                 ((16, 24, 32), False, 0), ((40, 40, 40), True, 2)])
def test_step_stencils_equal_operator_chain(precision, shape, forcing, width):
    import sopht_gb300.simulator as sps
    from sopht_gb300 import _lib as L
    rt = np.float32 if precision == "single" else np.float64
    tdt = torch.float32 if rt == np.float32 else torch.float64
    sgt = 0 if rt == np.float32 else 1
    nz, ny, nx = shape
    sim = sps.UnboundedNavierStokesFlowSimulator3D(shape, 1.0, 2e-3, real_t=rt, with_forcing=forcing,
                                                   penalty_zone_width=width)
    r = np.random.default_rng(5)
    w = torch.as_tensor(r.standard_normal((3, *shape)), dtype=tdt, device="cuda")
    u = torch.as_tensor(r.standard_normal((3, *shape)), dtype=tdt, device="cuda")
    f = torch.as_tensor(r.standard_normal((3, *shape)), dtype=tdt, device="cuda")
    sim.vorticity_field.copy_(w)
    sim.velocity_field.copy_(u)
    if forcing:
        sim.eul_grid_forcing_field.copy_(f)
    dt = 1.3e-3
    sc = sim._scalars(dt, (0.0, 0.0, 0.0))
    sim._step(ctypes.byref(sc), None)
    torch.cuda.synchronize()
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    n = int(np.prod(shape))
    w1 = torch.empty_like(w)
    if forcing:
        L.call("sg_forcing_curl_update_3d", sgt, nz, ny, nx, _p(w), _p(w1), _p(f), sc.forcing_prefac, s)
    else:
        w1.copy_(w)
    cr = torch.empty_like(w)
    L.call("sg_cross_3d", sgt, n, _p(u), _p(w1), _p(cr), s)
    w2 = torch.empty_like(w)
    L.call("sg_forcing_curl_update_3d", sgt, nz, ny, nx, _p(w1), _p(w2), _p(cr), sc.advection_prefac, s)
    w3 = torch.empty_like(w)
    L.call("sg_diffusion_step_3d", sgt, nz, ny, nx, _p(w2), _p(w3), sc.diffusion_prefac, s)
    wp = torch.empty_like(w)
    tabs = [torch.as_tensor(t, device="cuda") for t in sim._coef_tables] if width > 0 else [None] * 3
    L.call("sg_penalise_3d", sgt, nz, ny, nx, _p(w3), _p(wp), width, *[_p(t) for t in tabs], s)
    torch.cuda.synchronize()
    assert torch.equal(sim.vorticity_field, wp)
