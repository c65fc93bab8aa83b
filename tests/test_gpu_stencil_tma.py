"""The 3D rotational update and diffusion with tensor-copy-staged inputs against the direct-load
kernels.

``sg_rotational_update_3d(staged=1)`` stages (u, w1) planes in shared memory by TMA and forms
u x w1 once per point; ``sg_diffusion_3d_staged``, ``sg_forcing_curl_3d_staged`` and
``sg_curl_3d_staged`` stage the diffused field's, the forcing's and the stream function's planes
(the last with the free stream and the max of sum |u_d| as the step's curl takes them);
``staged=0`` runs the direct-load kernels.  Each pair does the same arithmetic per cell, so the
outputs must agree to the bit, on grids whose x, y and z extents are not multiples of the block
tiles (partial tiles, out-of-range halo fills) and on the smallest grid the staged forms take.
The status words stay zero (no copy wait ran out): the caller's, the 3D step's plan's and the
operator entries' (the 3D passive step takes the staged diffusion).
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _lib():
    from sopht_gb300 import _lib as L
    from sopht_gb300.build import build
    build()
    L.load()
    return L


@pytest.mark.parametrize("shape", [(3, 3, 4), (5, 9, 12), (17, 70, 36), (33, 20, 64), (40, 36, 128), (64, 64, 64)])
def test_staged_rotational_update_is_bitwise_the_direct_kernel(shape):
    L = _lib()
    nz, ny, nx = shape
    rng = np.random.default_rng(nz * 1000 + ny * 10 + nx)
    w1 = torch.from_numpy(rng.standard_normal((3, nz, ny, nx)).astype(np.float32)).cuda()
    u = torch.from_numpy(rng.standard_normal((3, nz, ny, nx)).astype(np.float32)).cuda()
    direct = torch.full_like(w1, np.nan)
    staged = torch.full_like(w1, np.nan)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    pc = 0.0137
    L.call("sg_rotational_update_3d", L.SG_F32, nz, ny, nx, w1.data_ptr(), u.data_ptr(), direct.data_ptr(), pc, 0,
           None, s)
    L.call("sg_rotational_update_3d", L.SG_F32, nz, ny, nx, w1.data_ptr(), u.data_ptr(), staged.data_ptr(), pc, 1,
           status.data_ptr(), s)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    assert torch.equal(direct, staged)
    # the update against a numpy restatement (u x w1, then the curl differences; tolerance for the
    # device's fused multiply-adds)
    a, b = w1.cpu().numpy().astype(np.float64), u.cpu().numpy().astype(np.float64)
    c = np.stack([b[1] * a[2] - a[1] * b[2], b[2] * a[0] - a[2] * b[0], b[0] * a[1] - a[0] * b[1]])
    ref = a.copy()
    i = (slice(1, -1),) * 3
    sh = lambda f, d, k: np.roll(f, -k, axis=d)  # noqa: E731
    curl = np.stack([sh(c[2], 1, 1) - sh(c[2], 1, -1) - sh(c[1], 0, 1) + sh(c[1], 0, -1),
                     sh(c[0], 0, 1) - sh(c[0], 0, -1) - sh(c[2], 2, 1) + sh(c[2], 2, -1),
                     sh(c[1], 2, 1) - sh(c[1], 2, -1) - sh(c[0], 1, 1) + sh(c[0], 1, -1)])
    for d in range(3):
        ref[d][i] = a[d][i] + pc * curl[d][i]
    np.testing.assert_allclose(staged.cpu().numpy(), ref, rtol=0, atol=1e-5 * np.abs(ref).max())


def test_staged_form_refuses_what_it_cannot_copy():
    L = _lib()
    w1 = torch.zeros((3, 8, 8, 10), device="cuda")  # nx = 10: rows of 40 bytes, not a 16-byte stride
    out = torch.zeros_like(w1)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    lib = L.load()
    assert lib.sg_rotational_update_3d(L.SG_F32, 8, 8, 10, ctypes.c_void_p(w1.data_ptr()),
                                       ctypes.c_void_p(w1.data_ptr() + 0), ctypes.c_void_p(out.data_ptr()), 0.1, 1,
                                       ctypes.c_void_p(status.data_ptr()), None) == 1
    assert b"multiple of 4" in lib.sg_last_error()


def test_three_d_step_leaves_its_status_word_zero():
    import sopht_gb300.simulator as sps
    L = _lib()
    sim = sps.UnboundedNavierStokesFlowSimulator3D(grid_size=(32, 48, 64), x_range=1.0, kinematic_viscosity=1e-3,
                                                   real_t=np.float32, with_forcing=True, with_free_stream_flow=True)
    rng = np.random.default_rng(3)
    sim.vorticity_field.copy_(torch.from_numpy(rng.standard_normal(sim.vorticity_field.shape).astype(np.float32)))
    for _ in range(3):
        dt = sim.compute_stable_timestep(dt_prefac=0.5)
        sim.time_step(dt=dt, free_stream_velocity=np.array([1.0, 0.0, 0.0]))
    torch.cuda.synchronize()
    st = ctypes.c_int32(-1)
    assert L.load().sg_flow_kernel_status(sim._plan, ctypes.byref(st)) == 0
    assert st.value == 0


@pytest.mark.parametrize("ncomp", [1, 3])
@pytest.mark.parametrize("shape", [(3, 3, 4), (17, 70, 36), (40, 36, 128), (64, 64, 64)])
def test_staged_diffusion_is_bitwise_the_direct_kernel(shape, ncomp):
    L = _lib()
    nz, ny, nx = shape
    rng = np.random.default_rng(nz + ny + nx + ncomp)
    w = torch.from_numpy(rng.standard_normal((ncomp, nz, ny, nx)).astype(np.float32)).cuda()
    direct = torch.full_like(w, np.nan)
    staged = torch.full_like(w, np.nan)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    k = 0.0931
    L.call("sg_diffusion_3d_staged", L.SG_F32, nz, ny, nx, ncomp, w.data_ptr(), direct.data_ptr(), k, 0, None, s)
    L.call("sg_diffusion_3d_staged", L.SG_F32, nz, ny, nx, ncomp, w.data_ptr(), staged.data_ptr(), k, 1,
           status.data_ptr(), s)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    assert torch.equal(direct, staged)
    a = w.cpu().numpy().astype(np.float64)
    ref = a.copy()
    i = (slice(None),) + (slice(1, -1),) * 3
    lap = (a[:, 2:, 1:-1, 1:-1] + a[:, :-2, 1:-1, 1:-1] + a[:, 1:-1, 2:, 1:-1] + a[:, 1:-1, :-2, 1:-1] +
           a[:, 1:-1, 1:-1, 2:] + a[:, 1:-1, 1:-1, :-2] - 6 * a[i])
    ref[i] = a[i] + k * lap
    np.testing.assert_allclose(staged.cpu().numpy(), ref, rtol=0, atol=1e-5 * np.abs(ref).max())


def test_passive_step_takes_the_staged_diffusion_and_leaves_the_status_word_zero():
    L = _lib()
    nz, ny, nx = 32, 40, 64
    rng = np.random.default_rng(5)
    field = torch.from_numpy(rng.standard_normal((3, nz, ny, nx)).astype(np.float32)).cuda()
    vel = torch.from_numpy(0.1 * rng.standard_normal((3, nz, ny, nx)).astype(np.float32)).cuda()
    scratch = torch.empty_like(field)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    L.call("sg_passive_transport_step", L.SG_F32, 3, nz, ny, nx, 3, field.data_ptr(), scratch.data_ptr(),
           vel.data_ptr(), 0.05, 0.01, s)
    torch.cuda.synchronize()
    assert torch.isfinite(field).all()
    st = ctypes.c_int32(-1)
    assert L.load().sg_ops_kernel_status(ctypes.byref(st)) == 0
    assert st.value == 0


@pytest.mark.parametrize("shape", [(3, 3, 4), (17, 70, 36), (40, 36, 128), (64, 64, 64)])
def test_staged_forcing_curl_is_bitwise_the_direct_kernel(shape):
    L = _lib()
    nz, ny, nx = shape
    rng = np.random.default_rng(7 * nz + ny + nx)
    w = torch.from_numpy(rng.standard_normal((3, nz, ny, nx)).astype(np.float32)).cuda()
    f = torch.from_numpy(rng.standard_normal((3, nz, ny, nx)).astype(np.float32)).cuda()
    direct = torch.full_like(w, np.nan)
    staged = torch.full_like(w, np.nan)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    pf = 0.0217
    L.call("sg_forcing_curl_3d_staged", L.SG_F32, nz, ny, nx, w.data_ptr(), direct.data_ptr(), f.data_ptr(), pf, 0,
           None, s)
    L.call("sg_forcing_curl_3d_staged", L.SG_F32, nz, ny, nx, w.data_ptr(), staged.data_ptr(), f.data_ptr(), pf, 1,
           status.data_ptr(), s)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    assert torch.equal(direct, staged)
    a, b = w.cpu().numpy().astype(np.float64), f.cpu().numpy().astype(np.float64)
    sh = lambda q, d, k: np.roll(q, -k, axis=d)  # noqa: E731
    curl = np.stack([sh(b[2], 1, 1) - sh(b[2], 1, -1) - sh(b[1], 0, 1) + sh(b[1], 0, -1),
                     sh(b[0], 0, 1) - sh(b[0], 0, -1) - sh(b[2], 2, 1) + sh(b[2], 2, -1),
                     sh(b[1], 2, 1) - sh(b[1], 2, -1) - sh(b[0], 1, 1) + sh(b[0], 1, -1)])
    ref = a.copy()
    i = (slice(1, -1),) * 3
    for d in range(3):
        ref[d][i] = a[d][i] + pf * curl[d][i]
    np.testing.assert_allclose(staged.cpu().numpy(), ref, rtol=0, atol=1e-5 * np.abs(ref).max())


@pytest.mark.parametrize("free", [False, True])
@pytest.mark.parametrize("shape", [(3, 3, 4), (17, 70, 36), (40, 36, 128), (64, 64, 64)])
def test_staged_velocity_curl_is_bitwise_the_direct_kernel(shape, free):
    L = _lib()
    nz, ny, nx = shape
    rng = np.random.default_rng(11 * nz + ny + nx + free)
    psi = torch.from_numpy(rng.standard_normal((3, nz, ny, nx)).astype(np.float32)).cuda()
    direct = torch.full_like(psi, np.nan)
    staged = torch.full_like(psi, np.nan)
    umax = torch.zeros(2, dtype=torch.float32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    fs = (ctypes.c_double * 3)(1.0, -0.25, 0.5) if free else None
    pref = 0.5 * nx
    L.call("sg_curl_3d_staged", L.SG_F32, nz, ny, nx, psi.data_ptr(), direct.data_ptr(), pref, fs, umax.data_ptr(),
           0, None, s)
    L.call("sg_curl_3d_staged", L.SG_F32, nz, ny, nx, psi.data_ptr(), staged.data_ptr(), pref, fs,
           umax.data_ptr() + 4, 1, status.data_ptr(), s)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    assert torch.equal(direct, staged)
    m = umax.cpu().numpy()
    assert m[0] == m[1] == np.abs(staged.cpu().numpy()).sum(axis=0).max()
