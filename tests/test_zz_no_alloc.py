"""The allocation-free 2D Poisson entry point against the plan-based one.

``sg_poisson2d_solve_noalloc`` exists for callers that must not allocate
device memory (work issued during CUDA graph capture, hosts whose device
memory belongs to another framework's pool, embeddings that forbid allocation
after start-up).  It keeps its workspace and Green's table in a fixed
file-scope device array.  This test calls it through the C ABI twice in a row
on different right-hand sides, compares each result with ``sg_poisson_solve``
of a regular plan at the tolerance of the other GPU tests, and checks that a
grid beyond the array's limit is rejected.  The file name makes pytest collect
it after every other test.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _rel_l2(a, b):
    return float(torch.linalg.vector_norm((a - b).double()) / torch.linalg.vector_norm(b.double()))


def test_noalloc_matches_plan_solve_twice():
    from sopht_gb300 import _lib
    from sopht_gb300.build import build

    build()
    lib = _lib.load()
    ny, nx, x_range = 96, 192, 1.0
    stream = torch.cuda.current_stream().cuda_stream
    plan = ctypes.c_void_p()
    assert lib.sg_poisson_plan_create(2, 1, ny, nx, x_range, _lib.SG_F32, 1, ctypes.byref(plan)) == 0
    try:
        gen = torch.Generator(device="cuda").manual_seed(1234)
        for call in range(2):
            rhs = torch.randn((ny, nx), generator=gen, device="cuda", dtype=torch.float32)
            ref = torch.empty_like(rhs)
            out = torch.full_like(rhs, float("nan"))
            assert lib.sg_poisson_solve(plan, rhs.data_ptr(), ref.data_ptr(), 1, 0, stream) == 0
            status = lib.sg_poisson2d_solve_noalloc(ny, nx, x_range, rhs.data_ptr(), out.data_ptr(), stream)
            assert status == 0, lib.sg_last_error()
            torch.cuda.synchronize()
            assert torch.isfinite(out).all(), f"call {call}: non-finite output"
            assert _rel_l2(out, ref) < 1e-5, f"call {call}"
            tol = float(np.float32(1e3) * np.finfo(np.float32).eps)
            assert float((out - ref).abs().max()) < tol, f"call {call}"
    finally:
        lib.sg_poisson_plan_destroy(plan)


def test_noalloc_rejects_grids_beyond_its_limit():
    from sopht_gb300 import _lib

    lib = _lib.load()
    big = torch.zeros((512, 1024), device="cuda")
    status = lib.sg_poisson2d_solve_noalloc(512, 1024, 1.0, big.data_ptr(), big.data_ptr(),
                                            torch.cuda.current_stream().cuda_stream)
    assert status == _lib.SG_ERR_SHAPE
    assert b"limit" in lib.sg_last_error()


def test_noalloc_grid_changes_rebuild_the_table():
    """Grids A, B, then A again: each call rebuilds the shared Green's table for its own grid, and
    each result matches the plan-based solve of that grid."""
    from sopht_gb300 import _lib

    lib = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    gen = torch.Generator(device="cuda").manual_seed(99)
    for ny, nx, x_range in ((64, 128, 1.0), (96, 160, 0.8), (64, 128, 1.0)):
        plan = ctypes.c_void_p()
        assert lib.sg_poisson_plan_create(2, 1, ny, nx, x_range, _lib.SG_F32, 1, ctypes.byref(plan)) == 0
        try:
            rhs = torch.randn((ny, nx), generator=gen, device="cuda", dtype=torch.float32)
            ref = torch.empty_like(rhs)
            out = torch.full_like(rhs, float("nan"))
            assert lib.sg_poisson_solve(plan, rhs.data_ptr(), ref.data_ptr(), 1, 0, stream) == 0
            assert lib.sg_poisson2d_solve_noalloc(ny, nx, x_range, rhs.data_ptr(), out.data_ptr(), stream) == 0, \
                lib.sg_last_error()
            torch.cuda.synchronize()
            assert _rel_l2(out, ref) < 1e-5, (ny, nx, x_range)
        finally:
            lib.sg_poisson_plan_destroy(plan)
