"""Index arithmetic of the register line FFT kernels, checked on the host.

``sopht_gb300/csrc/fft_reg.cuh`` writes the phases of its kernels as
host-and-device functions; ``tests/fft_reg_host.cu`` runs each block's 256
threads phase by phase on the CPU (the kernel's barriers between phases).
These tests lay out spectra the way the 3D Poisson passes do (y lines: slabs of
nx + 1 adjacent lines per z plane; z lines: one slab of 2 ny (nx + 1) lines per
component) and compare the forward, inverse and Green's-convolution passes
with numpy's FFT, in float32, including line counts that leave the last block
partly empty and the pruned (zero-padded input, cropped output) variants.
"""

from __future__ import annotations

import ctypes
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    out = tmp_path_factory.mktemp("rl") / "librl_host.so"
    cmd = [nvcc, "-O1", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC", "-shared",
           "-gencode", "arch=compute_103a,code=sm_103a", str(ROOT / "tests" / "fft_reg_host.cu"), "-o", str(out)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    h = ctypes.CDLL(str(out))
    h.rl_host_pass.restype = ctypes.c_int
    h.rl_host_pass.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                               ctypes.c_int, ctypes.c_longlong, ctypes.c_longlong, ctypes.c_int, ctypes.c_int,
                               ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_longlong,
                               ctypes.c_int, ctypes.c_int, ctypes.c_int]
    return h


def _twiddles(n):
    m = np.arange(n)
    return np.exp(-2j * np.pi * m / n).astype(np.complex64)


def _run(h, mode, N, buf, n_lines, slab_lines, slab_stride, stride, n_in, n_out, table=None,
         g_kstride=0, g_mstride=0, g_div=1, g_mmod=0, interleave=1):
    tw = _twiddles(N)
    g = table if table is not None else np.zeros(1, np.float32)
    rc = h.rl_host_pass(mode, N, buf.ctypes.data, buf.ctypes.data, n_lines, slab_lines, slab_stride, stride,
                        n_in, n_out, tw.ctypes.data, g.ctypes.data, g_kstride, g_mstride, g_div, g_mmod,
                        interleave)
    assert rc == 0


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("N,ncomp,ny,nx,interleave", [(512, 2, 3, 6, 1), (256, 3, 2, 4, 1), (512, 1, 8, 1, 1),
                                                       (512, 3, 4, 7, 3), (256, 2, 8, 3, 2)])
def test_z_convolution_pass(lib, N, ncomp, ny, nx, interleave):
    """interleave > 1: consecutive blocks take the same lines of consecutive components."""
    rng = np.random.default_rng(N + ny)
    nz = N // 2
    nxp = nx + 1
    plane = 2 * ny * nxp
    spec = np.zeros((ncomp, nz, 2 * ny, nxp), np.complex64)
    spec[...] = (rng.standard_normal(spec.shape) + 1j * rng.standard_normal(spec.shape)).astype(np.complex64)
    table = rng.uniform(0.5, 1.5, (nz + 1, ny + 1, nxp)).astype(np.float32)
    x = np.zeros((ncomp, N, 2 * ny, nxp), np.complex128)
    x[:, :nz] = spec
    X = np.fft.fft(x, axis=1)
    k = np.arange(N)
    ks = np.minimum(k, N - k)
    m = np.arange(2 * ny)
    ms = np.minimum(m, 2 * ny - m)
    X *= table[ks][:, ms, :][None]
    ref = (np.fft.ifft(X, axis=1) * N)[:, :nz]
    buf = spec.copy()
    _run(lib, 2, N, buf, ncomp * plane, plane, nz * plane, plane, nz, nz, table,
         g_kstride=(ny + 1) * nxp, g_mstride=nxp, g_div=nxp, g_mmod=2 * ny, interleave=interleave)
    assert _rel(buf, ref) < 2e-6


@pytest.mark.parametrize("N,ncomp,nz,nx,half_in", [(512, 2, 3, 6, True), (256, 3, 2, 5, True),
                                                    (512, 1, 2, 3, False), (256, 1, 1, 16, False)])
def test_y_forward_pass(lib, N, ncomp, nz, nx, half_in):
    rng = np.random.default_rng(N + nz + nx)
    ny = N // 2
    nxp = nx + 1
    spec = np.zeros((ncomp, nz, N, nxp), np.complex64)
    n_in = ny if half_in else N
    spec[:, :, :n_in] = (rng.standard_normal((ncomp, nz, n_in, nxp))
                         + 1j * rng.standard_normal((ncomp, nz, n_in, nxp))).astype(np.complex64)
    ref = np.fft.fft(spec.astype(np.complex128), axis=2)
    buf = spec.copy()
    _run(lib, 0, N, buf, ncomp * nz * nxp, nxp, N * nxp, nxp, n_in, N)
    assert _rel(buf, ref) < 2e-6


@pytest.mark.parametrize("N,ncomp,nz,nx,half_out", [(512, 2, 3, 6, True), (256, 3, 2, 5, True),
                                                     (512, 1, 2, 3, False), (256, 2, 1, 8, False)])
def test_y_inverse_pass(lib, N, ncomp, nz, nx, half_out):
    rng = np.random.default_rng(7 * N + nz + nx)
    nxp = nx + 1
    spec = (rng.standard_normal((ncomp, nz, N, nxp))
            + 1j * rng.standard_normal((ncomp, nz, N, nxp))).astype(np.complex64)
    n_out = N // 2 if half_out else N
    ref = (np.fft.ifft(spec.astype(np.complex128), axis=2) * N)[:, :, :n_out]
    buf = spec.copy()
    _run(lib, 1, N, buf, ncomp * nz * nxp, nxp, N * nxp, nxp, N, n_out)
    assert _rel(buf[:, :, :n_out], ref) < 2e-6
    if half_out:  # points beyond the crop are left as they were
        np.testing.assert_array_equal(buf[:, :, n_out:], spec[:, :, n_out:])


@pytest.mark.parametrize("n_rows,n_out", [(40, 256), (16, 200)])
def test_rows_complex_to_real(lib, n_rows, n_out):
    """Rows of 257 bins (the x spectrum of 512-real rows) back to their first n_out reals, against
    numpy's irfft scaled by the unnormalised length (the library folds 1/N into the Green's table)."""
    lib.rl_host_rows_c2r.restype = ctypes.c_int
    lib.rl_host_rows_c2r.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_void_p, ctypes.c_void_p]
    M = 256
    rng = np.random.default_rng(n_rows)
    x = rng.standard_normal((n_rows, 2 * M))
    spec = np.fft.rfft(x, axis=1).astype(np.complex64)  # (n_rows, M + 1)
    tw_m = np.exp(-2j * np.pi * np.arange(M) / M).astype(np.complex64)
    tw_l = np.exp(-2j * np.pi * np.arange(M + 1) / (2 * M)).astype(np.complex64)
    out = np.full((n_rows, M), np.nan, np.float32)
    assert lib.rl_host_rows_c2r(spec.ctypes.data, out.ctypes.data, n_rows, M, n_out, tw_m.ctypes.data,
                                tw_l.ctypes.data) == 0
    ref = np.fft.irfft(spec.astype(np.complex128), n=2 * M, axis=1) * (2 * M)
    assert _rel(out[:, :n_out].astype(np.float64), ref[:, :n_out]) < 2e-6
    assert np.isnan(out[:, n_out:]).all()


@pytest.mark.parametrize("width", [0, 2])
def test_flow_load_pass(lib, width):
    """The 3D load pass on a (3, 5, 3, 256) field: penalised vorticity written back (the fast load's
    arithmetic, bitwise), the forcing zeroed, and the x spectrum of each penalised row against
    numpy's rfft of the row zero-padded to 512 reals."""
    lib.rl_host_flow_load.restype = ctypes.c_int
    lib.rl_host_flow_load.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 9
    nz, ny, nx = 5, 3, 256
    rng = np.random.default_rng(width)
    src = rng.standard_normal((3, nz, ny, nx)).astype(np.float32)
    dst = np.full_like(src, np.nan)
    forcing = np.ones_like(src)
    cx = rng.uniform(0.2, 1.0, nx).astype(np.float32)
    cy = rng.uniform(0.2, 1.0, ny).astype(np.float32)
    cz = rng.uniform(0.2, 1.0, nz).astype(np.float32)
    spec = np.zeros((3, nz, 2 * ny, nx + 1), np.complex64)
    tw_m = np.exp(-2j * np.pi * np.arange(nx) / nx).astype(np.complex64)
    tw_l = np.exp(-2j * np.pi * np.arange(nx + 1) / (2 * nx)).astype(np.complex64)
    assert lib.rl_host_flow_load(nz, ny, width, src.ctypes.data, dst.ctypes.data, forcing.ctypes.data,
                                 cx.ctypes.data, cy.ctypes.data, cz.ctypes.data, spec.ctypes.data,
                                 tw_m.ctypes.data, tw_l.ctypes.data) == 0

    def band(i, n):
        return i if width <= 0 else min(max(i, width - 1), n - width)

    pen = np.empty_like(src)
    for z in range(nz):
        for y in range(ny):
            row = src[:, band(z, nz), band(y, ny)][:, [band(x, nx) for x in range(nx)]]
            if width > 0:
                row = row * cx[None]
                row = row * cy[y]
                row = row * cz[z]
            pen[:, z, y] = row
    np.testing.assert_array_equal(dst, pen)
    assert not forcing.any()
    padded = np.zeros((3, nz, ny, 2 * nx))
    padded[..., :nx] = pen
    ref = np.fft.rfft(padded, axis=-1)
    assert _rel(spec[:, :, :ny].astype(np.complex128), ref) < 2e-6
    assert not spec[:, :, ny:].any()
