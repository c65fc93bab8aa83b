"""Unbounded (free-space) Poisson solves by domain doubling (oracle only).

Restates ``poisson_solver_2d/UnboundedPoissonSolverPYFFTW2D.py:8-129`` and
``poisson_solver_3d/UnboundedPoissonSolverPYFFTW3D.py:9-172`` with
``scipy.fft.rfftn/irfftn`` in place of the pyfftw plans (the inverse is
normalised by 1/N, as pyfftw's default ``normalise_idft``).  The Green's
function table is built in ``real_t`` exactly as the reference builds it, or in
float64 when ``greens_dtype=np.float64`` is asked for.
"""

from __future__ import annotations

import os

import numpy as np
import scipy.fft

_WORKERS = os.cpu_count() or 1


def greens_function_2d(ny, nx, x_range, real_t):
    """Even-reflected -ln(r)/(2 pi) on the doubled grid, regularised at r=0.

    UnboundedPoissonSolverPYFFTW2D.py:47-64
    """
    dx = real_t(x_range / nx)
    y_range = x_range * (ny / nx)
    xd = np.linspace(0, 2 * x_range - dx, 2 * nx).astype(real_t)
    yd = np.linspace(0, 2 * y_range - dx, 2 * ny).astype(real_t)
    xg, yg = np.meshgrid(xd, yd)
    r = np.sqrt(np.minimum(xg, 2 * x_range - xg) ** 2 + np.minimum(yg, 2 * y_range - yg) ** 2)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        g = -np.log(r) / (2 * np.pi)
    g[0, 0] = -(2 * np.log(dx / np.sqrt(np.pi)) - 1) / (4 * np.pi)
    return g, dx


def greens_function_3d(nz, ny, nx, x_range, real_t):
    """Even-reflected 1/(4 pi r) on the doubled grid, G(0) = 1/(4 pi dx).

    UnboundedPoissonSolverPYFFTW3D.py:56-79
    """
    dx = real_t(x_range / nx)
    y_range = x_range * (ny / nx)
    z_range = x_range * (nz / nx)
    xd = np.linspace(0, 2 * x_range - dx, 2 * nx).astype(real_t)
    yd = np.linspace(0, 2 * y_range - dx, 2 * ny).astype(real_t)
    zd = np.linspace(0, 2 * z_range - dx, 2 * nz).astype(real_t)
    zg, yg, xg = np.meshgrid(zd, yd, xd, indexing="ij")
    r = np.sqrt(np.minimum(xg, 2 * x_range - xg) ** 2 + np.minimum(yg, 2 * y_range - yg) ** 2
                + np.minimum(zg, 2 * z_range - zg) ** 2)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        g = (1 / r) / (4 * np.pi)
    g[0, 0, 0] = 1 / (4 * np.pi * dx)
    return g, dx


class UnboundedPoisson2D:
    """-lap(psi) = rhs on an unbounded 2D domain (oracle of the pyfftw solver)."""

    def __init__(self, ny, nx, x_range=1.0, real_t=np.float32, greens_dtype=None):
        self.ny, self.nx, self.real_t = ny, nx, real_t
        gdt = real_t if greens_dtype is None else greens_dtype
        g, dx = greens_function_2d(ny, nx, x_range, gdt)
        self.dx = real_t(x_range / nx)
        # UnboundedPoissonSolverPYFFTW2D.py:42-44: G_hat * dx^2
        self.greens_hat = (scipy.fft.rfftn(g, workers=_WORKERS) * (dx ** 2)).astype(
            np.complex64 if real_t == np.float32 else np.complex128)

    def solve(self, rhs):
        """UnboundedPoissonSolverPYFFTW2D.py:95-129"""
        big = np.zeros((2 * self.ny, 2 * self.nx), dtype=self.real_t)
        big[: self.ny, : self.nx] = rhs
        spec = scipy.fft.rfftn(big, workers=_WORKERS)
        spec = spec * self.greens_hat
        out = scipy.fft.irfftn(spec, s=big.shape, workers=_WORKERS)
        return out[: self.ny, : self.nx].astype(self.real_t)


class UnboundedPoisson3D:
    """-lap(psi) = rhs on an unbounded 3D domain (oracle of the pyfftw solver)."""

    def __init__(self, nz, ny, nx, x_range=1.0, real_t=np.float32, greens_dtype=None):
        self.shape = (nz, ny, nx)
        self.real_t = real_t
        gdt = real_t if greens_dtype is None else greens_dtype
        g, dx = greens_function_3d(nz, ny, nx, x_range, gdt)
        self.dx = real_t(x_range / nx)
        self.greens_hat = (scipy.fft.rfftn(g, workers=_WORKERS) * (dx ** 3)).astype(
            np.complex64 if real_t == np.float32 else np.complex128)

    def solve(self, rhs):
        """UnboundedPoissonSolverPYFFTW3D.py:111-149"""
        nz, ny, nx = self.shape
        big = np.zeros((2 * nz, 2 * ny, 2 * nx), dtype=self.real_t)
        big[:nz, :ny, :nx] = rhs
        spec = scipy.fft.rfftn(big, workers=_WORKERS)
        spec *= self.greens_hat
        out = scipy.fft.irfftn(spec, s=big.shape, workers=_WORKERS)
        return out[:nz, :ny, :nx].astype(self.real_t)

    def vector_solve(self, rhs):
        """UnboundedPoissonSolverPYFFTW3D.py:151-172: three scalar solves."""
        return np.stack([self.solve(rhs[c]) for c in range(3)])
