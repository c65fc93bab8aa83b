"""The oracle's 3D flow step with its sweeps run on every host core (test infrastructure).

The reference runs its 3D stencils as OpenMP-parallel pystencils kernels and
its FFTs on FFTW threads.  The oracle's FFTs already use every core
(``scipy.fft`` workers) but its numpy sweeps run on one thread, which would
understate the reference's speed on a many-core host.  This subclass splits
each sweep of the 3D step (forcing and rotational curl updates, the u x w
product, diffusion, velocity recovery, free stream, the stable-dt maximum)
into z-slabs run by a thread pool, and runs the three Poisson solves at once; numpy releases the GIL inside its array
loops, so the slabs run in parallel.  Each slab calls the oracle's own
function on a view with a one-plane halo (or, for elementwise work, on its
planes), so every cell is computed by the same operations in the same order
as the serial oracle: the results are bitwise identical.  Only ``bench.py``'s
CPU legs and the tests use it.  ``ThreadedPassiveTransportOracle`` does the same
for the 3D passive-transport step (ENO3 advection with a two-plane halo, then
diffusion).
"""

from __future__ import annotations

import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from . import stencils as st
from .flow import NavierStokes3DOracle, PassiveTransportOracle


def _split(lo: int, hi: int, parts: int):
    bounds = np.linspace(lo, hi, parts + 1).round().astype(int)
    return [(int(a), int(b)) for a, b in zip(bounds[:-1], bounds[1:]) if b > a]


class ThreadedNavierStokes3DOracle(NavierStokes3DOracle):
    """``NavierStokes3DOracle`` with slab-parallel sweeps (``threads`` workers, default all cores)."""

    def __init__(self, *args, threads=None, **kwargs):
        super().__init__(*args, **kwargs)
        if threads is None:
            threads = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
        self.threads = threads
        nz = self.grid_size[0]
        self._interior = _split(1, nz - 1, self.threads)  # z planes with both neighbours
        self._planes = _split(0, nz, self.threads)
        self._pool = ThreadPoolExecutor(self.threads)

    def _run(self, fn, ranges):
        return list(self._pool.map(fn, ranges))

    def __del__(self):
        pool = getattr(self, "_pool", None)
        if pool is not None:
            pool.shutdown(wait=False)

    # ------------------------------------------------------------ sweeps

    def _forcing_curl(self, w, f, prefactor):
        """``st.forcing_curl_update_3d`` per slab: reads f around the slab, updates only the slab's w."""
        self._run(lambda r: st.forcing_curl_update_3d(w[:, r[0] - 1:r[1] + 1], f[:, r[0] - 1:r[1] + 1], prefactor),
                  self._interior)

    def _cross(self, a, b):
        out = np.empty_like(a)

        def run(r):
            out[:, r[0]:r[1]] = st.cross_3d(a[:, r[0]:r[1]], b[:, r[0]:r[1]])

        self._run(run, self._planes)
        return out

    def _diffusion(self, w, prefactor):
        """``st.diffusion_step_3d`` per slab on a copy with its halo, then written back: every slab
        reads the field before any slab writes it, as the serial sweep does."""
        def compute(r):
            sub = w[:, r[0] - 1:r[1] + 1].copy()
            st.diffusion_step_3d(sub, prefactor)
            return sub[:, 1:-1]

        results = self._run(compute, self._interior)

        def write(item):
            (z0, z1), sub = item
            w[:, z0:z1] = sub

        self._run(write, list(zip(self._interior, results)))

    def _curl(self, psi, prefactor, out):
        def run(r):
            out[:, r[0]:r[1]] = st.curl_3d(psi[:, r[0] - 1:r[1] + 1], prefactor)[:, 1:-1]

        self._run(run, self._interior)
        out[:, 0] = 0
        out[:, -1] = 0

    def compute_stable_timestep(self, dt_prefac=1.0):
        """The serial formula with the maximum of sum |u_d| taken slab by slab (a max is exact)."""
        u = self.velocity_field
        umax = max(self._run(lambda r: np.amax(np.sum(np.fabs(u[:, r[0]:r[1]]), axis=0)), self._planes))
        tol = 10 * np.finfo(self.real_t).eps
        dt = min(self.cfl * self.dx / (umax + tol), 0.9 * self.dx ** 2 / (2 * 3) / self.nu + tol)
        return dt * dt_prefac

    # -------------------------------------------------------------- step

    def _ns_step(self, dt, free_stream_velocity):
        rt, dx = self.real_t, self.dx
        w = self.vorticity_field
        c = self._cross(self.velocity_field, w)
        self._forcing_curl(w, c, rt(dt / (2 * dx)))
        self._diffusion(w, rt(self.nu * dt / dx / dx))
        if self.filter is not None:
            st.laplacian_filter_3d(w, self.filter["order"], self.filter["type"])
        p = self.position_field
        for comp in range(3):
            st.penalise_3d(w[comp], self.width, dx, p[0], p[1], p[2])
        # the three scalar solves at once: their padding, spectral products and crops overlap
        solved = self._run(lambda c: self.poisson.solve(w[c]), range(3))
        for comp in range(3):
            self.stream_func_field[comp] = solved[comp]
        self._curl(self.stream_func_field, rt(0.5 / dx), self.velocity_field)
        if self.with_free_stream_flow:
            fs = np.asarray(free_stream_velocity)
            u = self.velocity_field

            def add(r):
                for comp in range(3):
                    u[comp, r[0]:r[1]] = u[comp, r[0]:r[1]] + fs[comp]

            self._run(add, self._planes)

    def time_step(self, dt, free_stream_velocity=(0.0, 0.0, 0.0)):
        if self.with_forcing:
            self._forcing_curl(self.vorticity_field, self.eul_grid_forcing_field,
                               self.real_t(dt / (2 * self.dx * self.rho)))
        self._ns_step(dt, free_stream_velocity)
        if self.with_forcing:
            self.eul_grid_forcing_field[...] = 0
        self.time += dt


def _default_threads():
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)


class ThreadedPassiveTransportOracle(PassiveTransportOracle):
    """``PassiveTransportOracle`` with the 3D ENO3 advection and diffusion sweeps on z-slabs.

    Advection: each slab computes ``st.eno3_flux_3d`` on a view with a two-plane
    halo and keeps its own planes; once every slab has its flux, the field is
    updated (the serial step also reads the whole field before writing it).
    Diffusion as in ``ThreadedNavierStokes3DOracle``.  2D steps run serially."""

    def __init__(self, *args, threads=None, **kwargs):
        super().__init__(*args, **kwargs)
        self.threads = _default_threads() if threads is None else threads
        nz = self.grid_size[0]
        self._pool = ThreadPoolExecutor(self.threads)
        self._eno3 = _split(2, nz - 2, self.threads) if self.grid_dim == 3 else []
        self._interior = _split(1, nz - 1, self.threads) if self.grid_dim == 3 else []

    def _run(self, fn, ranges):
        return list(self._pool.map(fn, ranges))

    def __del__(self):
        pool = getattr(self, "_pool", None)
        if pool is not None:
            pool.shutdown(wait=False)

    def _advect(self, field, inv_dx):
        u = self.velocity_field
        fluxes = self._run(lambda r: st.eno3_flux_3d(field[r[0] - 2:r[1] + 2], u[:, r[0] - 2:r[1] + 2],
                                                     inv_dx)[2:-2], self._eno3)

        def write(item):
            (z0, z1), flux = item
            field[z0:z1] = field[z0:z1] + flux

        self._run(write, list(zip(self._eno3, fluxes)))

    def _diffuse(self, comps, prefactor):
        def compute(r):
            sub = comps[:, r[0] - 1:r[1] + 1].copy()
            st.diffusion_step_3d(sub, prefactor)
            return sub[:, 1:-1]

        results = self._run(compute, self._interior)

        def write(item):
            (z0, z1), sub = item
            comps[:, z0:z1] = sub

        self._run(write, list(zip(self._interior, results)))

    def time_step(self, dt):
        if self.grid_dim == 2:
            return super().time_step(dt)
        rt, dx = self.real_t, self.dx
        dt_by_dx = rt(dt / dx)
        comps = self.primary_field[None] if self.field_type == "scalar" else self.primary_field
        for c in range(comps.shape[0]):
            self._advect(comps[c], -dt_by_dx)
        self._diffuse(comps, rt(self.nu * dt / dx / dx))
        self.time += dt
        return None
