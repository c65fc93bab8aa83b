"""Many independent 2D flows advanced together (no counterpart in the reference).

``BatchedFlowSimulator2D`` takes already-built 2D simulators (any mix of
256/512/768/1024-cell x extents with 2 ny in the same set, any viscosity) and
their virtual-boundary interactors, and advances all of them with one
persistent launch per fused operator (8 launches per step for the whole
batch).  Each instance keeps its own stable dt, evaluated on the GPU from its
own velocity, exactly as ``compute_stable_timestep`` would give it, so every
instance follows the same trajectory it would follow stepped on its own with
``device_stable_timestep`` / ``time_step_device``.

The step is graph-capturable.  ``autotune`` times the launch-shape candidates
(sweep tile height 8 or 16 rows; persistent blocks per SM; 256- or 512-thread
blocks for the FFT passes) on the actual batch and keeps the fastest.
"""

from __future__ import annotations

import ctypes
import itertools

import numpy as np
import torch

from .. import _lib
from ..numeric.immersed_boundary_ops import KERNEL_TYPES
from ..utils import ptr, stream_ptr
from .flow import UnboundedNavierStokesFlowSimulator2D


class BatchedFlowSimulator2D:
    """Batch of 2D fp32 simulators with one immersed body each (or none)."""

    def __init__(self, simulators, interactors=None, free_stream_velocities=None, dt_prefac=1.0):
        n = len(simulators)
        if n == 0:
            raise ValueError("empty batch")
        interactors = list(interactors) if interactors is not None else [None] * n
        if len(interactors) != n:
            raise ValueError("one interactor (or None) per simulator")
        if free_stream_velocities is None:
            free_stream_velocities = [np.zeros(2)] * n
        self.simulators = list(simulators)
        self.interactors = interactors
        self.device = self.simulators[0].device
        members = (_lib.Batch2DMember * n)()
        for i, (sim, inter, fs) in enumerate(zip(self.simulators, interactors, free_stream_velocities,
                                                 strict=True)):
            if not isinstance(sim, UnboundedNavierStokesFlowSimulator2D):
                raise ValueError("batch members must be UnboundedNavierStokesFlowSimulator2D")
            if sim.real_t != np.float32 or not sim.with_forcing:
                raise ValueError("batch members must be fp32 simulators with forcing")
            if sim.device != self.device:
                raise ValueError("all batch members must live on one device")
            m = members[i]
            m.plan = sim._plan.value
            m.vorticity = ptr(sim.vorticity_field)
            m.velocity = ptr(sim.velocity_field)
            m.forcing = ptr(sim.eul_grid_forcing_field)
            m.stream_func = ptr(sim.stream_func_field)
            m.cfl, m.nu, m.flow_density, m.dt_prefac = sim.cfl, sim.kinematic_viscosity, sim.flow_density, dt_prefac
            v = np.zeros(2)
            if sim.with_free_stream_flow:
                v[:] = np.asarray(fs, dtype=np.float64).reshape(-1)[:2]
            m.free_stream[0], m.free_stream[1] = float(v[0]), float(v[1])
            if inter is not None:
                if inter.eul_grid_forcing_field.data_ptr() != sim.eul_grid_forcing_field.data_ptr():
                    raise ValueError(f"interactor {i} does not force simulator {i}")
                inter.upload_kinematics()
                m.n_lag = inter.num_lag_nodes
                m.kernel_type = KERNEL_TYPES[inter.interp_kernel_type]
                m.dx, m.shift = float(inter.dx), float(inter.eul_grid_coord_shift)
                m.position = ptr(inter._pos_stage.dev)
                m.body_velocity = ptr(inter._vel_stage.dev)
                m.nearest = ptr(inter.nearest_eul_grid_index_to_lag_grid)
                m.weights = ptr(inter.interp_weights)
                m.flow_velocity = ptr(inter.lag_grid_flow_velocity_field)
                m.velocity_mismatch = ptr(inter.lag_grid_velocity_mismatch_field)
                m.position_mismatch = ptr(inter.lag_grid_position_mismatch_field)
                m.lag_forcing = ptr(inter.lag_grid_forcing_field)
                m.stiffness = float(inter.virtual_boundary_stiffness_coeff)
                m.damping = float(inter.virtual_boundary_damping_coeff)
                m.status = ptr(inter._status)
        self._members = members
        self._batch = ctypes.c_void_p()
        _lib.call("sg_batch2d_create", n, members, ctypes.byref(self._batch))
        self.tuning = (16, 8, 256)
        self._primed = False

    def __len__(self):
        return len(self.simulators)

    def __del__(self):
        b = getattr(self, "_batch", None)
        if b is not None and b.value:
            try:
                _lib.load().sg_batch2d_destroy(b)
            except Exception:
                pass
            self._batch = None

    @property
    def cells(self) -> int:
        return int(sum(np.prod(s.grid_size) for s in self.simulators))

    def prime(self) -> None:
        """Evaluate every instance's velocity max once (before the first step)."""
        for sim in self.simulators:
            sim.prime_velocity_max()
        self._primed = True

    def set_tuning(self, sweep_tile_y: int, blocks_per_sm: int, fft_threads: int = 256) -> None:
        _lib.call("sg_batch2d_set_tuning", self._batch, int(sweep_tile_y), int(blocks_per_sm), int(fft_threads))
        self.tuning = (int(sweep_tile_y), int(blocks_per_sm), int(fft_threads))

    def step(self) -> None:
        """One coupled step of every instance (no synchronisation)."""
        if not self._primed:
            self.prime()
        _lib.call("sg_batch2d_step", self._batch, stream_ptr(self.device))

    def times(self) -> np.ndarray:
        """Simulated time of every instance, as accumulated on the GPU (synchronises)."""
        out = []
        for sim in self.simulators:
            out.append(sim.device_time())
        return np.asarray(out)

    def autotune(self, steps: int = 4, candidates=None) -> tuple:
        """Time the launch-shape candidates on this batch; keep the fastest.

        The candidates advance the batch (``steps`` steps each), like any
        other steps.  Returns (sweep tile height, blocks per SM, FFT block size)."""
        if candidates is None:
            candidates = list(itertools.product((16, 8), (0, 2, 4, 8, 16), (256, 512)))
        if not self._primed:
            self.prime()
        best, best_ms = None, float("inf")
        start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for cand in candidates:
            self.set_tuning(*cand)
            self.step()  # warm
            start.record()
            for _ in range(steps):
                self.step()
            stop.record()
            stop.synchronize()
            ms = start.elapsed_time(stop) / steps
            if ms < best_ms:
                best, best_ms = cand, ms
        self.set_tuning(*best)
        self.autotune_ms = best_ms
        return best
