"""Virtual-boundary forcing on CUDA tensors (mirrors sopht/numeric/immersed_boundary_ops).

``VirtualBoundaryForcing`` keeps the reference's constructor, buffers and
methods (immersed_boundary_ops/VirtualBoundaryForcing.py:20-283).  The
Lagrangian buffers live on the GPU in ``real_t``; marker positions and body
velocities are float64 (host numpy arrays are staged through pinned memory).
Support, weights, interpolation, mismatch and force are one warp-per-marker
kernel; spreading is a deterministic owner-ordered kernel without atomics.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from .. import _lib
from ..utils import default_device, normalize_real_t, ptr, sg_dtype, stream_ptr, torch_dtype

KERNEL_TYPES = {"cosine": 0, "peskin": 1}


class _PinnedStage:
    """Pinned host staging of a float64 (..., dim, n) array, reused across calls.

    Before the buffer is overwritten, the event recorded after the previous
    copy is waited on, so an in-flight upload never sees new data.  ``dev``
    may be a view into a larger device buffer (``_KinematicsStage``)."""

    def __init__(self, shape, device, dev=None):
        self.host = torch.empty(shape, dtype=torch.float64, pin_memory=True)
        self.dev = torch.empty(shape, dtype=torch.float64, device=device) if dev is None else dev
        self.event = torch.cuda.Event()
        self.pending = False

    def _wait(self):
        if self.pending:
            self.event.synchronize()

    def _send(self):
        self.dev.copy_(self.host, non_blocking=True)
        self.event.record()
        self.pending = True

    def upload(self, arr) -> torch.Tensor:
        if isinstance(arr, torch.Tensor) and arr.is_cuda:
            if arr.dtype == torch.float64 and arr.is_contiguous():
                return arr
            self.dev.copy_(arr)
            return self.dev
        self._wait()
        self.host.numpy()[...] = np.asarray(arr if not isinstance(arr, torch.Tensor) else arr.numpy())
        self._send()
        return self.dev


class _KinematicsStage:
    """Marker positions and velocities staged together: one pinned copy per call.

    ``pos`` and ``vel`` are the per-array stages; their device buffers are the
    two halves of one (2, dim, n) device array, so a call that has both on the
    host sends them in a single transfer."""

    def __init__(self, dim, n, device):
        self.both = _PinnedStage((2, dim, n), device)
        self.pos = _PinnedStage((dim, n), device, dev=self.both.dev[0])
        self.vel = _PinnedStage((dim, n), device, dev=self.both.dev[1])

    def upload(self, position, velocity):
        host_pair = not (isinstance(position, torch.Tensor) and position.is_cuda) and not (
            isinstance(velocity, torch.Tensor) and velocity.is_cuda)
        if not host_pair:
            return self.pos.upload(position), self.vel.upload(velocity)
        self.pos._wait()
        self.vel._wait()
        self.both._wait()
        h = self.both.host.numpy()
        h[0] = np.asarray(position if not isinstance(position, torch.Tensor) else position.numpy())
        h[1] = np.asarray(velocity if not isinstance(velocity, torch.Tensor) else velocity.numpy())
        self.both._send()
        return self.pos.dev, self.vel.dev


class _IBBinding:
    """Native binding of one interactor's buffers (``sg_ib_bind``).

    Owns two pinned staging slots for the marker kinematics, used in turn, and
    a pinned buffer receiving the Lagrangian forcing; ``step`` is one native
    call (kinematics upload, interaction, spreading, forcing copy)."""

    def __init__(self, vbf, key, eul_velocity):
        nz, ny, nx = vbf._extent(eul_velocity)
        dim, n = vbf.grid_dim, vbf.num_lag_nodes
        self.key = key
        self.handle = ctypes.c_void_p()
        with torch.cuda.device(vbf.device):
            _lib.call("sg_ib_bind", sg_dtype(vbf.real_t), dim, nz, ny, nx, float(vbf.dx),
                      float(vbf.eul_grid_coord_shift), n, KERNEL_TYPES[vbf.interp_kernel_type],
                      ptr(vbf.nearest_eul_grid_index_to_lag_grid), ptr(vbf.interp_weights),
                      ptr(vbf.lag_grid_flow_velocity_field), ptr(vbf._du), ptr(vbf._xi),
                      ptr(vbf.lag_grid_forcing_field), ptr(vbf._status), ptr(vbf._kin_stage.both.dev),
                      ctypes.byref(self.handle))
        self._lib = _lib.load()
        s0, s1, fh = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        _lib.call("sg_ib_binding_buffers", self.handle, ctypes.byref(s0), ctypes.byref(s1), ctypes.byref(fh))
        dbl = ctypes.POINTER(ctypes.c_double)
        self.kin = [np.ctypeslib.as_array(ctypes.cast(a.value, dbl), shape=(2, dim, n)) for a in (s0, s1)]
        self.kin_ptr = [s0.value, s1.value]
        ftype = ctypes.c_float if vbf.real_t == np.float32 else ctypes.c_double
        self.forcing = np.ctypeslib.as_array(ctypes.cast(fh.value, ctypes.POINTER(ftype)), shape=(dim, n))
        self.slot = 1
        self.used = [False, False]

    def wait(self, which: int) -> None:
        st = self._lib.sg_ib_binding_wait(self.handle, which)
        if st != _lib.SG_OK:
            _lib.call("sg_ib_binding_wait", self.handle, which)  # raises with the library's message

    def next_slot(self) -> int:
        """The next staging slot, once its previous upload has run."""
        slot = self.slot ^ 1
        self.slot = slot
        if self.used[slot]:
            self.wait(slot)
        self.used[slot] = True
        return slot

    def stage(self, position, velocity) -> int:
        """Write the kinematics into the next staging slot (after its previous upload ran)."""
        slot = self.next_slot()
        v = self.kin[slot]
        v[0] = position
        v[1] = velocity
        return slot

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                self._lib.sg_ib_unbind(h)
            except Exception:
                pass
            self.handle = None


class VirtualBoundaryForcing:
    """Feedback F = K xi + C dU between a Lagrangian body and the Eulerian flow.

    ``time_step(dt)`` (xi += dt * dU) is deferred and folded into the next
    interaction launch, which applies the same update in the same precision
    before it reads xi.  Any access to ``lag_grid_position_mismatch_field`` or
    ``lag_grid_velocity_mismatch_field`` in between first applies the pending
    update on its own, so every read sees the reference's order of operations.
    The pending update runs on the stream current at the time it is applied.
    """

    _pending_xi_dt = None
    _xi = None
    _du = None

    def __init__(self, virtual_boundary_stiffness_coeff, virtual_boundary_damping_coeff, grid_dim, dx,
                 num_lag_nodes, real_t, eul_grid_coord_shift=None, interp_kernel_width=None,
                 enable_eul_grid_forcing_reset=True, num_threads=False, start_time=0.0,
                 interp_kernel_type="cosine", device=None):
        if grid_dim not in (2, 3):
            raise ValueError("Invalid grid dimensions, must be either 2 or 3")
        real_t = normalize_real_t(real_t)
        if interp_kernel_width is None:
            interp_kernel_width = 2
        if interp_kernel_width != 2:
            raise ValueError("Interpolation kernel inconsistent with interpolation kernel width!")
        if interp_kernel_type not in KERNEL_TYPES:
            raise ValueError("Invalid interpolation kernel type. Current supported types are'cosine' and 'peskin'.")
        self.grid_dim = grid_dim
        self.virtual_boundary_stiffness_coeff = virtual_boundary_stiffness_coeff
        self.virtual_boundary_damping_coeff = virtual_boundary_damping_coeff
        self.time = start_time
        self.real_t = real_t
        self.dx = dx
        self.eul_grid_coord_shift = real_t(dx / 2) if eul_grid_coord_shift is None else eul_grid_coord_shift
        self.interp_kernel_width = interp_kernel_width
        self.interp_kernel_type = interp_kernel_type
        self.num_lag_nodes = num_lag_nodes
        self.device = default_device(device)
        dev, tdt = self.device, torch_dtype(real_t)
        n = num_lag_nodes
        self.nearest_eul_grid_index_to_lag_grid = torch.zeros((grid_dim, n), dtype=torch.int32, device=dev)
        self.interp_weights = torch.zeros(((2 * interp_kernel_width) ** grid_dim, n), dtype=tdt, device=dev)
        self.lag_grid_flow_velocity_field = torch.zeros((grid_dim, n), dtype=tdt, device=dev)
        self._xi = torch.zeros_like(self.lag_grid_flow_velocity_field)
        self._du = torch.zeros_like(self.lag_grid_flow_velocity_field)
        self._n_interactions = 0
        self.lag_grid_forcing_field = torch.zeros_like(self.lag_grid_flow_velocity_field)
        self._status = torch.zeros(1, dtype=torch.int32, device=dev)
        self._kin_stage = _KinematicsStage(grid_dim, n, dev)
        self._pos_stage = self._kin_stage.pos
        self._vel_stage = self._kin_stage.vel
        self.enable_eul_grid_forcing_reset = enable_eul_grid_forcing_reset
        if enable_eul_grid_forcing_reset:
            self.compute_interaction_forcing = (
                self.compute_interaction_force_on_eul_and_lag_grid_with_eul_grid_forcing_reset)
        else:
            self.compute_interaction_forcing = self.compute_interaction_force_on_eul_and_lag_grid

    @property
    def lag_grid_position_mismatch_field(self) -> torch.Tensor:
        self._flush_time_step()
        return self._xi

    @lag_grid_position_mismatch_field.setter
    def lag_grid_position_mismatch_field(self, value: torch.Tensor) -> None:
        self._flush_time_step()
        self._xi = value

    @property
    def lag_grid_velocity_mismatch_field(self) -> torch.Tensor:
        self._flush_time_step()
        return self._du

    @lag_grid_velocity_mismatch_field.setter
    def lag_grid_velocity_mismatch_field(self, value: torch.Tensor) -> None:
        self._flush_time_step()
        self._du = value

    def _flush_time_step(self) -> None:
        """Apply a deferred ``time_step`` now (its own kernel)."""
        dt = self._pending_xi_dt
        if dt is not None:
            self._pending_xi_dt = None
            _lib.call("sg_ib_mismatch_step", sg_dtype(self.real_t), self.grid_dim * self.num_lag_nodes,
                      ptr(self._xi), ptr(self._du), dt, stream_ptr(self.device))

    # -- grid extent of a field (component first)
    def _extent(self, field):
        if self.grid_dim == 2:
            _, ny, nx = field.shape
            return 1, ny, nx
        _, nz, ny, nx = field.shape
        return nz, ny, nx

    def _interaction(self, eul_velocity, position, body_velocity, xi_step=False, xi_dt=0.0, dev_scalars=None):
        if eul_velocity.dtype != torch_dtype(self.real_t):
            raise ValueError("Eulerian velocity dtype does not match real_t")
        pending = self._pending_xi_dt
        if pending is not None:
            if xi_step or dev_scalars is not None:
                self._flush_time_step()
            else:  # the deferred time_step rides on this launch
                self._pending_xi_dt = None
                xi_step, xi_dt = True, pending
        pos, vel = self._kin_stage.upload(position, body_velocity)
        nz, ny, nx = self._extent(eul_velocity)
        self._n_interactions += 1
        _lib.call("sg_ib_interaction", sg_dtype(self.real_t), self.grid_dim, nz, ny, nx, float(self.dx),
                  float(self.eul_grid_coord_shift), self.num_lag_nodes, KERNEL_TYPES[self.interp_kernel_type],
                  ptr(pos), ptr(vel), ptr(eul_velocity), ptr(self.nearest_eul_grid_index_to_lag_grid),
                  ptr(self.interp_weights), ptr(self.lag_grid_flow_velocity_field),
                  ptr(self._du), ptr(self._xi),
                  ptr(self.lag_grid_forcing_field), float(self.virtual_boundary_stiffness_coeff),
                  float(self.virtual_boundary_damping_coeff), int(xi_step), float(xi_dt), dev_scalars,
                  ptr(self._status), stream_ptr(self.device))

    # from this many markers on, spreading sorts the (marker, cell) pairs by cell (O(n log n)) instead of
    # scanning the lower-index markers of every pair (O(n^2)); both sum each cell in marker order.  On
    # a 256^3 grid (3D, markers of 100-element rods, launches replayed from a CUDA graph) the scan
    # takes 36, 75 and 120 us at 1024, 1600 and 2048 markers and the sort 54, 58 and 60 us (its radix
    # passes dominate), so they cross near 1300.
    SORTED_SPREAD_MIN_MARKERS = 1300
    _sorted_scratch = None

    def _spread(self, eul_forcing, reset: bool):
        nz, ny, nx = self._extent(eul_forcing)
        n = self.num_lag_nodes
        if n >= self.SORTED_SPREAD_MIN_MARKERS:
            key = (nz, ny, nx)
            if self._sorted_scratch is None or self._sorted_scratch[0] != key:
                nbytes = int(_lib.load().sg_ib_spread_sorted_scratch_bytes(self.grid_dim, nz, ny, nx, n))
                if nbytes > 0:
                    self._sorted_scratch = (key, torch.empty(nbytes, dtype=torch.uint8, device=self.device))
            if self._sorted_scratch is not None and self._sorted_scratch[0] == key:
                scratch = self._sorted_scratch[1]
                _lib.call("sg_ib_spread_sorted", sg_dtype(self.real_t), self.grid_dim, nz, ny, nx, n,
                          ptr(self.nearest_eul_grid_index_to_lag_grid), ptr(self.interp_weights),
                          ptr(self.lag_grid_forcing_field), ptr(eul_forcing), int(reset), scratch.data_ptr(),
                          scratch.numel(), stream_ptr(self.device))
                return
        _lib.call("sg_ib_spread", sg_dtype(self.real_t), self.grid_dim, nz, ny, nx, n,
                  ptr(self.nearest_eul_grid_index_to_lag_grid), ptr(self.interp_weights),
                  ptr(self.lag_grid_forcing_field), ptr(eul_forcing), int(reset), stream_ptr(self.device))

    def check_markers_in_domain(self) -> None:
        """Raise if any marker's interpolation support left the grid (synchronises)."""
        status = int(self._status.item())
        if status != 0:
            self._status.zero_()
            raise ValueError("an immersed-boundary marker's support lies outside the Eulerian grid")

    def compute_interaction_force_on_lag_grid(self, eul_grid_velocity_field, lag_grid_position_field,
                                              lag_grid_velocity_field):
        """VirtualBoundaryForcing.py:187-230."""
        self._interaction(eul_grid_velocity_field, lag_grid_position_field, lag_grid_velocity_field)

    def compute_interaction_force_on_eul_and_lag_grid(self, eul_grid_forcing_field, eul_grid_velocity_field,
                                                      lag_grid_position_field, lag_grid_velocity_field):
        """VirtualBoundaryForcing.py:232-253."""
        self._interaction(eul_grid_velocity_field, lag_grid_position_field, lag_grid_velocity_field)
        self._spread(eul_grid_forcing_field, reset=False)

    def compute_interaction_force_on_eul_and_lag_grid_with_eul_grid_forcing_reset(
            self, eul_grid_forcing_field, eul_grid_velocity_field, lag_grid_position_field,
            lag_grid_velocity_field):
        """VirtualBoundaryForcing.py:255-274."""
        self._interaction(eul_grid_velocity_field, lag_grid_position_field, lag_grid_velocity_field)
        self._spread(eul_grid_forcing_field, reset=True)

    # The three elementwise steps of the feedback law as the reference exposes them
    # (VirtualBoundaryForcing.py:132-185), in place on the first argument, for numpy arrays and
    # tensors alike.  The interaction launch computes all three fused; these serve callers that
    # compose the law themselves.

    @staticmethod
    def compute_lag_grid_velocity_mismatch_field(lag_grid_velocity_mismatch_field, lag_grid_flow_velocity_field,
                                                 lag_grid_body_velocity_field):
        """dU = U_flow - U_body."""
        lag_grid_velocity_mismatch_field[...] = lag_grid_flow_velocity_field - lag_grid_body_velocity_field

    @staticmethod
    def update_lag_grid_position_mismatch_field_via_euler_forward(lag_grid_position_mismatch_field,
                                                                  lag_grid_velocity_mismatch_field, dt):
        """xi += dt * dU."""
        lag_grid_position_mismatch_field[...] = (lag_grid_position_mismatch_field
                                                 + dt * lag_grid_velocity_mismatch_field)

    @staticmethod
    def compute_lag_grid_forcing_field(lag_grid_forcing_field, lag_grid_position_mismatch_field,
                                       lag_grid_velocity_mismatch_field, virtual_boundary_stiffness_coeff,
                                       virtual_boundary_damping_coeff):
        """F = K xi + C dU."""
        lag_grid_forcing_field[...] = (virtual_boundary_stiffness_coeff * lag_grid_position_mismatch_field
                                       + virtual_boundary_damping_coeff * lag_grid_velocity_mismatch_field)

    def time_step(self, dt):
        """VirtualBoundaryForcing.py:276-283: xi += dt * dU (deferred to the next interaction)."""
        self._flush_time_step()
        self._pending_xi_dt = float(self.real_t(dt))
        self.time += dt
