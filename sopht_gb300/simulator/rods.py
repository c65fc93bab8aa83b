"""A batch of Cosserat rods advanced on the GPU (``sg_rod_batch_step``).

The rods' state and material arrays are gathered once into FP64 device tensors
with the rod index first (the ``sg_rod_batch`` layout), from rod objects with
pyelastica's ``CosseratRod`` attribute names (``position_collection``,
``velocity_collection``, ``director_collection``, ``omega_collection``,
``mass``, ``rest_lengths``, ``rest_voronoi_lengths``, ``shear_matrix``,
``bend_matrix``, ``mass_second_moment_of_inertia``,
``inv_mass_second_moment_of_inertia``, ``rest_sigma``, ``rest_kappa``,
``external_forces``, ``external_torques``).  ``step`` runs every sub-step of a
call in one launch; ``upload_loads`` refreshes the external forces and torques
(the flow forces change every sub-step in the coupled loop of
flow_past_rod_case.py:231-250); ``element_markers`` and ``set_element_loads``
are the element-centric forcing grid of the whole batch on the device (markers
laid out for one VirtualBoundaryForcing over the batch, reaction loads read
back from its forcing); ``download_into`` copies the state back.

A clamped rod keeps node 0 and the directors of element 0 where they were when
the batch was made (pyelastica's ``OneEndFixedBC`` at the start of the rod).
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from .. import _lib
from ..numeric.immersed_boundary_ops import KERNEL_TYPES, VirtualBoundaryForcing
from ..utils import default_device, ptr, sg_dtype, stream_ptr

STATE = ("position_collection", "velocity_collection", "director_collection", "omega_collection")
MATERIAL = ("mass", "rest_lengths", "rest_voronoi_lengths", "shear_matrix", "bend_matrix",
            "mass_second_moment_of_inertia", "inv_mass_second_moment_of_inertia", "rest_sigma", "rest_kappa")
LOADS = ("external_forces", "external_torques")
# sg_rod_batch field of each array
_FIELD = {"position_collection": "position", "velocity_collection": "velocity", "director_collection": "directors",
          "omega_collection": "omega", "mass": "mass", "rest_lengths": "rest_lengths",
          "rest_voronoi_lengths": "rest_voronoi_lengths", "shear_matrix": "shear_matrix",
          "bend_matrix": "bend_matrix", "mass_second_moment_of_inertia": "mass_second_moment",
          "inv_mass_second_moment_of_inertia": "inv_mass_second_moment", "rest_sigma": "rest_sigma",
          "rest_kappa": "rest_kappa", "external_forces": "external_forces", "external_torques": "external_torques"}


SHEAR_COEFFICIENT = 4.0 / 3.0  # shear correction factor of a circular cross-section


class StraightRod:
    """A straight Cosserat rod at rest, with pyelastica's ``CosseratRod`` attribute names.

    Pyelastica (``CosseratRod.straight_rod``) builds the rods SophT couples to its flows; it is not
    a dependency of this package, so this class lays out the same discrete model for the GPU batch:
    n elements of rest length L / n between n + 1 nodes from ``start`` along ``direction``, directors
    with rows (normal, direction x normal, direction), a circular cross-section of radius r (A = pi
    r^2, I = pi r^4 / 4), node masses from the element masses rho A l0 (half to each end node),
    shear/stretch matrix diag(4/3 G A, 4/3 G A, E A), bend/twist matrix diag(E I, E I, G 2I) averaged
    onto the Voronoi regions with the rest-length weights, mass second moment rho l0 diag(I, I, 2I)
    and straight rest configuration.  ``G`` defaults to E / 3 (incompressible, Poisson ratio 1/2).
    """

    def __init__(self, n_elements, start, direction, normal, base_length, base_radius, density, youngs_modulus,
                 shear_modulus=None):
        n = int(n_elements)
        if n < 1:
            raise ValueError("a rod needs at least one element")
        direction = np.asarray(direction, dtype=np.float64)
        normal = np.asarray(normal, dtype=np.float64)
        direction = direction / np.linalg.norm(direction)
        normal = normal / np.linalg.norm(normal)
        if abs(float(direction @ normal)) > 1e-12:
            raise ValueError("the normal must be perpendicular to the rod direction")
        g = youngs_modulus / 3.0 if shear_modulus is None else float(shear_modulus)
        s = np.linspace(0.0, float(base_length), n + 1)
        self.n_elems = n
        self.position_collection = np.asarray(start, dtype=np.float64)[:, None] + np.outer(direction, s)
        self.velocity_collection = np.zeros((3, n + 1))
        frame = np.stack([normal, np.cross(direction, normal), direction])
        self.director_collection = np.repeat(frame[:, :, None], n, axis=2)
        self.omega_collection = np.zeros((3, n))
        self.rest_lengths = np.diff(s)
        self.lengths = self.rest_lengths.copy()
        self.rest_voronoi_lengths = 0.5 * (self.rest_lengths[1:] + self.rest_lengths[:-1])
        self.radius = np.full(n, float(base_radius))
        area = np.pi * self.radius**2
        inertia = area**2 / (4.0 * np.pi)
        element_mass = density * area * self.rest_lengths
        self.mass = np.zeros(n + 1)
        self.mass[:-1] += 0.5 * element_mass
        self.mass[1:] += 0.5 * element_mass
        eye = np.eye(3)[:, :, None]
        self.shear_matrix = eye * np.stack([SHEAR_COEFFICIENT * g * area, SHEAR_COEFFICIENT * g * area,
                                            youngs_modulus * area])[None]
        bend = eye * np.stack([youngs_modulus * inertia, youngs_modulus * inertia, 2.0 * g * inertia])[None]
        w = self.rest_lengths
        self.bend_matrix = (bend[..., 1:] * w[1:] + bend[..., :-1] * w[:-1]) / (w[1:] + w[:-1])
        self.mass_second_moment_of_inertia = eye * np.stack([inertia, inertia, 2.0 * inertia])[None] * (
            density * self.rest_lengths)
        self.inv_mass_second_moment_of_inertia = eye / np.stack(
            [inertia, inertia, 2.0 * inertia])[None] / (density * self.rest_lengths)
        self.rest_sigma = np.zeros((3, n))
        self.rest_kappa = np.zeros((3, n - 1))
        self.external_forces = np.zeros((3, n + 1))
        self.external_torques = np.zeros((3, n))


class CosseratRodBatch:
    """Rods of one element count, their arrays on ``device`` (FP64, rod index first)."""

    def __init__(self, rods, clamped=None, device=None):
        rods = list(rods)
        if not rods:
            raise ValueError("a rod batch needs at least one rod")
        n = int(rods[0].n_elems)
        if any(int(r.n_elems) != n for r in rods):
            raise ValueError("every rod of a batch has the same number of elements")
        if not 1 <= n <= 1024:
            raise ValueError("rods of 1 to 1024 elements")
        self.n_rods, self.n_elems = len(rods), n
        self.device = torch.device(device) if device is not None else default_device()
        if self.device.type == "cuda" and self.device.index is None:  # tensors report their device index
            self.device = torch.device("cuda", torch.cuda.current_device())
        self.arrays = {}
        for name in STATE + MATERIAL + LOADS:
            host = np.stack([np.asarray(getattr(r, name), dtype=np.float64) for r in rods])
            self.arrays[name] = torch.from_numpy(np.ascontiguousarray(host)).to(self.device)
        flags = [False] * len(rods) if clamped is None else [bool(c) for c in clamped]
        if len(flags) != len(rods):
            raise ValueError("one clamp flag per rod")
        self.clamped = torch.tensor(flags, dtype=torch.int32, device=self.device)
        self.clamp_position = self.arrays["position_collection"][:, :, 0].clone()
        self.clamp_directors = self.arrays["director_collection"][..., 0].clone()
        self._batch = self._struct()

    def _struct(self):
        b = _lib.RodBatch()
        b.n_rods, b.n_elems = self.n_rods, self.n_elems
        for name, t in self.arrays.items():
            setattr(b, _FIELD[name], t.data_ptr())
        b.clamped = self.clamped.data_ptr()
        b.clamp_position = self.clamp_position.data_ptr()
        b.clamp_directors = self.clamp_directors.data_ptr()
        return b

    def upload_loads(self, rods) -> None:
        """Copy each rod's ``external_forces`` and ``external_torques`` to the device."""
        for name in LOADS:
            host = np.stack([np.asarray(getattr(r, name), dtype=np.float64) for r in rods])
            self.arrays[name].copy_(torch.from_numpy(host))

    def step(self, dt: float, n_substeps: int = 1, damping_rate: float = 0.0) -> None:
        """``n_substeps`` position-Verlet steps of ``dt`` for every rod, in one launch on the
        current stream; loads stay fixed over the call."""
        self._require_cuda()
        _lib.call("sg_rod_batch_step", ctypes.byref(self._batch), int(n_substeps), float(dt), float(damping_rate),
                  stream_ptr(self.device))

    def element_markers(self, position, velocity, dim: int = 3) -> None:
        """The element-centric markers of every rod into ``position`` and ``velocity``, float64 CUDA
        tensors (dim, n_rods * n_elems) (marker r * n + e): one launch, on the current stream."""
        for name, t in (("position", position), ("velocity", velocity)):
            self._check_marker_array(name, t, dim, (torch.float64,))
        self._require_cuda(position, velocity)
        _lib.call("sg_rod_batch_element_markers", ctypes.byref(self._batch), int(dim), position.data_ptr(),
                  velocity.data_ptr(), stream_ptr(self.device))

    def set_element_loads(self, lag_forcing, dim: int = 3) -> None:
        """Each rod's external forces from the Lagrangian forcing of its element markers (the
        reaction, half on each node) and its external torques zeroed: one launch."""
        self._check_marker_array("lag_forcing", lag_forcing, dim, (torch.float32, torch.float64))
        self._require_cuda(lag_forcing)
        dtype = _lib.SG_F32 if lag_forcing.dtype == torch.float32 else _lib.SG_F64
        _lib.call("sg_rod_batch_element_loads", ctypes.byref(self._batch), int(dim), dtype, lag_forcing.data_ptr(),
                  stream_ptr(self.device))

    def _check_marker_array(self, name, t, dim, dtypes):
        """The native entries write or read (dim, n_rods * n_elems) elements of the marker arrays as
        raw pointers: the dtype, shape, layout and device are checked here, before any launch."""
        if dim not in (2, 3):
            raise ValueError(f"dim must be 2 or 3 (got {dim})")
        if not isinstance(t, torch.Tensor):
            raise ValueError(f"{name} must be a torch tensor")
        if t.dtype not in dtypes:
            raise ValueError(f"{name} must be {' or '.join(str(d) for d in dtypes)} (got {t.dtype})")
        shape = (dim, self.n_rods * self.n_elems)
        if tuple(t.shape) != shape:
            raise ValueError(f"{name} must have shape {shape} (got {tuple(t.shape)})")
        if not t.is_contiguous():
            raise ValueError(f"{name} must be C-contiguous")
        if t.device != self.device:
            raise ValueError(f"{name} lives on {t.device}; the batch lives on {self.device}")

    def _require_cuda(self, *tensors):
        if self.device.type != "cuda":
            raise RuntimeError(f"CosseratRodBatch runs on a CUDA device; this batch lives on {self.device}")
        for t in tensors:
            if not (isinstance(t, torch.Tensor) and t.is_cuda and t.is_contiguous()):
                raise ValueError("marker arrays must be C-contiguous CUDA tensors")

    def download_into(self, rods) -> None:
        """Copy the batch's positions, velocities, directors and angular velocities into the rods."""
        host = {name: self.arrays[name].cpu().numpy() for name in STATE}
        for i, r in enumerate(rods):
            for name in STATE:
                getattr(r, name)[...] = host[name][i]


class CosseratRodBatchFlowInteraction(VirtualBoundaryForcing):
    """The element-centric forcing grid of every rod of a ``CosseratRodBatch``, in one interactor.

    The reference couples each rod through a ``CosseratRodFlowInteraction`` with a
    ``CosseratRodElementCentricForcingGrid`` (cosserat_rod_flow_interaction.py:9-58,
    cosserat_rod_forcing_grids.py:82-130) and integrates it with pyelastica on the host, calling
    ``FlowForces.apply_forces`` (flow_forces.py:22-25) inside every rod sub-step.  Here the markers of
    the whole batch (marker r * n + e: element e of rod r) share one set of Lagrangian buffers, the
    stiffness and damping are rescaled by the largest element length squared as
    immersed_body_flow_interaction.py:83-86 does for each rod, and the rods stay on the GPU:

    * ``advance_rods(flow_dt, rod_dt)`` is the rod loop of one flow step (flow_past_rod_case.py:231-243):
      ``int(flow_dt / min(flow_dt, rod_dt))`` sub-steps, each a position-Verlet step whose flow forces
      are evaluated at the half-step configuration, followed by ``time_step`` of the mismatch -- one
      launch for every rod;
    * ``__call__()`` is the interaction and spreading of the final configuration;
    * ``device_call(dev_scalars, dev_time)`` does both with the flow step's dt and time read on the
      GPU, for steps captured in a CUDA graph.

    The flow forces are the rods' only external loads (``external_forces`` and ``external_torques`` are
    overwritten by the reaction each sub-step).  ``set_base_drive`` makes the clamps of clamped rods
    turn their base about a lab axis by theta(t) = amplitude sin(2 pi frequency t + phase).
    """

    def __init__(self, rod_batch, eul_grid_forcing_field, eul_grid_velocity_field, virtual_boundary_stiffness_coeff,
                 virtual_boundary_damping_coeff, dx, real_t=np.float64, eul_grid_coord_shift=None,
                 interp_kernel_width=None, enable_eul_grid_forcing_reset=False, num_threads=False, start_time=0.0,
                 interp_kernel_type="cosine"):
        if not isinstance(eul_grid_forcing_field, torch.Tensor) or not eul_grid_forcing_field.is_cuda:
            raise ValueError("eul_grid_forcing_field must be the simulator's CUDA tensor")
        if eul_grid_forcing_field.dim() != 4 or eul_grid_forcing_field.shape[0] != 3:
            raise ValueError("the rod batch couples to a 3D flow: (3, nz, ny, nx) fields")
        if rod_batch.n_elems > 256:
            raise ValueError("the coupled rod sub-steps take rods of 1 to 256 elements")
        self.rod_batch = rod_batch
        pos = rod_batch.arrays["position_collection"]
        max_len = float(torch.linalg.vector_norm(pos[:, :, 1:] - pos[:, :, :-1], dim=1).max())
        virtual_boundary_stiffness_coeff *= max_len ** 2
        virtual_boundary_damping_coeff *= max_len ** 2
        n_markers = rod_batch.n_rods * rod_batch.n_elems
        super().__init__(virtual_boundary_stiffness_coeff, virtual_boundary_damping_coeff, 3, dx, n_markers, real_t,
                         eul_grid_coord_shift, interp_kernel_width, enable_eul_grid_forcing_reset, num_threads,
                         start_time, interp_kernel_type=interp_kernel_type, device=eul_grid_forcing_field.device)
        if rod_batch.device != self.device:
            raise ValueError(f"the rod batch lives on {rod_batch.device}, the flow on {self.device}")
        self.eul_grid_forcing_field = eul_grid_forcing_field
        self.eul_grid_velocity_field = eul_grid_velocity_field
        self.position_field = torch.zeros((3, n_markers), dtype=torch.float64, device=self.device)
        self.velocity_field = torch.zeros_like(self.position_field)
        self._drive = None
        self.compute_lag_grid_kinematics()

    def set_base_drive(self, amplitude, frequency, phases, axis=(0.0, 1.0, 0.0)) -> None:
        """Clamped rods turn their base by amplitude sin(2 pi frequency t + phases[rod]) about ``axis``."""
        phases = np.asarray(phases, dtype=np.float64)
        if phases.shape != (self.rod_batch.n_rods,):
            raise ValueError(f"one phase per rod ({self.rod_batch.n_rods})")
        axis = np.asarray(axis, dtype=np.float64)
        axis = axis / np.linalg.norm(axis)
        self._drive = (float(amplitude), float(frequency), torch.from_numpy(phases).to(self.device), axis)

    def compute_lag_grid_kinematics(self) -> None:
        """The element centres and mass-weighted element velocities of every rod (one launch)."""
        self.rod_batch.element_markers(self.position_field, self.velocity_field, dim=3)

    def __call__(self) -> None:
        """immersed_body_flow_interaction.py:113-122 for the whole batch."""
        self.compute_lag_grid_kinematics()
        self.compute_interaction_forcing(eul_grid_forcing_field=self.eul_grid_forcing_field,
                                         eul_grid_velocity_field=self.eul_grid_velocity_field,
                                         lag_grid_position_field=self.position_field,
                                         lag_grid_velocity_field=self.velocity_field)

    def compute_flow_forces_and_torques(self) -> None:
        """immersed_body_flow_interaction.py:124-131: the interaction on the markers and its reaction
        as every rod's external forces (on the device)."""
        self.compute_lag_grid_kinematics()
        self.compute_interaction_force_on_lag_grid(self.eul_grid_velocity_field, self.position_field,
                                                   self.velocity_field)
        self.rod_batch.set_element_loads(self.lag_grid_forcing_field, dim=3)

    def _coupling(self, flow_dt, flow_time, rod_dt, damping_rate, dev_scalars=None, dev_time=None):
        u = self.eul_grid_velocity_field
        if u.dtype != self.lag_grid_forcing_field.dtype or not u.is_contiguous() or tuple(u.shape[:1]) != (3,):
            raise ValueError("the flow velocity must be a contiguous (3, nz, ny, nx) tensor of real_t")
        c = _lib.RodCoupling()
        c.dtype = sg_dtype(self.real_t)
        c.nz, c.ny, c.nx = (int(x) for x in u.shape[1:])
        c.dx, c.shift = float(self.dx), float(self.eul_grid_coord_shift)
        c.kernel_type = KERNEL_TYPES[self.interp_kernel_type]
        c.flow_velocity = ptr(u)
        c.marker_position, c.marker_velocity = ptr(self.position_field), ptr(self.velocity_field)
        c.nearest = ptr(self.nearest_eul_grid_index_to_lag_grid)
        c.weights = ptr(self.interp_weights)
        c.flow_velocity_lag = ptr(self.lag_grid_flow_velocity_field)
        c.velocity_mismatch, c.position_mismatch = ptr(self._du), ptr(self._xi)
        c.lag_forcing = ptr(self.lag_grid_forcing_field)
        c.stiffness = float(self.virtual_boundary_stiffness_coeff)
        c.damping = float(self.virtual_boundary_damping_coeff)
        c.flow_dt, c.flow_time = float(flow_dt), float(flow_time)
        c.dev_scalars, c.dev_time_end = dev_scalars, dev_time
        c.max_rod_dt, c.damping_rate = float(rod_dt), float(damping_rate)
        if self._drive is not None:
            amp, freq, phases, axis = self._drive
            c.drive_phase = phases.data_ptr()
            c.drive_amplitude, c.drive_frequency = amp, freq
            c.drive_axis[:] = [float(a) for a in axis]
        c.status = ptr(self._status)
        return c

    def advance_rods(self, flow_dt: float, rod_dt: float, flow_time: float = None, damping_rate: float = 0.0) -> int:
        """The rod loop of one flow step (flow_past_rod_case.py:231-243) for every rod, in one launch;
        returns the number of rod sub-steps, int(flow_dt / min(flow_dt, rod_dt))."""
        self._flush_time_step()
        if flow_time is None:
            flow_time = self.time
        c = self._coupling(flow_dt, flow_time, rod_dt, damping_rate)
        _lib.call("sg_rod_batch_coupled_substeps", ctypes.byref(self.rod_batch._batch), ctypes.byref(c),
                  stream_ptr(self.device))
        self.time += flow_dt
        return int(flow_dt / min(flow_dt, rod_dt))

    def device_call(self, dev_scalars: int, dev_time: int, rod_dt: float, time_origin: float = 0.0,
                    damping_rate: float = 0.0) -> None:
        """``advance_rods`` and ``__call__`` with the flow step's dt and time read on the GPU.

        ``dev_scalars`` is the device address ``device_stable_timestep`` returned, ``dev_time`` the
        flow plan's device time slot (``sg_flow_device_time_slot``) and ``time_origin`` the time it
        counts from.  Nothing here reads the GPU back, so the call can be captured in a CUDA graph."""
        self._flush_time_step()
        c = self._coupling(0.0, time_origin, rod_dt, damping_rate, dev_scalars=dev_scalars, dev_time=dev_time)
        _lib.call("sg_rod_batch_coupled_substeps", ctypes.byref(self.rod_batch._batch), ctypes.byref(c),
                  stream_ptr(self.device))
        self.compute_lag_grid_kinematics()
        self._interaction(self.eul_grid_velocity_field, self.position_field, self.velocity_field)
        self._spread(self.eul_grid_forcing_field, reset=self.enable_eul_grid_forcing_reset)

    def get_grid_deviation_error_l2_norm(self) -> float:
        """immersed_body_flow_interaction.py:133-141."""
        xi = self.lag_grid_position_mismatch_field.double()
        return float(torch.linalg.vector_norm(xi).item()) / np.sqrt(self.num_lag_nodes)
