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
from ..utils import default_device, stream_ptr

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
