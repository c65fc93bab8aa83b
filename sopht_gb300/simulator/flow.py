"""Unbounded vorticity Navier-Stokes flow simulators on the GPU.

Drop-in counterparts of ``sopht/simulator/flow`` (flow_simulators.py,
navier_stokes_flow_simulators.py, flow_simulators_{2,3}d.py): same
constructors, attributes and methods.  Fields are C-contiguous CUDA tensors of
``real_t``; ``position_field`` stays a host numpy array as in the reference.
One call of ``time_step`` is one fused flow step of ``libsopht_gb300.so``.

Additions beside the reference API (the plain API is unchanged):
  * ``device_stable_timestep(dt_prefac)`` evaluates the stable dt on the GPU and
    returns the device struct the step kernels read, so a whole coupled step
    can be replayed from a CUDA graph without a host round trip;
  * ``time_step_device(dev_scalars)`` is the step reading that struct.
"""

from __future__ import annotations

import ctypes
import logging
from typing import Literal

import numpy as np
import torch

from .. import _lib
from ..numeric.eulerian_grid_ops import _check_width, penalisation_factors
from ..utils import default_device, normalize_real_t, ptr, sg_dtype, stream_ptr, torch_dtype

logger = logging.getLogger(__name__)

_zeros_2 = np.zeros(2, dtype=np.float64)
_zeros_3 = np.zeros(3, dtype=np.float64)


class FlowSimulator:
    """flow_simulators.py:9-133: domain, fields, kernels, step driver."""

    def __init__(self, grid_dim, grid_size, x_range, real_t=np.float32, num_threads=1, time=0.0, device=None):
        if grid_dim not in [2, 3]:
            raise ValueError("Invalid grid dimensions. Supported values include 2 and 3.")
        self.grid_dim = grid_dim
        self.grid_size = tuple(int(g) for g in grid_size)
        self.x_range = x_range
        self.real_t = normalize_real_t(real_t)
        self.num_threads = num_threads
        self.time = time
        self.device = default_device(device)
        self._tdtype = torch_dtype(self.real_t)
        self._init_domain()
        self._init_fields()
        self._compile_kernels()
        self._finalise_flow_time_step()

    def _init_domain(self):
        """flow_simulators.py:50-95: cell-centred coordinates, component 0 = x."""
        grid_size_x = self.grid_size[-1]
        self.dx = self.real_t(self.x_range / grid_size_x)
        shift = self.dx / 2.0
        axes = []
        for n in self.grid_size:
            extent = self.x_range * n / grid_size_x
            axes.append(np.linspace(shift, extent - shift, n).astype(self.real_t))
        if self.grid_dim == 2:
            self.y_range = self.x_range * self.grid_size[0] / grid_size_x
        else:
            self.y_range = self.x_range * self.grid_size[1] / grid_size_x
            self.z_range = self.x_range * self.grid_size[0] / grid_size_x
        self.position_field = np.flipud(np.array(np.meshgrid(*axes, indexing="ij")))
        logger.info(
            "\n==================================================\n%dD flow domain initialized with "
            "dx = %s\nPlease initialize bodies within these bounds!\n"
            "==================================================", self.grid_dim, self.dx)

    def _zeros(self, *shape):
        return torch.zeros(shape, dtype=self._tdtype, device=self.device)

    def _init_fields(self):
        raise NotImplementedError

    def _compile_kernels(self):
        raise NotImplementedError

    def _finalise_flow_time_step(self):
        raise NotImplementedError

    def compute_stable_timestep(self, dt_prefac: float = 1.0):
        raise NotImplementedError

    def _update_simulator_time(self, dt):
        self.time += dt

    def time_step(self, dt, **kwargs):
        """flow_simulators.py:130-133."""
        self._flow_time_step(dt=dt, **kwargs)
        self._update_simulator_time(dt=dt)


class _UnboundedNavierStokesBase(FlowSimulator):
    _filter_type = 0
    _filter_order = 0

    def _make_plan(self):
        w = self.penalty_zone_width
        _check_width(w)
        pos = self.position_field
        if self.grid_dim == 2:
            nz, (ny, nx) = 1, self.grid_size
            cx = penalisation_factors(w, self.dx, pos[0][0, :], self.real_t)
            cy = penalisation_factors(w, self.dx, pos[1][:, 0], self.real_t)
            cz = None
        else:
            nz, ny, nx = self.grid_size
            cx = penalisation_factors(w, self.dx, pos[0][0, 0, :], self.real_t)
            cy = penalisation_factors(w, self.dx, pos[1][0, :, 0], self.real_t)
            cz = penalisation_factors(w, self.dx, pos[2][:, 0, 0], self.real_t)
        self._coef_tables = (cx, cy, cz)
        host = [c.ctypes.data_as(ctypes.c_void_p) if c is not None else None for c in (cx, cy, cz)]
        self._plan = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.call("sg_flow_plan_create", self.grid_dim, nz, ny, nx, float(self.x_range), sg_dtype(self.real_t),
                      int(w), host[0] if w > 0 else None, host[1] if w > 0 else None,
                      host[2] if w > 0 else None, self._filter_type, self._filter_order, ctypes.byref(self._plan))
        self._host_max = ctypes.c_double()
        self._host_max_ref = ctypes.byref(self._host_max)
        self._checked_fields = None

    @property
    def device_bytes(self) -> int:
        """Device memory held by the step plan (FFT workspace, Green's table, scratch)."""
        return int(_lib.load().sg_flow_plan_bytes(self._plan))

    def __del__(self):
        plan = getattr(self, "_plan", None)
        if plan is not None and plan.value:
            try:
                _lib.load().sg_flow_plan_destroy(plan)
            except Exception:
                pass
            self._plan = None

    def _check_fields(self):
        for name in ("vorticity_field", "velocity_field", "stream_func_field"):
            t = getattr(self, name)
            if t.dtype != self._tdtype or not t.is_contiguous() or t.device != self.device:
                raise ValueError(f"{name} must stay a contiguous {self._tdtype} tensor on {self.device}")

    def _scalars(self, dt, free_stream_velocity) -> _lib.StepScalars:
        rt, dx = self.real_t, self.dx
        sc = _lib.StepScalars()
        sc.dt = float(dt)
        if self.with_forcing:
            sc.forcing_prefac = float(rt(dt / (2 * dx * self.flow_density)))
        if self.grid_dim == 2:
            sc.advection_prefac = float(rt(dt / dx))
        else:
            sc.advection_prefac = float(rt(dt / (2 * dx)))
        sc.diffusion_prefac = float(rt(self.kinematic_viscosity * dt / dx / dx))
        if self.with_free_stream_flow:
            fs = np.asarray(free_stream_velocity, dtype=np.float64).reshape(-1)
            for c in range(self.grid_dim):
                sc.free_stream[c] = float(rt(fs[c]))
        return sc

    def _step(self, scalars_ptr, dev_scalars):
        forcing = self.eul_grid_forcing_field if self.with_forcing else None
        w, u, psi = self.vorticity_field, self.velocity_field, self.stream_func_field
        key = (w, u, psi, forcing, w.data_ptr(), u.data_ptr(), psi.data_ptr())
        c = self._checked_fields
        if c is None or any(a is not b for a, b in zip(c[:4], key[:4])) or c[4:] != key[4:]:
            # dtype, layout and device are checked again only when a field object or its storage changes
            self._check_fields()
            self._checked_fields = key
        _lib.call("sg_flow_step", self._plan, key[4], key[5], ptr(forcing), key[6], scalars_ptr, dev_scalars,
                  stream_ptr(self.device))

    def _flow_time_step(self, dt, free_stream_velocity=None):
        if free_stream_velocity is None:
            free_stream_velocity = _zeros_2 if self.grid_dim == 2 else _zeros_3
        sc = self._scalars(dt, free_stream_velocity)
        self._step(ctypes.byref(sc), None)

    def compute_stable_timestep(self, dt_prefac: float = 1.0):
        """navier_stokes_flow_simulators.py:212-223 / :501-512 (synchronises).

        The max of sum_d |u_d| is reduced on the GPU and read back through a
        pinned word of the plan (one call, one stream drain); the dt formula of
        passive_transport_flow_simulators.py:139-155 is then evaluated on the
        host with the reference's numpy scalar types, so the value is the same.
        """
        _lib.call("sg_flow_host_max", self._plan, ptr(self.velocity_field), self._host_max_ref,
                  stream_ptr(self.device))
        umax = self.real_t(self._host_max.value)
        rt = self.real_t
        tol = 10 * np.finfo(rt).eps
        dt = min(self.cfl * self.dx / (umax + tol),
                 0.9 * self.dx**2 / (2 * self.grid_dim) / self.kinematic_viscosity + tol)
        return dt * dt_prefac

    # ---- device-resident additions
    def device_stable_timestep(self, dt_prefac: float = 1.0, free_stream_velocity=None, recompute_max=True):
        """Stable dt and step prefactors evaluated on the GPU (no synchronisation).

        Returns the device address of the ``sg_step_scalars`` struct that
        ``time_step_device`` and the interactors' device-mode calls read.  With
        ``recompute_max=False`` the max of the velocity left by the previous
        step is used (the flow step records it), which is what a captured time
        loop does.
        """
        fs_arr = np.zeros(3, dtype=np.float64)
        if free_stream_velocity is not None and self.with_free_stream_flow:
            v = np.asarray(free_stream_velocity, dtype=np.float64).reshape(-1)[: self.grid_dim]
            fs_arr[: v.shape[0]] = v
        fs = (ctypes.c_double * 3)(*fs_arr.tolist())
        out = ctypes.c_void_p()
        _lib.call("sg_flow_device_dt", self._plan, ptr(self.velocity_field) if recompute_max else None,
                  float(self.cfl), float(self.kinematic_viscosity), float(self.flow_density), float(dt_prefac), fs,
                  ctypes.byref(out), stream_ptr(self.device))
        return out.value

    def prime_velocity_max(self) -> None:
        """Record max sum_d |u_d| of the current velocity for the first device-resident dt."""
        _lib.call("sg_flow_prime_max", self._plan, ptr(self.velocity_field), stream_ptr(self.device))

    def device_time_slot(self) -> int:
        """Device address of the time the device-resident dt accumulates (seconds since the plan was
        made, the end of the current step once its dt is computed)."""
        out = ctypes.c_void_p()
        _lib.call("sg_flow_device_time_slot", self._plan, ctypes.byref(out))
        return out.value

    def device_time(self) -> float:
        """Time accumulated on the GPU by the device-resident dt (synchronises)."""
        out = ctypes.c_double()
        _lib.call("sg_flow_read_device_time", self._plan, ctypes.byref(out))
        return self.time + out.value

    def time_step_device(self, dev_scalars: int) -> None:
        """One flow step with dt and prefactors read from device memory."""
        self._step(None, ctypes.c_void_p(dev_scalars))


class UnboundedNavierStokesFlowSimulator2D(_UnboundedNavierStokesBase):
    """navier_stokes_flow_simulators.py:24-223."""

    def __init__(self, grid_size, x_range, kinematic_viscosity, cfl=0.1, real_t=np.float32, num_threads=1,
                 time=0.0, with_forcing=False, with_free_stream_flow=False, flow_density=1.0, **kwargs):
        self.kinematic_viscosity = kinematic_viscosity
        self.cfl = cfl
        self.with_forcing = with_forcing
        self.with_free_stream_flow = with_free_stream_flow
        self.flow_density = flow_density
        self.penalty_zone_width = kwargs.get("penalty_zone_width", 2)
        super().__init__(grid_dim=2, grid_size=grid_size, x_range=x_range, real_t=real_t, num_threads=num_threads,
                         time=time, device=kwargs.get("device"))

    def _init_fields(self):
        self.vorticity_field = self._zeros(*self.grid_size)
        self.velocity_field = self._zeros(self.grid_dim, *self.grid_size)
        self.buffer_scalar_field = self._zeros(*self.grid_size)
        self.stream_func_field = self._zeros(*self.grid_size)
        if self.with_forcing:
            self.eul_grid_forcing_field = self._zeros(self.grid_dim, *self.grid_size)

    def _compile_kernels(self):
        self._make_plan()

    def _finalise_flow_time_step(self):
        pass


class UnboundedNavierStokesFlowSimulator3D(_UnboundedNavierStokesBase):
    """navier_stokes_flow_simulators.py:226-522."""

    def __init__(self, grid_size, x_range, kinematic_viscosity, cfl=0.1, real_t=np.float32, num_threads=1,
                 time=0.0, with_forcing=False, with_free_stream_flow=False, filter_vorticity=False,
                 flow_density=1.0,
                 poisson_solver_type: Literal["greens_function_convolution",
                                              "fast_diagonalisation"] = "greens_function_convolution",
                 **kwargs):
        self.kinematic_viscosity = kinematic_viscosity
        self.cfl = cfl
        self.with_forcing = with_forcing
        self.with_free_stream_flow = with_free_stream_flow
        self.penalty_zone_width = kwargs.get("penalty_zone_width", 2)
        self.filter_vorticity = filter_vorticity
        if self.filter_vorticity:
            self.filter_setting_dict = kwargs.get("filter_setting_dict", {"order": 2, "type": "multiplicative"})
            logger.info("Vorticity filtering is turned on: order = %s, type = %s",
                        self.filter_setting_dict["order"], self.filter_setting_dict["type"])
            types = {"multiplicative": 1, "convolution": 2}
            if self.filter_setting_dict["type"] not in types:
                raise ValueError("Invalid filter type")
            self._filter_type = types[self.filter_setting_dict["type"]]
            self._filter_order = int(self.filter_setting_dict["order"])
        self.flow_density = flow_density
        if poisson_solver_type not in ("greens_function_convolution", "fast_diagonalisation"):
            raise ValueError("Invalid Poisson solver type given")
        if poisson_solver_type == "fast_diagonalisation":
            raise NotImplementedError(
                "the fast-diagonalisation Poisson solver is outside the GPU flow-step path; "
                "use poisson_solver_type='greens_function_convolution'")
        self.poisson_solver_type = poisson_solver_type
        super().__init__(grid_dim=3, grid_size=grid_size, x_range=x_range, real_t=real_t, num_threads=num_threads,
                         time=time, device=kwargs.get("device"))

    def _init_fields(self):
        self.vorticity_field = self._zeros(self.grid_dim, *self.grid_size)
        self.velocity_field = torch.zeros_like(self.vorticity_field)
        self.buffer_vector_field = torch.zeros_like(self.vorticity_field)
        self.buffer_scalar_field = self.buffer_vector_field[0]
        self.stream_func_field = torch.zeros_like(self.vorticity_field)
        if self.with_forcing:
            self.eul_grid_forcing_field = torch.zeros_like(self.velocity_field)

    def _compile_kernels(self):
        self._make_plan()

    def _finalise_flow_time_step(self):
        pass

    def get_vorticity_divergence_l2_norm(self) -> float:
        """navier_stokes_flow_simulators.py:514-522."""
        nz, ny, nx = self.grid_size
        div = self.buffer_scalar_field
        _lib.call("sg_divergence_3d", sg_dtype(self.real_t), nz, ny, nx, ptr(self.vorticity_field), ptr(div),
                  float(self.real_t(1.0 / self.dx)), stream_ptr(self.device))
        return float(torch.linalg.vector_norm(div.double()).item()) * self.dx ** (self.grid_dim / 2.0)


def create_unbounded_flow_simulator_2d(grid_size, x_range, kinematic_viscosity, cfl=0.1,
                                       flow_type="navier_stokes", real_t=np.float32, num_threads=1, time=0.0,
                                       **kwargs):
    """flow_simulators_2d.py:8-55."""
    match flow_type:
        case "navier_stokes":
            with_forcing = False
        case "navier_stokes_with_forcing":
            with_forcing = True
        case _:
            raise ValueError("Invalid flow type given")
    return UnboundedNavierStokesFlowSimulator2D(
        grid_size=grid_size, x_range=x_range, kinematic_viscosity=kinematic_viscosity, cfl=cfl, real_t=real_t,
        num_threads=num_threads, time=time, with_forcing=with_forcing, **kwargs)


def create_unbounded_flow_simulator_3d(grid_size, x_range, kinematic_viscosity, cfl=0.1,
                                       flow_type="navier_stokes", real_t=np.float32, num_threads=1,
                                       filter_vorticity=False,
                                       poisson_solver_type="greens_function_convolution", time=0.0, **kwargs):
    """flow_simulators_3d.py:8-65."""
    match flow_type:
        case "navier_stokes":
            with_forcing = False
        case "navier_stokes_with_forcing":
            with_forcing = True
        case _:
            raise ValueError("Invalid flow type given")
    return UnboundedNavierStokesFlowSimulator3D(
        grid_size=grid_size, x_range=x_range, kinematic_viscosity=kinematic_viscosity, cfl=cfl, real_t=real_t,
        num_threads=num_threads, time=time, with_forcing=with_forcing, filter_vorticity=filter_vorticity,
        poisson_solver_type=poisson_solver_type, **kwargs)


def compute_advection_diffusion_stable_timestep(velocity_field, velocity_magnitude_field, grid_dim, dx, cfl,
                                                kinematic_viscosity, real_t=np.float32):
    """passive_transport_flow_simulators.py:139-155 (synchronises).

    The max of sum_d |u_d| is reduced by the library's kernel; as in the reference,
    ``velocity_magnitude_field`` receives sum_d |u_d|."""
    real_t = normalize_real_t(real_t)
    torch.sum(torch.abs(velocity_field), dim=0, out=velocity_magnitude_field)
    slot = torch.zeros(1, dtype=torch.float64, device=velocity_field.device)
    _lib.call("sg_max_abs_sum", sg_dtype(real_t), grid_dim, int(velocity_field[0].numel()), ptr(velocity_field),
              ptr(slot), stream_ptr(velocity_field.device))
    umax = real_t(slot.item())
    tol = 10 * np.finfo(real_t).eps
    return min(cfl * dx / (umax + tol), 0.9 * dx**2 / (2 * grid_dim) / kinematic_viscosity + tol)


class PassiveTransportFlowSimulator(FlowSimulator):
    """passive_transport_flow_simulators.py:14-136: advection (ENO3) and diffusion of a passive
    scalar (2D, 3D) or vector (3D) ``primary_field`` in a given ``velocity_field``.

    One ``time_step`` is one ``sg_passive_transport_step`` call, in place: in 2D one fused sweep
    through ``buffer_scalar_field``; in 3D one advection kernel (a vector field's three components
    per thread) into a scratch field and one diffusion kernel back (the scratch of a vector field is
    a private three-component buffer)."""

    def __init__(self, kinematic_viscosity, grid_dim, grid_size, x_range, cfl=0.1, real_t=np.float32,
                 num_threads=1, time=0.0, field_type: Literal["scalar", "vector"] = "scalar", **kwargs):
        if field_type not in ["scalar", "vector"]:
            raise ValueError("Invalid field type. Supported values include 'scalar' and 'vector'")
        if grid_dim == 2 and field_type == "vector":
            raise ValueError("Passive transport of vector 2D fields not supported yet.")
        self.kinematic_viscosity = kinematic_viscosity
        self.cfl = cfl
        self.field_type = field_type
        super().__init__(grid_dim=grid_dim, grid_size=grid_size, x_range=x_range, real_t=real_t,
                         num_threads=num_threads, time=time, device=kwargs.get("device"))

    def _init_fields(self):
        if self.field_type == "scalar":
            self.primary_field = self._zeros(*self.grid_size)
        else:
            self.primary_field = self._zeros(self.grid_dim, *self.grid_size)
        self.velocity_field = self._zeros(self.grid_dim, *self.grid_size)
        # the reference's shared advection / diffusion flux buffer; here the step's scratch field
        self.buffer_scalar_field = self._zeros(*self.grid_size)
        self._vector_scratch = self._zeros(self.grid_dim, *self.grid_size) if self.field_type == "vector" else None
        self._max_slot = torch.zeros(1, dtype=torch.float64, device=self.device)

    def _compile_kernels(self):
        pass

    def _advection_and_diffusion_time_step(self, dt, **kwargs):
        """passive_transport_flow_simulators.py:104-118."""
        del kwargs
        for name in ("primary_field", "velocity_field", "buffer_scalar_field"):
            t = getattr(self, name)
            if t.dtype != self._tdtype or not t.is_contiguous() or t.device != self.device:
                raise ValueError(f"{name} must stay a contiguous {self._tdtype} tensor on {self.device}")
        dt_by_dx = self.real_t(dt / self.dx)
        nu_dt_by_dx2 = self.real_t(self.kinematic_viscosity * dt / self.dx / self.dx)
        if self.grid_dim == 2:
            nz, (ny, nx) = 1, self.grid_size
        else:
            nz, ny, nx = self.grid_size
        ncomp = 1 if self.field_type == "scalar" else self.grid_dim
        scratch = self.buffer_scalar_field if ncomp == 1 else self._vector_scratch
        _lib.call("sg_passive_transport_step", sg_dtype(self.real_t), self.grid_dim, nz, ny, nx, ncomp,
                  ptr(self.primary_field), ptr(scratch), ptr(self.velocity_field),
                  float(dt_by_dx), float(nu_dt_by_dx2), stream_ptr(self.device))

    def _finalise_flow_time_step(self):
        self._flow_time_step = self._advection_and_diffusion_time_step

    def compute_stable_timestep(self, dt_prefac: float = 1.0):
        """passive_transport_flow_simulators.py:125-136 (synchronises; the magnitude field is not kept)."""
        n = int(np.prod(self.grid_size))
        _lib.call("sg_max_abs_sum", sg_dtype(self.real_t), self.grid_dim, n, ptr(self.velocity_field),
                  ptr(self._max_slot), stream_ptr(self.device))
        umax = self.real_t(self._max_slot.item())
        rt = self.real_t
        tol = 10 * np.finfo(rt).eps
        dt = min(self.cfl * self.dx / (umax + tol),
                 0.9 * self.dx**2 / (2 * self.grid_dim) / self.kinematic_viscosity + tol)
        return dt * dt_prefac
