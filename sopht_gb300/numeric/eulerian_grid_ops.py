"""Eulerian grid operators on CUDA tensors (mirrors sopht/numeric/eulerian_grid_ops).

The reference exposes its stencils as kernel *factories* ``gen_*(real_t, ...)``
returning a callable that updates caller arrays in place
(sopht/numeric/eulerian_grid_ops/__init__.py).  The factories here keep those
names, arguments and in-place semantics, on C-contiguous CUDA tensors, and
dispatch to the sm_103a kernels of ``libsopht_gb300.so``.  ``num_threads`` and
``fixed_grid_size`` are accepted for compatibility and ignored.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from .. import _lib
from ..utils import normalize_real_t, ptr, sg_dtype, stream_ptr, torch_dtype


def penalisation_factors(width: int, dx, coords: np.ndarray, real_t) -> np.ndarray:
    """Per-index factor of the boundary penalisation along one axis.

    penalise_field_boundary_2d.py:40-140 multiplies the band values by
    sin((pi/2)/(width dx) * (x - x_first)) at the front and by
    sin((pi/2)/(width dx) * (x_last - x)) at the back; every other index keeps
    factor 1 (an exact no-op multiply).  ``coords`` are the cell-centre
    coordinates of that axis in ``real_t``.
    """
    real_t = normalize_real_t(real_t)
    coords = np.asarray(coords, dtype=real_t)
    fac = np.ones(coords.shape[0], dtype=real_t)
    if width > 0:
        sine_prefactor = (np.pi / 2) / (width * dx)
        fac[:width] = np.sin(sine_prefactor * (coords[:width] - coords[0]))
        fac[-width:] = np.sin(sine_prefactor * (coords[-1] - coords[-width:]))
    return fac


def _check_width(width) -> None:
    if not isinstance(width, (int, np.integer)) or width < 0:
        raise ValueError("Invalid zone width, must be a non-negative integer")
    if width == 1:
        # penalise_field_boundary_2d.py:131 copies field[:, -1:0] (an empty
        # slice) into the back band, so the reference cannot run width 1
        raise ValueError("Invalid zone width 1: the back band copy field[:, -1:0] is empty")


class _PoissonBase:
    def __init__(self, dim, nz, ny, nx, x_range, real_t):
        self.real_t = normalize_real_t(real_t)
        self.dx = self.real_t(x_range / nx)
        self._plan = ctypes.c_void_p()
        _lib.call("sg_poisson_plan_create", dim, nz, ny, nx, float(x_range), sg_dtype(self.real_t),
                  3 if dim == 3 else 1, ctypes.byref(self._plan))

    @property
    def device_bytes(self) -> int:
        return int(_lib.load().sg_poisson_plan_bytes(self._plan))

    def __del__(self):
        plan = getattr(self, "_plan", None)
        if plan is not None and plan.value:
            try:
                _lib.load().sg_poisson_plan_destroy(plan)
            except Exception:
                pass
            self._plan = None

    def _solve(self, sol: torch.Tensor, rhs: torch.Tensor, ncomp: int, comp_stride: int) -> None:
        dt = torch_dtype(self.real_t)
        if sol.dtype != dt or rhs.dtype != dt:
            raise ValueError("field dtype does not match the solver's real_t")
        _lib.call("sg_poisson_solve", self._plan, ptr(rhs), ptr(sol), ncomp, comp_stride, stream_ptr(rhs.device))


class UnboundedPoissonSolver2D(_PoissonBase):
    """UnboundedPoissonSolverPYFFTW2D (poisson_solver_2d/UnboundedPoissonSolverPYFFTW2D.py:8-129)."""

    def __init__(self, grid_size_y, grid_size_x, x_range=1.0, num_threads=1, real_t=np.float64):
        self.grid_size_y, self.grid_size_x = grid_size_y, grid_size_x
        self.x_range = x_range
        self.y_range = x_range * (grid_size_y / grid_size_x)
        super().__init__(2, 1, grid_size_y, grid_size_x, x_range, real_t)

    def solve(self, solution_field: torch.Tensor, rhs_field: torch.Tensor) -> None:
        """-lap(solution) = rhs on the unbounded domain (:95-129)."""
        self._solve(solution_field, rhs_field, 1, 0)


class UnboundedPoissonSolver3D(_PoissonBase):
    """UnboundedPoissonSolverPYFFTW3D (poisson_solver_3d/UnboundedPoissonSolverPYFFTW3D.py:9-172)."""

    def __init__(self, grid_size_z, grid_size_y, grid_size_x, x_range=1.0, num_threads=1, real_t=np.float64):
        self.grid_size_z, self.grid_size_y, self.grid_size_x = grid_size_z, grid_size_y, grid_size_x
        self.x_range = x_range
        super().__init__(3, grid_size_z, grid_size_y, grid_size_x, x_range, real_t)

    def solve(self, solution_field: torch.Tensor, rhs_field: torch.Tensor) -> None:
        """One scalar solve (:111-149)."""
        self._solve(solution_field, rhs_field, 1, 0)

    def vector_field_solve(self, solution_vector_field: torch.Tensor, rhs_vector_field: torch.Tensor) -> None:
        """Three component solves in one batched pass (:151-172)."""
        n = rhs_vector_field[0].numel()
        self._solve(solution_vector_field, rhs_vector_field, 3, n)


# names the reference's simulators and users import
UnboundedPoissonSolverPYFFTW2D = UnboundedPoissonSolver2D
UnboundedPoissonSolverPYFFTW3D = UnboundedPoissonSolver3D


# ---------------------------------------------------------------- factories


def _scratch_like(t: torch.Tensor, cache: dict) -> torch.Tensor:
    key = (tuple(t.shape), t.dtype, t.device)
    buf = cache.get(key)
    if buf is None:
        buf = torch.empty_like(t)
        cache[key] = buf
    return buf


def gen_advection_timestep_euler_forward_conservative_eno3_pyst_kernel_2d(
        real_t, num_threads=False, fixed_grid_size=False):
    """advection_timestep_2d.py:10-55: field += ENO3 flux(field, velocity) with inv_dx = -dt/dx."""
    real_t = normalize_real_t(real_t)

    def kernel(field, advection_flux, velocity, dt_by_dx):
        ny, nx = field.shape
        _lib.call("sg_advection_eno3_step_2d", sg_dtype(real_t), ny, nx, ptr(field), ptr(advection_flux),
                  ptr(velocity), float(real_t(dt_by_dx)), stream_ptr(field.device))
        field.copy_(advection_flux)

    return kernel


def gen_diffusion_timestep_euler_forward_pyst_kernel_2d(real_t, num_threads=False, fixed_grid_size=False):
    """diffusion_timestep_2d.py:10-43: field += nu dt/dx^2 * lap(field) on the interior."""
    real_t = normalize_real_t(real_t)

    def kernel(field, diffusion_flux, nu_dt_by_dx2):
        ny, nx = field.shape
        _lib.call("sg_diffusion_step_2d", sg_dtype(real_t), ny, nx, ptr(field), ptr(diffusion_flux),
                  float(real_t(nu_dt_by_dx2)), stream_ptr(field.device))
        field.copy_(diffusion_flux)

    return kernel


def gen_update_vorticity_from_velocity_forcing_pyst_kernel_2d(real_t, num_threads=False, fixed_grid_size=False):
    """update_vorticity_from_velocity_forcing_2d.py:12-71."""
    real_t = normalize_real_t(real_t)
    cache: dict = {}

    def kernel(vorticity_field, velocity_forcing_field, prefactor):
        ny, nx = vorticity_field.shape
        tmp = _scratch_like(vorticity_field, cache)
        _lib.call("sg_forcing_curl_update_2d", sg_dtype(real_t), ny, nx, ptr(vorticity_field), ptr(tmp),
                  ptr(velocity_forcing_field), float(real_t(prefactor)), stream_ptr(vorticity_field.device))
        vorticity_field.copy_(tmp)

    return kernel


def gen_outplane_field_curl_pyst_kernel_2d(real_t, num_threads=False, fixed_grid_size=False,
                                           reset_ghost_zone=True):
    """outplane_field_curl_2d.py:13-100 (ghost ring of the curl set to zero)."""
    real_t = normalize_real_t(real_t)

    def kernel(curl, field, prefactor):
        ny, nx = field.shape
        _lib.call("sg_outplane_curl_2d", sg_dtype(real_t), ny, nx, ptr(field), ptr(curl),
                  float(real_t(prefactor)), stream_ptr(field.device))

    return kernel


def gen_penalise_field_boundary_pyst_kernel_2d(width, dx, x_grid_field, y_grid_field, real_t, num_threads=False,
                                               fixed_grid_size=False):
    """penalise_field_boundary_2d.py:12-142 (X pass then Y pass, in place)."""
    _check_width(width)
    real_t = normalize_real_t(real_t)
    xg = np.asarray(x_grid_field.cpu() if isinstance(x_grid_field, torch.Tensor) else x_grid_field)
    yg = np.asarray(y_grid_field.cpu() if isinstance(y_grid_field, torch.Tensor) else y_grid_field)
    cx = penalisation_factors(width, dx, xg[0, :], real_t)
    cy = penalisation_factors(width, dx, yg[:, 0], real_t)
    cache: dict = {}

    def kernel(field):
        if width == 0:
            return
        ny, nx = field.shape
        dev = field.device
        tabs = cache.setdefault(("tabs", dev), (torch.from_numpy(cx).to(dev), torch.from_numpy(cy).to(dev)))
        tmp = _scratch_like(field, cache)
        _lib.call("sg_penalise_2d", sg_dtype(real_t), ny, nx, ptr(field), ptr(tmp), int(width), ptr(tabs[0]),
                  ptr(tabs[1]), stream_ptr(dev))
        field.copy_(tmp)

    return kernel


def gen_curl_pyst_kernel_3d(real_t, num_threads=False, fixed_grid_size=False, reset_ghost_zone=True):
    """curl_3d.py:13-132."""
    real_t = normalize_real_t(real_t)

    def kernel(curl, field, prefactor):
        _, nz, ny, nx = field.shape
        _lib.call("sg_curl_3d", sg_dtype(real_t), nz, ny, nx, ptr(field), ptr(curl), float(real_t(prefactor)),
                  stream_ptr(field.device))

    return kernel


def gen_update_vorticity_from_velocity_forcing_pyst_kernel_3d(real_t, num_threads=False, fixed_grid_size=False):
    """update_vorticity_from_velocity_forcing_3d.py:12-132."""
    real_t = normalize_real_t(real_t)
    cache: dict = {}

    def kernel(vorticity_field, velocity_forcing_field, prefactor):
        _, nz, ny, nx = vorticity_field.shape
        tmp = _scratch_like(vorticity_field, cache)
        _lib.call("sg_forcing_curl_update_3d", sg_dtype(real_t), nz, ny, nx, ptr(vorticity_field), ptr(tmp),
                  ptr(velocity_forcing_field), float(real_t(prefactor)), stream_ptr(vorticity_field.device))
        vorticity_field.copy_(tmp)

    return kernel


def gen_elementwise_cross_product_pyst_kernel_3d(real_t, num_threads=False, fixed_grid_size=False):
    """elementwise_ops_3d.py:390-449."""
    real_t = normalize_real_t(real_t)

    def kernel(result_field, field_1, field_2):
        n = field_1[0].numel()
        _lib.call("sg_cross_3d", sg_dtype(real_t), n, ptr(field_1), ptr(field_2), ptr(result_field),
                  stream_ptr(field_1.device))

    return kernel


def gen_diffusion_timestep_euler_forward_pyst_kernel_3d(real_t, num_threads=False, fixed_grid_size=False,
                                                        field_type="scalar"):
    """diffusion_timestep_3d.py:12-80 (scalar or vector field)."""
    real_t = normalize_real_t(real_t)
    if field_type not in ("scalar", "vector"):
        raise ValueError("Invalid field type")
    cache: dict = {}

    def _step(f, k):
        v = f if f.dim() == 4 else f.unsqueeze(0)
        if v.shape[0] != 3:
            # scalar field: run the vector kernel on a zero-padded 3-component buffer
            buf = cache.setdefault(("v3", tuple(v.shape[1:]), v.dtype, v.device),
                                   torch.zeros((3, *v.shape[1:]), dtype=v.dtype, device=v.device))
            buf[0].copy_(v[0])
            v3 = buf
        else:
            v3 = v
        out = _scratch_like(v3, cache)
        _, nz, ny, nx = v3.shape
        _lib.call("sg_diffusion_step_3d", sg_dtype(real_t), nz, ny, nx, ptr(v3), ptr(out), float(real_t(k)),
                  stream_ptr(f.device))
        if v3 is v:
            f.copy_(out.view_as(f))
        else:
            f.copy_(out[0].view_as(f))

    if field_type == "scalar":
        def kernel(field, diffusion_flux, nu_dt_by_dx2):
            _step(field, nu_dt_by_dx2)
    else:
        def kernel(vector_field, diffusion_flux, nu_dt_by_dx2):
            _step(vector_field, nu_dt_by_dx2)
    return kernel


def gen_advection_flux_conservative_eno3_pyst_kernel_3d(real_t, num_threads=False, fixed_grid_size=False):
    """advection_flux_3d.py:12-233: advection_flux += the six ENO3 face fluxes of a scalar field."""
    real_t = normalize_real_t(real_t)

    def kernel(advection_flux, field, velocity, inv_dx):
        nz, ny, nx = field.shape
        _lib.call("sg_advection_eno3_flux_3d", sg_dtype(real_t), nz, ny, nx, ptr(field), ptr(advection_flux),
                  ptr(velocity), float(real_t(inv_dx)), stream_ptr(field.device))

    return kernel


def gen_advection_timestep_euler_forward_conservative_eno3_pyst_kernel_3d(
        real_t, num_threads=False, fixed_grid_size=False, field_type="scalar"):
    """advection_timestep_3d.py:12-99: field += ENO3 flux with inv_dx = -dt/dx, scalar or per
    component of a vector field.  The scalar ``advection_flux`` buffer receives each component's
    new values before they are copied back."""
    real_t = normalize_real_t(real_t)
    if field_type not in ("scalar", "vector"):
        raise ValueError("Invalid field type")

    def _step(f, buf, velocity, dt_by_dx):
        nz, ny, nx = f.shape[-3:]
        ncomp = 1 if f.dim() == 3 else f.shape[0]
        for c in range(ncomp):
            src = f if ncomp == 1 else f[c]
            _lib.call("sg_advection_eno3_step_3d", sg_dtype(real_t), nz, ny, nx, 1, ptr(src), ptr(buf),
                      ptr(velocity), float(real_t(dt_by_dx)), stream_ptr(f.device))
            src.copy_(buf)

    if field_type == "scalar":
        def kernel(field, advection_flux, velocity, dt_by_dx):
            _step(field, advection_flux, velocity, dt_by_dx)
    else:
        def kernel(vector_field, advection_flux, velocity, dt_by_dx):
            _step(vector_field, advection_flux, velocity, dt_by_dx)
    return kernel


def gen_penalise_field_boundary_pyst_kernel_3d(width, dx, x_grid_field, y_grid_field, z_grid_field, real_t,
                                               num_threads=False, fixed_grid_size=False, field_type="scalar"):
    """penalise_field_boundary_3d.py:13-240 (X, Y then Z pass)."""
    if not isinstance(width, (int, np.integer)) or width < 0:
        raise ValueError("Invalid width for boundary zone, must be a non-negative integer")
    if field_type not in ("scalar", "vector"):
        raise ValueError("Invalid field type")
    real_t = normalize_real_t(real_t)
    host = [np.asarray(g.cpu() if isinstance(g, torch.Tensor) else g) for g in (x_grid_field, y_grid_field,
                                                                              z_grid_field)]
    cx = penalisation_factors(width, dx, host[0][0, 0, :], real_t)
    cy = penalisation_factors(width, dx, host[1][0, :, 0], real_t)
    cz = penalisation_factors(width, dx, host[2][:, 0, 0], real_t)
    cache: dict = {}

    def _apply(v):
        if width == 0:
            return
        dev = v.device
        tabs = cache.setdefault(("tabs", dev), tuple(torch.from_numpy(c).to(dev) for c in (cx, cy, cz)))
        v3 = v if v.dim() == 4 else v.unsqueeze(0)
        if v3.shape[0] != 3:
            buf = cache.setdefault(("v3", tuple(v3.shape[1:]), v.dtype, dev),
                                   torch.zeros((3, *v3.shape[1:]), dtype=v.dtype, device=dev))
            buf[0].copy_(v3[0])
            src = buf
        else:
            src = v3
        out = _scratch_like(src, cache)
        _, nz, ny, nx = src.shape
        _lib.call("sg_penalise_3d", sg_dtype(real_t), nz, ny, nx, ptr(src), ptr(out), int(width), ptr(tabs[0]),
                  ptr(tabs[1]), ptr(tabs[2]), stream_ptr(dev))
        if src is v3:
            v.copy_(out.view_as(v))
        else:
            v.copy_(out[0].view_as(v))

    if field_type == "scalar":
        def kernel(field):
            _apply(field)
    else:
        def kernel(vector_field):
            _apply(vector_field)
    return kernel


def gen_laplacian_filter_kernel_3d(filter_order, filter_flux_buffer, field_buffer, real_t, num_threads=False,
                                   fixed_grid_size=False, field_type="scalar", filter_type="multiplicative",
                                   filter_flux_buffer_boundary_width=1):
    """laplacian_filter_3d.py:13-194 (multiplicative or convolution)."""
    if not isinstance(filter_order, (int, np.integer)) or filter_order < 0:
        raise ValueError("Invalid filter order, must be a non-negative integer")
    if not isinstance(filter_flux_buffer_boundary_width, int) or filter_flux_buffer_boundary_width <= 0:
        raise ValueError("Invalid value for filter flux buffer boundary zone, must be a positive integer")
    types = {"multiplicative": 1, "convolution": 2}
    if filter_type not in types:
        raise ValueError("Invalid filter type")
    if field_type not in ("scalar", "vector"):
        raise ValueError("Invalid field type")
    real_t = normalize_real_t(real_t)
    cache: dict = {}

    def _apply(v):
        v3 = v if v.dim() == 4 else v.unsqueeze(0)
        if v3.shape[0] != 3:
            buf = cache.setdefault(("v3", tuple(v3.shape[1:]), v.dtype, v.device),
                                   torch.zeros((3, *v3.shape[1:]), dtype=v.dtype, device=v.device))
            buf[0].copy_(v3[0])
            tgt = buf
        else:
            tgt = v3
        _, nz, ny, nx = tgt.shape
        _lib.call("sg_laplacian_filter_3d", sg_dtype(real_t), nz, ny, nx, ptr(tgt), types[filter_type],
                  int(filter_order), ptr(filter_flux_buffer), ptr(field_buffer), stream_ptr(v.device))
        if tgt is not v3:
            v.copy_(tgt[0].view_as(v))

    if field_type == "scalar":
        def kernel(scalar_field):
            _apply(scalar_field)
    else:
        def kernel(vector_field):
            _apply(vector_field)
    return kernel


def gen_divergence_pyst_kernel_3d(real_t, num_threads=False, fixed_grid_size=False, reset_ghost_zone=True):
    """divergence_3d.py:13-98: central divergence on [1:-1]^3; the one-cell ring of the output is
    set to 0 (``reset_ghost_zone``, the default) or left as it was."""
    real_t = normalize_real_t(real_t)
    cache: dict = {}

    def kernel(divergence, field, inv_dx):
        _, nz, ny, nx = field.shape
        out = divergence
        if not reset_ghost_zone:  # the kernel zeroes the ring: compute aside, keep the caller's ring
            key = (tuple(divergence.shape), divergence.dtype, divergence.device)
            out = cache.get(key)
            if out is None:
                out = cache[key] = torch.empty(divergence.shape, dtype=divergence.dtype, device=divergence.device)
        _lib.call("sg_divergence_3d", sg_dtype(real_t), nz, ny, nx, ptr(field), ptr(out),
                  float(real_t(inv_dx)), stream_ptr(field.device))
        if out is not divergence:
            divergence[1:-1, 1:-1, 1:-1] = out[1:-1, 1:-1, 1:-1]

    return kernel


# ------------------------------------------------- elementwise and flux-form factories
# stencil_ops_{2,3}d/elementwise_ops_{2,3}d.py, diffusion_flux_{2,3}d.py, advection_flux_2d.py.
# Each callable is one launch over C-contiguous CUDA tensors of real_t (a vector field's
# components are handled in the same launch unless they take different values).

_EW_SET, _EW_ADD_FIXED, _EW_COPY, _EW_SUM, _EW_SAXPBY, _EW_COMPLEX_PRODUCT = range(6)


def _contig(*tensors):
    for t in tensors:
        if not (isinstance(t, torch.Tensor) and t.is_cuda and t.is_contiguous()):
            raise ValueError("field arguments must be C-contiguous CUDA tensors")


def _ew(real_t, op, n, a, b, out, alpha=0.0, beta=0.0, device=None):
    _lib.call("sg_elementwise", sg_dtype(real_t), op, int(n), ptr(a), ptr(b), ptr(out), float(alpha), float(beta),
              stream_ptr(device))


def _check_field_type(field_type):
    if field_type not in ("scalar", "vector"):
        raise ValueError("Invalid field type")


def _gen_elementwise_sum(real_t, field_type="scalar"):
    real_t = normalize_real_t(real_t)
    _check_field_type(field_type)

    def kernel(sum_field, field_1, field_2):
        _contig(sum_field, field_1, field_2)
        _ew(real_t, _EW_SUM, sum_field.numel(), field_1, field_2, sum_field, device=sum_field.device)

    return kernel


def _gen_set_fixed_val(real_t, field_type="scalar"):
    real_t = normalize_real_t(real_t)
    _check_field_type(field_type)
    if field_type == "scalar":
        def kernel(field, fixed_val):
            _contig(field)
            _ew(real_t, _EW_SET, field.numel(), None, None, field, real_t(fixed_val), device=field.device)
    else:
        def kernel(vector_field, fixed_vals):
            _contig(vector_field)
            for c in range(vector_field.shape[0]):
                _ew(real_t, _EW_SET, vector_field[c].numel(), None, None, vector_field[c], real_t(fixed_vals[c]),
                    device=vector_field.device)
    return kernel


def _gen_elementwise_copy(real_t):
    real_t = normalize_real_t(real_t)

    def kernel(field, rhs_field):
        _contig(field, rhs_field)
        _ew(real_t, _EW_COPY, field.numel(), rhs_field, None, field, device=field.device)

    return kernel


def _gen_elementwise_complex_product(real_t):
    real_t = normalize_real_t(real_t)

    def kernel(product_field, field_1, field_2):
        _contig(product_field, field_1, field_2)
        if not (product_field.is_complex() and field_1.is_complex() and field_2.is_complex()):
            raise ValueError("complex product: the fields must be complex tensors")
        _ew(real_t, _EW_COMPLEX_PRODUCT, product_field.numel(), field_1, field_2, product_field,
            device=product_field.device)

    return kernel


def _gen_set_fixed_val_at_boundaries(real_t, width, dim, field_type="scalar"):
    real_t = normalize_real_t(real_t)
    if not isinstance(width, (int, np.integer)) or isinstance(width, bool) or width <= 0:
        raise ValueError("Invalid width for boundary zone, must be a positive integer")
    _check_field_type(field_type)

    def _one(f, val):
        ext = f.shape[-dim:]
        nz, ny, nx = (1, *ext) if dim == 2 else ext
        _lib.call("sg_set_boundary_zone", sg_dtype(real_t), dim, nz, ny, nx, int(width), ptr(f),
                  float(real_t(val)), stream_ptr(f.device))

    if field_type == "scalar":
        def kernel(field, fixed_val):
            _contig(field)
            _one(field, fixed_val)
    else:
        def kernel(vector_field, fixed_vals):
            _contig(vector_field)
            for c in range(vector_field.shape[0]):
                _one(vector_field[c], fixed_vals[c])
    return kernel


def _gen_add_fixed_val(real_t, field_type="scalar"):
    real_t = normalize_real_t(real_t)
    _check_field_type(field_type)
    if field_type == "scalar":
        def kernel(sum_field, field, fixed_val):
            _contig(sum_field, field)
            _ew(real_t, _EW_ADD_FIXED, field.numel(), field, None, sum_field, real_t(fixed_val), device=field.device)
    else:
        def kernel(sum_field, vector_field, fixed_vals):
            _contig(sum_field, vector_field)
            for c in range(vector_field.shape[0]):
                _ew(real_t, _EW_ADD_FIXED, vector_field[c].numel(), vector_field[c], None, sum_field[c],
                    real_t(fixed_vals[c]), device=vector_field.device)
    return kernel


def _gen_elementwise_saxpby(real_t, field_type="scalar"):
    real_t = normalize_real_t(real_t)
    _check_field_type(field_type)

    def kernel(sum_field, field_1, field_2, field_1_prefac, field_2_prefac):
        _contig(sum_field, field_1, field_2)
        _ew(real_t, _EW_SAXPBY, sum_field.numel(), field_1, field_2, sum_field, real_t(field_1_prefac),
            real_t(field_2_prefac), device=sum_field.device)

    return kernel


def gen_elementwise_sum_pyst_kernel_2d(real_t, num_threads=False, fixed_grid_size=False, field_type="scalar"):
    """elementwise_ops_2d.py:13-57: sum_field = field_1 + field_2."""
    return _gen_elementwise_sum(real_t, field_type)


def gen_elementwise_sum_pyst_kernel_3d(real_t, num_threads=False, fixed_grid_size=False, field_type="scalar"):
    """elementwise_ops_3d.py:13-57."""
    return _gen_elementwise_sum(real_t, field_type)


def gen_set_fixed_val_pyst_kernel_2d(real_t, num_threads=False, fixed_grid_size=False, field_type="scalar"):
    """elementwise_ops_2d.py:60-114: field = fixed_val (per component for a vector field)."""
    return _gen_set_fixed_val(real_t, field_type)


def gen_set_fixed_val_pyst_kernel_3d(real_t, num_threads=False, fixed_grid_size=False, field_type="scalar"):
    """elementwise_ops_3d.py:60-119."""
    return _gen_set_fixed_val(real_t, field_type)


def gen_elementwise_copy_pyst_kernel_2d(real_t, num_threads=False, fixed_grid_size=False):
    """elementwise_ops_2d.py:117-138: field = rhs_field."""
    return _gen_elementwise_copy(real_t)


def gen_elementwise_copy_pyst_kernel_3d(real_t, num_threads=False, fixed_grid_size=False):
    """elementwise_ops_3d.py:122-143."""
    return _gen_elementwise_copy(real_t)


def gen_elementwise_complex_product_pyst_kernel_2d(real_t, num_threads=False, fixed_grid_size=False):
    """elementwise_ops_2d.py:141-190: product_field = field_1 * field_2 (complex tensors)."""
    return _gen_elementwise_complex_product(real_t)


def gen_elementwise_complex_product_pyst_kernel_3d(real_t, num_threads=False, fixed_grid_size=False):
    """elementwise_ops_3d.py:146-197."""
    return _gen_elementwise_complex_product(real_t)


def gen_set_fixed_val_at_boundaries_pyst_kernel_2d(real_t, width, num_threads=False, field_type="scalar"):
    """elementwise_ops_2d.py:193-253: the band of `width` cells along every edge set to fixed_val."""
    return _gen_set_fixed_val_at_boundaries(real_t, width, 2, field_type)


def gen_set_fixed_val_at_boundaries_pyst_kernel_3d(real_t, width, num_threads=False, field_type="scalar"):
    """elementwise_ops_3d.py:200-268."""
    return _gen_set_fixed_val_at_boundaries(real_t, width, 3, field_type)


def gen_add_fixed_val_pyst_kernel_2d(real_t, num_threads=False, fixed_grid_size=False, field_type="scalar"):
    """elementwise_ops_2d.py:256-313: sum_field = field + fixed_val (per component for a vector field)."""
    return _gen_add_fixed_val(real_t, field_type)


def gen_add_fixed_val_pyst_kernel_3d(real_t, num_threads=False, fixed_grid_size=False, field_type="scalar"):
    """elementwise_ops_3d.py:271-334."""
    return _gen_add_fixed_val(real_t, field_type)


def gen_elementwise_saxpby_pyst_kernel_2d(real_t, num_threads=False, fixed_grid_size=False, field_type="scalar"):
    """elementwise_ops_2d.py:316-370: sum_field = field_1_prefac field_1 + field_2_prefac field_2."""
    return _gen_elementwise_saxpby(real_t, field_type)


def gen_elementwise_saxpby_pyst_kernel_3d(real_t, num_threads=False, fixed_grid_size=False, field_type="scalar"):
    """elementwise_ops_3d.py:337-387."""
    return _gen_elementwise_saxpby(real_t, field_type)


def gen_diffusion_flux_pyst_kernel_2d(real_t, num_threads=False, fixed_grid_size=False, reset_ghost_zone=True):
    """diffusion_flux_2d.py:13-72: diffusion_flux = prefactor lap(field) on [1:-1]^2 (ring zeroed when
    reset_ghost_zone, else left unchanged)."""
    real_t = normalize_real_t(real_t)

    def kernel(diffusion_flux, field, prefactor):
        _contig(diffusion_flux, field)
        ny, nx = field.shape
        _lib.call("sg_diffusion_flux", sg_dtype(real_t), 2, 1, ny, nx, ptr(field), ptr(diffusion_flux),
                  float(real_t(prefactor)), int(bool(reset_ghost_zone)), stream_ptr(field.device))

    return kernel


def gen_diffusion_flux_pyst_kernel_3d(real_t, num_threads=False, fixed_grid_size=False, field_type="scalar",
                                      reset_ghost_zone=True):
    """diffusion_flux_3d.py:14-115: scalar, or per component of a vector field."""
    real_t = normalize_real_t(real_t)
    _check_field_type(field_type)

    def _one(flux, f, prefactor):
        nz, ny, nx = f.shape
        _lib.call("sg_diffusion_flux", sg_dtype(real_t), 3, nz, ny, nx, ptr(f), ptr(flux),
                  float(real_t(prefactor)), int(bool(reset_ghost_zone)), stream_ptr(f.device))

    if field_type == "scalar":
        def kernel(diffusion_flux, field, prefactor):
            _contig(diffusion_flux, field)
            _one(diffusion_flux, field, prefactor)
    else:
        def kernel(vector_field_diffusion_flux, vector_field, prefactor):
            _contig(vector_field_diffusion_flux, vector_field)
            for c in range(vector_field.shape[0]):
                _one(vector_field_diffusion_flux[c], vector_field[c], prefactor)
    return kernel


def gen_advection_flux_conservative_eno3_pyst_kernel_2d(real_t, num_threads=False, fixed_grid_size=False):
    """advection_flux_2d.py:12-165: advection_flux += the four ENO3 face fluxes (in place)."""
    real_t = normalize_real_t(real_t)

    def kernel(advection_flux, field, velocity, inv_dx):
        _contig(advection_flux, field, velocity)
        ny, nx = field.shape
        _lib.call("sg_advection_eno3_flux_2d", sg_dtype(real_t), ny, nx, ptr(field), ptr(advection_flux),
                  ptr(velocity), float(real_t(inv_dx)), stream_ptr(field.device))

    return kernel
