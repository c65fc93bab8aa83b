"""Eulerian stencil operators of the reference, restated with numpy (oracle only).

Conventions shared with the reference (pystencils kernels iterate the interior
with ``g`` ghost layers on every axis, ``g`` = largest stencil offset):

* arrays are C-ordered, 2D ``(ny, nx)``, 3D ``(nz, ny, nx)``; vector fields put
  the component first with 0 = x;
* ENO3 advection writes the interior ``[2:-2]`` on every axis; the diffusion
  flux and curl write ``[1:-1]`` and their ghost ring is set to zero; the
  forcing-curl update leaves its ring unchanged.
"""

from __future__ import annotations

import numpy as np

# ---------------------------------------------------------------------------
# 2D
# ---------------------------------------------------------------------------


def forcing_curl_update_2d(vorticity, forcing, prefactor):
    """vorticity += prefactor * curl_h(forcing) on [1:-1]^2, in place.

    stencil_ops_2d/update_vorticity_from_velocity_forcing_2d.py:28-44
    """
    fx, fy = forcing[0], forcing[1]
    vorticity[1:-1, 1:-1] = vorticity[1:-1, 1:-1] + (
        fy[1:-1, 2:] - fy[1:-1, :-2] - fx[2:, 1:-1] + fx[:-2, 1:-1]
    ) * prefactor


# When set, every ENO3 upwind choice (the boolean mask u_0 > -u_{+1} of a face pass) goes through
# this callable, which returns the mask to use: ``oracle.adjoint.frozen_branches`` records the masks
# of a base trajectory and replays them, so that finite differences see one smooth branch of the map.
BRANCH_HOOK = None


def _eno3_face_flux(q_m1, q_0, q_p1, q_p2, u_0, u_p1, real_t):
    """ENO3 flux through the face between cells 0 and +1 along one axis.

    advection_flux_2d.py:35-47: upwind on the left when u_0 > -u_{+1}.
    """
    third, five6, sixth = real_t(1 / 3), real_t(5 / 6), real_t(1 / 6)
    left = third * q_p1 + five6 * q_0 - sixth * q_m1
    right = third * q_0 + five6 * q_p1 - sixth * q_p2
    mask = u_0 > -u_p1
    if BRANCH_HOOK is not None:
        mask = BRANCH_HOOK(mask)
    return np.where(mask, left, right)


def eno3_flux_2d(field, velocity, inv_dx, out=None):
    """Conservative ENO3 advection flux on [2:-2]^2 (zero elsewhere).

    advection_flux_2d.py:12-165 (four directional passes accumulated in the
    order x-front, x-back, y-front, y-back into a zeroed buffer).
    """
    real_t = field.dtype.type
    flux = np.zeros_like(field) if out is None else out
    s = slice(2, -2)
    ux, uy = velocity[0], velocity[1]
    qx = field * ux
    qy = field * uy

    def sh(a, dy, dx):
        ny, nx = a.shape
        return a[2 + dy: ny - 2 + dy, 2 + dx: nx - 2 + dx]

    east = _eno3_face_flux(sh(qx, 0, -1), sh(qx, 0, 0), sh(qx, 0, 1), sh(qx, 0, 2),
                           sh(ux, 0, 0), sh(ux, 0, 1), real_t)
    west = _eno3_face_flux(sh(qx, 0, -2), sh(qx, 0, -1), sh(qx, 0, 0), sh(qx, 0, 1),
                           sh(ux, 0, -1), sh(ux, 0, 0), real_t)
    north = _eno3_face_flux(sh(qy, -1, 0), sh(qy, 0, 0), sh(qy, 1, 0), sh(qy, 2, 0),
                            sh(uy, 0, 0), sh(uy, 1, 0), real_t)
    south = _eno3_face_flux(sh(qy, -2, 0), sh(qy, -1, 0), sh(qy, 0, 0), sh(qy, 1, 0),
                            sh(uy, -1, 0), sh(uy, 0, 0), real_t)
    acc = inv_dx * east
    acc = acc - inv_dx * west
    acc = acc + inv_dx * north
    acc = acc - inv_dx * south
    flux[...] = 0
    flux[s, s] = acc
    return flux


def advection_step_2d(field, velocity, dt_by_dx):
    """field += ENO3 flux with inv_dx = -dt/dx, in place.

    advection_timestep_2d.py:35-53
    """
    flux = eno3_flux_2d(field, velocity, -dt_by_dx)
    field[...] = field + flux


def diffusion_flux_2d(field, prefactor):
    """prefactor * 5-point Laplacian on [1:-1]^2, zero ring.

    diffusion_flux_2d.py:30-72
    """
    flux = np.zeros_like(field)
    flux[1:-1, 1:-1] = prefactor * (
        field[2:, 1:-1] + field[:-2, 1:-1] + field[1:-1, 2:] + field[1:-1, :-2]
        - 4 * field[1:-1, 1:-1]
    )
    return flux


def diffusion_step_2d(field, nu_dt_by_dx2):
    """field += diffusion flux, in place.  diffusion_timestep_2d.py:28-42"""
    field[...] = field + diffusion_flux_2d(field, nu_dt_by_dx2)


def outplane_curl_2d(psi, prefactor, out=None):
    """u_x = (psi[y+1]-psi[y-1])*p, u_y = (psi[x-1]-psi[x+1])*p on [1:-1]^2, zero ring.

    outplane_field_curl_2d.py:171-240
    """
    u = np.zeros((2, *psi.shape), dtype=psi.dtype) if out is None else out
    u[...] = 0
    u[0, 1:-1, 1:-1] = (psi[2:, 1:-1] - psi[:-2, 1:-1]) * prefactor
    u[1, 1:-1, 1:-1] = (psi[1:-1, :-2] - psi[1:-1, 2:]) * prefactor
    return u


def penalise_2d(field, width, dx, x_grid, y_grid):
    """Sine ramp of the boundary band, X pass then Y pass, in place.

    penalise_field_boundary_2d.py:40-140: the band value copies column (row)
    ``width-1`` (``-width``) and is multiplied by sin((pi/2) d / (width dx)),
    d = distance from the first (last) cell centre.  Width 0 is a no-op.
    """
    if width == 0:
        return
    sine_prefactor = (np.pi / 2) / (width * dx)
    x0, x1 = x_grid[0, 0], x_grid[0, -1]
    y0, y1 = y_grid[0, 0], y_grid[-1, 0]
    field[:, :width] = field[:, width - 1: width]
    field[:, -width:] = field[:, -width: -width + 1]
    field[:, :width] = field[:, :width] * np.sin(sine_prefactor * (x_grid[:, :width] - x0))
    field[:, -width:] = field[:, -width:] * np.sin(sine_prefactor * (x1 - x_grid[:, -width:]))
    field[:width, :] = field[width - 1: width, :]
    field[-width:, :] = field[-width: -width + 1, :]
    field[:width, :] = field[:width, :] * np.sin(sine_prefactor * (y_grid[:width, :] - y0))
    field[-width:, :] = field[-width:, :] * np.sin(sine_prefactor * (y1 - y_grid[-width:, :]))


# ---------------------------------------------------------------------------
# 3D
# ---------------------------------------------------------------------------

_I = slice(1, -1)


def _d(a, axis, shift):
    """Interior view of ``a`` shifted by ``shift`` along ``axis`` (0=z,1=y,2=x)."""
    sl = [slice(1, -1)] * 3
    n = a.shape[axis]
    sl[axis] = slice(1 + shift, n - 1 + shift)
    return a[tuple(sl)]


def curl_3d(field, prefactor, out=None):
    """curl_h on [1:-1]^3 with zero ring.  stencil_ops_3d/curl_3d.py:30-132"""
    fx, fy, fz = field
    c = np.zeros_like(field) if out is None else out
    c[...] = 0
    c[0, _I, _I, _I] = prefactor * (_d(fz, 1, 1) - _d(fz, 1, -1) - _d(fy, 0, 1) + _d(fy, 0, -1))
    c[1, _I, _I, _I] = prefactor * (_d(fx, 0, 1) - _d(fx, 0, -1) - _d(fz, 2, 1) + _d(fz, 2, -1))
    c[2, _I, _I, _I] = prefactor * (_d(fy, 2, 1) - _d(fy, 2, -1) - _d(fx, 1, 1) + _d(fx, 1, -1))
    return c


def forcing_curl_update_3d(vorticity, forcing, prefactor):
    """vorticity += prefactor * curl_h(forcing) on [1:-1]^3, component by component.

    stencil_ops_3d/update_vorticity_from_velocity_forcing_3d.py:29-132
    """
    fx, fy, fz = forcing
    w = vorticity
    w[0, _I, _I, _I] = w[0, _I, _I, _I] + prefactor * (
        _d(fz, 1, 1) - _d(fz, 1, -1) - _d(fy, 0, 1) + _d(fy, 0, -1))
    w[1, _I, _I, _I] = w[1, _I, _I, _I] + prefactor * (
        _d(fx, 0, 1) - _d(fx, 0, -1) - _d(fz, 2, 1) + _d(fz, 2, -1))
    w[2, _I, _I, _I] = w[2, _I, _I, _I] + prefactor * (
        _d(fy, 2, 1) - _d(fy, 2, -1) - _d(fx, 1, 1) + _d(fx, 1, -1))


def cross_3d(a, b):
    """Elementwise a x b.  stencil_ops_3d/elementwise_ops_3d.py:390-449"""
    out = np.empty_like(a)
    out[0] = a[1] * b[2] - b[1] * a[2]
    out[1] = a[2] * b[0] - b[2] * a[0]
    out[2] = a[0] * b[1] - b[0] * a[1]
    return out


def diffusion_step_3d(vector_field, nu_dt_by_dx2):
    """Per component: += prefactor * 7-point Laplacian on [1:-1]^3 (zero ring flux).

    diffusion_timestep_3d.py:12-80, diffusion_flux_3d.py:31-115
    """
    for c in range(vector_field.shape[0]):
        f = vector_field[c]
        flux = np.zeros_like(f)
        flux[_I, _I, _I] = nu_dt_by_dx2 * (
            _d(f, 2, 1) + _d(f, 2, -1) + _d(f, 1, 1) + _d(f, 1, -1) + _d(f, 0, 1) + _d(f, 0, -1)
            - 6 * f[_I, _I, _I])
        vector_field[c] = f + flux


def eno3_flux_3d(field, velocity, inv_dx, out=None):
    """Conservative ENO3 advection flux of a scalar field on [2:-2]^3 (zero elsewhere).

    stencil_ops_3d/advection_flux_3d.py:12-233: six directional passes, each a
    face flux of ``_eno3_face_flux`` along one axis, accumulated in the order
    x-front, x-back, y-front, y-back, z-front, z-back into a zeroed buffer.
    """
    real_t = field.dtype.type
    flux = np.zeros_like(field) if out is None else out
    nz, ny, nx = field.shape

    def sh(a, dz, dy, dx):
        return a[2 + dz: nz - 2 + dz, 2 + dy: ny - 2 + dy, 2 + dx: nx - 2 + dx]

    acc = None
    for axis, u in ((2, velocity[0]), (1, velocity[1]), (0, velocity[2])):
        q = field * u

        def at(a, k, axis=axis):
            off = [0, 0, 0]
            off[axis] = k
            return sh(a, *off)

        front = _eno3_face_flux(at(q, -1), at(q, 0), at(q, 1), at(q, 2), at(u, 0), at(u, 1), real_t)
        back = _eno3_face_flux(at(q, -2), at(q, -1), at(q, 0), at(q, 1), at(u, -1), at(u, 0), real_t)
        acc = inv_dx * front if acc is None else acc + inv_dx * front
        acc = acc - inv_dx * back
    flux[...] = 0
    flux[2:-2, 2:-2, 2:-2] = acc
    return flux


def advection_step_3d(field, velocity, dt_by_dx):
    """Scalar field += ENO3 flux with inv_dx = -dt/dx, in place.

    stencil_ops_3d/advection_timestep_3d.py:38-57 (a vector field is advected
    component by component with the same velocity, :61-96).
    """
    flux = eno3_flux_3d(field, velocity, -dt_by_dx)
    field[...] = field + flux


def divergence_3d(field, inv_dx):
    """0.5*inv_dx * central divergence on [1:-1]^3, zero ring.  divergence_3d.py"""
    div = np.zeros_like(field[0])
    div[_I, _I, _I] = (
        _d(field[0], 2, 1) - _d(field[0], 2, -1) + _d(field[1], 1, 1) - _d(field[1], 1, -1)
        + _d(field[2], 0, 1) - _d(field[2], 0, -1)) * 0.5 * inv_dx
    return div


def penalise_3d(field, width, dx, x_grid, y_grid, z_grid):
    """Scalar sine-ramp penalisation, X then Y then Z pass, in place.

    penalise_field_boundary_3d.py:56-208
    """
    if width == 0:
        return
    sp = (np.pi / 2) / (width * dx)
    x0, x1 = x_grid[0, 0, 0], x_grid[0, 0, -1]
    y0, y1 = y_grid[0, 0, 0], y_grid[0, -1, 0]
    z0, z1 = z_grid[0, 0, 0], z_grid[-1, 0, 0]
    w = width
    field[:, :, :w] = field[:, :, w - 1: w]
    field[:, :, -w:] = field[:, :, -w: -w + 1]
    field[:, :, :w] = field[:, :, :w] * np.sin(sp * (x_grid[:, :, :w] - x0))
    field[:, :, -w:] = field[:, :, -w:] * np.sin(sp * (x1 - x_grid[:, :, -w:]))
    field[:, :w, :] = field[:, w - 1: w, :]
    field[:, -w:, :] = field[:, -w: -w + 1, :]
    field[:, :w, :] = field[:, :w, :] * np.sin(sp * (y_grid[:, :w, :] - y0))
    field[:, -w:, :] = field[:, -w:, :] * np.sin(sp * (y1 - y_grid[:, -w:, :]))
    field[:w, :, :] = field[w - 1: w, :, :]
    field[-w:, :, :] = field[-w: -w + 1, :, :]
    field[:w, :, :] = field[:w, :, :] * np.sin(sp * (z_grid[:w, :, :] - z0))
    field[-w:, :, :] = field[-w:, :, :] * np.sin(sp * (z1 - z_grid[-w:, :, :]))


def _filter_pass(buf, axis):
    """One 1D Laplacian filter pass on the [1:-1]^3 interior, zero ring.

    laplacian_filter_3d.py:55-73: g = 0.25*(2 f - f[+1] - f[-1]) along ``axis``.
    """
    out = np.zeros_like(buf)
    out[_I, _I, _I] = 0.25 * (-_d(buf, axis, 1) - _d(buf, axis, -1) + 2 * buf[_I, _I, _I])
    return out


def laplacian_filter_3d(vector_field, order, filter_type):
    """Multiplicative or convolution Laplacian filter, per component, in place.

    laplacian_filter_3d.py:90-165: multiplicative applies (Lz Ly Lx)^order and
    subtracts once; convolution applies Lx^order, subtracts, then y, then z.
    """
    for c in range(vector_field.shape[0]):
        f = vector_field[c]
        if filter_type == "multiplicative":
            buf = f.copy()
            flux = np.zeros_like(f)
            for _ in range(order):
                for axis in (2, 1, 0):
                    flux = _filter_pass(buf, axis)
                    buf = flux
            f -= flux
        elif filter_type == "convolution":
            for axis in (2, 1, 0):
                buf = f.copy()
                flux = np.zeros_like(f)
                for _ in range(order):
                    flux = _filter_pass(buf, axis)
                    buf = flux
                f -= flux
        else:
            raise ValueError("Invalid filter type")
