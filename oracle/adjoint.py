"""FP64 reference gradient of a time-integrated body force (test infrastructure only).

The reference has no adjoint.  This module differentiates the oracle's own 2D
coupled step -- ``oracle.flow.NavierStokes2DOracle`` with a
``VirtualBoundaryForcingOracle`` in the call order of the reference's example
loop (``examples/.../flow_past_cylinder.py``: ``interactor.time_step(dt)``,
``interactor()``, ``flow_sim.time_step(dt, free_stream)``) -- with hand-written
transposes written directly against the reference's slice operations:

* forcing curl:   stencil_ops_2d/update_vorticity_from_velocity_forcing_2d.py:28-44
* ENO3 advection: stencil_ops_2d/advection_flux_2d.py:12-165 (branch held fixed)
* diffusion:      stencil_ops_2d/diffusion_flux_2d.py:30-72
* penalisation:   stencil_ops_2d/penalise_field_boundary_2d.py:40-140 (X then Y)
* Poisson:        poisson_solver_2d/UnboundedPoissonSolverPYFFTW2D.py (symmetric)
* curl:           stencil_ops_2d/outplane_field_curl_2d.py:171-240
* IB:             immersed_boundary_ops/VirtualBoundaryForcing.py:132-283 and
                  EulerianLagrangianGridCommunicator2D.py:167-374

Objective: L = sum_n dt_n * d . (-sum_k F_k^n), the body force (reaction of the
virtual-boundary forcing, rigid_body_forcing_grids.py:58-75) along ``d``,
integrated over the steps with the dt sequence frozen.  Parameters: the
prescribed marker velocities V (2, n_lag) and the kinematic viscosity nu.
Everything here runs in float64; it is slow and meant for small grids.
"""

from __future__ import annotations

import numpy as np

from . import stencils as st
from .flow import NavierStokes2DOracle
from .ib import VirtualBoundaryForcingOracle, interpolate, spread

# ---------------------------------------------------------------- transposes


def curl_adj(u_bar, prefactor):
    """psi_bar = curl^T u_bar for outplane_curl_2d (ring of u is zero)."""
    ux = np.zeros_like(u_bar[0])
    uy = np.zeros_like(u_bar[1])
    ux[1:-1, 1:-1] = u_bar[0, 1:-1, 1:-1]
    uy[1:-1, 1:-1] = u_bar[1, 1:-1, 1:-1]
    psi = np.zeros_like(ux)
    psi[1:, :] += ux[:-1, :]
    psi[:-1, :] -= ux[1:, :]
    psi[:, :-1] += uy[:, 1:]
    psi[:, 1:] -= uy[:, :-1]
    return psi * prefactor


def _band_copy_adj(g, width, axis):
    """Transpose of field[:w] = field[w-1]; field[-w:] = field[-w] along ``axis``."""
    g = np.moveaxis(g.copy(), axis, 0)
    front = g[:width].sum(axis=0)
    back = g[-width:].sum(axis=0)
    g[:width] = 0
    g[-width:] = 0
    g[width - 1] += front
    g[-width] += back
    return np.moveaxis(g, 0, axis)


def penalise_adj(g, width, dx, x_grid, y_grid):
    """Transpose of oracle.stencils.penalise_2d (X pass then Y pass)."""
    if width == 0:
        return g.copy()
    sp = (np.pi / 2) / (width * dx)
    x0, x1 = x_grid[0, 0], x_grid[0, -1]
    y0, y1 = y_grid[0, 0], y_grid[-1, 0]
    g = g.copy()
    # Y pass, reversed: multiply, then the band copy
    g[:width, :] = g[:width, :] * np.sin(sp * (y_grid[:width, :] - y0))
    g[-width:, :] = g[-width:, :] * np.sin(sp * (y1 - y_grid[-width:, :]))
    g = _band_copy_adj(g, width, 0)
    # X pass, reversed
    g[:, :width] = g[:, :width] * np.sin(sp * (x_grid[:, :width] - x0))
    g[:, -width:] = g[:, -width:] * np.sin(sp * (x1 - x_grid[:, -width:]))
    return _band_copy_adj(g, width, 1)


def diffusion_adj(g, k, field=None):
    """Transpose of diffusion_step_2d; also d loss / d k when ``field`` is given."""
    gm = np.zeros_like(g)
    gm[1:-1, 1:-1] = g[1:-1, 1:-1]
    out = g - 4 * k * gm
    out[1:, :] += k * gm[:-1, :]
    out[:-1, :] += k * gm[1:, :]
    out[:, 1:] += k * gm[:, :-1]
    out[:, :-1] += k * gm[:, 1:]
    dk = None
    if field is not None:
        dk = float(np.sum(st.diffusion_flux_2d(field, 1.0) * g))
    return out, dk


def _face_adj(q_bar, u, face_bar, axis, left_at):
    """Scatter one directional face flux's adjoint into q_bar (helper of eno3_adj).

    The face flux of interior cell c uses q at offsets ``left_at + (-1, 0, 1)``
    on the left branch and ``left_at + (0, 1, 2)`` on the right, with the branch
    decided by u at offsets ``left_at`` and ``left_at + 1``.
    """
    ny, nx = q_bar.shape

    def sh(a, o):
        if axis == 1:
            return a[2:ny - 2, 2 + o: nx - 2 + o]
        return a[2 + o: ny - 2 + o, 2:nx - 2]

    def add(o, val):
        if axis == 1:
            q_bar[2:ny - 2, 2 + o: nx - 2 + o] += val
        else:
            q_bar[2 + o: ny - 2 + o, 2:nx - 2] += val

    left = sh(u, left_at) > -sh(u, left_at + 1)
    third, five6, sixth = 1.0 / 3.0, 5.0 / 6.0, 1.0 / 6.0
    fl = np.where(left, face_bar, 0.0)
    fr = np.where(left, 0.0, face_bar)
    add(left_at + 1, third * fl)
    add(left_at, five6 * fl)
    add(left_at - 1, -sixth * fl)
    add(left_at, third * fr)
    add(left_at + 1, five6 * fr)
    add(left_at + 2, -sixth * fr)


def eno3_adj(g, w, u, dt_by_dx):
    """Transpose of the linearised advection_step_2d at (w, u).

    Returns (w_bar, u_bar): w_bar = g + (d flux/d w)^T g, u_bar = (d flux/d u)^T g.
    advection_flux_2d.py accumulates inv_dx * (east - west + north - south) on
    the interior [2:-2]^2 with inv_dx = -dt/dx.
    """
    inv_dx = -dt_by_dx
    ny, nx = g.shape
    gi = g[2:ny - 2, 2:nx - 2]
    qx_bar = np.zeros_like(g)
    qy_bar = np.zeros_like(g)
    _face_adj(qx_bar, u[0], inv_dx * gi, 1, 0)     # east: face between 0 and +1
    _face_adj(qx_bar, u[0], -inv_dx * gi, 1, -1)   # west: face between -1 and 0
    _face_adj(qy_bar, u[1], inv_dx * gi, 0, 0)     # north
    _face_adj(qy_bar, u[1], -inv_dx * gi, 0, -1)   # south
    w_bar = g + u[0] * qx_bar + u[1] * qy_bar
    u_bar = np.stack([w * qx_bar, w * qy_bar])
    return w_bar, u_bar


def forcing_curl_adj(g, prefactor):
    """Transpose of forcing_curl_update_2d with respect to the forcing."""
    f_bar = np.zeros((2, *g.shape))
    gi = g[1:-1, 1:-1] * prefactor
    f_bar[1, 1:-1, 2:] += gi
    f_bar[1, 1:-1, :-2] -= gi
    f_bar[0, 2:, 1:-1] -= gi
    f_bar[0, :-2, 1:-1] += gi
    return f_bar


# ---------------------------------------------------------------- rollout


class DragProblem2D:
    """A 2D flow with one fixed body whose markers carry prescribed velocities.

    ``make_flow()`` returns a fresh ``NavierStokes2DOracle`` (float64, with
    forcing) in its initial state; ``positions`` (2, n_lag) are the marker
    positions; K and C the rescaled virtual-boundary coefficients.
    """

    def __init__(self, make_flow, positions, stiffness, damping, dts, free_stream, direction=(1.0, 0.0)):
        self.make_flow = make_flow
        self.positions = np.asarray(positions, dtype=np.float64)
        self.K, self.C = stiffness, damping
        self.dts = [float(d) for d in dts]
        self.free_stream = np.asarray(free_stream, dtype=np.float64)
        self.direction = np.asarray(direction, dtype=np.float64)

    def _new(self, nu):
        flow = self.make_flow()
        flow.nu = nu
        vbf = VirtualBoundaryForcingOracle(self.K, self.C, 2, flow.dx, self.positions.shape[1], np.float64,
                                           enable_eul_grid_forcing_reset=True)
        return flow, vbf

    def loss(self, body_velocity, nu, record=False):
        """Forward rollout; returns L (and the per-step tape when ``record``)."""
        flow, vbf = self._new(nu)
        V = np.asarray(body_velocity, dtype=np.float64)
        L = 0.0
        tape = []
        for dt in self.dts:
            vbf.time_step(dt)
            vbf.compute_interaction_forcing(flow.eul_grid_forcing_field, flow.velocity_field, self.positions, V)
            L += dt * float(-(self.direction @ vbf.lag_grid_forcing_field.sum(axis=1)))
            rec = _step_recorded(flow, dt, self.free_stream)
            if record:
                tape.append(rec)
        if record:
            return L, tape, vbf
        return L

    def gradient(self, body_velocity, nu):
        """(L, dL/dV (2, n_lag), dL/dnu) by the hand-written adjoint."""
        L, tape, vbf = self.loss(body_velocity, nu, record=True)
        flow, _ = self._new(nu)
        dx = flow.dx
        pos = flow.position_field
        nearest, weights = vbf.nearest, vbf.weights
        n_lag = self.positions.shape[1]
        w_bar = np.zeros(flow.grid_size)
        u_bar = np.zeros((2, *flow.grid_size))
        xi_bar = np.zeros((2, n_lag))
        carry = np.zeros((2, n_lag))
        V_bar = np.zeros((2, n_lag))
        nu_bar = 0.0
        for n in range(len(self.dts) - 1, -1, -1):
            dt = self.dts[n]
            w_a, w_b, u_n = tape[n]
            psi_bar = curl_adj(u_bar, 0.5 / dx)
            g = w_bar + flow.poisson.solve(psi_bar)
            g = penalise_adj(g, flow.width, dx, pos[0], pos[1])
            k = nu * dt / dx / dx
            g, dk = diffusion_adj(g, k, w_b)
            nu_bar += dk * dt / dx / dx
            g, u_adv = eno3_adj(g, w_a, u_n, dt / dx)
            f_bar = forcing_curl_adj(g, dt / (2 * dx * flow.rho))
            w_bar = g
            # virtual boundary: F_bar = spread^T f_bar + loss weight
            F_bar = np.zeros((2, n_lag))
            for i in range(n_lag):
                win = (slice(nearest[1, i] - 1, nearest[1, i] + 3), slice(nearest[0, i] - 1, nearest[0, i] + 3))
                for c in range(2):
                    F_bar[c, i] = np.sum(f_bar[c][win] * weights[..., i])
            F_bar += -dt * self.direction[:, None]
            xi_bar = xi_bar + self.K * F_bar
            dU_bar = self.C * F_bar + carry
            V_bar -= dU_bar
            u_ib = np.zeros_like(u_bar)
            spread(u_ib, dU_bar * dx**2, weights, nearest)
            u_bar = u_adv + u_ib
            carry = dt * xi_bar
        return L, V_bar, nu_bar


def _step_recorded(flow: NavierStokes2DOracle, dt, free_stream):
    """flow.time_step(dt, free_stream) returning (w after forcing curl, w after advection, u before)."""
    rt, dx = flow.real_t, flow.dx
    w = flow.vorticity_field
    u_n = flow.velocity_field.copy()
    st.forcing_curl_update_2d(w, flow.eul_grid_forcing_field, rt(dt / (2 * dx * flow.rho)))
    w_a = w.copy()
    st.advection_step_2d(w, flow.velocity_field, rt(dt / dx))
    w_b = w.copy()
    st.diffusion_step_2d(w, rt(flow.nu * dt / dx / dx))
    st.penalise_2d(w, flow.width, dx, flow.position_field[0], flow.position_field[1])
    flow.stream_func_field[...] = flow.poisson.solve(w)
    st.outplane_curl_2d(flow.stream_func_field, rt(0.5 / dx), out=flow.velocity_field)
    if flow.with_free_stream_flow:
        for c in range(2):
            flow.velocity_field[c] = flow.velocity_field[c] + free_stream[c]
    flow.eul_grid_forcing_field[...] = 0
    flow.time += dt
    return w_a, w_b, u_n


class frozen_branches:
    """Context manager holding every ENO3 upwind choice of a rollout to a base trajectory's.

    ``with frozen_branches() as fb: problem.loss(V, nu)`` records the masks of the base run (in call
    order); later ``with fb.replay(): problem.loss(V + h dV, nu)`` runs with exactly those masks.  The
    ENO3 flux is discontinuous where u_j = -u_{j+1}, so a finite step can move the flow across an
    upwind switch; with the branches frozen the forward map is smooth (the map the adjoint
    differentiates) and central differences converge at O(h^2) at any step size.
    """

    def __init__(self):
        self.masks = []
        self._replay = None

    def __enter__(self):
        st.BRANCH_HOOK = self._record
        return self

    def __exit__(self, *exc):
        st.BRANCH_HOOK = None
        return False

    def _record(self, mask):
        self.masks.append(mask.copy())
        return mask

    def replay(self):
        outer = self

        class _Replay:
            def __enter__(self):
                it = iter(outer.masks)
                st.BRANCH_HOOK = lambda mask: next(it)
                return outer

            def __exit__(self, *exc):
                st.BRANCH_HOOK = None
                return False

        return _Replay()


def interpolate_adj(lag_bar, weights, nearest, eul_shape, dx):
    """Transpose of oracle.ib.interpolate (2D): eul_bar = dx^2 spread(lag_bar)."""
    out = np.zeros(eul_shape)
    spread(out, lag_bar * dx**2, weights, nearest)
    return out


__all__ = ["DragProblem2D", "frozen_branches", "curl_adj", "penalise_adj", "diffusion_adj", "eno3_adj", "forcing_curl_adj",
           "interpolate_adj", "interpolate"]
