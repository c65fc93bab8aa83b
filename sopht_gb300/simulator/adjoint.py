"""Gradients of a time-integrated body force through the 2D coupled step.

No counterpart in the reference (it has no differentiation).  The objective is

    L = sum_n dt_n * d . (-sum_k F_k^n)

the force on a fixed immersed body (the reaction of its virtual-boundary
forcing, rigid_body_forcing_grids.py:58-75) along the direction ``d``,
integrated over a frozen sequence of steps of the reference's coupled loop
(``interactor.time_step(dt)``, ``interactor()``,
``flow_sim.time_step(dt, free_stream)``).  It is differentiated with respect to
the prescribed marker velocities V (2, n_lag) -- the body's Lagrangian
velocity field -- and the kinematic viscosity.

The forward pass runs the drop-in kernels and stores a checkpoint of the state
(vorticity, velocity, position and velocity mismatch) every
``checkpoint_every`` steps.  The backward pass walks the segments in reverse:
it restores a checkpoint, recomputes the segment's forward steps while recording
a tape (velocity at the step start, vorticity after the forcing curl and after
the advection update), then applies the hand-written transpose of each step:
curl^T, the (self-adjoint) Poisson solve, one fused reverse sweep
(penalisation^T, diffusion^T with the viscosity term, ENO3^T, forcing-curl^T)
and the virtual-boundary transpose (spreading^T, feedback law, interpolation^T).
The ENO3 upwind branch of every face is held at its forward choice.

``time_integrated_body_force(objective, V, nu)`` wraps this in a
``torch.autograd.Function``.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from .. import _lib
from ..utils import ptr, sg_dtype, stream_ptr
from .flow import UnboundedNavierStokesFlowSimulator2D


class BodyForceObjective2D:
    """Differentiable time-integrated body force of one fixed body in a 2D flow.

    The objective owns the simulator's and interactor's state while it runs:
    every forward pass starts from the state they had when the objective was
    built.  ``dt_sequence`` is the frozen list of step sizes.
    """

    def __init__(self, flow_sim, interactor, dt_sequence, free_stream_velocity=(0.0, 0.0), direction=(1.0, 0.0),
                 checkpoint_every=20, use_graphs=False):
        if not isinstance(flow_sim, UnboundedNavierStokesFlowSimulator2D) or not flow_sim.with_forcing:
            raise ValueError("the objective needs a 2D flow simulator with forcing")
        if interactor.eul_grid_forcing_field.data_ptr() != flow_sim.eul_grid_forcing_field.data_ptr():
            raise ValueError("the interactor does not force this simulator")
        if checkpoint_every < 1:
            raise ValueError("checkpoint_every must be >= 1")
        self.sim = flow_sim
        self.inter = interactor
        self.dts = [float(d) for d in dt_sequence]
        if not self.dts:
            raise ValueError("empty dt sequence")
        self.n_steps = len(self.dts)
        self.free_stream = np.asarray(free_stream_velocity, dtype=np.float64).reshape(2)
        self.direction = np.asarray(direction, dtype=np.float64).reshape(2)
        self.ck = int(checkpoint_every)
        self.use_graphs = use_graphs
        sim, inter = flow_sim, interactor
        dev = sim.device
        self.device = dev
        self.dtype = sim.vorticity_field.dtype
        self._sgt = sg_dtype(sim.real_t)
        ny, nx = sim.grid_size
        self.ny, self.nx = ny, nx
        n_lag = inter.num_lag_nodes
        self.n_lag = n_lag
        inter.upload_kinematics()
        # the state every forward pass starts from
        self._w0 = sim.vorticity_field.clone()
        self._u0 = sim.velocity_field.clone()
        self._xi0 = inter.lag_grid_position_mismatch_field.clone()
        self._du0 = inter.lag_grid_velocity_mismatch_field.clone()
        self._pos = inter._pos_stage.dev.clone()
        self._V = inter._vel_stage.dev.clone()
        f = dict(dtype=self.dtype, device=dev)
        n_ck = (self.n_steps + self.ck - 1) // self.ck
        self._ck_w = torch.zeros((n_ck, ny, nx), **f)
        self._ck_u = torch.zeros((n_ck, 2, ny, nx), **f)
        self._ck_xi = torch.zeros((n_ck, 2, n_lag), **f)
        self._ck_du = torch.zeros((n_ck, 2, n_lag), **f)
        self._tape_wa = torch.zeros((self.ck, ny, nx), **f)
        self._tape_wb = torch.zeros((self.ck, ny, nx), **f)
        self._tape_u = torch.zeros((self.ck, 2, ny, nx), **f)
        self._w_bar = [torch.zeros((ny, nx), **f), torch.zeros((ny, nx), **f)]
        self._u_bar = torch.zeros((2, ny, nx), **f)
        self._psi_bar = torch.zeros((ny, nx), **f)
        self._poisson_bar = torch.zeros((ny, nx), **f)
        self._f_bar = torch.zeros((2, ny, nx), **f)
        self._xi_bar = torch.zeros((2, n_lag), **f)
        self._carry = torch.zeros((2, n_lag), **f)
        self._u_flow_bar = torch.zeros((2, n_lag), **f)
        self._V_bar = torch.zeros((2, n_lag), dtype=torch.float64, device=dev)
        n_part = int(_lib.load().sg_adj_partials_count_2d(ny, nx))
        self._partials = torch.zeros((self.n_steps, n_part), dtype=torch.float64, device=dev)
        self._dk = torch.zeros(self.n_steps, dtype=torch.float64, device=dev)
        self._loss = torch.zeros(1, dtype=torch.float64, device=dev)
        self._n_part = n_part
        self._poisson_plan = _lib.load().sg_flow_poisson_plan(sim._plan)
        self._graphs = {}
        self.gpu_launches = {}

    # ------------------------------------------------------------ helpers
    def _restore(self, w, u, xi, du):
        sim, inter = self.sim, self.inter
        sim.vorticity_field.copy_(w)
        sim.velocity_field.copy_(u)
        sim.eul_grid_forcing_field.zero_()
        inter.lag_grid_position_mismatch_field.copy_(xi)
        inter.lag_grid_velocity_mismatch_field.copy_(du)

    def _forward_step(self, n, tape_slot=None, accumulate_loss=True):
        sim, inter = self.sim, self.inter
        dt = self.dts[n]
        if tape_slot is not None:
            self._tape_u[tape_slot].copy_(sim.velocity_field)
            _lib.call("sg_flow_set_tape", sim._plan, ptr(self._tape_wa[tape_slot]), ptr(self._tape_wb[tape_slot]))
        inter._interaction(sim.velocity_field, self._pos, self._V, xi_step=True, xi_dt=dt)
        inter._spread(sim.eul_grid_forcing_field, reset=True)
        if accumulate_loss:
            w3 = (ctypes.c_double * 3)(-dt * self.direction[0], -dt * self.direction[1], 0.0)
            _lib.call("sg_lag_weighted_sum", self._sgt, 2, self.n_lag, ptr(inter.lag_grid_forcing_field), w3,
                      ptr(self._loss), stream_ptr(self.device))
        sim._flow_time_step(dt, self.free_stream)

    def _reverse_step(self, n, slot, cur):
        sim, inter = self.sim, self.inter
        dt = self.dts[n]
        ny, nx = self.ny, self.nx
        s = stream_ptr(self.device)
        sc = sim._scalars(dt, self.free_stream)
        pref = float(sim.real_t(0.5) / sim.real_t(sim.dx))
        _lib.call("sg_outplane_curl_adj_2d", self._sgt, ny, nx, ptr(self._u_bar), ptr(self._psi_bar), pref, s)
        _lib.call("sg_poisson_solve_adj", self._poisson_plan, ptr(self._psi_bar), ptr(self._poisson_bar), 1, 0, s)
        _lib.call("sg_ns2d_reverse_sweep", sim._plan, ptr(self._w_bar[cur]), ptr(self._poisson_bar),
                  ptr(self._tape_wa[slot]), ptr(self._tape_wb[slot]), ptr(self._tape_u[slot]), ctypes.byref(sc),
                  ptr(self._w_bar[1 - cur]), ptr(self._u_bar), ptr(self._f_bar), ptr(self._partials[n]), s)
        _lib.call("sg_sum_partials", self._n_part, ptr(self._partials[n]), ptr(self._dk[n:n + 1]), s)
        fc = (ctypes.c_double * 3)(-dt * self.direction[0], -dt * self.direction[1], 0.0)
        _lib.call("sg_ib_interaction_adj", self._sgt, 2, 1, ny, nx, float(sim.dx), self.n_lag,
                  ptr(inter.nearest_eul_grid_index_to_lag_grid), ptr(inter.interp_weights), ptr(self._f_bar), fc,
                  float(inter.virtual_boundary_stiffness_coeff), float(inter.virtual_boundary_damping_coeff), dt,
                  ptr(self._xi_bar), ptr(self._carry), ptr(self._V_bar), ptr(self._u_flow_bar), s)
        _lib.call("sg_ib_interp_adj", self._sgt, 2, 1, ny, nx, self.n_lag,
                  ptr(inter.nearest_eul_grid_index_to_lag_grid), ptr(inter.interp_weights), ptr(self._u_flow_bar),
                  ptr(self._u_bar), s)
        return 1 - cur

    def _forward_pass(self):
        self._restore(self._w0, self._u0, self._xi0, self._du0)
        self._loss.zero_()
        for n in range(self.n_steps):
            if n % self.ck == 0:
                k = n // self.ck
                self._ck_w[k].copy_(self.sim.vorticity_field)
                self._ck_u[k].copy_(self.sim.velocity_field)
                self._ck_xi[k].copy_(self.inter.lag_grid_position_mismatch_field)
                self._ck_du[k].copy_(self.inter.lag_grid_velocity_mismatch_field)
            self._forward_step(n)

    def _backward_pass(self):
        for t in (self._w_bar[0], self._u_bar, self._xi_bar, self._carry, self._V_bar, self._dk):
            t.zero_()
        cur = 0
        n_ck = self._ck_w.shape[0]
        for k in range(n_ck - 1, -1, -1):
            n0, n1 = k * self.ck, min(self.n_steps, (k + 1) * self.ck)
            self._restore(self._ck_w[k], self._ck_u[k], self._ck_xi[k], self._ck_du[k])
            for n in range(n0, n1):
                self._forward_step(n, tape_slot=n - n0, accumulate_loss=False)
            for n in range(n1 - 1, n0 - 1, -1):
                cur = self._reverse_step(n, n - n0, cur)

    def _run(self, name, fn):
        if not self.use_graphs:
            fn()
            return
        key = (name, float(self.sim.kinematic_viscosity))
        g = self._graphs.get(key)
        if g is None:
            for k in [k for k in self._graphs if k[0] == name]:
                del self._graphs[k]
            stream = torch.cuda.Stream(self.device)
            stream.wait_stream(torch.cuda.current_stream(self.device))
            with torch.cuda.stream(stream):
                fn()  # warm-up outside capture (lazy allocations, attribute setup)
            torch.cuda.current_stream(self.device).wait_stream(stream)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=stream):
                fn()
            self._graphs[key] = g
        g.replay()

    # ------------------------------------------------------------ public
    def forward(self, body_velocity, nu: float) -> torch.Tensor:
        """Run the forward pass; returns L as a 1-element float64 device tensor."""
        V = torch.as_tensor(body_velocity, dtype=torch.float64, device=self.device).reshape(2, self.n_lag)
        self._V.copy_(V)
        self.sim.kinematic_viscosity = float(nu)
        self._run("forward", self._forward_pass)
        return self._loss

    def backward(self):
        """Gradient of the last forward pass: (dL/dV (2, n_lag) float64 tensor, dL/dnu float)."""
        self._run("backward", self._backward_pass)
        dk = self._dk.cpu().numpy()
        dx2 = float(self.sim.dx) ** 2
        nu_bar = float(np.sum(dk * np.asarray(self.dts) / dx2))
        return self._V_bar.clone(), nu_bar

    def value_and_grad(self, body_velocity, nu: float):
        loss = float(self.forward(body_velocity, nu).item())
        gV, gnu = self.backward()
        return loss, gV, gnu


class _TimeIntegratedBodyForce(torch.autograd.Function):
    @staticmethod
    def forward(ctx, body_velocity, nu, objective):
        loss = objective.forward(body_velocity.detach(), float(nu))
        ctx.objective = objective
        ctx.v_shape = body_velocity.shape
        ctx.v_dtype = body_velocity.dtype
        ctx.nu_dtype = nu.dtype if isinstance(nu, torch.Tensor) else torch.float64
        return loss.clone().reshape(())

    @staticmethod
    def backward(ctx, grad_out):
        gV, gnu = ctx.objective.backward()
        g = grad_out.to(torch.float64)
        dV = (g * gV).reshape(ctx.v_shape).to(ctx.v_dtype)
        dnu = (g * gnu).to(ctx.nu_dtype)
        return dV, dnu, None


def time_integrated_body_force(objective: BodyForceObjective2D, body_velocity: torch.Tensor, nu) -> torch.Tensor:
    """Differentiable L(V, nu) (a 0-d float64 tensor); gradients flow to both."""
    if not isinstance(nu, torch.Tensor):
        nu = torch.tensor(float(nu), dtype=torch.float64, device=objective.device)
    return _TimeIntegratedBodyForce.apply(body_velocity, nu, objective)
