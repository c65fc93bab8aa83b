"""Discrete Cosserat rod dynamics (oracle for a batched rod integrator; test infrastructure).

SophT couples its rods through pyelastica 0.3.3.post2, which is not installed on
either machine this repository is tested on.  This module restates the
published discrete model that pyelastica implements: Gazzola, Dudte,
McCormick & Mahadevan (2018), "Forward and inverse problems in the mechanics
of soft filaments", R. Soc. Open Sci. 5:171628, with the position-Verlet
stepper.  Parity against pyelastica itself is unpinned; the tests pin the
model to analytic solutions instead (cantilever deflection, axial vibration
frequency, energy conservation, rigid-motion invariance).

Layout, as pyelastica's and SophT's forcing grids use it: n elements, n + 1
nodes; ``position``/``velocity`` (3, n+1); ``directors`` Q (3, 3, n) with rows
d1, d2, d3 (a lab vector v has local components Q v); ``omega`` (3, n) in the
local frame.

The model, per element i (local frame unless marked lab):

- l_i = |x_{i+1} - x_i|, t_i the unit tangent, e_i = l_i / l0_i;
- shear/stretch strain sigma_i = e_i Q_i t_i - e3, stress n_i = S_i sigma_i with
  S = diag(a G A, a G A, E A), a = 4/3;
- curvature on the n - 1 Voronoi regions: kappa_i = -log(Q_{i+1} Q_i^T)^v / D0_i
  (D0 the rest Voronoi length), bending couple m_i = B_i kappa_i with B the
  rest-length-weighted average of the two elements' diag(E I, E I, G 2I);
- nodal force: the difference over elements of Q^T n / e (lab);
- element couple: the difference over Voronoi regions of m / eps^3, the average of
  (kappa x m) D0 / eps^3, (Q t x n) l0, (J omega / e) x omega and
  (J omega / e^2) de/dt, where eps is the Voronoi dilatation and J the mass
  second moment rho l0 diag(I, I, 2I);
- m dv/dt = F + F_ext; (J / e) domega/dt = couple + C_ext.

Time step (position Verlet): x += v h/2 and Q <- exp(-[omega] h/2) Q; forces
at the midpoint; v += a h, omega += alpha h; x += v h/2 and Q <- exp(-[omega] h/2) Q.
"""

from __future__ import annotations

import numpy as np

SHEAR_FACTOR = 4.0 / 3.0


def _matvec(m, v):
    return np.einsum("ijk,jk->ik", m, v)


def _tmatvec(m, v):
    return np.einsum("jik,jk->ik", m, v)


def rotation_exp(v):
    """exp([v]x) for rotation vectors v (3, k), Rodrigues' formula."""
    theta = np.linalg.norm(v, axis=0)
    small = theta < 1e-12
    safe = np.where(small, 1.0, theta)
    k = v / safe
    s, c = np.sin(theta), np.cos(theta)
    kx = np.zeros((3, 3, v.shape[1]))
    kx[0, 1], kx[0, 2], kx[1, 0] = -k[2], k[1], k[2]
    kx[1, 2], kx[2, 0], kx[2, 1] = -k[0], -k[1], k[0]
    kx2 = np.einsum("ijk,jlk->ilk", kx, kx)
    eye = np.eye(3)[:, :, None]
    return eye + s * kx + (1.0 - c) * kx2


def rotation_log(r):
    """The rotation vector a with exp([a]x) = r, for rotations r (3, 3, k) of angle below pi."""
    cos = np.clip((np.einsum("iik->k", r) - 1.0) / 2.0, -1.0, 1.0)
    theta = np.arccos(cos)
    vee = np.stack([r[2, 1] - r[1, 2], r[0, 2] - r[2, 0], r[1, 0] - r[0, 1]])
    s = np.sin(theta)
    factor = np.where(theta < 1e-6, 0.5 + theta ** 2 / 12.0, theta / (2.0 * np.where(s == 0, 1.0, s)))
    return factor * vee


class CosseratRod:
    """One rod's state and material; ``step(dt)`` advances it by position Verlet."""

    def __init__(self, n_elements, start, direction, normal, length, radius, density, youngs_modulus,
                 shear_modulus=None, damping_rate=0.0):
        n = n_elements
        direction = np.asarray(direction, float) / np.linalg.norm(direction)
        normal = np.asarray(normal, float) / np.linalg.norm(normal)
        s = np.linspace(0.0, length, n + 1)
        self.n = n
        self.position = np.asarray(start, float)[:, None] + np.outer(direction, s)
        self.velocity = np.zeros((3, n + 1))
        d2 = np.cross(direction, normal)
        self.directors = np.repeat(np.stack([normal, d2, direction])[:, :, None], n, axis=2)
        self.omega = np.zeros((3, n))
        self.radius = np.full(n, float(radius)) if np.ndim(radius) == 0 else np.asarray(radius, float)
        self.density = density
        g = youngs_modulus / 3.0 if shear_modulus is None else shear_modulus
        self.rest_lengths = np.diff(s)
        self.rest_voronoi = 0.5 * (self.rest_lengths[1:] + self.rest_lengths[:-1])
        area = np.pi * self.radius ** 2
        inertia = area ** 2 / (4.0 * np.pi)  # pi r^4 / 4
        element_mass = density * area * self.rest_lengths
        self.mass = np.zeros(n + 1)
        self.mass[:-1] += 0.5 * element_mass
        self.mass[1:] += 0.5 * element_mass
        diag = lambda a, b, c: np.einsum("ij,k->ijk", np.eye(3), np.ones(n)) * np.stack([a, b, c])[None]  # noqa: E731
        self.shear_matrix = diag(SHEAR_FACTOR * g * area, SHEAR_FACTOR * g * area, youngs_modulus * area)
        bend = diag(youngs_modulus * inertia, youngs_modulus * inertia, g * 2.0 * inertia)
        w = self.rest_lengths
        self.bend_matrix = (bend[..., 1:] * w[1:] + bend[..., :-1] * w[:-1]) / (w[1:] + w[:-1])
        self.mass_second_moment = diag(inertia, inertia, 2.0 * inertia) * density * self.rest_lengths
        self.inv_mass_second_moment = np.linalg.inv(self.mass_second_moment.transpose(2, 0, 1)).transpose(1, 2, 0)
        self.rest_sigma = np.zeros((3, n))
        self.rest_kappa = np.zeros((3, n - 1))
        self.external_forces = np.zeros((3, n + 1))
        self.external_torques = np.zeros((3, n))
        self.damping_rate = damping_rate
        self.clamped = None  # (position of node 0, directors of element 0) when clamped
        self.drive = None  # (amplitude, frequency, phase, unit lab axis) of a clamp that turns the base
        self.time = 0.0

    def clamp_start(self) -> None:
        """Fix node 0 and the directors of element 0 where they are now."""
        self.clamped = (self.position[:, 0].copy(), self.directors[..., 0].copy())

    # -------------------------------------------------------------- geometry

    def _geometry(self):
        d = np.diff(self.position, axis=1)
        lengths = np.linalg.norm(d, axis=0)
        tangents = d / lengths
        dilatation = lengths / self.rest_lengths
        voronoi_dilatation = 0.5 * (lengths[1:] + lengths[:-1]) / self.rest_voronoi
        return lengths, tangents, dilatation, voronoi_dilatation

    def curvature(self):
        q = self.directors
        relative = np.einsum("ijk,ljk->ilk", q[..., 1:], q[..., :-1])  # Q_{i+1} Q_i^T
        return -rotation_log(relative) / self.rest_voronoi

    def strains(self):
        _, tangents, dilatation, _ = self._geometry()
        return dilatation * _matvec(self.directors, tangents) - np.array([0.0, 0.0, 1.0])[:, None]

    # ---------------------------------------------------------------- forces

    def internal_loads(self):
        """Nodal forces (lab) and element couples (local) from the current state."""
        lengths, tangents, e, eps = self._geometry()
        local_tangent = _matvec(self.directors, tangents)
        sigma = e * local_tangent - np.array([0.0, 0.0, 1.0])[:, None]
        stress = _matvec(self.shear_matrix, sigma - self.rest_sigma)
        lab = _tmatvec(self.directors, stress) / e
        force = np.zeros((3, self.n + 1))
        force[:, :-1] += lab
        force[:, 1:] -= lab
        kappa = self.curvature()
        moment = _matvec(self.bend_matrix, kappa - self.rest_kappa)
        couple = np.zeros((3, self.n))
        bend = moment / eps ** 3
        couple[:, :-1] += bend
        couple[:, 1:] -= bend
        twist = np.cross(kappa, moment, axis=0) * self.rest_voronoi / eps ** 3
        couple[:, :-1] += 0.5 * twist
        couple[:, 1:] += 0.5 * twist
        couple += np.cross(local_tangent, stress, axis=0) * self.rest_lengths
        j_omega = _matvec(self.mass_second_moment, self.omega)
        couple += np.cross(j_omega, self.omega, axis=0) / e
        dilatation_rate = np.einsum("ik,ik->k", tangents, np.diff(self.velocity, axis=1)) / self.rest_lengths
        couple += j_omega / e ** 2 * dilatation_rate
        return force, couple

    # ------------------------------------------------------------------ step

    def _rotate(self, h):
        self.directors = np.einsum("ijk,jlk->ilk", rotation_exp(-h * self.omega), self.directors)

    def _clamp_frame(self, t):
        """Directors and local angular velocity of element 0 at time t: fixed, or turned about the lab
        axis a by theta(t) = A sin(2 pi f t + phi) (each director d -> R d, so Q0 R^T, and omega =
        Q (theta' a))."""
        q0 = self.clamped[1]
        if self.drive is None:
            return q0, np.zeros(3)
        amp, freq, phase, axis = self.drive
        arg = 2.0 * np.pi * freq * t + phase
        theta, rate = amp * np.sin(arg), amp * 2.0 * np.pi * freq * np.cos(arg)
        rot = rotation_exp((theta * np.asarray(axis, float))[:, None])[..., 0]
        q = q0 @ rot.T
        return q, q @ (rate * np.asarray(axis, float))

    def _apply_clamp(self, t=None):
        if self.clamped is not None:
            q, w = self._clamp_frame(self.time if t is None else t)
            self.position[:, 0] = self.clamped[0]
            self.directors[..., 0] = q
            self.velocity[:, 0] = 0.0
            self.omega[:, 0] = w

    def step(self, dt: float, midpoint_loads=None) -> None:
        """One position-Verlet step.  ``midpoint_loads(rod)``, when given, sets the external loads from
        the half-step configuration (pyelastica evaluates its forcing there, inside do_step)."""
        half = 0.5 * dt
        self.position += half * self.velocity
        self._rotate(half)
        self._apply_clamp(self.time + half)
        if midpoint_loads is not None:
            midpoint_loads(self)
        force, couple = self.internal_loads()
        _, _, e, _ = self._geometry()
        self.velocity += dt * (force + self.external_forces) / self.mass
        self.omega += dt * e * _matvec(self.inv_mass_second_moment, couple + self.external_torques)
        if self.damping_rate:
            decay = np.exp(-self.damping_rate * dt)
            self.velocity *= decay
            self.omega *= decay
        self._apply_clamp(self.time + half)
        self.position += half * self.velocity
        self._rotate(half)
        self._apply_clamp(self.time + dt)
        self.time += dt

    # ---------------------------------------------------------------- energy

    def energy(self) -> float:
        """Kinetic (translation and rotation) plus shear/stretch and bending/twist strain energy."""
        _, _, e, _ = self._geometry()
        kinetic = 0.5 * np.sum(self.mass * np.sum(self.velocity ** 2, axis=0))
        kinetic += 0.5 * np.sum(self.omega * _matvec(self.mass_second_moment, self.omega) / e)
        sigma = self.strains() - self.rest_sigma
        strain = 0.5 * np.sum(sigma * _matvec(self.shear_matrix, sigma) * self.rest_lengths)
        kappa = self.curvature() - self.rest_kappa
        strain += 0.5 * np.sum(kappa * _matvec(self.bend_matrix, kappa) * self.rest_voronoi)
        return float(kinetic + strain)


class _ElementCentricView:
    """A rod under the attribute names the element-centric forcing grid reads."""

    def __init__(self, rod):
        self.rod = rod
        self.n_elems = rod.n

    @property
    def position_collection(self):
        return self.rod.position

    @property
    def velocity_collection(self):
        return self.rod.velocity

    @property
    def mass(self):
        return self.rod.mass

    @property
    def lengths(self):
        return np.linalg.norm(np.diff(self.rod.position, axis=1), axis=0)


def coupled_rod_loop(rods, interactors, flow_dt, rod_dt):
    """The rod loop of one flow step of the reference examples (flow_past_rod_case.py:231-243): each
    sub-step is one position-Verlet step of every rod with FlowForces.apply_forces (flow_forces.py:
    22-25: compute_flow_forces_and_torques, then the body forces as the rod's external loads) at the
    half step, then every interactor's time_step.  ``interactors[i]`` is an
    ``oracle.flow.ImmersedBodyInteractionOracle`` over ``RodElementCentricGridOracle`` of rod i
    (wrapped by ``element_centric_view``); the flow forces are the rods' only loads."""
    n_sub = int(flow_dt / min(flow_dt, rod_dt))
    h = flow_dt / n_sub

    def loads(inter):
        def apply(rod):
            inter.compute_flow_forces_and_torques()
            rod.external_forces[...] = inter.body_flow_forces
            rod.external_torques[...] = inter.body_flow_torques
        return apply

    for _ in range(n_sub):
        for rod, inter in zip(rods, interactors, strict=True):
            rod.step(h, midpoint_loads=loads(inter))
        for inter in interactors:
            inter.time_step(h)
    return n_sub


def element_centric_view(rod):
    """``rod`` as the element-centric forcing grid oracle expects it."""
    return _ElementCentricView(rod)
