"""The Cosserat rod oracle against analytic solutions (its parity with pyelastica is unpinned).

Rotation maps, rigid-motion invariance (a translating rod spinning about its
axis keeps its shape and spins at the set rate), the static cantilever tip
deflection P l^3 / (3 E I) + P l / (a G A) and the first bending frequency
3.516 sqrt(E I / (rho A l^4)) of the released beam, the first axial and torsional
frequencies of a clamped-free rod ((pi / 2L) sqrt(E / rho) and
(pi / 2l) sqrt(G / rho)), and energy conservation of a free bending vibration.
Fixing element 0's directors clamps bending and twist at that element's centre,
so l = L - l0 / 2 where they are concerned (axial motion lives on the nodes).
Tolerances are the discretisation error of 20 elements (about 1 %).
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle.rod import CosseratRod, rotation_exp, rotation_log

L, R, RHO, E = 1.0, 0.05, 1.0, 1.0e3
N = 20


def _rod(**kw):
    return CosseratRod(N, start=[0.0, 0.0, 0.0], direction=[0.0, 0.0, 1.0], normal=[1.0, 0.0, 0.0], length=L,
                       radius=R, density=RHO, youngs_modulus=E, **kw)


def _dt():
    return 0.3 * (L / N) / np.sqrt(E / RHO)


def _zero_crossings(t, y):
    s = np.sign(y)
    idx = np.nonzero(s[1:] * s[:-1] < 0)[0]
    return t[idx] - y[idx] * (t[idx + 1] - t[idx]) / (y[idx + 1] - y[idx])


def test_rotation_exp_log_round_trip():
    rng = np.random.default_rng(0)
    v = rng.standard_normal((3, 50))
    v *= (rng.uniform(0.0, 3.0, 50) / np.linalg.norm(v, axis=0))
    v[:, :3] = [[0, 1e-9, 0], [0, 0, 2e-7], [0, 0, 0]]
    r = rotation_exp(v)
    np.testing.assert_allclose(np.einsum("ijk,ljk->ilk", r, r), np.broadcast_to(np.eye(3)[:, :, None], r.shape),
                               atol=1e-14)
    np.testing.assert_allclose(rotation_log(r), v, atol=1e-9)


def test_rigid_motion_keeps_shape_and_spin():
    rod = _rod()
    v, spin = np.array([0.3, -0.2, 0.1]), 2.0
    rod.velocity[...] = v[:, None]
    rod.omega[2] = spin
    x0, d1 = rod.position.copy(), rod.directors[0].copy()
    force, couple = rod.internal_loads()
    assert np.abs(force).max() < 1e-12 and np.abs(couple).max() < 1e-12
    dt = _dt()
    for _ in range(200):
        rod.step(dt)
    np.testing.assert_allclose(rod.position, x0 + v[:, None] * rod.time, atol=1e-12)
    angle = spin * rod.time
    expected = np.stack([np.cos(angle) * d1[0], np.sin(angle) * d1[0], d1[2]])  # d1 = e_x spun about e_z
    np.testing.assert_allclose(rod.directors[0], expected, atol=1e-10)


def test_cantilever_tip_deflection():
    inertia = np.pi * R ** 4 / 4.0
    area = np.pi * R ** 2
    g = E / 3.0
    load = 1.5e-5
    omega1 = 3.516 * np.sqrt(E * inertia / (RHO * area * L ** 4))
    rod = _rod(damping_rate=2.0 * omega1)
    rod.clamp_start()
    rod.external_forces[0, -1] = load
    dt = _dt()
    for _ in range(int(4.0 / dt)):
        rod.step(dt)
    # fixing element 0's directors clamps the beam at that element's centre: free length L - l0 / 2
    free = L - 0.5 * L / N
    expected = load * free ** 3 / (3.0 * E * inertia) + load * free / (4.0 / 3.0 * g * area)
    assert rod.position[0, -1] == pytest.approx(expected, rel=1e-2)
    assert np.abs(rod.velocity).max() < 1e-3 * expected
    # released, the bent beam swings at the first bending frequency 3.516 sqrt(E I / (rho A l^4))
    # (rotary inertia and shear of this thick beam, L / r = 20, lower it by under 1 %)
    rod.external_forces[...] = 0.0
    rod.damping_rate = 0.0
    t0 = rod.time
    period = _first_period(rod, lambda r: r.position[0, -1], int(3.2 * 2 * np.pi / omega1 / dt))
    assert rod.time > t0
    assert period == pytest.approx(2 * np.pi / (3.516 * np.sqrt(E * inertia / (RHO * area * free ** 4))), rel=2e-2)


def _first_period(rod, probe, steps):
    dt = _dt()
    t, y = [], []
    for _ in range(steps):
        rod.step(dt)
        t.append(rod.time)
        y.append(probe(rod))
    crossings = _zero_crossings(np.array(t), np.array(y))
    return 2.0 * np.mean(np.diff(crossings))


def test_axial_frequency():
    rod = _rod()
    rod.clamp_start()
    s = np.linspace(0.0, L, N + 1)
    rod.velocity[2] = 1e-4 * np.sin(np.pi * s / (2 * L))  # first axial mode, started from rest length
    period = _first_period(rod, lambda r: r.velocity[2, -1], int(3 * 4 * L / np.sqrt(E / RHO) / _dt()))
    assert period == pytest.approx(4 * L / np.sqrt(E / RHO), rel=1e-2)


def test_torsional_frequency():
    rod = _rod()
    rod.clamp_start()
    centres = (np.arange(N) + 0.5) * L / N
    rod.omega[2] = 1e-4 * np.sin(np.pi * centres / (2 * L))  # first torsional mode
    speed = np.sqrt(E / 3.0 / RHO)
    period = _first_period(rod, lambda r: r.omega[2, -1], int(3 * 4 * L / speed / _dt()))
    # twist lives on the element centres and element 0 (centre at l0 / 2) is fixed: free length L - l0 / 2
    assert period == pytest.approx(4 * (L - 0.5 * L / N) / speed, rel=1e-2)


def test_bending_vibration_conserves_energy():
    rod = _rod()
    rod.clamp_start()
    s = np.linspace(0.0, L, N + 1)
    rod.velocity[0] = 1e-3 * (s / L) ** 2
    e0 = rod.energy()
    dt = _dt()
    energies = []
    for _ in range(3000):
        rod.step(dt)
        energies.append(rod.energy())
    assert np.max(np.abs(np.array(energies) - e0)) < 1e-3 * e0


def _bent_twisted_free_rod():
    """A free rod laid on an arc of curvature 1 in the xz plane, twisted 1.5 rad per unit length
    about its tangent and stretched 1 %, at rest: it holds bending, twist and stretch energy."""
    rod = _rod()
    s = np.linspace(0.0, L, N + 1) * 1.01
    rod.position = np.stack([1.0 - np.cos(s), 0.0 * s, np.sin(s)])
    centres = (np.arange(N) + 0.5) / N * L
    for i, c in enumerate(centres):
        bend = rotation_exp(np.array([[0.0], [c], [0.0]]))[:, :, 0]
        twist = rotation_exp((bend @ np.array([0.0, 0.0, 1.5 * c]))[:, None])[:, :, 0]
        rod.directors[:, :, i] = (twist @ bend).T
    return rod


def _momenta(rod):
    e = rod._geometry()[2]
    linear = np.sum(rod.mass * rod.velocity, axis=1)
    spin = np.einsum("ijk,jk->ik", rod.mass_second_moment, rod.omega) / e
    angular = np.sum(rod.mass * np.cross(rod.position, rod.velocity, axis=0), axis=1)
    angular += np.einsum("jik,jk->ik", rod.directors, spin).sum(axis=1)
    scale = np.sum(rod.mass * np.linalg.norm(rod.velocity, axis=0)) * L
    return linear, angular, scale


def test_free_rod_conserves_momenta():
    """Released from rest, the bent and twisted rod moves but its total linear momentum and its
    angular momentum (node momenta plus element spins Q^T J omega / e) stay zero: below 2e-4 of
    the motion's momentum scale (sum m |v| L; 3.8e-5 measured).  The couple's kappa x m,
    transport and dilatation terms are what keep it there: flipping or dropping any one of
    them raises it 1.5 to 50 times above the bound."""
    rod = _bent_twisted_free_rod()
    dt = _dt()
    worst_linear = worst_angular = top = 0.0
    for _ in range(3000):
        rod.step(dt)
        linear, angular, scale = _momenta(rod)
        top = max(top, scale)
        worst_linear = max(worst_linear, np.abs(linear).max())
        worst_angular = max(worst_angular, np.abs(angular).max())
    assert top > 1e-3  # it moves
    assert worst_linear < 1e-12
    assert worst_angular < 2e-4 * top
