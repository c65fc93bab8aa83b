"""The oracle's FP64 adjoint, pinned to finite differences of the oracle's forward.

The reference has no adjoint.  Each hand-written transpose is checked with a
dot-product test against the oracle's forward operator (itself pinned to the
reference by the golden fixtures), and the whole rollout gradient against
central differences of the oracle's forward rollout.
"""

import numpy as np
import pytest

from oracle import stencils as st
from oracle.adjoint import (DragProblem2D, _step_recorded, curl_adj, diffusion_adj, eno3_adj, forcing_curl_adj,
                            interpolate_adj, penalise_adj)
from oracle.flow import CircularCylinderOracle, NavierStokes2DOracle, position_field
from oracle.ib import cosine_weights, interpolate, nearest_index_and_support

SHAPE = (20, 28)


def _rng(seed=0):
    return np.random.default_rng(seed)


def dot(a, b):
    return float(np.sum(a * b))


def test_curl_adjoint_dot_product():
    r = _rng(1)
    psi = r.standard_normal(SHAPE)
    ubar = r.standard_normal((2, *SHAPE))
    u = st.outplane_curl_2d(psi, 0.7)
    assert dot(u, ubar) == pytest.approx(dot(psi, curl_adj(ubar, 0.7)), rel=1e-12)


@pytest.mark.parametrize("width", [0, 2, 3])
def test_penalise_adjoint_dot_product(width):
    r = _rng(2)
    dx, pos = position_field(SHAPE, 1.0, np.float64)
    x = r.standard_normal(SHAPE)
    y = r.standard_normal(SHAPE)
    px = x.copy()
    st.penalise_2d(px, width, dx, pos[0], pos[1])
    assert dot(px, y) == pytest.approx(dot(x, penalise_adj(y, width, dx, pos[0], pos[1])), rel=1e-12)


def test_diffusion_adjoint_dot_product_and_k_derivative():
    r = _rng(3)
    x = r.standard_normal(SHAPE)
    y = r.standard_normal(SHAPE)
    k = 0.13
    fx = x.copy()
    st.diffusion_step_2d(fx, k)
    xa, dk = diffusion_adj(y, k, x)
    assert dot(fx, y) == pytest.approx(dot(x, xa), rel=1e-12)
    # d/dk <step(x; k), y> = <lap(x), y>
    h = 1e-6
    a, b = x.copy(), x.copy()
    st.diffusion_step_2d(a, k + h)
    st.diffusion_step_2d(b, k - h)
    assert (dot(a, y) - dot(b, y)) / (2 * h) == pytest.approx(dk, rel=1e-7)


def test_forcing_curl_adjoint_dot_product():
    r = _rng(4)
    f = r.standard_normal((2, *SHAPE))
    g = r.standard_normal(SHAPE)
    w = np.zeros(SHAPE)
    st.forcing_curl_update_2d(w, f, 0.3)
    assert dot(w, g) == pytest.approx(dot(f, forcing_curl_adj(g, 0.3)), rel=1e-12)


def test_eno3_adjoint_matches_linearisation():
    """The advection step is bilinear in (w, u) for fixed upwind branches, so a
    central difference with a small step is exact up to round-off."""
    r = _rng(5)
    w = r.standard_normal(SHAPE)
    u = r.standard_normal((2, *SHAPE)) + np.array([0.7, -0.4])[:, None, None]
    dw = r.standard_normal(SHAPE)
    du = r.standard_normal((2, *SHAPE))
    g = r.standard_normal(SHAPE)
    c = 0.21
    eps = 1e-7

    def step(ww, uu):
        out = ww.copy()
        st.advection_step_2d(out, uu, c)
        return out

    jv = (step(w + eps * dw, u + eps * du) - step(w - eps * dw, u - eps * du)) / (2 * eps)
    w_bar, u_bar = eno3_adj(g, w, u, c)
    assert dot(jv, g) == pytest.approx(dot(dw, w_bar) + dot(du, u_bar), rel=1e-7)


def test_interpolation_adjoint_dot_product():
    r = _rng(6)
    dx = 1.0 / SHAPE[1]
    pos = np.stack([r.uniform(0.2, 0.8, 9), r.uniform(0.2, 0.5, 9)])
    nearest, support, _ = nearest_index_and_support(pos, dx, dx / 2)
    wts = cosine_weights(support, dx, np.float64)
    u = r.standard_normal((2, *SHAPE))
    lag_bar = r.standard_normal((2, 9))
    U = interpolate(u, wts, nearest, dx)
    assert dot(U, lag_bar) == pytest.approx(dot(u, interpolate_adj(lag_bar, wts, nearest, u.shape, dx)), rel=1e-12)


def _tiny_problem(n_steps=6, ny=32, nx=64):
    r = np.random.default_rng(42)
    w0 = r.normal(0.0, 1e-3, (ny, nx))

    def make_flow():
        f = NavierStokes2DOracle((ny, nx), 1.0, 5e-4, real_t=np.float64, with_forcing=True,
                                 with_free_stream_flow=True)
        f.vorticity_field[...] = w0
        return f

    cyl = CircularCylinderOracle((0.25, 0.5 * ny / nx), 0.1, 24)
    h = cyl.get_maximum_lagrangian_grid_spacing()
    dx = 1.0 / nx
    prob = DragProblem2D(make_flow, cyl.position_field, -5e4 * h, -20.0 * h, [0.1 * dx] * n_steps, (1.0, 0.0))
    theta = np.linspace(0, 2 * np.pi, 24, endpoint=False)
    V = 0.1 * np.stack([-np.sin(theta), np.cos(theta)]) * r.uniform(0, 1, 24)
    return prob, V


def test_recorded_step_equals_oracle_step():
    prob, _ = _tiny_problem()
    a = prob.make_flow()
    b = prob.make_flow()
    forcing = 0.01 * np.random.default_rng(7).standard_normal(a.eul_grid_forcing_field.shape)
    for f in (a, b):
        f.eul_grid_forcing_field[...] = forcing
    a.time_step(1e-3, (1.0, 0.0))
    _step_recorded(b, 1e-3, np.array([1.0, 0.0]))
    np.testing.assert_array_equal(a.vorticity_field, b.vorticity_field)
    np.testing.assert_array_equal(a.velocity_field, b.velocity_field)


def test_rollout_gradient_matches_central_differences():
    prob, V = _tiny_problem()
    nu = 5e-4
    L, gV, gnu = prob.gradient(V, nu)
    assert L == pytest.approx(prob.loss(V, nu), rel=1e-14)
    r = np.random.default_rng(11)
    for _ in range(2):
        dV = r.standard_normal(V.shape)
        # small step: larger ones flip ENO3 upwind branches where u_j ~ -u_{j+1}
        # (the flux is discontinuous there), which the linearisation ignores
        h = 1e-6
        fd = (prob.loss(V + h * dV, nu) - prob.loss(V - h * dV, nu)) / (2 * h)
        assert fd == pytest.approx(dot(gV, dV), rel=1e-6)
    h = 1e-7
    fd_nu = (prob.loss(V, nu + h) - prob.loss(V, nu - h)) / (2 * h)
    assert fd_nu == pytest.approx(gnu, rel=1e-5)


def test_gradient_matches_frozen_branch_differences_at_the_configuration_step():
    """At h = 1e-3 (the configuration's finite-difference step) plain central differences cross ENO3
    upwind switches; with every upwind choice held to the base trajectory's the forward map is smooth
    and the central differences match the adjoint to O(h^2): within 1e-3."""
    from oracle.adjoint import frozen_branches
    prob, V = _tiny_problem()
    nu = 5e-4
    with frozen_branches() as fb:
        L0 = prob.loss(V, nu)
    assert fb.masks
    _, gV, gnu = prob.gradient(V, nu)
    r = np.random.default_rng(5)
    h = 1e-3
    for _ in range(3):
        dV = r.standard_normal(V.shape)
        with fb.replay():
            lp = prob.loss(V + h * dV, nu)
        with fb.replay():
            lm = prob.loss(V - h * dV, nu)
        assert (lp - lm) / (2 * h) == pytest.approx(dot(gV, dV), rel=1e-3)
    with fb.replay():
        lp = prob.loss(V, nu * (1 + h))
    with fb.replay():
        lm = prob.loss(V, nu * (1 - h))
    assert (lp - lm) / (2 * h * nu) == pytest.approx(gnu, rel=1e-3)
    with fb.replay():
        assert prob.loss(V, nu) == L0  # replaying the base masks reproduces the base run
