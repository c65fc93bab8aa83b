"""GPU adjoints: per-operator transposes, the fused reverse sweep, and the
step-level gradient against the oracle's FP64 adjoint and finite differences.

Per-operator checks are dot-product tests in FP64 against the forward
entry points, <A x, y> = <x, A^T y>; the advection step is bilinear in (w, u)
for fixed upwind branches, so its central difference is exact to round-off.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

NY, NX = 40, 72


@pytest.fixture(scope="module", autouse=True)
def _built():
    from sopht_gb300.build import build
    build()


def _lib():
    from sopht_gb300 import _lib as L
    return L


def _cuda(a, dtype=torch.float64):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def _p(t):
    """Raw device pointer of a tensor the caller keeps alive (a temporary's memory
    can be reused by the next allocation before the kernel runs)."""
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _s():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def dot(a, b):
    return float(torch.sum(a.double() * b.double()).item())


F64 = 1  # SG_F64


def test_curl_adjoint_dot_product():
    L = _lib()
    r = np.random.default_rng(1)
    psi, ubar = _cuda(r.standard_normal((NY, NX))), _cuda(r.standard_normal((2, NY, NX)))
    u = torch.zeros_like(ubar)
    psib = torch.zeros_like(psi)
    L.call("sg_outplane_curl_2d", F64, NY, NX, _p(psi), _p(u), 0.7, _s())
    L.call("sg_outplane_curl_adj_2d", F64, NY, NX, _p(ubar), _p(psib), 0.7, _s())
    assert dot(u, ubar) == pytest.approx(dot(psi, psib), rel=1e-12)


@pytest.mark.parametrize("width", [0, 2, 3, 4])
def test_penalise_adjoint_dot_product(width):
    from sopht_gb300.numeric.eulerian_grid_ops import penalisation_factors
    L = _lib()
    r = np.random.default_rng(2)
    dx = 1.0 / NX
    cx = _cuda(penalisation_factors(width, dx, (np.arange(NX) + 0.5) * dx, np.float64))
    cy = _cuda(penalisation_factors(width, dx, (np.arange(NY) + 0.5) * dx, np.float64))
    x, y = _cuda(r.standard_normal((NY, NX))), _cuda(r.standard_normal((NY, NX)))
    px, ay = torch.zeros_like(x), torch.zeros_like(y)
    L.call("sg_penalise_2d", F64, NY, NX, _p(x), _p(px), width, _p(cx), _p(cy), _s())
    L.call("sg_penalise_adj_2d", F64, NY, NX, _p(y), _p(ay), width, _p(cx), _p(cy), _s())
    assert dot(px, y) == pytest.approx(dot(x, ay), rel=1e-12)


def test_penalise_adjoint_matches_oracle_transpose():
    from oracle.adjoint import penalise_adj
    from oracle.flow import position_field
    from sopht_gb300.numeric.eulerian_grid_ops import penalisation_factors
    L = _lib()
    r = np.random.default_rng(3)
    dx, pos = position_field((NY, NX), 1.0, np.float64)
    cx = _cuda(penalisation_factors(2, dx, pos[0][0, :], np.float64))
    cy = _cuda(penalisation_factors(2, dx, pos[1][:, 0], np.float64))
    y = r.standard_normal((NY, NX))
    yd = _cuda(y)  # keep every device buffer alive while the kernel may run
    out = torch.zeros((NY, NX), dtype=torch.float64, device="cuda")
    L.call("sg_penalise_adj_2d", F64, NY, NX, _p(yd), _p(out), 2, _p(cx), _p(cy), _s())
    np.testing.assert_allclose(out.cpu().numpy(), penalise_adj(y, 2, dx, pos[0], pos[1]), rtol=1e-13, atol=1e-15)


def test_diffusion_adjoint_dot_product_and_partials():
    L = _lib()
    r = np.random.default_rng(4)
    x, y = _cuda(r.standard_normal((NY, NX))), _cuda(r.standard_normal((NY, NX)))
    k = 0.11
    fx, ay = torch.zeros_like(x), torch.zeros_like(y)
    n_part = int(L.load().sg_adj_partials_count_2d(NY, NX))
    part = torch.zeros(n_part, dtype=torch.float64, device="cuda")
    acc = torch.zeros(1, dtype=torch.float64, device="cuda")
    L.call("sg_diffusion_step_2d", F64, NY, NX, _p(x), _p(fx), k, _s())
    L.call("sg_diffusion_adj_2d", F64, NY, NX, _p(y), _p(ay), k, _p(x), _p(part), _s())
    L.call("sg_sum_partials", n_part, _p(part), _p(acc), _s())
    assert dot(fx, y) == pytest.approx(dot(x, ay), rel=1e-12)
    # the step is affine in k: <step(x; k), y> = <x, y> + k <lap x, y>
    fx0 = torch.zeros_like(x)
    L.call("sg_diffusion_step_2d", F64, NY, NX, _p(x), _p(fx0), 0.0, _s())
    assert (dot(fx, y) - dot(fx0, y)) / k == pytest.approx(acc.item(), rel=1e-10)


def test_forcing_curl_adjoint_dot_product():
    L = _lib()
    r = np.random.default_rng(5)
    f, g = _cuda(r.standard_normal((2, NY, NX))), _cuda(r.standard_normal((NY, NX)))
    zero = torch.zeros((NY, NX), dtype=torch.float64, device="cuda")
    w = torch.zeros_like(zero)
    fb = torch.zeros_like(f)
    L.call("sg_forcing_curl_update_2d", F64, NY, NX, _p(zero), _p(w), _p(f), 0.3, _s())
    L.call("sg_forcing_curl_adj_2d", F64, NY, NX, _p(g), _p(fb), 0.3, _s())
    assert dot(w, g) == pytest.approx(dot(f, fb), rel=1e-12)


def test_eno3_adjoint_matches_linearisation():
    L = _lib()
    r = np.random.default_rng(6)
    w = _cuda(r.standard_normal((NY, NX)))
    u = _cuda(r.standard_normal((2, NY, NX)) + np.array([0.7, -0.4])[:, None, None])
    dw, du = _cuda(r.standard_normal((NY, NX))), _cuda(r.standard_normal((2, NY, NX)))
    g = _cuda(r.standard_normal((NY, NX)))
    c, eps = 0.21, 1e-7

    def step(ww, uu):
        out = torch.zeros_like(ww)
        L.call("sg_advection_eno3_step_2d", F64, NY, NX, _p(ww), _p(out), _p(uu), c, _s())
        return out

    jv = (step(w + eps * dw, u + eps * du) - step(w - eps * dw, u - eps * du)) / (2 * eps)
    wb, ub = torch.zeros_like(w), torch.zeros_like(u)
    L.call("sg_advection_eno3_adj_2d", F64, NY, NX, _p(w), _p(u), c, _p(g), _p(wb), _p(ub), _s())
    assert dot(jv, g) == pytest.approx(dot(dw, wb) + dot(du, ub), rel=1e-7)


def test_eno3_adjoint_matches_oracle_transpose():
    from oracle.adjoint import eno3_adj
    L = _lib()
    r = np.random.default_rng(7)
    w, u, g = r.standard_normal((NY, NX)), r.standard_normal((2, NY, NX)) + 0.3, r.standard_normal((NY, NX))
    wd, ud, gd = _cuda(w), _cuda(u), _cuda(g)
    wb = torch.zeros((NY, NX), dtype=torch.float64, device="cuda")
    ub = torch.zeros((2, NY, NX), dtype=torch.float64, device="cuda")
    L.call("sg_advection_eno3_adj_2d", F64, NY, NX, _p(wd), _p(ud), 0.17, _p(gd), _p(wb), _p(ub), _s())
    ow, ou = eno3_adj(g, w, u, 0.17)
    np.testing.assert_allclose(wb.cpu().numpy(), ow, rtol=1e-12, atol=1e-13)
    np.testing.assert_allclose(ub.cpu().numpy(), ou, rtol=1e-12, atol=1e-13)


def test_poisson_is_self_adjoint_on_gpu():
    from sopht_gb300.numeric import UnboundedPoissonSolver2D
    r = np.random.default_rng(8)
    P = UnboundedPoissonSolver2D(NY, NX, x_range=1.0, real_t=np.float64)
    x, y = _cuda(r.standard_normal((NY, NX))), _cuda(r.standard_normal((NY, NX)))
    px, py = torch.zeros_like(x), torch.zeros_like(y)
    P.solve(solution_field=px, rhs_field=x)
    P.solve(solution_field=py, rhs_field=y)
    assert dot(px, y) == pytest.approx(dot(x, py), rel=1e-12)


def test_ib_transposes_dot_product():
    """Spreading^T (in sg_ib_interaction_adj) and interpolation^T (sg_ib_interp_adj)."""
    from sopht_gb300.numeric.immersed_boundary_ops import VirtualBoundaryForcing
    L = _lib()
    r = np.random.default_rng(9)
    n, dx = 11, 1.0 / NX
    vbf = VirtualBoundaryForcing(0.0, 1.0, 2, dx, n, np.float64, device="cuda")
    pos = np.stack([r.uniform(0.2, 0.8, n), r.uniform(0.1, 0.45, n)])
    u = _cuda(r.standard_normal((2, NY, NX)))
    vbf.compute_interaction_force_on_lag_grid(u, pos, np.zeros((2, n)))
    U = vbf.lag_grid_flow_velocity_field.clone()
    nearest, wts = vbf.nearest_eul_grid_index_to_lag_grid, vbf.interp_weights
    # interpolation^T: <interp u, Ub> = <u, spread(dx^2 Ub)>
    Ub = _cuda(r.standard_normal((2, n)))
    Ub_scaled = Ub * dx * dx
    ub = torch.zeros_like(u)
    L.call("sg_ib_interp_adj", F64, 2, 1, NY, NX, n, _p(nearest), _p(wts), _p(Ub_scaled), _p(ub), _s())
    assert dot(U, Ub) == pytest.approx(dot(u, ub), rel=1e-12)
    # spreading^T: with K = 0, C = 1 and no carry, V_bar = -spread^T(f_bar)
    F = _cuda(r.standard_normal((2, n)))
    f = torch.zeros_like(u)
    L.call("sg_ib_spread", F64, 2, 1, NY, NX, n, _p(nearest), _p(wts), _p(F), _p(f), 1, _s())
    fb = _cuda(r.standard_normal((2, NY, NX)))
    xi_b, carry, ufb = (torch.zeros((2, n), dtype=torch.float64, device="cuda") for _ in range(3))
    vb = torch.zeros((2, n), dtype=torch.float64, device="cuda")
    L.call("sg_ib_interaction_adj", F64, 2, 1, NY, NX, dx, n, _p(nearest), _p(wts), _p(fb), None, 0.0, 1.0, 0.0,
           _p(xi_b), _p(carry), _p(vb), _p(ufb), _s())
    assert dot(f, fb) == pytest.approx(-dot(F, vb), rel=1e-12)


@pytest.mark.parametrize("width", [0, 2])
def test_reverse_sweep_equals_operator_composition(width):
    import sopht_gb300.simulator as sps
    L = _lib()
    r = np.random.default_rng(10)
    sim = sps.UnboundedNavierStokesFlowSimulator2D((NY, NX), 1.0, 1e-3, real_t=np.float64, with_forcing=True,
                                                   penalty_zone_width=width)
    ny, nx = NY, NX
    g0, g1 = _cuda(r.standard_normal((ny, nx))), _cuda(r.standard_normal((ny, nx)))
    wa, wb = _cuda(r.standard_normal((ny, nx))), _cuda(r.standard_normal((ny, nx)))
    u = _cuda(r.standard_normal((2, ny, nx)) + 0.2)
    sc = sim._scalars(3e-3, (0.0, 0.0))
    n_part = int(L.load().sg_adj_partials_count_2d(ny, nx))
    part = torch.zeros(n_part, dtype=torch.float64, device="cuda")
    acc_f = torch.zeros(1, dtype=torch.float64, device="cuda")
    out_w, out_u, out_f = torch.zeros_like(g0), torch.zeros_like(u), torch.zeros_like(u)
    L.call("sg_ns2d_reverse_sweep", sim._plan, _p(g0), _p(g1), _p(wa), _p(wb), _p(u), ctypes.byref(sc), _p(out_w),
           _p(out_u), _p(out_f), _p(part), _s())
    L.call("sg_sum_partials", n_part, _p(part), _p(acc_f), _s())
    # the same chain through the single-operator adjoints
    cx, cy = (torch.as_tensor(t, device="cuda") if t is not None else None for t in sim._coef_tables[:2])
    g = g0 + g1
    gc = torch.zeros_like(g)
    L.call("sg_penalise_adj_2d", F64, ny, nx, _p(g), _p(gc), width, _p(cx), _p(cy), _s())
    gb = torch.zeros_like(g)
    part2 = torch.zeros(n_part, dtype=torch.float64, device="cuda")
    acc_c = torch.zeros(1, dtype=torch.float64, device="cuda")
    L.call("sg_diffusion_adj_2d", F64, ny, nx, _p(gc), _p(gb), sc.diffusion_prefac, _p(wb), _p(part2), _s())
    L.call("sg_sum_partials", n_part, _p(part2), _p(acc_c), _s())
    ga = torch.zeros_like(g)
    ub = torch.zeros_like(u)
    L.call("sg_advection_eno3_adj_2d", F64, ny, nx, _p(wa), _p(u), sc.advection_prefac, _p(gb), _p(ga), _p(ub), _s())
    fb = torch.zeros_like(u)
    L.call("sg_forcing_curl_adj_2d", F64, ny, nx, _p(ga), _p(fb), sc.forcing_prefac, _s())
    for a, b in ((out_w, ga), (out_u, ub), (out_f, fb)):
        torch.testing.assert_close(a, b, rtol=1e-13, atol=1e-13)
    assert acc_f.item() == pytest.approx(acc_c.item(), rel=1e-12)


# ---------------------------------------------------------------- step level


def _drag_problem(real_t, ny=32, nx=64, n_steps=6, checkpoint_every=4, use_graphs=False, n_mk=24, dt=None,
                  radius=0.1, amplitude=0.1):
    """The oracle's tiny drag problem and the same problem on the GPU path."""
    import sopht_gb300.simulator as sps
    from oracle.adjoint import DragProblem2D
    from oracle.flow import CircularCylinderOracle, NavierStokes2DOracle
    r = np.random.default_rng(42)
    w0 = r.normal(0.0, 1e-3, (ny, nx))
    nu = 5e-4
    centre = (0.25, 0.5 * ny / nx)

    def make_flow():
        f = NavierStokes2DOracle((ny, nx), 1.0, nu, real_t=np.float64, with_forcing=True, with_free_stream_flow=True)
        f.vorticity_field[...] = w0
        return f

    cyl_o = CircularCylinderOracle(centre, radius, n_mk)
    h = cyl_o.get_maximum_lagrangian_grid_spacing()
    dx = 1.0 / nx
    dts = [0.1 * dx if dt is None else dt] * n_steps
    prob = DragProblem2D(make_flow, cyl_o.position_field, -5e4 * h, -20.0 * h, dts, (1.0, 0.0))
    theta = np.linspace(0, 2 * np.pi, n_mk, endpoint=False)
    V = amplitude * np.stack([-np.sin(theta), np.cos(theta)]) * r.uniform(0, 1, n_mk)

    sim = sps.UnboundedNavierStokesFlowSimulator2D((ny, nx), 1.0, nu, real_t=real_t, with_forcing=True,
                                                   with_free_stream_flow=True)
    sim.vorticity_field.copy_(torch.as_tensor(w0.astype(real_t)))
    cyl = sps.Cylinder([centre[0], centre[1], 0.0], base_radius=radius)
    inter = sps.RigidBodyFlowInteraction(
        rigid_body=cyl, eul_grid_forcing_field=sim.eul_grid_forcing_field, eul_grid_velocity_field=sim.velocity_field,
        virtual_boundary_stiffness_coeff=-5e4, virtual_boundary_damping_coeff=-20.0, dx=sim.dx, grid_dim=2,
        real_t=real_t, forcing_grid_cls=sps.CircularCylinderForcingGrid, num_forcing_points=n_mk,
        enable_eul_grid_forcing_reset=True)
    obj = sps.BodyForceObjective2D(sim, inter, dts, free_stream_velocity=(1.0, 0.0),
                                   checkpoint_every=checkpoint_every, use_graphs=use_graphs)
    return prob, obj, V, nu


@pytest.mark.parametrize("precision", ["double", "single"])
def test_step_gradient_vs_oracle_adjoint(precision):
    rt = np.float64 if precision == "double" else np.float32
    prob, obj, V, nu = _drag_problem(rt)
    L_o, gV_o, gnu_o = prob.gradient(V, nu)
    L_g, gV_g, gnu_g = obj.value_and_grad(torch.as_tensor(V, device="cuda"), nu)
    gV_g = gV_g.cpu().numpy()
    tol = 1e-9 if rt == np.float64 else 2e-3
    assert L_g == pytest.approx(L_o, rel=tol)
    assert np.linalg.norm(gV_g - gV_o) <= tol * np.linalg.norm(gV_o)
    assert gnu_g == pytest.approx(gnu_o, rel=tol)


def test_graph_mode_is_bitwise_equal_to_eager():
    _, obj_e, V, nu = _drag_problem(np.float32)
    _, obj_g, _, _ = _drag_problem(np.float32, use_graphs=True)
    Vt = torch.as_tensor(V, device="cuda")
    Le, gVe, gnue = obj_e.value_and_grad(Vt, nu)
    Lg, gVg, gnug = obj_g.value_and_grad(Vt, nu)
    Lg2, gVg2, gnug2 = obj_g.value_and_grad(Vt, nu)  # replay
    assert Le == Lg == Lg2
    assert torch.equal(gVe, gVg) and torch.equal(gVg, gVg2)
    assert gnue == gnug == gnug2


def test_autograd_function_and_fd_on_gpu():
    import sopht_gb300.simulator as sps
    # 48 markers keep the Lagrangian spacing inside [0.5, 2] dx; dt at the scale the stable-timestep rule
    # gives the 256 x 512 flow (a larger one lets the stiff feedback law blow up within 30 steps)
    _, obj, V, nu = _drag_problem(np.float64, ny=48, nx=96, n_steps=30, checkpoint_every=8, n_mk=48, dt=2e-4)
    Vt = torch.as_tensor(V, device="cuda").requires_grad_(True)
    nut = torch.tensor(nu, dtype=torch.float64, device="cuda", requires_grad=True)
    loss = sps.time_integrated_body_force(obj, Vt, nut)
    loss.backward()
    gV, gnu = Vt.grad.detach().clone(), float(nut.grad.item())
    r = np.random.default_rng(3)
    dV = torch.as_tensor(r.standard_normal(V.shape), device="cuda")
    h = 1e-7  # small enough that no ENO3 upwind branch flips (FP64 round-off ~1e-10 here)
    fd = (obj.forward(Vt.detach() + h * dV, nu).item() - obj.forward(Vt.detach() - h * dV, nu).item()) / (2 * h)
    assert fd == pytest.approx(float(torch.sum(gV * dV).item()), rel=1e-6)
    hn = 1e-8
    fdn = (obj.forward(Vt.detach(), nu + hn).item() - obj.forward(Vt.detach(), nu - hn).item()) / (2 * hn)
    assert fdn == pytest.approx(gnu, rel=1e-5)


def test_gradient_at_the_configuration_step_with_frozen_branches():
    """The drag gradient of the 256 x 512 cylinder flow (96 markers with a tangential wall velocity of
    amplitude up to 0.2, 200 frozen-dt steps, checkpoint every 20) on the GPU in FP64, against central
    differences at the configuration's step h = 1e-3 of the oracle's forward map with every ENO3
    upwind choice held to the base trajectory's (without that, steps of 1e-3 cross upwind switches and
    plain differences are off by several per cent): within 1e-3, in two directions and for nu."""
    from oracle.adjoint import frozen_branches
    prob, obj, V, nu = _drag_problem(np.float64, ny=256, nx=512, n_steps=200, checkpoint_every=20, n_mk=96,
                                     dt=1.9e-4, radius=0.05, amplitude=0.2)
    _, gV, gnu = obj.value_and_grad(torch.as_tensor(V, device="cuda"), nu)
    gV = gV.cpu().numpy()
    with frozen_branches() as fb:
        prob.loss(V, nu)
    h = 1e-3
    r = np.random.default_rng(17)
    for _ in range(2):
        dV = r.standard_normal(V.shape)
        with fb.replay():
            lp = prob.loss(V + h * dV, nu)
        with fb.replay():
            lm = prob.loss(V - h * dV, nu)
        assert (lp - lm) / (2 * h) == pytest.approx(float(np.sum(gV * dV)), rel=1e-3)
    with fb.replay():
        lp = prob.loss(V, nu * (1 + h))
    with fb.replay():
        lm = prob.loss(V, nu * (1 - h))
    assert (lp - lm) / (2 * h * nu) == pytest.approx(gnu, rel=1e-3)
