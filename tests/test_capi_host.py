"""CPU checks of the C ABI and of the host-side reformulations (no GPU needed).

* the library loads, and exports exactly the entry points ``include/*.h``
  declares (and the ctypes binding knows each of them);
* argument validation fails with the documented status before any CUDA call;
* the GPU path's reformulations, restated in numpy, agree with the oracle:
  penalisation as one clamped gather times per-index factors, and the
  domain-doubled Poisson solve as row R2C -> column convolution -> row C2R
  without materialising the doubled box.
"""

from __future__ import annotations

import ctypes
import re
from pathlib import Path

import numpy as np
import pytest
from conftest import load_golden, real_t_of, ref_tol

from oracle import stencils as st
from oracle.poisson import UnboundedPoisson2D, UnboundedPoisson3D, greens_function_2d, greens_function_3d

REPO = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def lib():
    from sopht_gb300 import _lib
    from sopht_gb300.build import LIB, build
    if not LIB.exists():
        build()
    return _lib.load()


def _header_symbols():
    syms = set()
    for h in (REPO / "include").glob("*.h"):
        text = h.read_text()
        syms |= set(re.findall(r"\b(sg_[a-z0-9_]+)\s*\(", text))
    return syms


def test_library_exports_every_declared_symbol(lib):
    from sopht_gb300 import _lib
    declared = _header_symbols()
    assert len(declared) >= 25
    for name in declared:
        assert hasattr(lib, name), f"{name} declared in include/ but not exported"
    assert declared == set(_lib.declared_symbols()), "ctypes binding out of sync with the header"
    assert lib.sg_version() >= 100


def test_every_entry_names_what_it_replaces():
    """Each function the header declares is listed in tests/golden/c_entries.json with the reference
    interface it replaces (file:line) or the reason it has no counterpart, and nothing else is."""
    import json
    entries = json.loads((REPO / "tests" / "golden" / "c_entries.json").read_text())
    assert set(entries) == _header_symbols()
    for name, what in entries.items():
        assert re.search(r"\.py(:\d+)?|no reference counterpart|pyelastica", what), name


def test_argument_validation_without_gpu(lib):
    plan = ctypes.c_void_p()
    assert lib.sg_poisson_plan_create(4, 8, 8, 8, 1.0, 0, 1, ctypes.byref(plan)) == 1
    assert b"dim" in lib.sg_last_error()
    assert lib.sg_poisson_plan_create(2, 1, 8, 7, 1.0, 0, 1, ctypes.byref(plan)) == 2  # odd nx
    assert lib.sg_poisson_plan_create(2, 1, 8, 8, 1.0, 7, 1, ctypes.byref(plan)) == 1  # bad dtype
    assert lib.sg_poisson_plan_create(2, 1, 10, 22, 1.0, 0, 1, ctypes.byref(plan)) == 4  # nx = 2*11
    assert lib.sg_flow_plan_create(2, 1, 4, 4, 1.0, 0, 2, None, None, None, 0, 0, ctypes.byref(plan)) == 2
    assert lib.sg_ib_spread(0, 5, 1, 8, 8, 3, None, None, None, None, 0, None) == 1


def test_argument_validation_of_the_operator_entries(lib):
    """Each call fails a check that precedes every launch (the pointers are never dereferenced)."""
    a, b, c = 16, 32, 48  # distinct non-null placeholders
    assert lib.sg_elementwise(0, 9, 8, None, None, None, 0.0, 0.0, None) == 1  # unknown op
    assert lib.sg_elementwise(0, 3, 8, a, None, c, 0.0, 0.0, None) == 1  # sum without a second input
    assert lib.sg_elementwise(0, 2, -1, a, None, c, 0.0, 0.0, None) == 1  # negative count
    assert lib.sg_set_boundary_zone(0, 4, 1, 8, 8, 1, None, 0.0, None) == 1  # dim
    assert lib.sg_set_boundary_zone(0, 3, 8, 8, 8, 0, a, 0.0, None) == 1  # width 0
    assert lib.sg_set_boundary_zone(0, 3, 0, 8, 8, 1, a, 0.0, None) == 2  # empty extent
    assert lib.sg_set_boundary_zone(7, 3, 8, 8, 8, 1, a, 0.0, None) == 1  # dtype
    assert lib.sg_diffusion_flux(0, 5, 8, 8, 8, a, b, 0.1, 1, None) == 1  # dim
    assert lib.sg_diffusion_flux(7, 3, 8, 8, 8, a, b, 0.1, 1, None) == 1  # dtype
    assert lib.sg_diffusion_flux(0, 3, 8, 8, 8, a, a, 0.1, 1, None) == 1  # aliasing
    assert lib.sg_advection_eno3_flux_2d(0, 8, 8, a, b, None, 0.1, None) == 1  # no velocity
    assert lib.sg_advection_eno3_flux_3d(0, 8, 8, 8, a, b, None, 0.1, None) == 1
    assert lib.sg_advection_eno3_step_3d(0, 8, 8, 8, 0, a, b, c, 0.1, None) == 2  # no components
    assert lib.sg_passive_transport_step(0, 2, 1, 8, 8, 3, a, b, c, 0.1, 0.1, None) == 4  # 2D vector
    assert lib.sg_passive_transport_step(0, 3, 8, 8, 8, 2, a, b, c, 0.1, 0.1, None) == 1  # 2 components
    assert lib.sg_passive_transport_step(0, 4, 8, 8, 8, 1, a, b, c, 0.1, 0.1, None) == 1  # dim
    assert b"dim" in lib.sg_last_error()
    # the rod batch entries
    from sopht_gb300._lib import RodBatch
    rb = RodBatch()
    assert lib.sg_rod_batch_step(None, 1, 1e-5, 0.0, None) == 1
    rb.n_rods, rb.n_elems = 2, 0
    assert lib.sg_rod_batch_step(ctypes.byref(rb), 1, 1e-5, 0.0, None) == 2  # no elements
    rb.n_elems = 2000
    assert lib.sg_rod_batch_step(ctypes.byref(rb), 1, 1e-5, 0.0, None) == 2  # above 1024 elements
    rb.n_elems = 8
    assert lib.sg_rod_batch_step(ctypes.byref(rb), 1, 1e-5, 0.0, None) == 1  # null arrays
    for field in ("position", "velocity", "mass", "external_forces", "external_torques"):
        setattr(rb, field, a)
    assert lib.sg_rod_batch_element_markers(ctypes.byref(rb), 4, b, c, None) == 1  # dim
    assert lib.sg_rod_batch_element_markers(ctypes.byref(rb), 3, None, c, None) == 1  # no output
    assert lib.sg_rod_batch_element_loads(ctypes.byref(rb), 3, 7, b, None) == 1  # dtype
    assert lib.sg_rod_batch_element_loads(ctypes.byref(rb), 2, 0, None, None) == 1  # no forcing
    # the coupled sub-steps hold one element per thread: 1 to 256 elements per rod
    from sopht_gb300._lib import RodCoupling
    for field in ("directors", "omega", "rest_lengths", "shear_matrix", "mass_second_moment",
                  "inv_mass_second_moment", "rest_sigma", "rest_voronoi_lengths", "bend_matrix", "rest_kappa"):
        setattr(rb, field, a)
    cp = RodCoupling()
    rb.n_elems = 300
    assert lib.sg_rod_batch_coupled_substeps(ctypes.byref(rb), ctypes.byref(cp), None) == 2
    assert b"256" in lib.sg_last_error()
    rb.n_elems = 8
    assert lib.sg_rod_batch_coupled_substeps(ctypes.byref(rb), None, None) == 1  # no coupling


def _clamped_penalise(field, width, cx, cy, cz=None):
    """Penalisation as the fused kernels do it: gather from the clamped index, times factors."""
    def clamp(i, n):
        return np.clip(i, width - 1, n - width) if width > 0 else i

    if field.ndim == 2:
        ny, nx = field.shape
        yy, xx = np.meshgrid(clamp(np.arange(ny), ny), clamp(np.arange(nx), nx), indexing="ij")
        out = field[yy, xx] * cx[None, :]
        return out * cy[:, None]
    nz, ny, nx = field.shape
    zz, yy, xx = np.meshgrid(clamp(np.arange(nz), nz), clamp(np.arange(ny), ny), clamp(np.arange(nx), nx),
                             indexing="ij")
    out = field[zz, yy, xx] * cx[None, None, :]
    out = out * cy[None, :, None]
    return out * cz[:, None, None]


@pytest.mark.parametrize("width", [0, 2, 3, 4])
def test_penalise_as_clamped_gather(precision, width):
    from sopht_gb300.numeric.eulerian_grid_ops import penalisation_factors
    g = load_golden("stencils2d", precision)
    rt = real_t_of(precision)
    for tag in ("sq", "rect"):
        f = g[f"{tag}/field"]
        pos = g[f"{tag}/position"]
        dx = rt(1.0 / f.shape[1])
        ref = f.copy()
        st.penalise_2d(ref, width, dx, pos[0], pos[1])
        cx = penalisation_factors(width, dx, pos[0][0, :], rt)
        cy = penalisation_factors(width, dx, pos[1][:, 0], rt)
        np.testing.assert_array_equal(_clamped_penalise(f, width, cx, cy), ref)
    g3 = load_golden("stencils3d", precision)
    f = g3["rect/field"][0]
    pos = g3["rect/position"]
    dx = rt(1.0 / f.shape[2])
    ref = f.copy()
    st.penalise_3d(ref, width, dx, pos[0], pos[1], pos[2])
    cx = penalisation_factors(width, dx, pos[0][0, 0, :], rt)
    cy = penalisation_factors(width, dx, pos[1][0, :, 0], rt)
    cz = penalisation_factors(width, dx, pos[2][:, 0, 0], rt)
    np.testing.assert_array_equal(_clamped_penalise(f, width, cx, cy, cz), ref)


def _split_solve_2d(rhs, ny, nx, x_range):
    """Row R2C (implicit zero pad) -> column FFT * G_sym * IFFT, crop -> row C2R, crop."""
    g, dx = greens_function_2d(ny, nx, x_range, np.float64)
    ghat = np.fft.rfft2(g).real[: ny + 1, :] * dx**2 / (4 * ny * nx)
    a = np.fft.rfft(rhs, n=2 * nx, axis=1)                     # (ny, nx+1)
    b = np.fft.fft(a, n=2 * ny, axis=0)                        # (2ny, nx+1)
    ks = np.minimum(np.arange(2 * ny), 2 * ny - np.arange(2 * ny))
    b = b * ghat[ks, :]
    c = np.fft.ifft(b, axis=0)[:ny] * (2 * ny)                 # unnormalised inverse, crop
    return np.fft.irfft(c, n=2 * nx, axis=1)[:, :nx] * (2 * nx)


def _split_solve_3d(rhs, nz, ny, nx, x_range):
    g, dx = greens_function_3d(nz, ny, nx, x_range, np.float64)
    ghat = np.fft.rfftn(g).real[: nz + 1, : ny + 1, :] * dx**3 / (8 * nz * ny * nx)
    a = np.fft.rfft(rhs, n=2 * nx, axis=2)
    a = np.fft.fft(a, n=2 * ny, axis=1)
    a = np.fft.fft(a, n=2 * nz, axis=0)
    kz = np.minimum(np.arange(2 * nz), 2 * nz - np.arange(2 * nz))
    ky = np.minimum(np.arange(2 * ny), 2 * ny - np.arange(2 * ny))
    a = a * ghat[kz][:, ky, :]
    a = np.fft.ifft(a, axis=0)[:nz] * (2 * nz)
    a = np.fft.ifft(a, axis=1)[:, :ny] * (2 * ny)
    return np.fft.irfft(a, n=2 * nx, axis=2)[..., :nx] * (2 * nx)


def test_split_poisson_matches_doubled_box():
    rng = np.random.default_rng(5)
    for ny, nx, xr in ((12, 24, 1.0), (16, 16, 2.0), (6, 12, 1.0)):
        rhs = rng.standard_normal((ny, nx))
        ref = UnboundedPoisson2D(ny, nx, xr, np.float64).solve(rhs)
        np.testing.assert_allclose(_split_solve_2d(rhs, ny, nx, xr), ref, rtol=0, atol=1e-13)
    for nz, ny, nx in ((6, 8, 12), (8, 8, 8)):
        rhs = rng.standard_normal((nz, ny, nx))
        ref = UnboundedPoisson3D(nz, ny, nx, 1.0, np.float64).solve(rhs)
        np.testing.assert_allclose(_split_solve_3d(rhs, nz, ny, nx, 1.0), ref, rtol=0, atol=1e-13)


def test_ghat_is_real_and_symmetric():
    """The even-reflected Green's function has a real, even transform (table storage)."""
    g, _ = greens_function_3d(6, 8, 10, 1.0, np.float64)
    gh = np.fft.rfftn(g)
    assert np.abs(gh.imag).max() < 1e-12 * np.abs(gh.real).max()
    np.testing.assert_allclose(gh.real[1:6], gh.real[-1:-6:-1], rtol=1e-12, atol=1e-14)


def test_rod_element_kinematics_matches_numpy(lib):
    """The host-side element-centric rod kinematics against the grid's numpy formulas, bitwise, for
    contiguous node arrays and for rows strided inside a larger block; the staging slot gets both."""
    from sopht_gb300.simulator.immersed_body import _node_to_element_velocity
    rng = np.random.default_rng(6)
    n = 37
    block = rng.standard_normal((3, 3 * (n + 1)))
    cases = [(rng.standard_normal((3, n + 1)), rng.standard_normal((3, n + 1))),
             (block[:, n + 1: 2 * (n + 1)], block[:, 2 * (n + 1):])]
    mass = rng.random(n + 1) + 0.5
    for pos, vel in cases:
        for dim in (2, 3):
            po = np.empty((dim, n))
            vo = np.empty((dim, n))
            stage = np.full((2, dim, n), np.nan)
            st_ = lib.sg_rod_element_kinematics(dim, n, pos.ctypes.data, pos.strides[0] // 8, vel.ctypes.data,
                                                vel.strides[0] // 8, mass.ctypes.data, po.ctypes.data,
                                                vo.ctypes.data, stage.ctypes.data)
            assert st_ == 0
            ref_p = (pos[:dim, 1:] + pos[:dim, :-1]) / 2.0
            ref_v = _node_to_element_velocity(mass, vel)[:dim]
            np.testing.assert_array_equal(po, ref_p)
            np.testing.assert_array_equal(vo, ref_v)
            np.testing.assert_array_equal(stage[0], ref_p)
            np.testing.assert_array_equal(stage[1], ref_v)
    bad = lib.sg_rod_element_kinematics(3, n, cases[0][0].ctypes.data, n, cases[0][1].ctypes.data, n + 1,
                                        mass.ctypes.data, po.ctypes.data, vo.ctypes.data, None)
    assert bad == 1  # a row stride shorter than a row is rejected
