"""GPU parity of the lower-level factories: elementwise operations and the flux-form stencils.

Against the fixtures made by running the reference (the ENO3 and diffusion flux forms
and the vector add-fixed-value of ``golden_stencils2d_*``) at 1e3 eps absolute, and
against numpy / the oracle elsewhere: exact for set, copy, sum and add; 1e3 eps for
the products.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch
from conftest import load_golden, real_t_of, ref_tol

from oracle import stencils as st

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from sopht_gb300 import _lib
    from sopht_gb300.build import build
    build()
    _lib.load()
    assert torch.cuda.is_available()


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("tag", ["sq", "rect"])
def test_flux_forms_2d_vs_reference(precision, tag):
    from sopht_gb300.numeric import eulerian_grid_ops as ops
    g = load_golden("stencils2d", precision)
    rt = real_t_of(precision)
    tol = ref_tol(precision)
    f, v = g[f"{tag}/field"], g[f"{tag}/velocity"]
    flux = torch.zeros_like(dev(f))
    ops.gen_advection_flux_conservative_eno3_pyst_kernel_2d(real_t=rt)(
        advection_flux=flux, field=dev(f), velocity=dev(v), inv_dx=rt(0.1))
    np.testing.assert_allclose(host(flux), g[f"{tag}/eno3_flux"], atol=tol)
    # the flux form accumulates into whatever the buffer holds
    base = np.random.default_rng(1).standard_normal(f.shape).astype(rt)
    flux = dev(base)
    ops.gen_advection_flux_conservative_eno3_pyst_kernel_2d(real_t=rt)(
        advection_flux=flux, field=dev(f), velocity=dev(v), inv_dx=rt(0.1))
    np.testing.assert_allclose(host(flux), base + st.eno3_flux_2d(f, v, rt(0.1)), atol=tol)
    # diffusion flux: the fixture started from a garbage buffer, so its ring must read 0
    dflux = torch.from_numpy(np.random.default_rng(2).standard_normal(f.shape).astype(rt)).cuda()
    ops.gen_diffusion_flux_pyst_kernel_2d(real_t=rt)(diffusion_flux=dflux, field=dev(f), prefactor=rt(0.1))
    np.testing.assert_allclose(host(dflux), g[f"{tag}/diffusion_flux"], atol=tol)
    keep = torch.full_like(dflux, 7.0)
    ops.gen_diffusion_flux_pyst_kernel_2d(real_t=rt, reset_ghost_zone=False)(
        diffusion_flux=keep, field=dev(f), prefactor=rt(0.1))
    out = host(keep)
    np.testing.assert_allclose(out[1:-1, 1:-1], g[f"{tag}/diffusion_flux"][1:-1, 1:-1], atol=tol)
    assert (out[0] == 7.0).all() and (out[:, -1] == 7.0).all()
    # add a fixed value per component (elementwise_ops_2d.py:256-313)
    out = dev(v)
    ops.gen_add_fixed_val_pyst_kernel_2d(real_t=rt, field_type="vector")(
        sum_field=out, vector_field=out, fixed_vals=[1.5, -0.25])
    np.testing.assert_allclose(host(out), g[f"{tag}/add_fixed_val"], atol=tol)


@pytest.mark.parametrize("ftype", ["scalar", "vector"])
def test_diffusion_flux_3d_vs_oracle(precision, ftype):
    from sopht_gb300.numeric import eulerian_grid_ops as ops
    rt = real_t_of(precision)
    rng = np.random.default_rng(3)
    shape = (10, 12, 14)
    f = rng.standard_normal((3, *shape) if ftype == "vector" else shape).astype(rt)
    flux = dev(rng.standard_normal(f.shape).astype(rt))
    kern = ops.gen_diffusion_flux_pyst_kernel_3d(real_t=rt, field_type=ftype)
    if ftype == "vector":
        kern(vector_field_diffusion_flux=flux, vector_field=dev(f), prefactor=rt(0.2))
    else:
        kern(diffusion_flux=flux, field=dev(f), prefactor=rt(0.2))
    comps = f.reshape(-1, *shape)
    ref = np.zeros_like(comps)
    for c in range(comps.shape[0]):
        tmp = comps[c:c + 1].copy()
        st.diffusion_step_3d(tmp, rt(0.2))  # field + flux on the interior, field on the ring
        ref[c] = tmp[0] - comps[c]
        ref[c][0], ref[c][-1], ref[c][:, 0], ref[c][:, -1], ref[c][:, :, 0], ref[c][:, :, -1] = 0, 0, 0, 0, 0, 0
    np.testing.assert_allclose(host(flux).reshape(ref.shape), ref, atol=ref_tol(precision))


@pytest.mark.parametrize("dim", [2, 3])
def test_elementwise_ops_vs_numpy(precision, dim):
    from sopht_gb300.numeric import eulerian_grid_ops as ops
    rt = real_t_of(precision)
    tol = ref_tol(precision)
    rng = np.random.default_rng(dim)
    shape = (12, 20) if dim == 2 else (6, 8, 10)
    a = rng.standard_normal(shape).astype(rt)
    b = rng.standard_normal(shape).astype(rt)
    v = rng.standard_normal((dim, *shape)).astype(rt)
    sfx = f"_{dim}d"
    get = lambda name: getattr(ops, name.replace("_2d", sfx))  # noqa: E731
    out = torch.empty_like(dev(a))
    get("gen_elementwise_sum_pyst_kernel_2d")(real_t=rt)(sum_field=out, field_1=dev(a), field_2=dev(b))
    np.testing.assert_array_equal(host(out), a + b)
    get("gen_elementwise_saxpby_pyst_kernel_2d")(real_t=rt)(
        sum_field=out, field_1=dev(a), field_2=dev(b), field_1_prefac=0.3, field_2_prefac=-1.7)
    np.testing.assert_allclose(host(out), rt(0.3) * a + rt(-1.7) * b, atol=tol)
    get("gen_elementwise_copy_pyst_kernel_2d")(real_t=rt)(field=out, rhs_field=dev(b))
    np.testing.assert_array_equal(host(out), b)
    get("gen_set_fixed_val_pyst_kernel_2d")(real_t=rt)(field=out, fixed_val=2.5)
    assert (host(out) == rt(2.5)).all()
    vo = dev(v)
    get("gen_set_fixed_val_pyst_kernel_2d")(real_t=rt, field_type="vector")(
        vector_field=vo, fixed_vals=[1.0, -2.0, 3.0][:dim])
    for c in range(dim):
        assert (host(vo[c]) == rt([1.0, -2.0, 3.0][c])).all()
    get("gen_add_fixed_val_pyst_kernel_2d")(real_t=rt)(sum_field=out, field=dev(a), fixed_val=0.75)
    np.testing.assert_array_equal(host(out), a + rt(0.75))
    ca = (a + 1j * b).astype(np.complex64 if rt == np.float32 else np.complex128)
    cb = (b - 0.5j * a).astype(ca.dtype)
    cp = torch.empty_like(dev(ca))
    get("gen_elementwise_complex_product_pyst_kernel_2d")(real_t=rt)(product_field=cp, field_1=dev(ca),
                                                                     field_2=dev(cb))
    np.testing.assert_allclose(host(cp), ca * cb, atol=4 * tol)
    # boundary band: scalar and per component, width 2
    band = dev(a)
    get("gen_set_fixed_val_at_boundaries_pyst_kernel_2d")(real_t=rt, width=2)(field=band, fixed_val=-1.0)
    ref = a.copy()
    for axis in range(dim):
        sl = [slice(None)] * dim
        sl[axis] = slice(0, 2)
        ref[tuple(sl)] = -1.0
        sl[axis] = slice(-2, None)
        ref[tuple(sl)] = -1.0
    np.testing.assert_array_equal(host(band), ref)
    vb = dev(v)
    get("gen_set_fixed_val_at_boundaries_pyst_kernel_2d")(real_t=rt, width=1, field_type="vector")(
        vector_field=vb, fixed_vals=[0.0] * dim)
    got = host(vb)
    for c in range(dim):
        inner = tuple([c] + [slice(1, -1)] * dim)
        np.testing.assert_array_equal(got[inner], v[inner])
        assert got[c].sum() == pytest.approx(v[inner].sum(), rel=1e-5)


def test_factory_argument_errors():
    from sopht_gb300.numeric import eulerian_grid_ops as ops
    with pytest.raises(ValueError, match="width"):
        ops.gen_set_fixed_val_at_boundaries_pyst_kernel_2d(real_t=np.float32, width=0)
    with pytest.raises(ValueError):
        ops.gen_elementwise_sum_pyst_kernel_3d(real_t=np.float32, field_type="tensor")
    k = ops.gen_elementwise_copy_pyst_kernel_2d(real_t=np.float32)
    base = torch.zeros((8, 8), device="cuda")
    with pytest.raises(ValueError, match="contiguous"):
        k(field=base[:, ::2], rhs_field=torch.zeros((8, 4), device="cuda"))
