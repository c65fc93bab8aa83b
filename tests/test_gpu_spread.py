"""The sorted spreading (``sg_ib_spread_sorted``) against the owner-scan spreading and the oracle.

Both kernels add each cell's contributions in ascending marker order, so their sums must agree to
the bit; the sorted one is the path ``VirtualBoundaryForcing`` takes from
``SORTED_SPREAD_MIN_MARKERS`` markers on, where the owner scan grows quadratically.  The second test
spreads a Cosserat rod's capped surface grid of more than 10 000 markers and compares it with the
numpy oracle of the reference's serial spreading loop.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _lib():
    from sopht_gb300 import _lib as L
    from sopht_gb300.build import build
    build()
    L.load()
    return L


@pytest.mark.parametrize("dim,dtype,reset", [(2, np.float64, 0), (3, np.float32, 1), (3, np.float64, 0),
                                             (2, np.float32, 1)])
def test_sorted_spread_is_bitwise_the_owner_scan(dim, dtype, reset):
    L = _lib()
    rng = np.random.default_rng(dim * 10 + reset)
    grid = (24, 20, 28)[3 - dim:]
    n = 900
    cells = 4 ** dim
    # markers crowded into a small box so that many share cells; one marker's window leaves the grid
    lo = np.array(grid[::-1]) // 3
    nearest = np.stack([rng.integers(lo[d], lo[d] + 6, n) for d in range(dim)]).astype(np.int32)
    nearest[0, 5] = 0
    weights = rng.standard_normal((cells, n)).astype(dtype)
    forcing = rng.standard_normal((dim, n)).astype(dtype)
    base = rng.standard_normal((dim, *grid)).astype(dtype)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    near_d, w_d, f_d = dev(nearest), dev(weights), dev(forcing)
    out_scan, out_sort = dev(base), dev(base)
    nz, ny, nx = (1, *grid) if dim == 2 else grid
    sg = L.SG_F32 if dtype == np.float32 else L.SG_F64
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    L.call("sg_ib_spread", sg, dim, nz, ny, nx, n, near_d.data_ptr(), w_d.data_ptr(), f_d.data_ptr(),
           out_scan.data_ptr(), reset, s)
    nbytes = int(L.load().sg_ib_spread_sorted_scratch_bytes(dim, nz, ny, nx, n))
    assert nbytes > 0
    scratch = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    for _ in range(2):  # the scratch is reused: a second call gives the same bits
        out = dev(base)
        L.call("sg_ib_spread_sorted", sg, dim, nz, ny, nx, n, near_d.data_ptr(), w_d.data_ptr(), f_d.data_ptr(),
               out.data_ptr(), reset, scratch.data_ptr(), nbytes, s)
        torch.cuda.synchronize()
        assert torch.equal(out, out_scan)
    with pytest.raises(ValueError, match="scratch"):
        L.call("sg_ib_spread_sorted", sg, dim, nz, ny, nx, n, near_d.data_ptr(), w_d.data_ptr(), f_d.data_ptr(),
               out_sort.data_ptr(), reset, scratch.data_ptr(), nbytes - 1, s)


def test_surface_grid_of_ten_thousand_markers_vs_oracle():
    """A rod's capped surface grid (> 10 000 markers) through VirtualBoundaryForcing, which takes the
    sorted spreading at this size, against the oracle's interaction and serial spreading (FP64)."""
    import sopht_gb300.simulator as sps
    from oracle.ib import VirtualBoundaryForcingOracle
    from sopht_gb300.numeric import VirtualBoundaryForcing
    _lib()
    n = 48
    dx = 1.0 / n
    rod = sps.StraightRod(40, [0.25, 0.5, 0.2], [0.3, 0.0, 1.0], [0.0, 1.0, 0.0], 0.55, 0.12, 1.0, 1e4)
    rod.radius = np.full(40, 0.12)
    fg = sps.CosseratRodSurfaceForcingGrid(3, rod, surface_grid_density_for_largest_element=240, with_cap=True)
    m = fg.num_lag_nodes
    assert m > 10_000
    pos, vel = fg.position_field, fg.velocity_field
    rng = np.random.default_rng(4)
    u = rng.standard_normal((3, n, n, n))
    xi = 1e-3 * rng.standard_normal((3, m))
    vbf = VirtualBoundaryForcing(-2e4, -1e2, 3, dx, m, np.float64, enable_eul_grid_forcing_reset=True)
    assert m >= vbf.SORTED_SPREAD_MIN_MARKERS
    vbf.lag_grid_position_mismatch_field.copy_(torch.from_numpy(xi))
    f = torch.full((3, n, n, n), 3.0, dtype=torch.float64, device="cuda")
    vbf.compute_interaction_forcing(f, torch.from_numpy(u).cuda(), pos, vel)
    vbf.check_markers_in_domain()
    ora = VirtualBoundaryForcingOracle(-2e4, -1e2, 3, dx, m, np.float64, enable_eul_grid_forcing_reset=True)
    ora.lag_grid_position_mismatch_field[...] = xi
    f_o = np.full((3, n, n, n), 3.0)
    ora.compute_interaction_forcing(f_o, u, pos, vel)
    lag = vbf.lag_grid_forcing_field.cpu().numpy()
    np.testing.assert_allclose(lag, ora.lag_grid_forcing_field, rtol=1e-10, atol=1e-10 * np.abs(lag).max())
    got = f.cpu().numpy()
    assert np.abs(got - f_o).max() <= 1e-12 * np.abs(f_o).max()
