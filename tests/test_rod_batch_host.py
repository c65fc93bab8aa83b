"""The batched rod kernel's arithmetic, run on the host, against the numpy rod model.

``sopht_gb300/csrc/rod.cuh`` holds every pass of the batched Cosserat rod
kernel as host-and-device functions; ``tests/rod_host.cpp`` runs them in the
kernel's order on the host (built here with g++, no contraction of multiply-adds).
Three rods of one batch -- clamped and free, bent and twisted, with external
forces and torques and with damping -- are advanced for 300 sub-steps and
compared with ``oracle.rod.CosseratRod`` stepped one rod at a time: positions,
velocities, directors and angular velocities agree to 1e-10 of their scale
(8e-14 measured; the two sum in different orders, and a flipped twist term or a
dropped dilatation term moves them by 2e-2 to 3e-2).  The device launch itself
(one CTA per rod, barriers between passes) is exercised only on a GPU.
"""

from __future__ import annotations

import ctypes
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle.rod import CosseratRod, rotation_exp

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def host_lib(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    out = tmp_path_factory.mktemp("rodhost") / "librodhost.so"
    cmd = [gxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-ffp-contract=off", "-I", str(ROOT / "include"),
           str(ROOT / "tests" / "rod_host.cpp"), "-o", str(out)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    lib = ctypes.CDLL(str(out))
    from sopht_gb300._lib import RodBatch
    lib.rod_host_step.argtypes = [ctypes.POINTER(RodBatch), ctypes.c_int, ctypes.c_double, ctypes.c_double]
    lib.rod_host_step.restype = ctypes.c_int
    lib.rod_host_step_merged.argtypes = [ctypes.POINTER(RodBatch), ctypes.c_int, ctypes.c_double, ctypes.c_double]
    lib.rod_host_step_merged.restype = ctypes.c_int
    lib.rod_host_markers.argtypes = [ctypes.POINTER(RodBatch), ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lib.rod_host_loads.argtypes = [ctypes.POINTER(RodBatch), ctypes.c_int, ctypes.c_void_p]
    return lib


N = 16


def _rods():
    rng = np.random.default_rng(3)
    rods = []
    for i in range(3):
        rod = CosseratRod(N, start=[0.1 * i, 0.0, 0.0], direction=[0.0, 0.2 * i, 1.0], normal=[1.0, 0.0, 0.0],
                          length=0.5, radius=0.02 + 0.005 * i, density=1.0 + i, youngs_modulus=2e3)
        s = np.linspace(0.0, 0.5, N + 1)
        rod.position = rod.position + 0.01 * np.stack([np.sin(7 * s), np.cos(5 * s) - 1.0, 0.02 * s])
        centres = (np.arange(N) + 0.5) / N
        for e in range(N):
            rot = rotation_exp(np.array([[0.3 * centres[e]], [0.2 * i * centres[e]], [0.8 * centres[e]]]))[:, :, 0]
            rod.directors[:, :, e] = rot @ rod.directors[:, :, e]
        rod.velocity = 0.05 * rng.standard_normal(rod.velocity.shape)
        rod.omega = 0.5 * rng.standard_normal(rod.omega.shape)
        rod.external_forces = 1e-4 * rng.standard_normal(rod.external_forces.shape)
        rod.external_torques = 1e-6 * rng.standard_normal(rod.external_torques.shape)
        rod.rest_kappa = 0.1 * rng.standard_normal(rod.rest_kappa.shape)
        if i != 1:
            rod.clamp_start()
        rods.append(rod)
    return rods


def _batch(rods):
    keep = {}

    def stack(name, get=None, dtype=np.float64):
        arr = np.ascontiguousarray(np.stack([(get or (lambda r: getattr(r, name)))(r) for r in rods]), dtype=dtype)
        keep[name] = arr
        return arr.ctypes.data

    from sopht_gb300._lib import RodBatch
    b = RodBatch()
    b.n_rods, b.n_elems = len(rods), rods[0].n
    for field, attr in (("position", "position"), ("velocity", "velocity"), ("directors", "directors"),
                        ("omega", "omega"), ("mass", "mass"), ("rest_lengths", "rest_lengths"),
                        ("rest_voronoi_lengths", "rest_voronoi"), ("shear_matrix", "shear_matrix"),
                        ("bend_matrix", "bend_matrix"), ("mass_second_moment", "mass_second_moment"),
                        ("inv_mass_second_moment", "inv_mass_second_moment"), ("rest_sigma", "rest_sigma"),
                        ("rest_kappa", "rest_kappa"), ("external_forces", "external_forces"),
                        ("external_torques", "external_torques")):
        setattr(b, field, stack(attr))
    b.clamped = stack("clamped", lambda r: int(r.clamped is not None), np.int32)
    b.clamp_position = stack("clamp_x", lambda r: r.clamped[0] if r.clamped else np.zeros(3))
    b.clamp_directors = stack("clamp_q", lambda r: r.clamped[1] if r.clamped else np.eye(3))
    return b, keep


@pytest.mark.parametrize("damping", [0.0, 3.0])
def test_host_passes_match_the_rod_model(host_lib, damping):
    rods = _rods()
    b, arrays = _batch(rods)
    dt, steps = 2e-5, 300
    decay = float(np.exp(-damping * dt)) if damping else 1.0
    assert host_lib.rod_host_step(ctypes.byref(b), steps, dt, decay) == 0
    for r, rod in enumerate(rods):
        rod.damping_rate = damping
        for _ in range(steps):
            rod.step(dt)
        for name, ref in (("position", rod.position), ("velocity", rod.velocity), ("directors", rod.directors),
                          ("omega", rod.omega)):
            got = arrays[name][r]
            scale = max(np.abs(ref).max(), 1e-30)
            assert np.abs(got - ref).max() <= 1e-10 * scale, (r, name, np.abs(got - ref).max() / scale)
    # the rods moved, and the clamped ones kept their base
    assert np.abs(arrays["velocity"]).max() > 1e-3
    for r, rod in enumerate(rods):
        if rod.clamped is not None:
            np.testing.assert_array_equal(arrays["position"][r][:, 0], rod.clamped[0])


@pytest.mark.parametrize("damping", [0.0, 3.0])
def test_merged_half_drifts_are_bitwise_the_two_half_drifts(host_lib, damping):
    """The coupled kernel takes the closing half drift of a sub-step and the opening one of the next
    in one pass (drift_node_twice, rotate_element_twice: one rotation exponential applied twice);
    over 300 sub-steps of bent, twisted, clamped and free rods that gives the bits of the plain
    sequence."""
    dt, steps = 2e-5, 300
    decay = float(np.exp(-damping * dt)) if damping else 1.0
    b1, a1 = _batch(_rods())
    b2, a2 = _batch(_rods())
    assert host_lib.rod_host_step(ctypes.byref(b1), steps, dt, decay) == 0
    assert host_lib.rod_host_step_merged(ctypes.byref(b2), steps, dt, decay) == 0
    for name in ("position", "velocity", "directors", "omega"):
        np.testing.assert_array_equal(a1[name], a2[name])
    assert np.abs(a1["velocity"]).max() > 1e-3


@pytest.mark.parametrize("n", [1, 2])
def test_host_passes_short_rods(host_lib, n):
    """One element (no Voronoi region) and two elements (one), free and clamped."""
    rng = np.random.default_rng(n)
    rods = []
    for clamp in (False, True):
        rod = CosseratRod(n, start=[0.0, 0.0, 0.0], direction=[0.1, 0.0, 1.0], normal=[1.0, 0.0, 0.0],
                          length=0.1 * n, radius=0.02, density=1.0, youngs_modulus=1e3)
        rod.velocity = 0.05 * rng.standard_normal(rod.velocity.shape)
        rod.omega = 0.5 * rng.standard_normal(rod.omega.shape)
        rod.external_forces = 1e-4 * rng.standard_normal(rod.external_forces.shape)
        if clamp:
            rod.clamp_start()
        rods.append(rod)
    b, arrays = _batch(rods)
    assert host_lib.rod_host_step(ctypes.byref(b), 200, 1e-5, 1.0) == 0
    for r, rod in enumerate(rods):
        for _ in range(200):
            rod.step(1e-5)
        for name, ref in (("position", rod.position), ("velocity", rod.velocity),
                          ("directors", rod.directors), ("omega", rod.omega)):
            scale = max(np.abs(ref).max(), 1e-30)
            assert np.abs(arrays[name][r] - ref).max() <= 1e-10 * scale, (n, r, name)


class _PyelasticaNamed:
    """An oracle rod seen through pyelastica's CosseratRod attribute names."""

    def __init__(self, rod):
        self.n_elems = rod.n
        self.position_collection, self.velocity_collection = rod.position, rod.velocity
        self.director_collection, self.omega_collection = rod.directors, rod.omega
        self.mass, self.rest_lengths, self.rest_voronoi_lengths = rod.mass, rod.rest_lengths, rod.rest_voronoi
        self.shear_matrix, self.bend_matrix = rod.shear_matrix, rod.bend_matrix
        self.mass_second_moment_of_inertia = rod.mass_second_moment
        self.inv_mass_second_moment_of_inertia = rod.inv_mass_second_moment
        self.rest_sigma, self.rest_kappa = rod.rest_sigma, rod.rest_kappa
        self.external_forces, self.external_torques = rod.external_forces, rod.external_torques


def test_rod_batch_layout_without_a_gpu():
    """CosseratRodBatch gathers the rods into the sg_rod_batch layout (checked on CPU tensors; its
    step needs a CUDA device and says so)."""
    import sopht_gb300.simulator as sps
    rods = _rods()
    named = [_PyelasticaNamed(r) for r in rods]
    batch = sps.CosseratRodBatch(named, clamped=[r.clamped is not None for r in rods], device="cpu")
    assert (batch.n_rods, batch.n_elems) == (3, N)
    for field in ("position", "velocity", "directors", "omega", "mass", "rest_lengths", "rest_voronoi_lengths",
                  "shear_matrix", "bend_matrix", "mass_second_moment", "inv_mass_second_moment", "rest_sigma",
                  "rest_kappa", "external_forces", "external_torques"):
        assert getattr(batch._batch, field)  # a pointer into the batch's own tensors
    np.testing.assert_array_equal(batch.arrays["director_collection"].numpy(), np.stack([r.directors for r in rods]))
    np.testing.assert_array_equal(batch.clamped.numpy(), [1, 0, 1])
    np.testing.assert_array_equal(batch.clamp_position.numpy()[0], rods[0].clamped[0])
    with pytest.raises(RuntimeError, match="CUDA device"):
        batch.step(1e-5)
    # the state goes back into the rods
    for r in named:
        r.velocity_collection[...] = 0.0
    batch.download_into(named)
    np.testing.assert_array_equal(named[2].velocity_collection, batch.arrays["velocity_collection"][2].numpy())
    with pytest.raises(ValueError, match="same number of elements"):
        sps.CosseratRodBatch([named[0], _PyelasticaNamed(CosseratRod(3, [0, 0, 0], [0, 0, 1], [1, 0, 0], 1.0,
                                                                     0.1, 1.0, 1e3))], device="cpu")


def test_rod_batch_marker_arrays_are_checked_before_any_launch():
    """The marker and forcing arrays go to the native entries as raw pointers, so their dtype, shape,
    layout and device are checked in Python (ValueError) before the CUDA requirement (RuntimeError)."""
    import torch

    import sopht_gb300.simulator as sps
    rods = _rods()
    batch = sps.CosseratRodBatch([_PyelasticaNamed(r) for r in rods], device="cpu")
    m = len(rods) * N
    good = torch.zeros((3, m), dtype=torch.float64)
    bad = {
        "float32 position": (torch.zeros((3, m), dtype=torch.float32), good),
        "short position": (torch.zeros((3, m - 1), dtype=torch.float64), good),
        "2D-shaped position for dim 3": (torch.zeros((2, m), dtype=torch.float64), good),
        "strided velocity": (good, torch.zeros((m, 3), dtype=torch.float64).t()),
        "numpy velocity": (good, np.zeros((3, m))),
    }
    for what, (pos, vel) in bad.items():
        with pytest.raises(ValueError):
            batch.element_markers(pos, vel, dim=3)
        assert what
    with pytest.raises(ValueError, match="dim"):
        batch.element_markers(good, good, dim=4)
    with pytest.raises(RuntimeError, match="CUDA device"):
        batch.element_markers(good, good.clone(), dim=3)
    for forcing in (torch.zeros((3, m), dtype=torch.float16), torch.zeros((3, m + 1)), torch.zeros((2, m)),
                    torch.zeros((3, m), dtype=torch.int64)):
        with pytest.raises(ValueError):
            batch.set_element_loads(forcing, dim=3)
    with pytest.raises(RuntimeError, match="CUDA device"):
        batch.set_element_loads(torch.zeros((2, m), dtype=torch.float32), dim=2)
    if torch.cuda.is_available():  # a tensor on another device than the batch's
        with pytest.raises(ValueError, match="lives on"):
            batch.set_element_loads(torch.zeros((3, m), device="cuda"), dim=3)


@pytest.mark.parametrize("dim", [2, 3])
def test_host_element_markers_and_loads_match_the_forcing_grid(host_lib, dim):
    """The batch's element-centric markers and reaction loads (rod.cuh) against the forcing grid's
    numpy formulas (cosserat_rod_forcing_grids.py:82-130), bitwise."""
    from sopht_gb300.simulator.immersed_body import _node_to_element_velocity
    rods = _rods()
    b, arrays = _batch(rods)
    n_markers = len(rods) * N
    pos, vel = np.zeros((dim, n_markers)), np.zeros((dim, n_markers))
    assert host_lib.rod_host_markers(ctypes.byref(b), dim, pos.ctypes.data, vel.ctypes.data) == 0
    for r, rod in enumerate(rods):
        p = rod.position
        np.testing.assert_array_equal(pos[:, r * N:(r + 1) * N], ((p[:dim, 1:] + p[:dim, :-1]) / 2.0))
        np.testing.assert_array_equal(vel[:, r * N:(r + 1) * N],
                                      _node_to_element_velocity(rod.mass, rod.velocity)[:dim])
    forcing = np.random.default_rng(7).standard_normal((dim, n_markers))
    assert host_lib.rod_host_loads(ctypes.byref(b), dim, forcing.ctypes.data) == 0
    for r in range(len(rods)):
        f = forcing[:, r * N:(r + 1) * N]
        ref = np.zeros((3, N + 1))
        ref[:dim, 1:] -= 0.5 * f
        ref[:dim, :-1] -= 0.5 * f
        np.testing.assert_array_equal(arrays["external_forces"][r], ref)
        assert not arrays["external_torques"][r].any()
