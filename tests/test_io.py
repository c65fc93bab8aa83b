"""HDF5 + XDMF field IO and restart against the reference's IO.

h5py is not installed here or on the GPU machines, so both the reference's IO
(when the fixtures were made) and this package's IO run against the
in-memory h5py stand-in ``tests/golden/memory_h5.py``.  The fixtures
``golden_io_*`` hold the tree of datasets and attributes the reference wrote
for three cases (3D fields with two Lagrangian grids, a 2D simulator grid, a
rod) and its XDMF text.  Checked: the same tree with the same dtypes and
values (exact), XDMF files with the same elements, attributes and values
(whitespace and float formatting aside), loading the reference's files back
into numpy arrays and torch tensors in place, the reference's error cases, and
``restart_simulation`` with a stand-in for pyelastica's ``load_state``.
"""

from __future__ import annotations

import sys
import types
import xml.etree.ElementTree as ET

import numpy as np
import pytest
import torch
from conftest import GOLDEN, load_golden

sys.path.insert(0, str(GOLDEN))
import memory_h5  # noqa: E402

import sopht_gb300.utils as spu  # noqa: E402


@pytest.fixture(autouse=True)
def _h5(monkeypatch, tmp_path):
    monkeypatch.setitem(sys.modules, "h5py", memory_h5)
    monkeypatch.chdir(tmp_path)


def _same_tree(got: dict, ref: dict) -> None:
    assert sorted(got) == sorted(ref)
    for key, value in ref.items():
        assert got[key].dtype == value.dtype, key
        np.testing.assert_array_equal(got[key], value, err_msg=key)


def _norm(text, digits):
    words = (text or "").split()
    try:
        return [round(float(w), digits) for w in words]
    except ValueError:
        return words


def _same_xdmf(got_text: str, ref_text: str, digits: int) -> None:
    a, b = ET.fromstring(got_text), ET.fromstring(ref_text)

    def walk(x, y, path):
        assert x.tag == y.tag, path
        assert sorted(x.attrib) == sorted(y.attrib), (path, x.attrib, y.attrib)
        for k in x.attrib:
            assert _norm(x.attrib[k], digits) == _norm(y.attrib[k], digits), (path, k)
        assert _norm(x.text, digits) == _norm(y.text, digits), (path, x.text, y.text)
        assert len(x) == len(y), path
        for i, (cx, cy) in enumerate(zip(x, y)):
            walk(cx, cy, f"{path}/{cx.tag}[{i}]")

    walk(a, b, a.tag)
    assert got_text.startswith('<?xml version="1.0" ?>\n<!DOCTYPE Xdmf SYSTEM "Xdmf.dtd" []>')


def _ref(g, case):
    pre = f"{case}/h5/"
    return {k[len(pre):]: v for k, v in g.items() if k.startswith(pre)}


def _save_3d(g, real_t, as_tensor=False):
    conv = (lambda a: torch.from_numpy(a.copy())) if as_tensor else (lambda a: a.copy())
    io = spu.IO(dim=3, real_dtype=real_t)
    io.define_eulerian_grid(origin=np.array([0.1, 0.2, 0.3]), dx=np.array([0.05, 0.05, 0.05]),
                            grid_size=np.array([8, 10, 12]))
    eul = {k: conv(g[f"eul3d/in/{k}"]) for k in ("vorticity_mag", "velocity")}
    io.add_as_eulerian_fields_for_io(**eul)
    lag = {k: conv(g[f"eul3d/in/{k}"]) for k in ("sphere_grid", "radius_field", "forcing", "rod_grid",
                                                  "rod_velocity")}
    io.add_as_lagrangian_fields_for_io(lagrangian_grid=lag["sphere_grid"], lagrangian_grid_name="sphere",
                                       radius_field=lag["radius_field"], forcing=lag["forcing"])
    io.add_as_lagrangian_fields_for_io(lagrangian_grid=lag["rod_grid"], lagrangian_grid_connect=True,
                                       rod_velocity=lag["rod_velocity"])
    io.save(h5_file_name="sopht_0003.h5", time=0.125)
    return io, eul, lag


@pytest.mark.parametrize("precision", ["single", "double"])
@pytest.mark.parametrize("as_tensor", [False, True])
def test_3d_fields_and_lagrangian_grids_like_reference(precision, as_tensor):
    g = load_golden("io", precision)
    real_t = np.float32 if precision == "single" else np.float64
    io, _, _ = _save_3d(g, real_t, as_tensor)
    _same_tree(memory_h5.dump("sopht_0003.h5"), _ref(g, "eul3d"))
    for name in ("eulerian", "sphere", "Lagrangian_grid_0"):
        with open(f"sopht_0003_{name}.xmf") as fh:
            _same_xdmf(fh.read(), str(g[f"eul3d/xmf/{name}"]), io.precision)


@pytest.mark.parametrize("precision", ["single", "double"])
def test_2d_simulator_grid_like_reference(precision):
    g = load_golden("io", precision)
    fields = {"vorticity": g["eul2d/in/vorticity"], "velocity": torch.from_numpy(g["eul2d/in/velocity"].copy())}
    io = spu.EulerianFieldIO(position_field=g["eul2d/in/position"], eulerian_fields_dict=fields)
    assert io.precision == 16  # decided on the position field's dtype object, as the reference does
    io.save(h5_file_name="flow_0001.h5", time=2.5)
    _same_tree(memory_h5.dump("flow_0001.h5"), _ref(g, "eul2d"))
    with open("flow_0001_eulerian.xmf") as fh:
        _same_xdmf(fh.read(), str(g["eul2d/xmf/eulerian"]), 16)


@pytest.mark.parametrize("precision", ["single", "double"])
def test_rod_like_reference(precision):
    g = load_golden("io", precision)
    real_t = np.float32 if precision == "single" else np.float64
    p = g["rod/in/position_collection"]
    rod = types.SimpleNamespace(n_elems=p.shape[1] - 1, position_collection=p - 0.01, radius=g["rod/in/radius"])
    io = spu.CosseratRodIO(cosserat_rod=rod, dim=3, real_dtype=real_t)
    rod.position_collection += 0.01  # save reads the rod as it is then
    io.save(h5_file_name="rod_0007.h5", time=1.0)
    _same_tree(memory_h5.dump("rod_0007.h5"), _ref(g, "rod"))
    with open("rod_0007_rod.xmf") as fh:
        _same_xdmf(fh.read(), str(g["rod/xmf/rod"]), io.precision)


@pytest.mark.parametrize("as_tensor", [False, True])
def test_load_reference_file_in_place(as_tensor):
    g = load_golden("io", "single")
    memory_h5.restore("sopht_0003.h5", _ref(g, "eul3d"))
    zeros = (lambda a: torch.zeros(a.shape, dtype=torch.from_numpy(a).dtype)) if as_tensor else np.zeros_like
    io = spu.IO(dim=3, real_dtype=np.float32)
    io.define_eulerian_grid(origin=np.array([0.1, 0.2, 0.3]), dx=np.array([0.05, 0.05, 0.05]),
                            grid_size=np.array([8, 10, 12]))
    eul = {k: zeros(g[f"eul3d/in/{k}"]) for k in ("vorticity_mag", "velocity")}
    lag = {k: zeros(g[f"eul3d/in/{k}"]) for k in ("sphere_grid", "radius_field", "forcing", "rod_grid",
                                                   "rod_velocity")}
    io.add_as_eulerian_fields_for_io(**eul)
    io.add_as_lagrangian_fields_for_io(lagrangian_grid=lag["sphere_grid"], lagrangian_grid_name="sphere",
                                       radius_field=lag["radius_field"], forcing=lag["forcing"])
    io.add_as_lagrangian_fields_for_io(lagrangian_grid=lag["rod_grid"], lagrangian_grid_connect=True,
                                       rod_velocity=lag["rod_velocity"])
    kept = {k: v for k, v in {**eul, **lag}.items()}
    assert io.load(h5_file_name="sopht_0003.h5") == 0.125
    for k, v in kept.items():
        assert v is (eul | lag)[k]  # filled in place
        got = v.numpy() if as_tensor else v
        np.testing.assert_array_equal(got, g[f"eul3d/in/{k}"], err_msg=k)
    np.testing.assert_array_equal(io.lagrangian_grid_connection["Lagrangian_grid_0"], np.arange(7))


def test_round_trip_and_restart_consistency():
    g = load_golden("io", "double")
    io, eul, lag = _save_3d(g, np.float64)
    for v in (*eul.values(), *lag.values()):
        v[...] = 0.0
    assert io.load("sopht_0003.h5") == 0.125
    np.testing.assert_array_equal(eul["velocity"], g["eul3d/in/velocity"])
    np.testing.assert_array_equal(lag["forcing"], g["eul3d/in/forcing"])
    io.eulerian_dx = np.array([0.05, 0.05, 0.06])
    with pytest.raises(ValueError, match="Eulerian dx does not match loaded file!"):
        io.load("sopht_0003.h5")
    io.eulerian_dx = np.array([0.05, 0.05, 0.05])
    io.eulerian_origin = np.array([0.0, 0.2, 0.3])
    with pytest.raises(ValueError, match="Eulerian origin does not match loaded file!"):
        io.load("sopht_0003.h5")


def test_registration_and_load_errors():
    with pytest.raises(ValueError, match="Invalid dimension"):
        spu.IO(dim=4)
    io = spu.IO(dim=2)
    with pytest.raises(ValueError, match="Eulerian mesh is not defined!"):
        io.add_as_eulerian_fields_for_io(w=np.zeros((4, 4)))
    with pytest.raises(TypeError, match="Invalid input types"):
        io.define_eulerian_grid(origin=[0.0, 0.0], dx=np.ones(2), grid_size=np.array([4, 4]))
    io.define_eulerian_grid(origin=np.zeros(2), dx=np.ones(2), grid_size=np.array([4, 6]))
    with pytest.raises(ValueError, match="Unable to identify eulerian field type"):
        io.add_as_eulerian_fields_for_io(w=np.zeros((4, 5)))
    with pytest.raises(ValueError, match="lagrangian grid has to be a 2D"):
        io.add_as_lagrangian_fields_for_io(lagrangian_grid=np.zeros(5))
    with pytest.raises(ValueError, match="Invalid lagrangian grid dimension"):
        io.add_as_lagrangian_fields_for_io(lagrangian_grid=np.zeros((3, 5)))
    with pytest.raises(ValueError, match="Unable to identify lagrangian field type"):
        io.add_as_lagrangian_fields_for_io(lagrangian_grid=np.zeros((2, 5)), f=np.zeros((3, 2)))
    # a file without the registered field
    io = spu.IO(dim=2)
    io.define_eulerian_grid(origin=np.zeros(2), dx=np.ones(2), grid_size=np.array([4, 6]))
    io.add_as_eulerian_fields_for_io(w=np.ones((4, 6)))
    io.save("a.h5", time=1.0)
    other = spu.IO(dim=2)
    other.define_eulerian_grid(origin=np.zeros(2), dx=np.ones(2), grid_size=np.array([4, 6]))
    other.add_as_eulerian_fields_for_io(u=np.zeros((2, 4, 6)))
    with pytest.raises(ValueError, match="Unable to find vector field u_0"):
        other.load("a.h5")
    lag_only = spu.IO(dim=2)
    lag_only.add_as_lagrangian_fields_for_io(lagrangian_grid=np.zeros((2, 3)), lagrangian_grid_name="body",
                                             s=np.zeros(3))
    with pytest.raises(ValueError, match="Unable to find grid 'body'"):
        lag_only.load("a.h5")


def test_restart_simulation_picks_latest(monkeypatch):
    def make(path, t):
        io = spu.IO(dim=2)
        io.define_eulerian_grid(origin=np.zeros(2), dx=np.ones(2), grid_size=np.array([3, 4]))
        io.add_as_eulerian_fields_for_io(w=np.full((3, 4), t))
        io.save(path, time=t)
        return io

    for n, t in ((2, 0.5), (11, 2.75)):
        for stem in ("sopht", "rod", "forcing_grid"):
            make(f"{stem}_{n:04d}.h5", t)
    fields = [np.zeros((3, 4)) for _ in range(3)]
    ios = []
    for f in fields:
        io = spu.IO(dim=2)
        io.define_eulerian_grid(origin=np.zeros(2), dx=np.ones(2), grid_size=np.array([3, 4]))
        io.add_as_eulerian_fields_for_io(w=f)
        ios.append(io)
    calls = []
    fake = types.ModuleType("elastica")
    fake.load_state = lambda sim, directory, verbose: calls.append((sim, directory, verbose)) or 2.75
    monkeypatch.setitem(sys.modules, "elastica", fake)
    assert spu.restart_simulation("sim", *ios, restart_dir="rods") == 2.75
    assert calls == [("sim", "rods", True)]
    for f in fields:
        assert (f == 2.75).all()
    fake.load_state = lambda *a: 1.0
    with pytest.raises(ValueError, match="not matched with the Elastica"):
        spu.restart_simulation("sim", *ios, restart_dir="rods")


def test_restart_simulation_without_files(tmp_path):
    with pytest.raises(FileNotFoundError, match="no file to load"):
        spu.restart_simulation(None, None, None, None, restart_dir=str(tmp_path))
