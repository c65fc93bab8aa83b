"""HDF5 + XDMF field IO for flow fields held on the GPU (sopht/utils/io.py:13-694).

The file layout is the reference's, so files move between the two packages
and ParaView reads the XDMF side files of either:

- root attribute ``time``;
- ``Eulerian/Scalar/<name>`` with shape (1, *grid) (the leading 1 makes
  ParaView place 2D fields in the XY plane), ``Eulerian/Vector/<name>_<i>``
  one dataset per component, ``Eulerian/Parameters`` with the attributes
  ``origin``, ``dx`` and ``grid_size`` (z, y, x order);
- ``Lagrangian/<grid>/Grid`` as (N, dim), ``Lagrangian/<grid>/Connection``
  (0..N-1) for polyline grids, ``Lagrangian/<grid>/Scalar/<name>`` and
  ``Lagrangian/<grid>/Vector/<name>`` as (N, dim);
- ``<file>_eulerian.xmf`` (a 3D co-rectilinear mesh, 2D grids as one slab) and
  ``<file>_<grid>.xmf`` per Lagrangian grid (polyline or polyvertex).

The Eulerian fields of this package's simulators are CUDA tensors.  ``save``
stages every registered device field into pinned host memory with
asynchronous copies and waits once, then writes; ``load`` reads each dataset
and copies it into the registered tensor in place, so a simulator restarts
from a file without re-creating its fields.  numpy arrays work as in the
reference.  h5py is imported when a file is first read or written.
"""

from __future__ import annotations

import xml.etree.ElementTree as ET
from pathlib import Path

import numpy as np
import torch

_XDMF_HEAD = '<?xml version="1.0" ?>\n<!DOCTYPE Xdmf SYSTEM "Xdmf.dtd" []>\n'


def _h5py():
    try:
        import h5py
    except ImportError as exc:  # pragma: no cover - depends on the environment
        raise ImportError("sopht_gb300.utils.IO reads and writes HDF5 files through h5py, which is not "
                          "installed") from exc
    return h5py


def _stage_to_host(fields: dict) -> dict:
    """Host numpy copies of the fields: one asynchronous device->host copy per CUDA
    tensor into pinned memory, one wait per device; numpy arrays pass through."""
    out, pending = {}, set()
    for name, f in fields.items():
        if isinstance(f, torch.Tensor):
            if f.is_cuda:
                host = torch.empty(f.shape, dtype=f.dtype, pin_memory=True)
                host.copy_(f.detach(), non_blocking=True)
                pending.add(f.device)
                out[name] = host
            else:
                out[name] = f.detach()
        else:
            out[name] = np.asarray(f)
    for device in pending:
        torch.cuda.current_stream(device).synchronize()
    return {k: (v.numpy() if isinstance(v, torch.Tensor) else v) for k, v in out.items()}


def _assign(target, value) -> None:
    """Write a host array into a registered field in place (host->device for CUDA tensors)."""
    if isinstance(target, torch.Tensor):
        target.copy_(torch.from_numpy(np.ascontiguousarray(value)).reshape(target.shape))
    else:
        target[...] = value


def _ints(values) -> str:
    return " ".join(str(int(v)) for v in values)


def _floats(values, digits: int) -> str:
    """Positional, at most ``digits`` fractional digits, shortest round trip in the values' own type."""
    return " ".join(np.format_float_positional(v, precision=digits, unique=True, trim=".")
                    for v in np.asarray(values).reshape(-1))


def _data_item(parent, text: str, **attrib) -> ET.Element:
    item = ET.SubElement(parent, "DataItem", attrib)
    item.text = text
    return item


def _write_xdmf(path: str, time, build) -> None:
    root = ET.Element("Xdmf", {"xmlns:xi": "http://www.w3.org/2003/XInclude", "Version": "2.2"})
    grid = ET.SubElement(ET.SubElement(root, "Domain"), "Grid", {"GridType": "Uniform"})
    ET.SubElement(grid, "Time", {"Value": f"{time}"})
    build(grid)
    ET.indent(root, space="    ")
    Path(path).write_text(_XDMF_HEAD + ET.tostring(root, encoding="unicode") + "\n")


class IO:
    """io.py:13-465: registered Eulerian and Lagrangian fields saved to / loaded from HDF5.

    ``precision`` (the XDMF ``Precision`` of floats) is 8 when ``real_dtype`` is
    ``np.float32`` itself and 16 otherwise, as the reference decides it."""

    def __init__(self, dim: int, real_dtype: type = np.float64) -> None:
        if dim not in (2, 3):
            raise ValueError("Invalid dimension (only 2D and 3D)")
        self.dim = dim
        self.real_dtype = real_dtype
        self.precision = 8 if real_dtype is np.float32 else 16
        self.eulerian_grid_defined = False
        self.eulerian_fields: dict = {}
        self.eulerian_fields_type: dict = {}
        self.lagrangian_fields: dict = {}
        self.lagrangian_fields_type: dict = {}
        self.lagrangian_grids: dict = {}
        self.lagrangian_fields_with_grid_name: dict = {}
        self.lagrangian_grid_count = 0
        self.lagrangian_grid_connection: dict = {}

    # ------------------------------------------------------------ registration

    def define_eulerian_grid(self, origin: np.ndarray, dx: np.ndarray, grid_size: np.ndarray) -> None:
        """Origin, spacing and size of the Eulerian grid, each (dim,) in z, y, x order."""
        if not all(isinstance(a, np.ndarray) for a in (origin, dx, grid_size)):
            raise TypeError("Invalid input types for Eulerian grid definition")
        self.eulerian_origin = origin
        self.eulerian_dx = dx
        self.eulerian_grid_size = grid_size
        self.eulerian_grid_defined = True

    def add_as_eulerian_fields_for_io(self, **fields_for_io) -> None:
        """Register Eulerian fields by keyword: shape grid_size is a scalar, (dim, *grid_size) a vector."""
        if not self.eulerian_grid_defined:
            raise ValueError("Eulerian mesh is not defined!")
        grid = tuple(int(n) for n in self.eulerian_grid_size)
        for name, field in fields_for_io.items():
            self.eulerian_fields[name] = field
            shape = tuple(field.shape)
            if shape == grid:
                self.eulerian_fields_type[name] = "Scalar"
            elif shape == (self.dim, *grid):
                self.eulerian_fields_type[name] = "Vector"
            else:
                raise ValueError(f"Unable to identify eulerian field type (scalar / vector) based on field "
                                 f"dimension {field.shape}")

    def add_as_lagrangian_fields_for_io(self, lagrangian_grid, lagrangian_grid_name: str | None = None,
                                        lagrangian_grid_connect: bool = False, **fields_for_io) -> None:
        """Register a Lagrangian grid (dim, N) and the fields on it: first axis N is a scalar,
        the grid's own shape a vector.  Unnamed grids are ``Lagrangian_grid_<count>``."""
        if len(lagrangian_grid.shape) != 2:
            raise ValueError("lagrangian grid has to be a 2D (dim, N) array.")
        if lagrangian_grid.shape[0] != self.dim:
            raise ValueError("Invalid lagrangian grid dimension (only 2D and 3D)")
        if lagrangian_grid_name is None:
            lagrangian_grid_name = f"Lagrangian_grid_{self.lagrangian_grid_count}"
            self.lagrangian_grid_count += 1
        n = lagrangian_grid.shape[1]
        if lagrangian_grid_connect:
            self.lagrangian_grid_connection[lagrangian_grid_name] = np.arange(n)
        self.lagrangian_grids[lagrangian_grid_name] = lagrangian_grid
        names = self.lagrangian_fields_with_grid_name[lagrangian_grid_name] = []
        for name, field in fields_for_io.items():
            self.lagrangian_fields[name] = field
            names.append(name)
            if field.shape[0] == n:
                self.lagrangian_fields_type[name] = "Scalar"
            elif tuple(field.shape) == tuple(lagrangian_grid.shape):
                self.lagrangian_fields_type[name] = "Vector"
            else:
                raise ValueError(f"Unable to identify lagrangian field type (scalar / vector) based on field "
                                 f"dimension {field.shape}")

    # ------------------------------------------------------------------- save

    def save(self, h5_file_name: str, time: float = 0.0) -> None:
        """Write every registered field at ``time`` (io.py:191-203)."""
        self._save(h5_file_name, time)

    def _save(self, h5_file_name: str, time: float = 0.0) -> None:
        eul = _stage_to_host(self.eulerian_fields) if self.eulerian_grid_defined else {}
        grids = _stage_to_host(self.lagrangian_grids)
        lag = _stage_to_host(self.lagrangian_fields)
        grid = tuple(int(n) for n in self.eulerian_grid_size) if self.eulerian_grid_defined else ()
        with _h5py().File(h5_file_name, "w") as f:
            f.attrs["time"] = time
            if self.eulerian_grid_defined:
                top = f.create_group("Eulerian")
                scalars, vectors = top.create_group("Scalar"), top.create_group("Vector")
                for name, field in eul.items():
                    if self.eulerian_fields_type[name] == "Scalar":
                        scalars.create_dataset(name, data=field.reshape(1, *grid))
                    else:
                        for c in range(self.dim):
                            vectors.create_dataset(f"{name}_{c}", data=field[c].reshape(1, *grid))
                params = top.create_group("Parameters")
                params.attrs["origin"] = self.eulerian_origin
                params.attrs["dx"] = self.eulerian_dx
                params.attrs["grid_size"] = self.eulerian_grid_size
            top = f.create_group("Lagrangian")
            for gname, points in grids.items():
                g = top.create_group(gname)
                g.create_dataset("Grid", data=points.T)
                if gname in self.lagrangian_grid_connection:
                    g.create_dataset("Connection", data=self.lagrangian_grid_connection[gname])
                scalars, vectors = g.create_group("Scalar"), g.create_group("Vector")
                for name in self.lagrangian_fields_with_grid_name[gname]:
                    if self.lagrangian_fields_type[name] == "Scalar":
                        scalars.create_dataset(name, data=lag[name])
                    else:
                        vectors.create_dataset(name, data=np.moveaxis(lag[name], 0, -1))
        if self.eulerian_fields:
            self.generate_xdmf_eulerian(h5_file_name=h5_file_name, time=time)
        if self.lagrangian_fields:
            self.generate_xdmf_lagrangian(h5_file_name=h5_file_name, time=time)

    # ------------------------------------------------------------------- load

    def load(self, h5_file_name: str) -> float:
        """Read the registered fields back in place and return the saved time (io.py:250-361).

        Raises ValueError for a missing field or grid, and when the file's Eulerian
        origin, spacing or size differ from this object's (restart consistency)."""
        with _h5py().File(h5_file_name, "r") as f:
            members: list = []
            f.visit(members.append)
            present = set(members)
            time = f.attrs["time"]
            if self.eulerian_fields:
                if not self.eulerian_grid_defined:
                    raise ValueError("Eulerian grid is not defined!")
                for name, field in self.eulerian_fields.items():
                    if self.eulerian_fields_type[name] == "Scalar":
                        if f"Eulerian/Scalar/{name}" not in present:
                            raise ValueError(f"Unable to find scalar field {name} in loaded file!")
                        _assign(field, f["Eulerian"]["Scalar"][name][0, ...])
                    else:
                        for c in range(self.dim):
                            if f"Eulerian/Vector/{name}_{c}" not in present:
                                raise ValueError(f"Unable to find vector field {name}_{c} in loaded file!")
                            _assign(field[c], f["Eulerian"]["Vector"][f"{name}_{c}"][0, ...])
                params = f["Eulerian"]["Parameters"].attrs
                for key, mine, what in (("origin", self.eulerian_origin, "origin"), ("dx", self.eulerian_dx, "dx"),
                                        ("grid_size", self.eulerian_grid_size, "grid size")):
                    if not np.allclose(mine, params[key]):
                        raise ValueError(f"Eulerian {what} does not match loaded file!")
            if self.lagrangian_fields:
                for gname, points in self.lagrangian_grids.items():
                    base = f"Lagrangian/{gname}"
                    if f"{base}/Grid" not in present:
                        raise ValueError(f"Unable to find grid '{gname}' in loaded file!")
                    _assign(points, np.transpose(f["Lagrangian"][gname]["Grid"][...]))
                    if f"{base}/Connection" in present:
                        self.lagrangian_grid_connection[gname] = f["Lagrangian"][gname]["Connection"][...]
                    for name in self.lagrangian_fields_with_grid_name[gname]:
                        kind = self.lagrangian_fields_type[name]
                        if f"{base}/{kind}/{name}" not in present:
                            raise ValueError(f"Unable to find {kind.lower()} field {name} on grid {gname} in "
                                             f"loaded file!")
                        data = f["Lagrangian"][gname][kind][name][...]
                        _assign(self.lagrangian_fields[name], data if kind == "Scalar" else np.moveaxis(data, -1, 0))
        return time

    # ------------------------------------------------------------------- XDMF

    def generate_xdmf_eulerian(self, h5_file_name: str, time: float = 0.0) -> None:
        """``<file>_eulerian.xmf``: a 3D co-rectilinear mesh (origin and spacing inline, 2D grids
        prefixed by one slab of zero spacing) and one node attribute per scalar or component."""
        pad = self.dim == 2
        size = _ints(([1] if pad else []) + [int(n) for n in self.eulerian_grid_size])
        origin = _floats(np.insert(self.eulerian_origin, 0, 0.0) if pad else self.eulerian_origin, self.precision)
        dx = _floats(np.insert(self.eulerian_dx, 0, 0.0) if pad else self.eulerian_dx, self.precision)
        prec = str(self.precision)

        def build(grid):
            ET.SubElement(grid, "Topology", {"TopologyType": "3DCORECTMesh", "Dimensions": size})
            geometry = ET.SubElement(grid, "Geometry", {"GeometryType": "ORIGIN_DXDYDZ"})
            for label, text in (("Origin", origin), ("Spacing", dx)):
                _data_item(geometry, text, Name=label, Dimensions=str(self.dim), NumberType="Float",
                           Precision=prec, Format="XML")
            for name, kind in self.eulerian_fields_type.items():
                parts = [name] if kind == "Scalar" else [f"{name}_{c}" for c in range(self.dim)]
                for part in parts:
                    attribute = ET.SubElement(grid, "Attribute", {"Name": part, "Active": "1",
                                                                  "AttributeType": "Scalar", "Center": "Node"})
                    _data_item(attribute, f"{h5_file_name}:/Eulerian/{kind}/{part}", Dimensions=size,
                               NumberType="Float", Precision=prec, Format="HDF")

        _write_xdmf(h5_file_name.replace(".h5", "_eulerian.xmf"), time, build)

    def generate_xdmf_lagrangian(self, h5_file_name: str, time: float) -> None:
        """``<file>_<grid>.xmf`` per Lagrangian grid: a polyline through the points in order when
        the grid is connected, else a polyvertex; XY or XYZ geometry; one attribute per field."""
        prec = str(self.precision)
        for gname, points in self.lagrangian_grids.items():
            n = int(points.shape[1])
            size = _ints([n, self.dim])
            source = f"{h5_file_name}:/Lagrangian/{gname}"

            def build(grid, gname=gname, n=n, size=size, source=source):
                if gname in self.lagrangian_grid_connection:
                    topology = ET.SubElement(grid, "Topology", {"TopologyType": "Polyline"})
                    _data_item(topology, f"{source}/Connection", DataType="Int", Dimensions=_ints([1, n]),
                               Format="HDF", Precision=prec)
                else:
                    ET.SubElement(grid, "Topology", {"TopologyType": "Polyvertex", "NumberOfElements": str(n)})
                geometry = ET.SubElement(grid, "Geometry", {"GeometryType": "XYZ" if self.dim == 3 else "XY"})
                _data_item(geometry, f"{source}/Grid", Dimensions=size, NumberType="Float", Precision=prec,
                           Format="HDF")
                for name in self.lagrangian_fields_with_grid_name[gname]:
                    kind = self.lagrangian_fields_type[name]
                    attribute = ET.SubElement(grid, "Attribute", {"Name": name, "Active": "1",
                                                                  "AttributeType": kind, "Center": "Node"})
                    _data_item(attribute, f"{source}/{kind}/{name}", Dimensions=str(n) if kind == "Scalar" else size,
                               NumberType="Float", Precision=prec, Format="HDF")

            _write_xdmf(h5_file_name.replace(".h5", f"_{gname}.xmf"), time, build)


class CosseratRodIO(IO):
    """io.py:576-611: a rod's element centres as a connected Lagrangian grid ``rod`` with
    the element radii (``scalar_3d``); ``save`` refreshes the centres from the rod first."""

    def __init__(self, cosserat_rod, dim: int, real_dtype: type = np.float64) -> None:
        super().__init__(dim, real_dtype)
        self.cosserat_rod = cosserat_rod
        self.rod_element_position = np.zeros((self.dim, cosserat_rod.n_elems))
        self._update_rod_element_position()
        self.add_as_lagrangian_fields_for_io(lagrangian_grid=self.rod_element_position, lagrangian_grid_name="rod",
                                             scalar_3d=self.cosserat_rod.radius, lagrangian_grid_connect=True)

    def save(self, h5_file_name: str, time: float = 0.0) -> None:
        self._update_rod_element_position()
        self._save(h5_file_name=h5_file_name, time=time)

    def _update_rod_element_position(self) -> None:
        p = self.cosserat_rod.position_collection
        self.rod_element_position[...] = 0.5 * (p[: self.dim, 1:] + p[: self.dim, :-1])


class EulerianFieldIO(IO):
    """io.py:614-694: the Eulerian grid read off a simulator's ``position_field``.

    Origin = the smallest coordinate along each axis (z, y, x order), spacing =
    the first x step, size = the field's grid shape; the fields of
    ``eulerian_fields_dict`` are registered by key."""

    def __init__(self, position_field, eulerian_fields_dict: dict) -> None:
        position = _stage_to_host({"p": position_field})["p"]
        grid_dim = position.shape[0]
        super().__init__(dim=grid_dim, real_dtype=position_field.dtype)  # raises unless 2D or 3D
        axes = (1, 0) if grid_dim == 2 else (2, 1, 0)  # y, x or z, y, x components of the position field
        origin = np.array([position[a].min() for a in axes])
        x = position[0].reshape(-1)
        dx = x[1] - x[0]
        self.define_eulerian_grid(origin=origin, dx=dx * np.ones(grid_dim), grid_size=np.array(position.shape[1:]))
        self.add_as_eulerian_fields_for_io(**eulerian_fields_dict)
