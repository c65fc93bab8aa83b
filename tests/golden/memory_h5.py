"""Test-only stand-in for the part of h5py's API that SophT's field IO uses.

This module is test infrastructure: h5py is not installed on either machine
this repository is tested on, so the IO tests and ``make_golden.py`` put this
module in ``sys.modules["h5py"]`` (or in the reference IO module's namespace)
to run the reference's IO and this package's IO against the same file model.
Nothing in the product imports it.

The model follows h5py's semantics for what the IO calls use: ``File(name,
mode)`` as a context manager ("w" truncates, "r" reads), groups with
``create_group``, ``create_dataset(name, data=...)`` (the data copied, dtype
kept), ``attrs`` (values stored as numpy scalars or arrays), path indexing
(``f["a"]["b"]`` and ``f["a/b"]``), ``in`` and ``visit`` (every member's path
relative to the group, groups before their members, in insertion order).
A file is kept on disk as a pickle of that tree, so that directory listings,
reopening and restart logic behave as with real files; the bytes are not HDF5.
"""

from __future__ import annotations

import pickle
from pathlib import Path

import numpy as np


class Dataset:
    def __init__(self, data) -> None:
        self._data = np.array(data, copy=True)
        self.attrs = _Attrs()

    @property
    def shape(self):
        return self._data.shape

    @property
    def dtype(self):
        return self._data.dtype

    def __getitem__(self, idx):
        return self._data[idx]


class _Attrs(dict):
    def __setitem__(self, key, value) -> None:
        super().__setitem__(key, np.array(value, copy=True) if np.ndim(value) else np.asarray(value)[()])


class Group:
    def __init__(self) -> None:
        self._members: dict[str, Group | Dataset] = {}
        self.attrs = _Attrs()

    def _new(self, name: str, obj):
        parent, _, leaf = name.rpartition("/")
        grp = self[parent] if parent else self
        if leaf in grp._members:
            raise ValueError(f"Unable to create {name!r} (name already exists)")
        grp._members[leaf] = obj
        return obj

    def create_group(self, name: str) -> Group:
        return self._new(name, Group())

    def create_dataset(self, name: str, data=None, **_) -> Dataset:
        return self._new(name, Dataset(data))

    def __getitem__(self, path: str):
        obj = self
        for part in (p for p in path.split("/") if p):
            obj = obj._members[part]
        return obj

    def __contains__(self, path: str) -> bool:
        try:
            self[path]
        except (KeyError, AttributeError):
            return False
        return True

    def keys(self):
        return self._members.keys()

    def visit(self, func):
        def walk(grp, prefix):
            for name, obj in grp._members.items():
                path = f"{prefix}{name}"
                out = func(path)
                if out is not None:
                    return out
                if isinstance(obj, Group):
                    out = walk(obj, path + "/")
                    if out is not None:
                        return out
            return None

        return walk(self, "")


class File(Group):
    def __init__(self, name, mode: str = "r") -> None:
        super().__init__()
        self.filename = str(name)
        self.mode = mode
        if mode == "r":
            path = Path(self.filename)
            if not path.exists():
                raise FileNotFoundError(f"Unable to open file {self.filename!r}")
            with path.open("rb") as fh:
                root = pickle.load(fh)
            self._members, self.attrs = root._members, root.attrs
        elif mode != "w":
            raise ValueError(f"mode {mode!r} is not modelled")

    def close(self) -> None:
        if self.mode == "w":
            root = Group()
            root._members, root.attrs = self._members, self.attrs
            with Path(self.filename).open("wb") as fh:
                pickle.dump(root, fh)
            self.mode = "closed"

    def __enter__(self) -> File:
        return self

    def __exit__(self, *exc) -> None:
        self.close()


def dump(path) -> dict:
    """Every dataset (by path) and attribute (``path@name``; the root's as ``@name``) of a file."""
    out = {}
    with File(path, "r") as f:
        def collect(grp, prefix):
            for key, value in grp.attrs.items():
                out[f"{prefix}@{key}"] = np.asarray(value)
            for name, obj in grp._members.items():
                p = f"{prefix}/{name}" if prefix else name
                if isinstance(obj, Group):
                    collect(obj, p)
                    out.setdefault(f"{p}/", np.array([]))
                else:
                    out[p] = obj[...]
        collect(f, "")
    return out


def restore(path, dumped: dict) -> None:
    """Write a file holding what ``dump`` returned (groups, datasets, attributes)."""
    with File(path, "w") as f:
        for key in sorted(k for k in dumped if k.endswith("/") and "@" not in k):
            parts = key.rstrip("/").split("/")
            grp = f
            for part in parts:
                grp = grp[part] if part in grp.keys() else grp.create_group(part)
        for key, value in dumped.items():
            if "@" in key:
                owner, _, name = key.partition("@")
                (f[owner] if owner else f).attrs[name] = value
            elif not key.endswith("/"):
                f.create_dataset(key, data=value)
