"""Test-only stand-ins that let the reference SophT package import and run here.

This module is test infrastructure. It is used only by ``make_golden.py`` in this
directory to execute the reference implementation's own Python code (its sympy
stencil definitions, its Poisson solver classes, its immersed-boundary loops and
its simulator step drivers) on seeded inputs, so that the outputs can be frozen
as golden fixtures.  Nothing in the product imports it.

The reference depends on four packages that are not installed in this image:

* ``pystencils`` 1.4 (pinned in the reference's ``uv.lock``) turns each
  ``@ps.kernel`` function into C code.  The stand-in below re-reads the kernel's
  source, turns ``lhs @= rhs`` into an assignment record and ``a if c else b``
  into ``sympy.Piecewise`` (the same two rewrites pystencils' kernel decorator
  performs), and evaluates each assignment with numpy over the iteration space
  pystencils would use: the full array minus ``g`` ghost layers on every side,
  where ``g`` is the largest absolute offset of any field access in the kernel,
  or the explicit ``iteration_slice`` when the config gives one.  Scalar kernel
  parameters are cast to the kernel's ``data_type`` as pystencils does.
* ``pyfftw`` 0.15 is replaced by ``scipy.fft`` R2C/C2R transforms in the same
  precision, with the inverse normalised by 1/N (pyfftw's ``normalise_idft``).
* ``numba`` 0.64: ``njit`` becomes the identity, so the loops run as Python.
* ``pyelastica`` 0.3.3.post2: only the names the reference imports, plus numpy
  restatements of the three helpers the forcing grids call
  (``_batch_cross``, ``_batch_matvec`` and the mass-weighted
  ``_node_to_element_velocity``).

``h5py``, ``matplotlib`` and ``ffmpeg`` are imported by the reference's IO and
plotting utilities only; they become empty modules.
"""

from __future__ import annotations

import ast
import inspect
import sys
import textwrap
import types

import numpy as np
import scipy.fft
import sympy as sp

# ----------------------------------------------------------------------------
# pystencils stand-in
# ----------------------------------------------------------------------------

_ACCESS_REGISTRY: dict[str, tuple[str, tuple[int, ...]]] = {}


def _offset_tag(o: int) -> str:
    return f"m{-o}" if o < 0 else f"p{o}"


class _Field:
    def __init__(self, name: str) -> None:
        self.name = name

    def __getitem__(self, idx):
        if not isinstance(idx, tuple):
            idx = (idx,)
        idx = tuple(int(i) for i in idx)
        sym_name = f"F__{self.name}__" + "_".join(_offset_tag(o) for o in idx)
        _ACCESS_REGISTRY[sym_name] = (self.name, idx)
        return sp.Symbol(sym_name, real=True)


def _fields(spec: str):
    names, _, _typ = spec.partition(":")
    fields = [_Field(n.strip()) for n in names.split(",") if n.strip()]
    return fields[0] if len(fields) == 1 else tuple(fields)


class _KernelRewrite(ast.NodeTransformer):
    def visit_FunctionDef(self, node):
        node.decorator_list = []
        self.generic_visit(node)
        return node

    def visit_AugAssign(self, node):
        self.generic_visit(node)
        if isinstance(node.op, ast.MatMult):
            target = node.target
            target.ctx = ast.Load()
            for sub in ast.walk(target):
                if hasattr(sub, "ctx"):
                    sub.ctx = ast.Load()
            call = ast.Call(
                func=ast.Name(id="__shim_assign__", ctx=ast.Load()),
                args=[target, node.value],
                keywords=[],
            )
            return ast.copy_location(ast.Expr(value=call), node)
        return node

    def visit_IfExp(self, node):
        self.generic_visit(node)
        call = ast.Call(
            func=ast.Name(id="__shim_piecewise__", ctx=ast.Load()),
            args=[node.body, node.test, node.orelse],
            keywords=[],
        )
        return ast.copy_location(call, node)


def _kernel(func):
    src = textwrap.dedent(inspect.getsource(func))
    tree = ast.parse(src)
    tree = _KernelRewrite().visit(tree)
    ast.fix_missing_locations(tree)
    assignments: list[tuple[sp.Symbol, sp.Expr]] = []
    namespace = dict(func.__globals__)
    if func.__closure__:
        for name, cell in zip(func.__code__.co_freevars, func.__closure__, strict=True):
            namespace[name] = cell.cell_contents
    namespace["__shim_assign__"] = lambda lhs, rhs: assignments.append((lhs, sp.sympify(rhs)))
    namespace["__shim_piecewise__"] = lambda a, c, b: sp.Piecewise((a, c), (b, True))
    exec(compile(tree, filename=f"<shim kernel {func.__name__}>", mode="exec"), namespace)
    namespace[func.__name__]()
    return assignments


class _CreateKernelConfig:
    def __init__(self, data_type="float64", default_number_float=None, cpu_openmp=False,
                 iteration_slice=None, **_):
        self.data_type = np.dtype(data_type)
        self.iteration_slice = iteration_slice


class _MakeSlice:
    def __getitem__(self, idx):
        return idx if isinstance(idx, tuple) else (idx,)


def _accesses(expr) -> list[str]:
    return [s.name for s in expr.free_symbols if s.name in _ACCESS_REGISTRY]


class _CompiledKernel:
    def __init__(self, assignments, config):
        self.assignments = assignments
        self.config = config or _CreateKernelConfig()
        offsets = []
        for lhs, rhs in assignments:
            for name in _accesses(lhs) + _accesses(rhs):
                offsets.extend(_ACCESS_REGISTRY[name][1])
        self.ghost_layers = int(max((abs(o) for o in offsets), default=0))

    def __call__(self, **kwargs):
        real_t = self.config.data_type.type
        results = []
        for lhs, rhs in self.assignments:
            lhs_field, lhs_off = _ACCESS_REGISTRY[lhs.name]
            shape = np.asarray(kwargs[lhs_field]).shape
            if self.config.iteration_slice is not None:
                region = [slice(*s.indices(n)[:2]) for s, n in
                          zip(self.config.iteration_slice, shape, strict=True)]
            else:
                g = self.ghost_layers
                region = [slice(g, n - g) for n in shape]
            args, vals = [], []
            for sym in sorted(rhs.free_symbols, key=lambda s: s.name):
                if sym.name in _ACCESS_REGISTRY:
                    fname, off = _ACCESS_REGISTRY[sym.name]
                    arr = kwargs[fname]
                    sl = tuple(slice(r.start + o, r.stop + o) for r, o in zip(region, off, strict=True))
                    vals.append(arr[sl])
                else:
                    vals.append(real_t(kwargs[sym.name]))
                args.append(sym)
            fn = sp.lambdify(args, rhs, modules="numpy")
            results.append((lhs_field, lhs_off, region, fn(*vals)))
        for lhs_field, lhs_off, region, value in results:
            arr = kwargs[lhs_field]
            sl = tuple(slice(r.start + o, r.stop + o) for r, o in zip(region, lhs_off, strict=True))
            arr[sl] = value


class _KernelAST:
    def __init__(self, assignments, config):
        self._k = _CompiledKernel(assignments, config)

    def compile(self):
        return self._k


def _create_kernel(assignments, config=None, **_):
    return _KernelAST(assignments, config)


def _make_pystencils() -> types.ModuleType:
    m = types.ModuleType("pystencils")
    m.fields = _fields
    m.kernel = _kernel
    m.create_kernel = _create_kernel
    m.CreateKernelConfig = _CreateKernelConfig
    m.make_slice = _MakeSlice()
    return m


# ----------------------------------------------------------------------------
# pyfftw stand-in
# ----------------------------------------------------------------------------


class _FFTW:
    def __init__(self, input_array, output_array, axes=(-1,), direction="FFTW_FORWARD",
                 flags=(), threads=1, **_):
        self.input_array = input_array
        self.output_array = output_array
        self.axes = tuple(axes)
        self.direction = direction

    def __call__(self, input_array=None, output_array=None, normalise_idft=True, **_):
        inp = self.input_array if input_array is None else input_array
        out = self.output_array if output_array is None else output_array
        if self.direction == "FFTW_FORWARD":
            out[...] = scipy.fft.rfftn(inp, axes=self.axes)
        else:
            s = [out.shape[a] for a in self.axes]
            out[...] = scipy.fft.irfftn(inp, s=s, axes=self.axes)
        return out


def _make_pyfftw() -> types.ModuleType:
    m = types.ModuleType("pyfftw")
    m.empty_aligned = lambda shape, dtype=np.float64, n=None: np.empty(shape, dtype=dtype)
    m.FFTW = _FFTW
    builders = types.ModuleType("pyfftw.builders")
    builders.rfftn = lambda a, threads=1, **_: (lambda x=None: scipy.fft.rfftn(a if x is None else x))
    builders.irfftn = lambda a, threads=1, **_: (lambda x=None: scipy.fft.irfftn(a if x is None else x))
    builders.fftn = lambda a, threads=1, **_: (lambda x=None: scipy.fft.fftn(a if x is None else x))
    builders.ifftn = lambda a, threads=1, **_: (lambda x=None: scipy.fft.ifftn(a if x is None else x))
    m.builders = builders
    return m


# ----------------------------------------------------------------------------
# numba, pyelastica and the plotting/IO stand-ins
# ----------------------------------------------------------------------------


def _njit(*args, **kwargs):
    if len(args) == 1 and callable(args[0]) and not kwargs:
        return args[0]
    return lambda f: f


class _StubMeta(type):
    def __getattr__(cls, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _StubMeta(name, (), {"__init__": lambda self, *a, **k: None})


class _StubModule(types.ModuleType):
    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        cls = _StubMeta(name, (), {"__init__": lambda self, *a, **k: None})
        setattr(self, name, cls)
        return cls


def _batch_cross(a, b):
    return np.cross(a, b, axis=0)


def _batch_matvec(matrix, vector):
    return np.einsum("ijk,jk->ik", matrix, vector)


def _batch_matrix_transpose(matrix):
    return np.transpose(matrix, (1, 0, 2))


def _node_to_element_velocity(mass, node_velocity_collection):
    # pyelastica: element velocity is the mass-weighted mean of its two nodes
    return (
        mass[1:] * node_velocity_collection[:, 1:] + mass[:-1] * node_velocity_collection[:, :-1]
    ) / (mass[1:] + mass[:-1])


def _elements_to_nodes_inplace(vector_in_element_frame, vector_in_node_frame):
    half = 0.5 * vector_in_element_frame
    vector_in_node_frame[..., :-1] += half
    vector_in_node_frame[..., 1:] += half


def install() -> None:
    """Register every stand-in in ``sys.modules`` (idempotent)."""
    if "pystencils" in sys.modules and getattr(sys.modules["pystencils"], "_is_shim", False):
        return
    ps = _make_pystencils()
    ps._is_shim = True
    sys.modules["pystencils"] = ps
    fftw = _make_pyfftw()
    sys.modules["pyfftw"] = fftw
    sys.modules["pyfftw.builders"] = fftw.builders
    numba = types.ModuleType("numba")
    numba.njit = _njit
    sys.modules["numba"] = numba

    ea = _StubModule("elastica")
    sys.modules["elastica"] = ea
    linalg = _StubModule("elastica._linalg")
    linalg._batch_cross = _batch_cross
    linalg._batch_matvec = _batch_matvec
    linalg._batch_matrix_transpose = _batch_matrix_transpose
    sys.modules["elastica._linalg"] = linalg
    inter = _StubModule("elastica.interaction")
    inter._node_to_element_velocity = _node_to_element_velocity
    inter._elements_to_nodes_inplace = _elements_to_nodes_inplace
    sys.modules["elastica.interaction"] = inter
    utils = _StubModule("elastica.utils")

    class MaxDimension:
        @staticmethod
        def value():
            return 3

    utils.MaxDimension = MaxDimension
    sys.modules["elastica.utils"] = utils
    sys.modules["elastica.rod"] = _StubModule("elastica.rod")
    sys.modules["elastica.rod.cosserat_rod"] = _StubModule("elastica.rod.cosserat_rod")
    for name in ("h5py", "ffmpeg", "matplotlib", "matplotlib.pyplot", "matplotlib.cm",
                 "matplotlib.colors", "matplotlib.animation", "matplotlib.patches"):
        sys.modules[name] = _StubModule(name)
    for name in list(sys.modules):
        if name.startswith(("matplotlib.", "elastica.", "pyfftw.")):
            parent, _, child = name.rpartition(".")
            if parent in sys.modules:
                setattr(sys.modules[parent], child, sys.modules[name])
