"""Precision, axis and device helpers (mirrors sopht/utils/precision.py and field.py)."""

from __future__ import annotations

import numpy as np
import torch

from .. import _lib


def get_real_t(precision: str = "single") -> type:
    """precision.py:6-13: 'single' -> np.float32, 'double' -> np.float64."""
    if precision == "single":
        return np.float32
    if precision == "double":
        return np.float64
    raise ValueError("Precision argument must be single or double")


def get_test_tol(precision: str = "single") -> float:
    """precision.py:16-19: 1e3 machine epsilons of the precision."""
    real_t = get_real_t(precision=precision)
    return real_t(1e3) * np.finfo(real_t).eps


class VectorField:
    """Component indices of vector fields (field.py): x = 0, y = 1, z = 2."""

    @staticmethod
    def x_axis_idx() -> int:
        return 0

    @staticmethod
    def y_axis_idx() -> int:
        return 1

    @staticmethod
    def z_axis_idx() -> int:
        return 2


def normalize_real_t(real_t) -> type:
    """Accept numpy or torch float types; return np.float32 / np.float64."""
    if real_t in (np.float32, torch.float32, "float32", "single"):
        return np.float32
    if real_t in (np.float64, torch.float64, "float64", "double"):
        return np.float64
    raise ValueError("Invalid real type")


def torch_dtype(real_t) -> torch.dtype:
    return torch.float32 if normalize_real_t(real_t) == np.float32 else torch.float64


def sg_dtype(real_t) -> int:
    return _lib.SG_F32 if normalize_real_t(real_t) == np.float32 else _lib.SG_F64


def default_device(device=None) -> torch.device:
    if device is not None:
        return torch.device(device)
    if not torch.cuda.is_available():
        raise RuntimeError("sopht_gb300 needs a CUDA device (sm_103a); none is available")
    return torch.device("cuda", torch.cuda.current_device())


_raw_stream = getattr(torch._C, "_cuda_getCurrentRawStream", None)
_cuda_ready = False


def stream_ptr(device: torch.device | None = None) -> int:
    """Raw cudaStream_t of torch's current stream on ``device``.

    Read straight from torch's C++ stream registry when that entry point exists
    (it does in the torch releases this package supports): the public
    ``torch.cuda.current_stream(device)`` builds a Stream object per call,
    which costs several microseconds on every operator call."""
    global _cuda_ready
    if _raw_stream is not None:
        if not _cuda_ready:
            torch.cuda.init()  # the raw lookup does not initialise CUDA itself
            _cuda_ready = True
        idx = device.index if device is not None and device.index is not None else torch.cuda.current_device()
        return _raw_stream(idx)
    return torch.cuda.current_stream(device).cuda_stream


def ptr(t: torch.Tensor | None) -> int | None:
    """Device pointer of a contiguous CUDA tensor (None passes through)."""
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError("expected a C-contiguous tensor")
    return t.data_ptr()


def as_device(x, dtype: torch.dtype, device: torch.device, out: torch.Tensor | None = None) -> torch.Tensor:
    """Copy a numpy array or tensor into ``out`` (or a new device tensor)."""
    if isinstance(x, torch.Tensor):
        src = x.to(dtype=dtype)
    else:
        src = torch.from_numpy(np.ascontiguousarray(np.asarray(x, dtype=torch.empty((), dtype=dtype).numpy().dtype)))
    if out is None:
        return src.to(device=device, non_blocking=True).contiguous()
    out.copy_(src, non_blocking=True)
    return out


from .io import IO, CosseratRodIO, EulerianFieldIO  # noqa: E402
from .restart_sim import restart_simulation  # noqa: E402
