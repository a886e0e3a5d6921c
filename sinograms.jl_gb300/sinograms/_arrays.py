"""Array plumbing between numpy / torch and the C ABI.

Host arrays (numpy, CPU tensors) are passed as host pointers; CUDA tensors as device
pointers with SGB_DEVICE_PTRS, enqueued on torch's current stream.  Outputs are created
in the same place as the main input.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

try:  # torch is optional for host-only use
    import torch
except Exception:  # pragma: no cover
    torch = None


def is_cuda(x) -> bool:
    return torch is not None and isinstance(x, torch.Tensor) and x.is_cuda


class Arr:
    """A float32 (or uint8) contiguous view of an input with its pointer and flags."""

    def __init__(self, x, dtype=np.float32):
        self.src = x
        if is_cuda(x):
            tdt = torch.float32 if dtype == np.float32 else torch.uint8
            self.obj = x.detach().to(tdt).contiguous()
            self.ptr = ctypes.c_void_p(self.obj.data_ptr())
            self.device = True
            self.shape = tuple(self.obj.shape)
        else:
            if torch is not None and isinstance(x, torch.Tensor):
                x = x.detach().cpu().numpy()
            self.obj = np.ascontiguousarray(x, dtype=dtype)
            self.ptr = ctypes.c_void_p(self.obj.ctypes.data)
            self.device = False
            self.shape = self.obj.shape


def flags_for(device: bool, sync: bool = True) -> int:
    return (_lib.SGB_DEVICE_PTRS | (0 if sync else _lib.SGB_ASYNC)) if device else 0


def stream_for(device: bool):
    if device:
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    return None


def plan_call(device: bool, sync: bool):
    """(flags, stream) of a plan call: with sync=False host buffers are also copied
    asynchronously, on torch's current stream (keep them alive, and pinned, until
    plan.sync())."""
    flags = (_lib.SGB_DEVICE_PTRS if device else 0) | (0 if sync else _lib.SGB_ASYNC)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream) if (device or not sync) else None
    return flags, st


def empty(shape, like: Arr, dtype=np.float32):
    if like.device:
        return torch.empty(shape, dtype=torch.float32, device=like.obj.device)
    return np.empty(shape, dtype=dtype)


def check_out(out, shape, device: bool):
    """Raise ValueError unless `out` can take the library's prod(shape) float32 writes: a
    C-contiguous float32 array of exactly `shape`, a CUDA tensor when `device` (the input is on
    the GPU), else a numpy array or CPU tensor."""
    shape = tuple(shape)
    if torch is not None and isinstance(out, torch.Tensor):
        ok = (out.is_cuda == device and out.dtype == torch.float32 and out.is_contiguous()
              and tuple(out.shape) == shape)
    else:
        ok = (not device and isinstance(out, np.ndarray) and out.dtype == np.float32
              and out.flags.c_contiguous and out.flags.writeable and out.shape == shape)
    if not ok:
        where = "a CUDA tensor" if device else "a host array"
        desc = f"{type(out).__name__} {getattr(out, 'dtype', '')} {tuple(getattr(out, 'shape', ()))}"
        raise ValueError(f"out must be {where}, float32, contiguous, of shape {shape}; got {desc}")
    return out


def out_buffer(out, shape, like: Arr):
    """The caller's `out` (checked by check_out) or a new array in the same place as the input."""
    if out is None:
        return empty(shape, like)
    if like.device and is_cuda(out) and out.device != like.obj.device:
        raise ValueError(f"out is on {out.device}, the input on {like.obj.device}")
    return check_out(out, shape, like.device)


def ptr(a):
    if a is None:
        return None
    if torch is not None and isinstance(a, torch.Tensor):
        return ctypes.c_void_p(a.data_ptr())
    return ctypes.c_void_p(a.ctypes.data)


def f64(v) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(v, dtype=np.float64))
