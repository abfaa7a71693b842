"""Device plumbing for the Python host layer: CUDA checks, streams, array
conversion and workspace buffers (PyTorch supplies device memory and
streams; all array arithmetic on the hot path runs in the ctgpu kernels)."""

from __future__ import annotations

import numpy as np
import torch

from . import _lib

_reduce_ws: dict[tuple[int, int], torch.Tensor] = {}


def require_cuda() -> torch.device:
    """Return the current CUDA device; raise if there is none (no CPU path)."""
    if not torch.cuda.is_available():
        raise RuntimeError(
            "scico_gb300 runs its operators on a CUDA device only and found none; "
            "there is no CPU fallback"
        )
    return torch.device("cuda", torch.cuda.current_device())


def stream() -> int:
    """Handle of the current torch CUDA stream (passed to the C ABI)."""
    return torch.cuda.current_stream().cuda_stream


def to_device(x, shape=None, name: str = "array") -> torch.Tensor:
    """float32, C-contiguous CUDA tensor view/copy of `x` (numpy or torch)."""
    dev = require_cuda()
    if isinstance(x, torch.Tensor):
        if x.dtype != torch.float32:
            raise ValueError(f"{name}: expected dtype float32, got {x.dtype}")
        t = x if x.device.type == "cuda" else x.to(dev)
    else:
        a = np.asarray(x)
        if a.dtype != np.float32:
            a = a.astype(np.float32)
        t = torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    if not t.is_contiguous():
        t = t.contiguous()
    if shape is not None and tuple(t.shape) != tuple(shape):
        raise ValueError(f"{name}: expected shape {tuple(shape)}, got {tuple(t.shape)}")
    return t


def empty(shape, dtype=torch.float32) -> torch.Tensor:
    return torch.empty(tuple(shape), dtype=dtype, device=require_cuda())


def zeros(shape, dtype=torch.float32) -> torch.Tensor:
    return torch.zeros(tuple(shape), dtype=dtype, device=require_cuda())


def workspace(nbytes: int) -> torch.Tensor:
    """Uninitialised scratch (the caching allocator returns 512-B aligned blocks)."""
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=require_cuda())


def reduce_workspace() -> torch.Tensor:
    """Zero-filled reduction workspace of the current device and stream.

    Each reduction leaves it zeroed again, so one buffer per (device, stream)
    serves every reduction issued on that stream.
    """
    dev = require_cuda()
    key = (dev.index, stream())
    ws = _reduce_ws.get(key)
    if ws is None:
        n = _lib.load().ct_reduce_workspace()
        ws = torch.zeros(int(n), dtype=torch.uint8, device=dev)
        _reduce_ws[key] = ws
    return ws
