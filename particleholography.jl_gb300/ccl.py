"""Host mirror of ParticleHolography.jl src/ccl.jl:186-238 over libphgb300.

``cu_connected_component_labeling`` labels 8-connected components of equal
value; pixels with value > 0 get ``1 + the minimum linear index`` of their
component, others 0 (UInt32) -- the reference's labels exactly.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib

__all__ = ["cu_connected_component_labeling", "count_labels", "cu_find_valid_labels"]


def cu_connected_component_labeling(input_img: torch.Tensor, reference_grid: bool = True) -> torch.Tensor:
    """ccl.jl:186-211.

    ``input_img``: CUDA Float32 or Bool tensor of shape ``(n_slow, n_fast)``
    (a Julia ``(n_fast, n_slow)`` array).  The reference labels the buffer as a
    grid of ``size(img,1)`` rows by ``size(img,2)`` columns in linear memory
    order; ``reference_grid=True`` (default) does the same, which equals true
    2-D 8-connectivity for square images.  ``reference_grid=False`` labels the
    true 2-D image for any shape.
    """
    img = input_img.data if hasattr(input_img, "data") and isinstance(input_img.data, torch.Tensor) else input_img
    if not img.is_cuda:
        raise TypeError("cu_connected_component_labeling works on CUDA tensors (CuArray)")
    if img.dim() != 2:
        raise ValueError("input must be 2-D")
    if not img.is_contiguous():
        img = img.contiguous()
    if img.dtype == torch.bool or img.dtype == torch.uint8:
        code = _lib.PH_BOOL
        img = img.view(torch.uint8) if img.dtype == torch.bool else img
    elif img.dtype == torch.float32:
        code = _lib.PH_F32
    else:
        raise TypeError(f"input must be Float32 or Bool, got {img.dtype}")
    n_slow, n_fast = int(img.shape[0]), int(img.shape[1])
    rows, cols = (n_fast, n_slow) if reference_grid else (n_slow, n_fast)
    out = torch.empty(img.shape, dtype=torch.int32, device=img.device)   # UInt32 bits
    dev = img.device.index if img.device.index is not None else torch.cuda.current_device()
    ctx = _lib.default_context(dev)
    ctx.call("ph_ccl", out.data_ptr(), img.data_ptr(), code, rows, cols, torch.cuda.current_stream(dev).cuda_stream)
    return out.view(torch.uint32) if hasattr(torch, "uint32") else out


def _labels_on_device(labels) -> torch.Tensor:
    if isinstance(labels, np.ndarray):
        labels = torch.from_numpy(np.ascontiguousarray(labels).view(np.int32)).cuda()
    if not labels.is_cuda:
        labels = labels.cuda()
    return labels.contiguous()


def _roots(labels, capacity: int):
    lab = _labels_on_device(labels)
    dev = lab.device.index if lab.device.index is not None else torch.cuda.current_device()
    ctx = _lib.default_context(dev)
    n = lab.numel()
    count = ctypes.c_int64(0)
    buf = np.empty(max(capacity, 0), dtype=np.int64)
    ctx.call("ph_ccl_roots", buf.ctypes.data if capacity > 0 else None, int(capacity), ctypes.byref(count),
             lab.data_ptr(), n, torch.cuda.current_stream(dev).cuda_stream)
    return int(count.value), buf


def count_labels(labels) -> int:
    """ccl.jl:213-221: number of indices i with ``labels[i] == i`` (1-based)."""
    c, _ = _roots(labels, 0)
    return c


def cu_find_valid_labels(labels) -> np.ndarray:
    """ccl.jl:224-238: sorted 1-based root indices as a host Int64 vector."""
    c, _ = _roots(labels, 0)
    _, buf = _roots(labels, c)
    return buf[:c]
