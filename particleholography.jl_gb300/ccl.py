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


def cu_connected_component_labeling_batch(vol: torch.Tensor) -> torch.Tensor:
    """The per-slice labeling of particle_bounding_boxes (particle_detection.jl:58-76)
    in one launch set: ``vol`` (CUDA Bool/Float32, shape ``(slices, n_slow, n_fast)``)
    -> UInt32 labels of the same shape, each slice labelled on its own (true 2-D
    8-connectivity of the slice)."""
    v = vol.contiguous()
    if v.dim() != 3 or not v.is_cuda:
        raise ValueError("expected a 3-D CUDA tensor (slices, n_slow, n_fast)")
    if v.dtype in (torch.bool, torch.uint8):
        code, v = _lib.PH_BOOL, v.view(torch.uint8)
    elif v.dtype == torch.float32:
        code = _lib.PH_F32
    else:
        raise TypeError(f"input must be Float32 or Bool, got {v.dtype}")
    out = torch.empty(v.shape, dtype=torch.int32, device=v.device)
    dev = v.device.index if v.device.index is not None else torch.cuda.current_device()
    _lib.default_context(dev).call("ph_ccl_batch", out.data_ptr(), v.data_ptr(), code, int(v.shape[0]),
                                   int(v.shape[1]), int(v.shape[2]), torch.cuda.current_stream(dev).cuda_stream)
    return out.view(torch.uint32) if hasattr(torch, "uint32") else out


def cu_bounding_rectangles(labels: torch.Tensor) -> np.ndarray:
    """get_bounding_rectangles (ccl.jl:240-264) on the device for every component
    of a label image ``(n_slow, n_fast)`` or label volume ``(slices, n_slow, n_fast)``.

    Returns an int64 array of rows ``(root, x_min, y_min, x_max, y_max)``: the
    global 1-based root index and the 1-based box, x the slow axis (the
    reference's column j) and y the fast axis (its row i), ordered by root.
    """
    lab = _labels_on_device(labels)
    shape = tuple(lab.shape)
    slices, rows, cols = (1,) + shape if len(shape) == 2 else shape
    dev = lab.device.index if lab.device.index is not None else torch.cuda.current_device()
    ctx = _lib.default_context(dev)
    s = torch.cuda.current_stream(dev).cuda_stream
    count = ctypes.c_int64(0)
    ctx.call("ph_ccl_boxes", None, 0, ctypes.byref(count), lab.data_ptr(), slices, rows, cols, s)
    out = np.empty((max(count.value, 1), 5), dtype=np.int64)
    ctx.call("ph_ccl_boxes", out.ctypes.data, int(count.value), ctypes.byref(count), lab.data_ptr(), slices, rows,
             cols, s)
    return out[:count.value]


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
