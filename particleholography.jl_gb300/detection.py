"""The device side of particle_bounding_boxes (particle_detection.jl:58-96):
the thresholded reconstruction volume and the per-slice component boxes.

The reference reconstructs a volume, thresholds it, then labels and boxes
every slice from a host loop (CCL, a device-to-host copy and CPU bounding
rectangles per slice).  Here the threshold is the reconstruction's own
epilogue (``ph_reconst_binary_vol``), all slices are labelled in one launch
set and the boxes are reduced on the device.  The merging of boxes across
slices into particle neighbourhoods (gen_particle_neighborhoods and its
UUID bookkeeping) is host logic and stays with the caller.
"""
from __future__ import annotations

import numpy as np
import torch

from .ccl import cu_bounding_rectangles, cu_connected_component_labeling_batch
from .holofunc import _check_same, _ctx_stream, _recon_args


def cu_get_reconst_binary_vol(wavefront, transfer_front, transfer_dz, slices: int, threshold: float,
                              return_proj: bool = False):
    """``cu_get_reconst_vol(..., Float32) .<= threshold`` (holofunc.jl:184-200)
    as a Bool volume of shape ``(slices, n_slow, n_fast)``, in one pass."""
    wf, tf, td = _recon_args(wavefront, transfer_front, transfer_dz)
    _check_same(wf, tf, td)
    vol = torch.empty((int(slices),) + tuple(wf.shape), dtype=torch.bool, device=wf.device)
    proj = torch.empty(wf.shape, dtype=torch.float32, device=wf.device) if return_proj else None
    ctx, s = _ctx_stream(wf)
    ctx.call("ph_reconst_binary_vol", vol.data_ptr(), float(threshold), proj.data_ptr() if proj is not None else None,
             wf.data_ptr(), tf.data_ptr(), td.data_ptr(), int(wf.shape[1]), int(wf.shape[0]), int(slices), s)
    return (vol, proj) if return_proj else vol


def slice_bounding_boxes(bin_vol: torch.Tensor) -> list:
    """Per slice of a binary volume ``(slices, n_slow, n_fast)``: an int64 array of
    rows ``(root, x_min, y_min, x_max, y_max)`` as get_bounding_rectangles
    (ccl.jl:240-264) gives for that slice's labels (root 1-based within the slice)."""
    labels = cu_connected_component_labeling_batch(bin_vol)
    boxes = cu_bounding_rectangles(labels)
    per = int(bin_vol.shape[1]) * int(bin_vol.shape[2])
    out = [np.empty((0, 5), dtype=np.int64) for _ in range(int(bin_vol.shape[0]))]
    if len(boxes):
        k = (boxes[:, 0] - 1) // per
        for s in np.unique(k):
            b = boxes[k == s].copy()
            b[:, 0] -= s * per
            out[int(s)] = b
    return out


def cu_reconst_subvolumes(wavefront, transfer_front, transfer_dz, slices: int, boxes) -> list:
    """The N0f8 sub-volumes particle_coordinates cuts out of ``cu_get_reconst_vol``
    (particle_detection.jl:146-208), computed without the volume.  ``boxes``:
    rows ``(x_min, y_min, z_min, x_max, y_max, z_max)`` (particle_bbs order,
    1-based inclusive, x the slow axis, y the fast axis).  Returns one uint8
    tensor per box, shape ``(z, x, y)`` (raw N0f8 levels)."""
    import ctypes
    wf, tf, td = _recon_args(wavefront, transfer_front, transfer_dz)
    _check_same(wf, tf, td)
    bx = np.ascontiguousarray(np.asarray(boxes, dtype=np.int64).reshape(-1, 6))
    count = len(bx)
    offs = np.zeros(count + 1, dtype=np.int64)
    ctx, s = _ctx_stream(wf)
    nx, ny = int(wf.shape[1]), int(wf.shape[0])
    ctx.call("ph_reconst_subvolumes", None, offs.ctypes.data, bx.ctypes.data if count else None, count, None, None,
             None, nx, ny, int(slices), s)
    out = torch.empty(max(int(offs[-1]), 1), dtype=torch.uint8, device=wf.device)
    if count:
        ctx.call("ph_reconst_subvolumes", out.data_ptr(), offs.ctypes.data, bx.ctypes.data, count, wf.data_ptr(),
                 tf.data_ptr(), td.data_ptr(), nx, ny, int(slices), s)
    res = []
    for i, (x0, y0, z0, x1, y1, z1) in enumerate(bx.tolist()):
        shape = (z1 - z0 + 1, x1 - x0 + 1, y1 - y0 + 1)
        res.append(out[int(offs[i]):int(offs[i + 1])].view(shape))
    return res


def _gaussian_kernel(sigma: float = 5.0) -> np.ndarray:
    """ImageFiltering's Kernel.gaussian((sigma,)): 4 ceil(sigma) + 1 taps, sum 1."""
    h = 2 * int(np.ceil(sigma))
    x = np.arange(-h, h + 1, dtype=np.float64)
    k = np.exp(-x * x / (2 * sigma * sigma))
    return k / k.sum()


def particle_coordinates(boxes, subvols, sigma: float = 5.0) -> np.ndarray:
    """particle_coordinates (particle_detection.jl:146-160) on device sub-volumes:
    per box, the Tamura depth profile (std / mean of each slice), smoothed with
    the Gaussian kernel (replicated ends), its first maximum z, and the centre of
    mass of that slice.  Returns rows (x, y, z) in the reference's 1-based
    volume coordinates (float64 host arithmetic)."""
    k = _gaussian_kernel(sigma)
    h = len(k) // 2
    out = []
    for (x0, y0, z0, *_), sv in zip(np.asarray(boxes, dtype=np.int64).reshape(-1, 6).tolist(), subvols):
        v = sv.cpu().numpy().astype(np.float64) / 255.0                     # (z, x, y)
        prof = np.array([sl.std(ddof=1) / sl.mean() if sl.size > 1 and sl.mean() != 0 else 0.0 for sl in v])
        padded = np.concatenate([np.full(h, prof[0]), prof, np.full(h, prof[-1])])
        smooth = np.array([np.dot(padded[i:i + len(k)], k) for i in range(len(prof))])
        z = int(np.argmax(smooth))
        sl = v[z]                                                            # (x = column j, y = row i)
        tot = sl.sum()
        jj, ii = np.meshgrid(np.arange(1, sl.shape[0] + 1), np.arange(1, sl.shape[1] + 1), indexing="ij")
        x = (jj * sl).sum() / tot
        y = (ii * sl).sum() / tot
        out.append((x + x0 - 1, y + y0 - 1, z + 1 + z0 - 1))
    return np.array(out, dtype=np.float64).reshape(-1, 3)
