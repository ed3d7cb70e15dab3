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
