"""Preprocessing of utils.jl on the device: the background images of a
recording (make_background, cu_make_background_mode) and pad_with_mean."""
from __future__ import annotations

import numpy as np
import torch

from .holofunc import _ctx_stream, _need


def _stack(images, device) -> torch.Tensor:
    if isinstance(images, torch.Tensor):
        st = images
    else:
        st = torch.from_numpy(np.ascontiguousarray(np.stack([np.asarray(i) for i in images])))
    if st.dtype != torch.uint8:
        # the reference's conversion of N0f8/Float images: round(UInt8, clamp(x * 255, 0, 255))
        st = torch.round(torch.clamp(st.float() * 255, 0, 255)).to(torch.uint8)
    dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
    return st.to(dev).contiguous()


def _background(entry: str, images, device) -> np.ndarray:
    st = _stack(images, device)
    if st.dim() != 3:
        raise ValueError("images must be a stack (count, n_slow, n_fast)")
    out = torch.empty(tuple(st.shape[1:]), dtype=torch.float64, device=st.device)
    ctx, s = _ctx_stream(st)
    ctx.call(entry, out.data_ptr(), st.data_ptr(), int(st.shape[0]), int(st.shape[2]), int(st.shape[1]), s)
    return out.cpu().numpy()


def cu_make_background_mode(grayimglist, device: int | None = None) -> np.ndarray:
    """utils.jl:279-317: the per-pixel intensity mode of a list of UInt8 (or
    N0f8 / Float) images, as a host Float64 array of value / 255."""
    return _background("ph_background_mode", grayimglist, device)


def make_background(images, mode: str = "mode", device: int | None = None) -> np.ndarray:
    """utils.jl:210-231 on images already loaded (the reference takes file paths):
    ``mode="mode"`` the per-pixel mode, ``mode="mean"`` the per-pixel mean."""
    if mode == "mode":
        return cu_make_background_mode(images, device)
    if mode == "mean":
        return _background("ph_background_mean", images, device)
    raise ValueError(f"mode must be 'mode' or 'mean'. Got {mode!r}")


def pad_with_mean(img: torch.Tensor, padsize: int) -> torch.Tensor:
    """utils.jl:319-325: a padsize x padsize Float32 array of mean(img) with
    ``img`` (CUDA Float32, shape (n_slow, n_fast)) placed in the centre."""
    t = _need(img, torch.float32, "img")
    out = torch.empty((int(padsize), int(padsize)), dtype=torch.float32, device=t.device)
    ctx, s = _ctx_stream(t)
    ctx.call("ph_pad_with_mean", out.data_ptr(), t.data_ptr(), int(t.shape[1]), int(t.shape[0]), int(padsize), s)
    return out
