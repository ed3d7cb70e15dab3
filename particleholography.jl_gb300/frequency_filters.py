"""Host mirror of ParticleHolography.jl src/frequency_filters.jl over libphgb300.

The masks are built by device kernels; applying one is a forward FFT, the
mask multiply folded into the column pass, and an inverse FFT.
"""
from __future__ import annotations

import torch

from .holofunc import _ctx_stream, _data, _need
from .types import CuLowPassFilter, CuWavefront

__all__ = ["cu_rectangle_filter", "cu_super_gaussian_filter", "cu_apply_low_pass_filter",
           "cu_apply_low_pass_filter_"]


def _mask(entry: str, prop_dist: float, wavlen: float, imglen: int, pixel_pitch: float, device) -> CuLowPassFilter:
    dev = torch.cuda.current_device() if device is None else device
    out = torch.empty((imglen, imglen), dtype=torch.float32, device=f"cuda:{dev}")
    ctx, s = _ctx_stream(out)
    ctx.call(entry, out.data_ptr(), int(imglen), float(prop_dist), float(wavlen), float(pixel_pitch), s)
    return CuLowPassFilter(out)


def cu_rectangle_filter(prop_dist: float, wavlen: float, imglen: int, pixel_picth: float,
                        device: int | None = None) -> CuLowPassFilter:
    """frequency_filters.jl:31-38."""
    return _mask("ph_lpf_rectangle", prop_dist, wavlen, imglen, pixel_picth, device)


def cu_super_gaussian_filter(prop_dist: float, wavlen: float, imglen: int, pixel_picth: float,
                             device: int | None = None) -> CuLowPassFilter:
    """frequency_filters.jl:66-74."""
    return _mask("ph_lpf_super_gaussian", prop_dist, wavlen, imglen, pixel_picth, device)


def _apply(out: torch.Tensor, holo: torch.Tensor, lpf: torch.Tensor) -> None:
    ctx, s = _ctx_stream(holo)
    ctx.call("ph_apply_lpf", out.data_ptr(), holo.data_ptr(), lpf.data_ptr(), int(holo.shape[1]),
             int(holo.shape[0]), s)


def cu_apply_low_pass_filter_(holo: CuWavefront, lpf: CuLowPassFilter) -> None:
    """frequency_filters.jl:88-91 (``cu_apply_low_pass_filter!``): in place."""
    h = _need(_data(holo), torch.complex64, "holo")
    m = _need(_data(lpf), torch.float32, "lpf")
    if tuple(h.shape) != tuple(m.shape):
        raise AssertionError(f"holo and lpf must have the same size. Got {tuple(h.shape)}, {tuple(m.shape)}.")
    _apply(h, h, m)


def cu_apply_low_pass_filter(holo: CuWavefront, lpf: CuLowPassFilter) -> CuWavefront:
    """frequency_filters.jl:105-107: a filtered copy."""
    h = _need(_data(holo), torch.complex64, "holo")
    m = _need(_data(lpf), torch.float32, "lpf")
    if tuple(h.shape) != tuple(m.shape):
        raise AssertionError(f"holo and lpf must have the same size. Got {tuple(h.shape)}, {tuple(m.shape)}.")
    out = torch.empty_like(h)
    _apply(out, h, m)
    return CuWavefront(out)
