"""Host mirror of ParticleHolography.jl src/holofunc.jl over libphgb300.

Same function names, argument order and meaning, and the same failures
(``AssertionError`` with the reference's message where it ``@assert``s,
``ValueError`` where it throws ``ArgumentError``).  Every function launches
the sm_103a kernels through the C ABI on the current torch CUDA stream of the
input's device; nothing here computes on the CPU.

Arrays are torch CUDA tensors; a Julia ``(n_fast, n_slow)`` array is a tensor
of shape ``(n_slow, n_fast)`` and a Julia ``(n_fast, n_slow, slices)`` volume
is ``(slices, n_slow, n_fast)``.
"""
from __future__ import annotations

import torch

from . import _lib
from .types import CuTransfer, CuTransferSqrtPart, CuWavefront, N0f8

__all__ = [
    "cu_transfer_sqrt_arr", "cu_transfer", "cu_transfer_fp64", "cu_gabor_wavefront", "cu_phase_retrieval_holo",
    "cu_get_reconst_vol", "cu_get_reconst_xyprojection", "cu_get_reconst_vol_and_xyprojection",
    "cu_get_reconst_complex_vol", "cu_asm_prop_", "cu_2d_pad", "cu_get_reconst_vol_and_xyprojection_padded",
]

_RETURN_DTYPES = {
    N0f8: (_lib.PH_N0F8, torch.uint8),
    torch.float16: (_lib.PH_F16, torch.float16),
    torch.float32: (_lib.PH_F32, torch.float32),
    torch.float64: (_lib.PH_F64, torch.float64),
}


def _device_index(t: torch.Tensor) -> int:
    if not t.is_cuda:
        raise TypeError("libphgb300 works on CUDA tensors (CuArray); got a CPU tensor")
    return t.device.index if t.device.index is not None else torch.cuda.current_device()


def _ctx_stream(t: torch.Tensor):
    dev = _device_index(t)
    return _lib.default_context(dev), torch.cuda.current_stream(dev).cuda_stream


def _data(x) -> torch.Tensor:
    return x.data if hasattr(x, "data") and isinstance(x.data, torch.Tensor) else x


def _need(t: torch.Tensor, dtype: torch.dtype, what: str) -> torch.Tensor:
    if t.dtype != dtype:
        raise TypeError(f"{what} must be {dtype}, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{what} must be contiguous")
    return t


def _jsize(t: torch.Tensor) -> tuple:
    """Julia-order size of a tensor (reversed shape)."""
    return tuple(int(s) for s in reversed(t.shape))


def _return_code(return_type):
    if return_type in _RETURN_DTYPES:
        return _RETURN_DTYPES[return_type]
    raise ValueError(f"return_type must be Subtype of AbstractFloat or N0f8. Got {return_type}")


# ------------------------------------------------------------------ transfer functions

def cu_transfer_sqrt_arr(datlen: int, wavlen: float, dx: float, device: int | None = None,
                         n_slow: int | None = None) -> CuTransferSqrtPart:
    """holofunc.jl:30-36: the Float32 square-root term of the transfer function.
    ``n_slow`` (an extension; the reference is square): rows of a datlen-wide grid."""
    dev = torch.cuda.current_device() if device is None else device
    ny = datlen if n_slow is None else int(n_slow)
    out = torch.empty((ny, datlen), dtype=torch.float32, device=f"cuda:{dev}")
    ctx, s = _ctx_stream(out)
    ctx.call("ph_transfer_sqrt", out.data_ptr(), datlen, ny, float(wavlen), float(dx), s)
    return CuTransferSqrtPart(out)


def cu_transfer(z0: float, datLen: int, wavLen: float, d_sqr: CuTransferSqrtPart) -> CuTransfer:
    """holofunc.jl:61-67: ``exp(2im*pi*z0/wavLen*sqrt(d_sqr))`` as ComplexF32."""
    d = _need(_data(d_sqr), torch.float32, "d_sqr")
    if d.dim() != 2 or int(d.shape[1]) != datLen:   # rows may differ (non-square grids from n_slow)
        raise AssertionError(f"d_sqr must have size ({datLen}, {datLen}). Got {_jsize(d)}.")
    ny = int(d.shape[0])
    out = torch.empty((ny, datLen), dtype=torch.complex64, device=d.device)
    ctx, s = _ctx_stream(out)
    ctx.call("ph_transfer", out.data_ptr(), d.data_ptr(), datLen, ny, float(z0), float(wavLen), s)
    return CuTransfer(out)


def cu_transfer_fp64(z: float, datlen: int, wavlen: float, dx: float, device: int | None = None,
                     n_slow: int | None = None) -> CuTransfer:
    """No reference counterpart: the transfer function with the square-root term
    in FP64 (exact physics) on the same centred grid as ``cu_transfer``."""
    dev = torch.cuda.current_device() if device is None else device
    ny = datlen if n_slow is None else int(n_slow)
    out = torch.empty((ny, datlen), dtype=torch.complex64, device=f"cuda:{dev}")
    ctx, s = _ctx_stream(out)
    ctx.call("ph_transfer_fp64", out.data_ptr(), datlen, ny, float(z), float(wavlen), float(dx), s)
    return CuTransfer(out)


# ------------------------------------------------------------------ wavefronts

def cu_gabor_wavefront(holo: torch.Tensor) -> CuWavefront:
    """holofunc.jl:80-82: ``ComplexF32.(sqrt.(holo) .+ 0.0im)``."""
    h = _need(_data(holo), torch.float32, "holo")
    out = torch.empty(h.shape, dtype=torch.complex64, device=h.device)
    ctx, s = _ctx_stream(h)
    ctx.call("ph_gabor_wavefront", out.data_ptr(), h.data_ptr(), int(h.shape[1]), int(h.shape[0]), s)
    return CuWavefront(out)


def cu_2d_pad(inarr) -> torch.Tensor:
    """holofunc.jl:139-149: pad to twice the size with the mean value."""
    x = _need(_data(inarr), torch.complex64, "inarr")
    n = int(x.shape[1])
    out = torch.empty((2 * n, 2 * n), dtype=torch.complex64, device=x.device)
    ctx, s = _ctx_stream(x)
    ctx.call("ph_pad2d", out.data_ptr(), x.data_ptr(), n, int(x.shape[0]), s)
    return out


def cu_phase_retrieval_holo(holo1: torch.Tensor, holo2: torch.Tensor, transfer: CuTransfer, invtransfer: CuTransfer,
                            priter: int, datlen: int, return_residual: bool = False):
    """holofunc.jl:100-129: Gerchberg-Saxton phase retrieval.

    With ``return_residual`` also returns ``|| |u2| - sqrt(I2) || / || sqrt(I2) ||``
    (FP64, before the last amplitude replacement at plane 2) as a 0-d CUDA
    float64 tensor -- a quantity the reference does not compute.
    """
    h1 = _need(_data(holo1), torch.float32, "holo1")
    h2 = _need(_data(holo2), torch.float32, "holo2")
    t = _need(_data(transfer), torch.complex64, "transfer")
    ti = _need(_data(invtransfer), torch.complex64, "invtransfer")
    shape = (datlen, datlen)
    if not (tuple(h1.shape) == tuple(h2.shape) == tuple(t.shape) == tuple(ti.shape) == shape):
        raise AssertionError(
            f"All arrays must have the same size as ({datlen}, {datlen}). Got {_jsize(h1)}, {_jsize(h2)}, "
            f"{_jsize(t)}, {_jsize(ti)}.")
    out = torch.empty(shape, dtype=torch.complex64, device=h1.device)
    res = torch.zeros((), dtype=torch.float64, device=h1.device) if return_residual else None
    ctx, s = _ctx_stream(h1)
    ctx.call("ph_phase_retrieval", out.data_ptr(), h1.data_ptr(), h2.data_ptr(), t.data_ptr(), ti.data_ptr(),
             datlen, datlen, int(priter), res.data_ptr() if res is not None else None, s)
    if return_residual:
        return CuWavefront(out), res
    return CuWavefront(out)


# ------------------------------------------------------------------ propagation / reconstruction

def cu_asm_prop_(outholo: CuWavefront, inholo: CuWavefront, d_sqr: CuTransferSqrtPart, zprop: float, datlen: int,
                 wavlen: float) -> None:
    """holofunc.jl:383-388 (``cu_asm_prop!``): propagate ``inholo`` by ``zprop`` into ``outholo``."""
    o = _need(_data(outholo), torch.complex64, "outholo")
    i = _need(_data(inholo), torch.complex64, "inholo")
    d = _need(_data(d_sqr), torch.float32, "d_sqr")
    if not (tuple(o.shape) == tuple(i.shape) == tuple(d.shape) == (datlen, datlen)):
        raise AssertionError(f"All arrays must have the same size as ({datlen}, {datlen}). "
                             f"Got {_jsize(o)}, {_jsize(i)}, {_jsize(d)}.")
    ctx, s = _ctx_stream(i)
    ctx.call("ph_asm_prop", o.data_ptr(), i.data_ptr(), d.data_ptr(), float(zprop), datlen, datlen, float(wavlen), s)


def _recon_args(wavefront, transfer_front, transfer_dz):
    wf = _need(_data(wavefront), torch.complex64, "wavefront")
    tf = _need(_data(transfer_front), torch.complex64, "transfer_front")
    td = _need(_data(transfer_dz), torch.complex64, "transfer_dz")
    return wf, tf, td


def _check_same(wf, tf, td):
    if not (tuple(wf.shape) == tuple(tf.shape) == tuple(td.shape)):
        raise AssertionError(f"All arrays must have the same size. Got {_jsize(wf)}, {_jsize(tf)}, {_jsize(td)}.")


def cu_get_reconst_xyprojection(wavefront: CuWavefront, transfer_front: CuTransfer, transfer_dz: CuTransfer,
                                slices: int, return_argmin: bool = False):
    """holofunc.jl:248-266: per-pixel minimum over slices of |slice|^2 (unclamped).

    ``return_argmin`` also returns the 0-based slice index of the first minimum
    (int32), which the reference does not compute.  The volume is never stored.
    """
    wf, tf, td = _recon_args(wavefront, transfer_front, transfer_dz)
    _check_same(wf, tf, td)
    proj = torch.empty(wf.shape, dtype=torch.float32, device=wf.device)
    arg = torch.empty(wf.shape, dtype=torch.int32, device=wf.device) if return_argmin else None
    ctx, s = _ctx_stream(wf)
    ctx.call("ph_reconst_xyproj", proj.data_ptr(), arg.data_ptr() if arg is not None else None, wf.data_ptr(),
             tf.data_ptr(), td.data_ptr(), int(wf.shape[1]), int(wf.shape[0]), int(slices), s)
    return (proj, arg) if return_argmin else proj


def cu_get_reconst_xyprojection_lpf(wavefront: CuWavefront, transfer_front: CuTransfer, transfer_dz: CuTransfer,
                                    lpf, slices: int, return_argmin: bool = False):
    """``cu_apply_low_pass_filter`` (frequency_filters.jl:88-107) then
    ``cu_get_reconst_xyprojection`` (holofunc.jl:248-266) in one call: the
    filter multiplies the spectrum the reconstruction already forms, so the
    filter's own inverse/forward FFT pair disappears."""
    wf, tf, td = _recon_args(wavefront, transfer_front, transfer_dz)
    _check_same(wf, tf, td)
    m = _need(_data(lpf), torch.float32, "lpf")
    if tuple(m.shape) != tuple(wf.shape):
        raise AssertionError(f"All arrays must have the same size. Got {_jsize(wf)}, {_jsize(m)}.")
    proj = torch.empty(wf.shape, dtype=torch.float32, device=wf.device)
    arg = torch.empty(wf.shape, dtype=torch.int32, device=wf.device) if return_argmin else None
    ctx, s = _ctx_stream(wf)
    ctx.call("ph_reconst_xyproj_lpf", proj.data_ptr(), arg.data_ptr() if arg is not None else None, wf.data_ptr(),
             tf.data_ptr(), td.data_ptr(), m.data_ptr(), int(wf.shape[1]), int(wf.shape[0]), int(slices), s)
    return (proj, arg) if return_argmin else proj


def _reconst_vol(wavefront, transfer_front, transfer_dz, slices, return_type, with_proj):
    wf, tf, td = _recon_args(wavefront, transfer_front, transfer_dz)
    _check_same(wf, tf, td)
    code, dtype = _return_code(return_type)
    vol = torch.empty((int(slices),) + tuple(wf.shape), dtype=dtype, device=wf.device)
    proj = torch.empty(wf.shape, dtype=torch.float32, device=wf.device) if with_proj else None
    ctx, s = _ctx_stream(wf)
    ctx.call("ph_reconst_vol", vol.data_ptr(), code, proj.data_ptr() if proj is not None else None, wf.data_ptr(),
             tf.data_ptr(), td.data_ptr(), int(wf.shape[1]), int(wf.shape[0]), int(slices), s)
    return (vol, proj) if with_proj else vol


def cu_get_reconst_vol(wavefront: CuWavefront, transfer_front: CuTransfer, transfer_dz: CuTransfer, slices: int,
                       return_type=N0f8) -> torch.Tensor:
    """holofunc.jl:184-200: the clamped intensity volume as ``return_type``
    (N0f8 -> uint8 raw)."""
    return _reconst_vol(wavefront, transfer_front, transfer_dz, slices, return_type, False)


def cu_get_reconst_complex_vol(wavefront: CuWavefront, transfer_front: CuTransfer, transfer_dz: CuTransfer,
                               slices: int) -> torch.Tensor:
    """holofunc.jl:216-232: the complex amplitude volume (ComplexF32)."""
    wf, tf, td = _recon_args(wavefront, transfer_front, transfer_dz)
    _check_same(wf, tf, td)
    vol = torch.empty((int(slices),) + tuple(wf.shape), dtype=torch.complex64, device=wf.device)
    ctx, s = _ctx_stream(wf)
    ctx.call("ph_reconst_vol", vol.data_ptr(), _lib.PH_C64, None, wf.data_ptr(), tf.data_ptr(), td.data_ptr(),
             int(wf.shape[1]), int(wf.shape[0]), int(slices), s)
    return vol


def cu_get_reconst_vol_and_xyprojection(wavefront: CuWavefront, transfer_front: CuTransfer, transfer_dz: CuTransfer,
                                        slices: int, return_type=N0f8):
    """holofunc.jl:300-321: the volume and its strict-< minimum projection (Float32)."""
    return _reconst_vol(wavefront, transfer_front, transfer_dz, slices, return_type, True)


def cu_get_reconst_vol_and_xyprojection_padded(wavefront: CuWavefront, transfer_front: CuTransfer,
                                               transfer_dz: CuTransfer, slices: int, return_type=N0f8):
    """holofunc.jl:339-364: mean-padded reconstruction, N0f8 centre-crop volume
    and its projection."""
    wf, tf, td = _recon_args(wavefront, transfer_front, transfer_dz)
    expected = tuple(2 * s for s in wf.shape)
    if not (expected == tuple(tf.shape) == tuple(td.shape)):
        raise AssertionError(
            "size(transfer_front.data) and size(transfer_dz.data) must be equal to 2*size(wavefront.data). "
            f"Got {_jsize(wf)}, {_jsize(tf)}, {_jsize(td)}.")
    code, _ = _return_code(return_type)
    datlen = int(wf.shape[1])
    vol = torch.empty((int(slices), datlen, datlen), dtype=torch.uint8, device=wf.device)
    proj = torch.empty((datlen, datlen), dtype=torch.float32, device=wf.device)
    ctx, s = _ctx_stream(wf)
    ctx.call("ph_reconst_vol_padded", vol.data_ptr(), proj.data_ptr(), wf.data_ptr(), tf.data_ptr(), td.data_ptr(),
             datlen, int(wf.shape[0]), int(slices), code, s)
    return vol, proj
