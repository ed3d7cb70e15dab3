"""Reference-semantics FP32 oracle of ParticleHolography.jl's reconstruction path.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``): imported by tests, by
``__graft_entry__.smoke()`` as the checker and by ``bench.py``'s CPU baseline.

Every function restates one function of the reference, step by step, on the
CPU with numpy / scipy.fft in complex64, so that the rounding points match the
reference's: Float32 square-root term, Float64 ``exp`` rounded to ComplexF32,
complex64 cumulative transfer products, ``clamp`` then ``round`` half-to-even
for N0f8, strict ``<`` when projecting a stored volume.

Array convention: a Julia array of size ``(n_fast, n_slow)`` (column-major) is
held here as a C-ordered numpy array of shape ``(n_slow, n_fast)``; element
``A[x, y]`` (1-based Julia) is ``a[y - 1, x - 1]``.  A volume of Julia size
``(n_fast, n_slow, slices)`` is held as shape ``(slices, n_slow, n_fast)``.
All reference functions are square-only (``datlen``); the shape is carried
per axis here so rectangular inputs follow the same formulas.

The FFT itself is scipy's single-precision pocketfft standing in for cuFFT
(which the reference calls through CUDA.jl, version unpinned): both round in
complex64, neither is bit-identical to the other.
"""
from __future__ import annotations

import os

import numpy as np
import scipy.fft as sfft

N0f8 = "N0f8"                       # FixedPointNumbers.N0f8 stand-in (UInt8 raw / 255)
RETURN_TYPES = (N0f8, np.float16, np.float32, np.float64)


def _workers() -> int:
    return len(os.sched_getaffinity(0))


def _fft2(x: np.ndarray) -> np.ndarray:
    """CUFFT.fft on a complex64 matrix: unnormalised forward 2-D DFT in FP32."""
    return sfft.fft2(np.asarray(x, dtype=np.complex64), workers=_workers())


def _ifft2(x: np.ndarray) -> np.ndarray:
    """CUFFT.ifft: inverse 2-D DFT normalised by 1/(n_fast*n_slow), in FP32."""
    return sfft.ifft2(np.asarray(x, dtype=np.complex64), workers=_workers())


fftshift = np.fft.fftshift        # AbstractFFTs.fftshift: circshift by floor(n/2)
ifftshift = np.fft.ifftshift      # AbstractFFTs.ifftshift: circshift by -floor(n/2)


# ---------------------------------------------------------------- transfer

def transfer_sqrt_arr(datlen: int, wavlen: float, dx: float, n_slow: int | None = None) -> np.ndarray:
    """``cu_transfer_sqrt_arr`` (holofunc.jl:30-36) and its kernel (holofunc.jl:8-15).

    ``Plane[x, y] = 1.0 - ((x - datLen/2 - 1.0)*wavLen/datLen/dx)^2
    - ((y - datLen/2 - 1.0)*wavLen/datLen/dx)^2`` evaluated in Float64 with the
    reference's left-to-right operation order and stored as Float32.
    """
    nx = int(datlen)
    ny = nx if n_slow is None else int(n_slow)
    x = np.arange(1, nx + 1, dtype=np.float64)
    y = np.arange(1, ny + 1, dtype=np.float64)
    tx = (((x - nx / 2) - 1.0) * wavlen) / nx / dx
    ty = (((y - ny / 2) - 1.0) * wavlen) / ny / dx
    plane = (1.0 - (tx * tx)[None, :]) - (ty * ty)[:, None]
    return plane.astype(np.float32)


def transfer(z0: float, datlen: int, wavlen: float, d_sqr: np.ndarray) -> np.ndarray:
    """``cu_transfer`` (holofunc.jl:61-67) and its kernel (holofunc.jl:38-45).

    ``exp(2im*pi*z0/wavLen*sqrt(d_sqr))``: the square root is taken in Float32
    on the Float32 ``d_sqr``; the product and ``exp`` are ComplexF64; the store
    rounds to ComplexF32.
    """
    d = np.asarray(d_sqr, dtype=np.float32)
    with np.errstate(invalid="ignore"):
        s = np.sqrt(d).astype(np.float64)             # Float32 sqrt, then promoted
    c = ((2.0 * np.pi) * z0) / wavlen
    phase = c * s
    return (np.cos(phase) + 1j * np.sin(phase)).astype(np.complex64)


def gabor_wavefront(holo: np.ndarray) -> np.ndarray:
    """``cu_gabor_wavefront`` (holofunc.jl:80-82): ``ComplexF32.(sqrt.(holo) .+ 0.0im)``."""
    return np.sqrt(np.asarray(holo, dtype=np.float32)).astype(np.complex64)


# ---------------------------------------------------------------- propagation

def _propagate(x: np.ndarray, tf: np.ndarray) -> np.ndarray:
    """``ifft(ifftshift(fftshift(fft(x)) .* tf))`` in complex64 (holofunc.jl:114,121,386)."""
    return _ifft2(ifftshift(fftshift(_fft2(x)) * np.asarray(tf, dtype=np.complex64))).astype(np.complex64)


def _amplitude_replace(sqrt_i: np.ndarray, light: np.ndarray) -> np.ndarray:
    """``sqrtI .* exp.(1.0im .* angle.(light))`` (holofunc.jl:115,118 and :122,125).

    ``angle`` is the Float32 ``atan(imag, real)`` (so ``angle(0) == 0``); the
    ``exp`` and the product are ComplexF64, rounded to ComplexF32 on store.
    """
    phi = np.angle(light).astype(np.float32).astype(np.float64)
    s = sqrt_i.astype(np.float64)
    return (s * np.cos(phi) + 1j * (s * np.sin(phi))).astype(np.complex64)


def phase_retrieval_holo(holo1, holo2, transfer_, invtransfer, priter: int, datlen: int,
                         return_residual: bool = False):
    """``cu_phase_retrieval_holo`` (holofunc.jl:100-129), Gerchberg-Saxton.

    Returns the retrieved wavefront at the plane of ``holo1``.  With
    ``return_residual`` it also returns ``|| |u2| - sqrt(I2) ||_2 / ||sqrt(I2)||_2``
    measured (in FP64) just before STEP2 of the last iteration -- a quantity the
    reference does not compute, added for the GS accuracy report.
    """
    holo1 = np.asarray(holo1, dtype=np.float32)
    holo2 = np.asarray(holo2, dtype=np.float32)
    shape = (datlen, datlen)
    if not (holo1.shape == holo2.shape == np.shape(transfer_) == np.shape(invtransfer) == shape):
        raise AssertionError(
            f"All arrays must have the same size as ({datlen}, {datlen}). Got {holo1.shape}, "
            f"{holo2.shape}, {np.shape(transfer_)}, {np.shape(invtransfer)}.")
    sqrt_i1 = np.sqrt(holo1)
    sqrt_i2 = np.sqrt(holo2)
    light1 = sqrt_i1.astype(np.complex64)
    residual = None
    for it in range(priter):
        light2 = _propagate(light1, transfer_)                       # STEP1
        if return_residual and it == priter - 1:
            a = np.abs(light2.astype(np.complex128))
            s2 = sqrt_i2.astype(np.float64)
            residual = float(np.linalg.norm(a - s2) / np.linalg.norm(s2))
        light2 = _amplitude_replace(sqrt_i2, light2)                 # STEP2
        light1 = _propagate(light2, invtransfer)                     # STEP3
        light1 = _amplitude_replace(sqrt_i1, light1)                 # STEP4
    if return_residual:
        return light1, residual
    return light1


def pad2d(inarr: np.ndarray) -> np.ndarray:
    """``cu_2d_pad`` (holofunc.jl:139-149): 2x size, filled with ``mean(inarr)``,
    input placed at 1-based rows/cols ``outlen÷4+1 : outlen÷4+inlen``."""
    inarr = np.asarray(inarr, dtype=np.complex64)
    inlen = inarr.shape[1]                      # size(inarr, 1): the fast axis
    outlen = 2 * inlen
    mean = np.complex64(inarr.astype(np.complex128).mean())
    out = np.full((outlen, outlen), mean, dtype=np.complex64)
    o = outlen // 4
    out[o:o + inarr.shape[0], o:o + inlen] = inarr
    return out


def asm_prop(inholo: np.ndarray, d_sqr: np.ndarray, zprop: float, datlen: int, wavlen: float) -> np.ndarray:
    """``cu_asm_prop!`` (holofunc.jl:383-388): builds ``cu_transfer(zprop, ...)``
    then ``ifft(ifftshift(fftshift(fft(in)) .* tf))``."""
    tf = transfer(zprop, datlen, wavlen, d_sqr)
    return _propagate(inholo, tf)


# ---------------------------------------------------------------- reconstruction

def _intensity(field: np.ndarray) -> np.ndarray:
    """``abs2`` of ComplexF32 (also equal to ``abs(x*conj(x))``, holofunc.jl:257)."""
    re = field.real.astype(np.float32)
    im = field.imag.astype(np.float32)
    return (re * re + im * im).astype(np.float32)


def normedfloat_to_n0f8(val: np.ndarray) -> np.ndarray:
    """``_normedfloat_to_N0f8`` (holofunc.jl:154-156): ``round(UInt8, clamp(v,0,1)*255)``,
    Float32 product, round half to even.  Returned as the raw UInt8."""
    v = np.clip(np.asarray(val, dtype=np.float32), np.float32(0.0), np.float32(1.0))
    return np.rint(v * np.float32(255.0)).astype(np.uint8)


def _convert(intensity_clamped: np.ndarray, return_type):
    if return_type is N0f8 or return_type == N0f8:
        return normedfloat_to_n0f8(intensity_clamped)
    if return_type in (np.float16, np.float32, np.float64):
        return intensity_clamped.astype(return_type)
    raise ValueError(f"return_type must be Subtype of AbstractFloat or N0f8. Got {return_type}")


def ifft_and_abs(fftholo: np.ndarray, return_type=N0f8) -> np.ndarray:
    """``_ifft_and_abs`` (holofunc.jl:158-166): ``clamp(abs2(ifft(ifftshift(X))), 0, 1)``
    converted to ``return_type``."""
    if not (return_type is N0f8 or return_type in (np.float16, np.float32, np.float64)):
        raise ValueError(f"return_type must be Subtype of AbstractFloat or N0f8. Got {return_type}")
    inten = _intensity(_ifft2(ifftshift(fftholo)))
    return _convert(np.clip(inten, np.float32(0.0), np.float32(1.0)), return_type)


def _check_same(wf, tf, tdz):
    if not (np.shape(wf) == np.shape(tf) == np.shape(tdz)):
        raise AssertionError(f"All arrays must have the same size. Got {np.shape(wf)}, {np.shape(tf)}, {np.shape(tdz)}.")


def spectrum(wf: np.ndarray, transfer_front: np.ndarray) -> np.ndarray:
    """``fftshift(fft(wavefront)) .* transfer_front`` (holofunc.jl:189-190, 254-255)."""
    return (fftshift(_fft2(wf)) * np.asarray(transfer_front, dtype=np.complex64)).astype(np.complex64)


def iter_slices(wf, transfer_front, transfer_dz, slices: int):
    """Yields the cumulative spectra ``X_k = fftshift(fft(wf)).*Hf.*Hdz^k`` for
    k = 0..slices-1, each a complex64 product of the previous one with ``Hdz``
    (holofunc.jl:194-197, 226-229, 259-263)."""
    tdz = np.asarray(transfer_dz, dtype=np.complex64)
    x = spectrum(wf, transfer_front)
    for k in range(slices):
        if k > 0:
            x = (x * tdz).astype(np.complex64)
        yield x


def reconst_vol(wf, transfer_front, transfer_dz, slices: int, return_type=N0f8) -> np.ndarray:
    """``cu_get_reconst_vol`` (holofunc.jl:184-200) -> shape ``(slices, n_slow, n_fast)``."""
    _check_same(wf, transfer_front, transfer_dz)
    return np.stack([ifft_and_abs(x, return_type) for x in iter_slices(wf, transfer_front, transfer_dz, slices)])


def reconst_complex_vol(wf, transfer_front, transfer_dz, slices: int) -> np.ndarray:
    """``cu_get_reconst_complex_vol`` (holofunc.jl:216-232)."""
    _check_same(wf, transfer_front, transfer_dz)
    return np.stack([_ifft2(ifftshift(x)).astype(np.complex64)
                     for x in iter_slices(wf, transfer_front, transfer_dz, slices)])


def reconst_xyprojection(wf, transfer_front, transfer_dz, slices: int, with_argmin: bool = False):
    """``cu_get_reconst_xyprojection`` (holofunc.jl:248-266): unclamped per-pixel
    minimum over slices of ``abs(x.*conj(x))``.

    ``with_argmin`` additionally returns the 0-based slice of the first minimum
    (ties keep the earlier slice), which the reference does not return.
    """
    _check_same(wf, transfer_front, transfer_dz)
    proj = None
    arg = None
    for k, x in enumerate(iter_slices(wf, transfer_front, transfer_dz, slices)):
        inten = _intensity(_ifft2(ifftshift(x)))
        if proj is None:
            proj = inten
            arg = np.zeros(inten.shape, dtype=np.int32)
        else:
            better = inten < proj
            arg[better] = k
            proj = np.minimum(proj, inten)
    if with_argmin:
        return proj, arg
    return proj


def xy_projection_from_vol(vol: np.ndarray) -> np.ndarray:
    """``_cu_get_xy_projection_from_vol!`` (holofunc.jl:268-282): strict ``<``
    minimum over slices, stored as Float32 (N0f8 raw ``i`` becomes ``i/255f0``)."""
    m = vol.min(axis=0)
    if vol.dtype == np.uint8:
        return (m.astype(np.float32) / np.float32(255.0)).astype(np.float32)
    return m.astype(np.float32)


def reconst_vol_and_xyprojection(wf, transfer_front, transfer_dz, slices: int, return_type=N0f8):
    """``cu_get_reconst_vol_and_xyprojection`` (holofunc.jl:300-321)."""
    vol = reconst_vol(wf, transfer_front, transfer_dz, slices, return_type)
    return vol, xy_projection_from_vol(vol)


def reconst_vol_and_xyprojection_padded(wf, transfer_front, transfer_dz, slices: int, return_type=N0f8):
    """``cu_get_reconst_vol_and_xyprojection_padded`` (holofunc.jl:339-364).

    The wavefront is mean-padded to 2N (``cu_2d_pad``); each slice is the
    centre crop (1-based ``N/2+1 : 3N/2``) of ``_ifft_and_abs``; the volume is
    always N0f8.
    """
    wf = np.asarray(wf, dtype=np.complex64)
    expected = tuple(2 * s for s in wf.shape)
    if not (expected == np.shape(transfer_front) == np.shape(transfer_dz)):
        raise AssertionError(
            "size(transfer_front.data) and size(transfer_dz.data) must be equal to 2*size(wavefront.data). "
            f"Got {wf.shape}, {np.shape(transfer_front)}, {np.shape(transfer_dz)}.")
    datlen = wf.shape[1]
    h = datlen // 2
    padded = pad2d(wf)
    vol = []
    for x in iter_slices(padded, transfer_front, transfer_dz, slices):
        tmp = ifft_and_abs(x, return_type)[h:3 * h, h:3 * h]
        if tmp.dtype != np.uint8:
            tmp = normedfloat_to_n0f8(tmp.astype(np.float32))
        vol.append(tmp)
    vol = np.stack(vol)
    return vol, xy_projection_from_vol(vol)


# ---------------------------------------------------------------- low-pass filters

def _lpf_maxi(prop_dist: float, wavlen: float, imglen: int, pitch: float) -> float:
    """frequency_filters.jl:33 / :68."""
    return 1 / wavlen * imglen ** 2 * pitch ** 2 / np.sqrt(4.0 * prop_dist ** 2 + imglen ** 2 * pitch ** 2)


def rectangle_filter(prop_dist: float, wavlen: float, imglen: int, pitch: float) -> np.ndarray:
    """``cu_rectangle_filter`` (frequency_filters.jl:31-38; kernel :5-15).

    ``arr[y, x] = 0`` where ``(x - datlen/2 + 1)^2 + (y - datlen/2)^2 >= maxi^2``
    (1-based x, y; note the asymmetric offsets), else 1.  ``arr[y, x]`` has y as
    the fast index, so it is ``a[x-1, y-1]`` here.
    """
    maxi = _lpf_maxi(prop_dist, wavlen, imglen, pitch)
    i = np.arange(1, imglen + 1, dtype=np.float64)
    xs = (i - imglen / 2 + 1)[:, None]        # x indexes the slow axis (rows of `a`)
    ys = (i - imglen / 2)[None, :]
    return np.where(xs ** 2 + ys ** 2 >= maxi ** 2, 0.0, 1.0).astype(np.float32)


def super_gaussian_filter(prop_dist: float, wavlen: float, imglen: int, pitch: float) -> np.ndarray:
    """``cu_super_gaussian_filter`` (frequency_filters.jl:66-74; kernel :40-50), FP64
    evaluation stored as Float32."""
    maxi = _lpf_maxi(prop_dist, wavlen, imglen, pitch)
    sigma = maxi / (imglen * pitch) / (2.0 * np.log(2.0)) ** (1 / 6)
    i = np.arange(1, imglen + 1, dtype=np.float64)
    t = (i - imglen / 2 + 1) / imglen / pitch / sigma
    r2 = (t ** 2)[:, None] + (t ** 2)[None, :]
    return np.exp(-1 / 2 * r2 ** 3).astype(np.float32)


def apply_low_pass_filter(holo: np.ndarray, lpf: np.ndarray) -> np.ndarray:
    """``cu_apply_low_pass_filter[!]`` (frequency_filters.jl:88-107):
    ``ifft(ifftshift(lpf .* fftshift(fft(holo))))``."""
    return _ifft2(ifftshift(np.asarray(lpf, np.float32) * fftshift(_fft2(holo)))).astype(np.complex64)


# ---------------------------------------------------------------- labels

def count_labels(labels: np.ndarray) -> int:
    """``count_labels`` (ccl.jl:213-221): number of i with ``labels[i+1] == i+1``."""
    flat = np.asarray(labels).reshape(-1).astype(np.int64)
    return int(np.count_nonzero(flat == np.arange(1, flat.size + 1, dtype=np.int64)))


def bounding_rectangles(labels: np.ndarray, valid_labels: np.ndarray) -> list:
    """``get_bounding_rectangles`` (ccl.jl:240-264) on a Julia ``(height, width)``
    label array held here as ``(width, height)``: for each valid label,
    ``(x_min, y_min, x_max, y_max)`` with x the column index j (our slow axis)
    and y the row index i (our fast axis), 1-based."""
    out = []
    for lab in valid_labels:
        xs, ys = np.nonzero(np.asarray(labels) == lab)     # xs: slow (j - 1), ys: fast (i - 1)
        out.append((int(xs.min()) + 1, int(ys.min()) + 1, int(xs.max()) + 1, int(ys.max()) + 1))
    return out


def find_valid_labels(labels: np.ndarray) -> np.ndarray:
    """``cu_find_valid_labels`` (ccl.jl:224-238): sorted 1-based linear indices
    ``i`` with ``labels[i] == i`` (the component roots), as Int64."""
    flat = np.asarray(labels).reshape(-1).astype(np.int64)
    return (np.nonzero(flat == np.arange(1, flat.size + 1, dtype=np.int64))[0] + 1).astype(np.int64)


# ---------------------------------------------------------------- preprocessing (utils.jl)

def make_background_mode(images) -> np.ndarray:
    """``cu_make_background_mode`` (utils.jl:279-317) and ``make_background(...;
    mode=:mode)`` (utils.jl:210-231): per-pixel most frequent UInt8 value over a
    stack of images (votes per value, the first maximum on ties), / 255 as Float64."""
    stack = np.asarray(images, dtype=np.uint8)
    votes = np.zeros((256,) + stack.shape[1:], dtype=np.int64)
    for img in stack:
        np.add.at(votes, (img.astype(np.int64),) + tuple(np.indices(img.shape)), 1)
    return np.argmax(votes, axis=0).astype(np.float64) / 255.0


def make_background_mean(images) -> np.ndarray:
    """``make_background(...; mode=:mean)`` (utils.jl:212-218): the mean of the
    images as Float64, each UInt8 image read as Float32(value / 255)
    (load_gray2float) and summed in image order."""
    stack = (np.asarray(images, dtype=np.uint8).astype(np.float32) / np.float32(255.0)).astype(np.float64)
    acc = np.zeros(stack.shape[1:], dtype=np.float64)
    for img in stack:          # in image order, as the reference's loop
        acc += img
    return acc / len(stack)


def pad_with_mean(img: np.ndarray, padsize: int) -> np.ndarray:
    """``pad_with_mean`` (utils.jl:319-325) on a Julia ``(h, w)`` image held here as
    ``(w, h)`` = ``(n_slow, n_fast)``: a padsize x padsize array of mean(img) with
    the image at Julia rows ``div(p,2)-div(h,2)+1 ..`` and columns
    ``div(p,2)-div(w,2)+1 ..``."""
    n_slow, n_fast = img.shape
    assert padsize > n_fast and padsize > n_slow, "Padsize should be larger than the image size."
    out = np.full((padsize, padsize), np.float32(np.mean(img, dtype=np.float64)), dtype=np.float32)
    o_fast, o_slow = padsize // 2 - n_fast // 2, padsize // 2 - n_slow // 2
    out[o_slow:o_slow + n_slow, o_fast:o_fast + n_fast] = img
    return out
