"""FP64 angular-spectrum physics and the seeded synthetic-hologram generator.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

* ``transfer_exact``: ``H = exp(i 2 pi z sqrt(1/lambda^2 - fx^2 - fy^2))`` in
  complex128 with the square-root term kept in FP64 -- the physics of
  ``docs/src/whats_inline_holography.md:8-14``, on the reference's centred
  frequency grid (the grid of ``holofunc.jl:12``); evanescent frequencies get 0.
* ``reconst_xyprojection_fp64``: per-slice exact transfer
  ``H(-(z0 + k dz))`` instead of cumulative complex64 products.
* ``phase_retrieval_fp64``: the Gerchberg-Saxton loop of holofunc.jl:100-129 in
  complex128.
* ``draw_discs`` / ``synth_hologram``: the seeded generator (docs
  ``whats_inline_holography.md:17-33``): opaque discs, plane wave of unit
  amplitude at the farthest disc, ``(1 - A_i)`` masks, ASM propagation between
  disc planes and on to the sensor at z = 0, intensity min-max normalised to
  [0, 1] plus N(0, sigma^2) noise, cast to Float32.
"""
from __future__ import annotations

import os
from dataclasses import dataclass

import numpy as np
import scipy.fft as sfft


def _w() -> int:
    return len(os.sched_getaffinity(0))


def sqr_exact(nx: int, ny: int, wavlen: float, dx: float) -> np.ndarray:
    """FP64 ``1 - (lambda fx)^2 - (lambda fy)^2`` on the centred grid, shape (ny, nx)."""
    x = np.arange(1, nx + 1, dtype=np.float64)
    y = np.arange(1, ny + 1, dtype=np.float64)
    tx = (x - nx / 2 - 1.0) * wavlen / nx / dx
    ty = (y - ny / 2 - 1.0) * wavlen / ny / dx
    return 1.0 - (tx * tx)[None, :] - (ty * ty)[:, None]


def transfer_exact(z: float, nx: int, wavlen: float, dx: float, ny: int | None = None) -> np.ndarray:
    """Exact transfer function on the reference's centred grid (complex128)."""
    ny = nx if ny is None else ny
    s = sqr_exact(nx, ny, wavlen, dx)
    ok = s >= 0
    phase = 2.0 * np.pi * z / wavlen * np.sqrt(np.where(ok, s, 0.0))
    return np.where(ok, np.exp(1j * phase), 0.0)


def transfer_natural(z: float, nx: int, ny: int, wavlen: float, dx: float) -> np.ndarray:
    """Exact transfer function in natural FFT order (``fftfreq`` grid), complex128."""
    fx = np.fft.fftfreq(nx, d=dx)
    fy = np.fft.fftfreq(ny, d=dx)
    s = 1.0 / wavlen ** 2 - fx[None, :] ** 2 - fy[:, None] ** 2
    ok = s >= 0
    return np.where(ok, np.exp(2j * np.pi * z * np.sqrt(np.where(ok, s, 0.0))), 0.0)


def propagate_natural(psi: np.ndarray, z: float, wavlen: float, dx: float) -> np.ndarray:
    ny, nx = psi.shape
    return sfft.ifft2(sfft.fft2(psi, workers=_w()) * transfer_natural(z, nx, ny, wavlen, dx), workers=_w())


# ---------------------------------------------------------------- reconstruction

def spectrum_fp64(wf: np.ndarray) -> np.ndarray:
    return np.fft.fftshift(sfft.fft2(np.asarray(wf, dtype=np.complex128), workers=_w()))


def reconst_slice_fp64(spec_centred: np.ndarray, z: float, wavlen: float, dx: float) -> np.ndarray:
    """Exact intensity of the slice at back-propagation distance ``z`` (use z < 0
    to reconstruct into the volume, as ``cu_transfer(-z0, ...)`` does)."""
    ny, nx = spec_centred.shape
    h = transfer_exact(z, nx, wavlen, dx, ny)
    u = sfft.ifft2(np.fft.ifftshift(spec_centred * h), workers=_w())
    return (u.real ** 2 + u.imag ** 2)


def reconst_xyprojection_fp64(wf, z0: float, dz: float, slices: int, wavlen: float, dx: float,
                              with_argmin: bool = False):
    """Exact-physics counterpart of ``cu_get_reconst_xyprojection`` with
    ``Hf = H(-z0)`` and ``Hdz = H(-dz)``: slice k is at ``-(z0 + k dz)``."""
    spec = spectrum_fp64(wf)
    proj = None
    arg = None
    for k in range(slices):
        inten = reconst_slice_fp64(spec, -(z0 + k * dz), wavlen, dx)
        if proj is None:
            proj, arg = inten, np.zeros(inten.shape, dtype=np.int32)
        else:
            better = inten < proj
            arg[better] = k
            proj = np.where(better, inten, proj)
    return (proj, arg) if with_argmin else proj


def phase_retrieval_fp64(holo1, holo2, dzp: float, priter: int, wavlen: float, dx: float,
                         return_residual: bool = False):
    """Gerchberg-Saxton (holofunc.jl:100-129) in complex128 with exact transfers
    ``H(+dzp)`` / ``H(-dzp)``."""
    ny, nx = np.shape(holo1)
    h = transfer_exact(dzp, nx, wavlen, dx, ny)
    hinv = transfer_exact(-dzp, nx, wavlen, dx, ny)
    s1 = np.sqrt(np.asarray(holo1, dtype=np.float64))
    s2 = np.sqrt(np.asarray(holo2, dtype=np.float64))

    def prop(x, tf):
        return sfft.ifft2(np.fft.ifftshift(np.fft.fftshift(sfft.fft2(x, workers=_w())) * tf), workers=_w())

    def replace(s, u):
        return s * np.exp(1j * np.angle(u))

    light1 = s1.astype(np.complex128)
    residual = None
    for it in range(priter):
        light2 = prop(light1, h)
        if it == priter - 1:
            residual = float(np.linalg.norm(np.abs(light2) - s2) / np.linalg.norm(s2))
        light2 = replace(s2, light2)
        light1 = replace(s1, prop(light2, hinv))
    return (light1, residual) if return_residual else light1


# ---------------------------------------------------------------- generator

@dataclass
class Discs:
    """Opaque discs: centres (um), diameters (um), depths (um)."""
    x: np.ndarray
    y: np.ndarray
    d: np.ndarray
    z: np.ndarray


def draw_discs(seed: int, n: int, count: int, dmin: float, dmax: float, zmin: float, zmax: float,
               dx: float, ny: int | None = None) -> Discs:
    """Seeded disc field: ``numpy.random.Generator(PCG64(seed))``; diameters
    U(dmin, dmax) um, centres U(0, N dx), depths U(zmin, zmax) um, drawn in
    that order."""
    ny = n if ny is None else ny
    rng = np.random.Generator(np.random.PCG64(seed))
    d = rng.uniform(dmin, dmax, count)
    x = rng.uniform(0.0, n * dx, count)
    y = rng.uniform(0.0, ny * dx, count)
    z = rng.uniform(zmin, zmax, count)
    return Discs(x=x, y=y, d=d, z=z)


def noise(seed: int, shape, sigma: float) -> np.ndarray:
    """Gaussian sensor noise; its own stream (seed + 1) so the disc draws do not
    depend on the image size."""
    rng = np.random.Generator(np.random.PCG64(seed + 1))
    return rng.normal(0.0, sigma, shape)


def disc_mask(discs: Discs, i: int, nx: int, ny: int, dx: float) -> np.ndarray:
    """``A_i``: 1 where the pixel centre ``(ix dx, iy dx)`` lies within the disc."""
    xs = np.arange(nx) * dx
    ys = np.arange(ny) * dx
    r = discs.d[i] / 2.0
    return ((xs[None, :] - discs.x[i]) ** 2 + (ys[:, None] - discs.y[i]) ** 2) <= r * r


def synth_field(discs: Discs, nx: int, ny: int, wavlen: float, dx: float, z_sensor: float = 0.0) -> np.ndarray:
    """Complex field at the sensor plane (FP64): unit plane wave at the farthest
    disc, ``(1 - A_i)`` at each disc plane, ASM between planes."""
    order = np.argsort(-discs.z, kind="stable")
    psi = np.ones((ny, nx), dtype=np.complex128)
    zc = discs.z[order[0]] if len(order) else z_sensor
    for i in order:
        if zc != discs.z[i]:
            psi = propagate_natural(psi, zc - discs.z[i], wavlen, dx)
            zc = discs.z[i]
        psi = psi * (1.0 - disc_mask(discs, i, nx, ny, dx))
    return propagate_natural(psi, zc - z_sensor, wavlen, dx)


def normalise_with_noise(intensity: np.ndarray, seed: int, sigma: float) -> np.ndarray:
    lo, hi = float(intensity.min()), float(intensity.max())
    scale = 1.0 / (hi - lo) if hi > lo else 0.0
    out = (intensity - lo) * scale + noise(seed, intensity.shape, sigma)
    return np.maximum(out, 0.0).astype(np.float32)      # a sensor records no negative intensity


def synth_hologram(seed: int, n: int, count: int, dmin: float, dmax: float, zmin: float, zmax: float,
                   wavlen: float = 0.6328, dx: float = 10.0, sigma: float = 0.01,
                   z_sensor: float = 0.0) -> np.ndarray:
    """One seeded Float32 hologram of shape (n, n) in FP64 physics."""
    discs = draw_discs(seed, n, count, dmin, dmax, zmin, zmax, dx)
    psi = synth_field(discs, n, n, wavlen, dx, z_sensor)
    return normalise_with_noise(np.abs(psi) ** 2, seed, sigma)
