"""Seeded synthetic inline holograms (no counterpart in the reference, which ships
no generator; the physics follows its docs, whats_inline_holography.md:17-33).

Discs are drawn on the host with ``numpy.random.Generator(PCG64(seed))``
(diameters U(dmin, dmax) um, centres U(0, N dx), depths U(zmin, zmax) um, in
that order; Gaussian sensor noise from the stream ``seed + 1``); the field is
built on the GPU by ``ph_synth_hologram``: unit plane wave at the farthest disc,
``(1 - A_i)`` at every disc plane, angular-spectrum propagation between planes
and on to the sensor, intensity min-max normalised to [0, 1], plus noise.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch

from . import _lib


@dataclass
class HologramSpec:
    """One synthetic hologram: size, particle field and optics (lengths in um)."""
    seed: int
    n: int
    count: int
    dmin: float
    dmax: float
    zmin: float
    zmax: float
    wavlen: float = 0.6328
    dx: float = 10.0
    sigma: float = 0.01
    z_sensor: float = 0.0
    n_slow: int | None = None   # rows (slow axis); None = n (square)

    @property
    def ny(self) -> int:
        return self.n if self.n_slow is None else self.n_slow


def draw_discs(spec: HologramSpec) -> np.ndarray:
    """``[count, 4]`` float64 array of (x, y, diameter, z) in um."""
    rng = np.random.Generator(np.random.PCG64(spec.seed))
    d = rng.uniform(spec.dmin, spec.dmax, spec.count)
    x = rng.uniform(0.0, spec.n * spec.dx, spec.count)
    y = rng.uniform(0.0, spec.ny * spec.dx, spec.count)
    z = rng.uniform(spec.zmin, spec.zmax, spec.count)
    return np.ascontiguousarray(np.stack([x, y, d, z], axis=1), dtype=np.float64)


def draw_noise(spec: HologramSpec, stream: int = 1) -> np.ndarray:
    """Sensor noise of the hologram: N(0, sigma^2) from the stream ``seed + stream``."""
    rng = np.random.Generator(np.random.PCG64(spec.seed + stream))
    return rng.normal(0.0, spec.sigma, (spec.ny, spec.n)).astype(np.float32)


def synth_hologram(spec: HologramSpec, device: int | None = None, noise: bool = True,
                   noise_stream: int = 1) -> torch.Tensor:
    """A Float32 CUDA tensor of shape (ny, n): the seeded hologram (noisy
    intensities clamped at 0, as a sensor records them)."""
    dev = torch.cuda.current_device() if device is None else device
    out = torch.empty((spec.ny, spec.n), dtype=torch.float32, device=f"cuda:{dev}")
    discs = draw_discs(spec)
    nz = torch.from_numpy(draw_noise(spec, noise_stream)).to(out.device) if noise and spec.sigma > 0 else None
    ctx = _lib.default_context(dev)
    ctx.call("ph_synth_hologram", out.data_ptr(), spec.n, spec.ny, discs.ctypes.data, int(spec.count),
             float(spec.wavlen), float(spec.dx), float(spec.z_sensor), nz.data_ptr() if nz is not None else None,
             torch.cuda.current_stream(dev).cuda_stream)
    if nz is not None:
        torch.cuda.current_stream(dev).synchronize()   # keep `nz` alive until the kernel has read it
    return out


def synth_pair(spec: HologramSpec, separation: float, device: int | None = None):
    """Two holograms of the same particle field recorded ``separation`` um apart:
    the first at ``spec.z_sensor`` (closer to the particles), the second
    ``separation`` further away.  Each gets its own noise."""
    from dataclasses import replace
    h1 = synth_hologram(spec, device)
    # same discs (same seed), the second sensor plane, independent noise stream
    h2 = synth_hologram(replace(spec, z_sensor=spec.z_sensor - separation), device, noise_stream=2)
    return h1, h2
