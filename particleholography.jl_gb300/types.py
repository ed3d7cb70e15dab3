"""Device data types of the hot path (mirrors ParticleHolography.jl src/types.jl:13-62).

Each wraps one 2-D CUDA tensor.  A Julia array of size ``(n_fast, n_slow)`` is
held as a C-ordered tensor of shape ``(n_slow, n_fast)`` over the same memory
order; ``size()`` reports the Julia-order size.
"""
from __future__ import annotations

import torch


class N0f8:
    """FixedPointNumbers.N0f8 marker: volumes of this type are UInt8 tensors
    whose value is ``raw / 255``."""


class _DeviceArray2D:
    _dtype: torch.dtype = torch.float32

    def __init__(self, data: torch.Tensor):
        if not isinstance(data, torch.Tensor) or data.dim() != 2:
            raise TypeError(f"{type(self).__name__} wraps a 2-D tensor")
        self.data = data

    def size(self) -> tuple[int, int]:
        """Julia-order size ``(n_fast, n_slow)`` (``Base.size``, types.jl:56)."""
        return (int(self.data.shape[1]), int(self.data.shape[0]))

    def axes(self):
        return tuple(range(n) for n in self.size())

    def ndims(self) -> int:
        return 2

    def eltype(self) -> torch.dtype:
        return self.data.dtype

    def __repr__(self) -> str:
        return f"{type(self).__name__}(size={self.size()}, dtype={self.data.dtype}, device={self.data.device})"


class CuTransferSqrtPart(_DeviceArray2D):
    """Square-root part of the transfer function (types.jl:13-15), Float32."""


class CuTransfer(_DeviceArray2D):
    """Transfer function (types.jl:25-27), ComplexF32."""


class CuWavefront(_DeviceArray2D):
    """Wavefront (types.jl:37-39), ComplexF32."""


class CuLowPassFilter(_DeviceArray2D):
    """Frequency-domain low-pass mask (types.jl:50-52), Float32."""
