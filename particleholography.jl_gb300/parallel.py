"""Depth sharding of the projection across ranks (no counterpart in the
reference, which runs one GPU and loops over slices on the host).

A reconstruction of S slices splits into contiguous slice ranges, one per
rank.  Each rank reduces its range to a packed per-pixel word
``(float bits of the minimum intensity) << 32 | slice`` -- intensities are
non-negative, so the bit pattern orders like the value and ties resolve to the
smaller slice, exactly the reference's first-minimum rule (holofunc.jl:276) --
and one all-reduce with MIN merges the ranks.  The words fit in a signed int64
(the sign bit of a non-negative float is 0), so any backend's int64 MIN works.

The library computes a rank's words directly: ``reconst_xyprojection_range``
(``ph_reconst_xyproj_range``) reconstructs slices [k0, k1) with their global
indices into packed words, and ``unpack_projection`` (``ph_unpack_projection``)
turns the merged words into the projection and argmin.  A rank with an empty
range contributes the merge identity ``PACKED_EMPTY`` (INT64_MAX).

Frames (independent holograms) need no exchange at all: ``bench.py --gpus N``
runs one replica per GPU.
"""
from __future__ import annotations

import numpy as np
import torch

PACKED_EMPTY = int(np.iinfo(np.int64).max)   # PH_PACKED_EMPTY (include/phgb300.h)


def shard_range(slices: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous slice range [k0, k1) of `rank` (sizes differ by at most one)."""
    base, extra = divmod(slices, world)
    k0 = rank * base + min(rank, extra)
    return k0, k0 + base + (1 if rank < extra else 0)


def pack(proj: torch.Tensor, argmin: torch.Tensor) -> torch.Tensor:
    """(float32 min, int32 slice) -> packed int64 words."""
    bits = proj.contiguous().view(torch.int32).to(torch.int64)
    return (bits << 32) | argmin.to(torch.int64)


def unpack(packed: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
    bits = (packed >> 32).to(torch.int32)
    return bits.view(torch.float32), (packed & 0xFFFFFFFF).to(torch.int32)


def empty_packed(shape, device=None) -> torch.Tensor:
    """The identity of the MIN merge (a rank with no slices contributes this)."""
    return torch.full(shape, PACKED_EMPTY, dtype=torch.int64, device=device)


def reconst_xyprojection_range(wavefront, transfer_front, transfer_dz, k0: int, k1: int,
                               packed: torch.Tensor | None = None, accumulate: bool = False) -> torch.Tensor:
    """Packed words of slices [k0, k1) of ``cu_get_reconst_xyprojection``
    (holofunc.jl:248-266) on the GPU, slice indices global.

    Returns ``packed`` (int64, the wavefront's shape; allocated when None).
    ``accumulate`` merges into the words already in ``packed`` instead of
    starting from the identity."""
    from . import holofunc
    wf, tf, td = holofunc._recon_args(wavefront, transfer_front, transfer_dz)
    holofunc._check_same(wf, tf, td)
    if packed is None:
        packed = torch.empty(wf.shape, dtype=torch.int64, device=wf.device)
    if tuple(packed.shape) != tuple(wf.shape) or packed.dtype != torch.int64 or not packed.is_contiguous():
        raise ValueError("packed must be a contiguous int64 tensor of the wavefront's shape")
    ctx, s = holofunc._ctx_stream(wf)
    ctx.call("ph_reconst_xyproj_range", packed.data_ptr(), wf.data_ptr(), tf.data_ptr(), td.data_ptr(),
             int(wf.shape[1]), int(wf.shape[0]), int(k0), int(k1), 1 if accumulate else 0, s)
    return packed


def unpack_projection(packed: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
    """Merged packed words -> (projection float32, argmin int32) on the GPU."""
    from . import holofunc
    if packed.dtype != torch.int64 or not packed.is_contiguous() or packed.dim() != 2:
        raise ValueError("packed must be a contiguous 2-D int64 tensor")
    proj = torch.empty(packed.shape, dtype=torch.float32, device=packed.device)
    arg = torch.empty(packed.shape, dtype=torch.int32, device=packed.device)
    ctx, s = holofunc._ctx_stream(packed)
    ctx.call("ph_unpack_projection", proj.data_ptr(), arg.data_ptr(), packed.data_ptr(), int(packed.shape[1]),
             int(packed.shape[0]), s)
    return proj, arg


def merge(packed: torch.Tensor, group=None) -> torch.Tensor:
    """All-reduce the packed words of every rank with MIN (in place)."""
    import torch.distributed as dist
    dist.all_reduce(packed, op=dist.ReduceOp.MIN, group=group)
    return packed
