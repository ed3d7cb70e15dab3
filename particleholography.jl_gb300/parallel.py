"""Depth sharding of the projection across ranks (no counterpart in the
reference, which runs one GPU and loops over slices on the host).

A reconstruction of S slices splits into contiguous slice ranges, one per
rank.  Each rank reduces its range to a packed per-pixel word
``(float bits of the minimum intensity) << 32 | slice`` -- intensities are
non-negative, so the bit pattern orders like the value and ties resolve to the
smaller slice, exactly the reference's first-minimum rule (holofunc.jl:276) --
and one all-reduce with MIN merges the ranks.  The words fit in a signed int64
(the sign bit of a non-negative float is 0), so any backend's int64 MIN works.

Frames (independent holograms) need no exchange at all: ``bench.py --gpus N``
runs one replica per GPU.
"""
from __future__ import annotations

import numpy as np
import torch


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
    return torch.full(shape, np.iinfo(np.int64).max, dtype=torch.int64, device=device)


def merge(packed: torch.Tensor, group=None) -> torch.Tensor:
    """All-reduce the packed words of every rank with MIN (in place)."""
    import torch.distributed as dist
    dist.all_reduce(packed, op=dist.ReduceOp.MIN, group=group)
    return packed
