"""Batches of projections: many ``cu_get_reconst_xyprojection`` calls
(holofunc.jl:248-266), one per hologram, each with its own size, transfer
functions and slice count, planned once and run as one CUDA graph
(``ph_batch_plan`` / ``ph_batch_run``).  The reference runs such a batch as a
host loop of single calls; results here equal those calls exactly.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from .holofunc import _ctx_stream, _data, _need, _jsize


class ReconBatch:
    """A planned batch.

    ``items``: a sequence of dicts with ``transfer_front``, ``transfer_dz``
    (CuTransfer or complex64 tensors of the hologram's shape), ``slices`` and
    either ``hologram`` (Float32; the wavefront is its square root, as
    ``cu_gabor_wavefront``) or ``wavefront`` (complex64).  Outputs are
    allocated once: ``proj[i]`` (Float32) and, with ``return_argmin``,
    ``argmin[i]`` (int32).  ``run()`` recomputes them from the items' current
    buffer contents; the buffers must stay alive while the plan exists.
    """

    def __init__(self, items, lanes: int = 4, return_argmin: bool = True):
        self._keep = []
        self.proj, self.argmin = [], []
        recs = (_lib.ReconItem * max(1, len(items)))()
        dev = None
        for i, it in enumerate(items):
            tf = _need(_data(it["transfer_front"]), torch.complex64, "transfer_front")
            td = _need(_data(it["transfer_dz"]), torch.complex64, "transfer_dz")
            if it.get("hologram") is not None:
                src = _need(_data(it["hologram"]), torch.float32, "hologram")
            else:
                src = _need(_data(it["wavefront"]), torch.complex64, "wavefront")
            if not (tuple(src.shape) == tuple(tf.shape) == tuple(td.shape)):
                raise AssertionError(f"All arrays must have the same size. Got {_jsize(src)}, {_jsize(tf)}, "
                                     f"{_jsize(td)}.")
            dev = src.device if dev is None else dev
            p = torch.empty(src.shape, dtype=torch.float32, device=src.device)
            a = torch.empty(src.shape, dtype=torch.int32, device=src.device) if return_argmin else None
            self.proj.append(p)
            self.argmin.append(a)
            self._keep += [src, tf, td]
            r = recs[i]
            r.hologram = src.data_ptr() if src.dtype == torch.float32 else None
            r.wavefront = src.data_ptr() if src.dtype == torch.complex64 else None
            r.tf_front, r.tf_dz = tf.data_ptr(), td.data_ptr()
            r.proj = p.data_ptr()
            r.argmin = a.data_ptr() if a is not None else None
            r.n_fast, r.n_slow, r.slices = int(src.shape[1]), int(src.shape[0]), int(it["slices"])
        if dev is None:
            raise ValueError("a batch needs at least one item")
        self._ctx, _ = _ctx_stream(self._keep[0])
        # the plan reads the item buffers when it runs; make the work that wrote them visible first
        torch.cuda.current_stream(dev).synchronize()
        h = ctypes.c_void_p()
        self._ctx.call("ph_batch_plan", ctypes.cast(recs, ctypes.c_void_p), len(items), int(lanes), ctypes.byref(h))
        self._handle = h

    @property
    def scratch_bytes(self) -> int:
        return int(_lib.lib().ph_batch_scratch_bytes(self._handle))

    def run(self):
        """Runs the batch on the current stream; returns (proj list, argmin list)."""
        _, s = _ctx_stream(self._keep[0])
        _lib.raise_for(_lib.lib().ph_batch_run(self._handle, s), self._ctx.handle)
        return self.proj, self.argmin

    def close(self) -> None:
        if getattr(self, "_handle", None):
            _lib.lib().ph_batch_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune(n_fast: int, n_slow: int, slices: int, allow_forms: bool = False, cache: str | None = None,
             device: int | None = None) -> dict:
    """The library's autotuner (``ph_autotune``) for one shape: times the
    projection's knobs once (slices per CTA, batch of intermediates and, with
    ``allow_forms``, the split-precision row-pass forms) and keeps the fastest
    in the device's context, so later reconstructions of the shape -- single
    calls, batch plans, servers -- use it.  With ``cache`` (a JSON path) the
    choice is read from / written to the file, keyed by device name and shape.
    Returns ``{"form", "group_cap", "batch_slices", "ms"}``."""
    dev = torch.cuda.current_device() if device is None else device
    ctx = _lib.default_context(dev)
    choice = (ctypes.c_int32 * 3)()
    ms = ctypes.c_double()
    s = torch.cuda.current_stream(dev).cuda_stream
    ctx.call("ph_autotune", int(n_fast), int(n_slow), int(slices), 1 if allow_forms else 0,
             cache.encode() if cache is not None else None, ctypes.addressof(choice), ctypes.byref(ms), s)
    return {"form": int(choice[0]), "group_cap": int(choice[1]), "batch_slices": int(choice[2]), "ms": ms.value}
