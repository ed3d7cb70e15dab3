"""Serving: a request queue in front of ``cu_get_reconst_xyprojection``
(holofunc.jl:248-266) for a stream of holograms (``ph_serve_*``).  Requests are
admitted in arrival order against the server's HBM budget (one scratch block
each, sized for the request) as work slots and memory free up, and run
concurrently on the slots' streams; transfer functions for recurring optics
come from the server's cache.  A request may carry an 8-bit camera frame
instead of a hologram: it is then decoded, background-corrected and
mean-padded on the device (``load_gray2float``, the docs' background removal,
``pad_with_mean``).
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from .holofunc import _ctx_stream, _data, _need


class Server:
    """``Server(max_shape=(n_slow, n_fast), max_slices, lanes)``: accepts requests
    up to that size.  ``submit`` returns a ticket at once; ``poll`` returns the
    request's latency in ms once it has finished (None while pending)."""

    def __init__(self, max_shape, max_slices: int, lanes: int = 3, tf_cache: int = 16, device: int | None = None,
                 budget_bytes: int = 0):
        dev = torch.cuda.current_device() if device is None else device
        self.device = dev
        self._ctx = _lib.default_context(dev)
        h = ctypes.c_void_p()
        ny, nx = int(max_shape[0]), int(max_shape[1])
        self._ctx.call("ph_serve_create", int(lanes), nx, ny, int(max_slices), int(tf_cache), int(budget_bytes),
                       ctypes.byref(h))
        self._handle = h
        self._live = {}

    def submit(self, hologram, proj: torch.Tensor, slices: int, z0: float, dz: float, wavlen: float = 0.6328,
               dx: float = 10.0, argmin: torch.Tensor | None = None) -> int:
        """Queues the projection of ``hologram`` (Float32, wavefront = its square
        root) over ``slices`` slices from ``z0`` in steps of ``dz`` (um) into
        ``proj`` (and ``argmin``).  Ordered after the work already on the
        current stream."""
        h = _need(_data(hologram), torch.float32, "hologram")
        p = _need(proj, torch.float32, "proj")
        if tuple(p.shape) != tuple(h.shape) or (argmin is not None and tuple(argmin.shape) != tuple(h.shape)):
            raise AssertionError("All arrays must have the same size.")
        req = _lib.ServeRequest(h.data_ptr(), p.data_ptr(), argmin.data_ptr() if argmin is not None else None,
                                int(h.shape[1]), int(h.shape[0]), int(slices), float(z0), float(dz), float(wavlen),
                                float(dx))
        return self._submit(req, h, (h, p, argmin))

    def submit_frame(self, frame: torch.Tensor, proj: torch.Tensor, slices: int, z0: float, dz: float,
                     wavlen: float = 0.6328, dx: float = 10.0, argmin: torch.Tensor | None = None,
                     background: torch.Tensor | None = None, background_offset: float = 0.0,
                     flip: bool = False) -> int:
        """Queues the projection of the hologram made on the device from an
        8-bit camera frame: ``frame`` uint8 ``(rows, cols)`` or ``(rows, cols,
        channels)`` row-major as a camera or image file stores it (rows
        bottom-up when ``flip``).  Levels / 255 (``load_gray2float``), minus
        ``background`` (float64, the library's layout ``(cols, rows)``) plus
        ``background_offset``, centred and padded with its mean to ``proj``'s
        shape ``(n_slow, n_fast)`` = ``(>= cols, >= rows)``."""
        f = _need(frame, torch.uint8, "frame")
        p = _need(proj, torch.float32, "proj")
        rows, cols = int(f.shape[0]), int(f.shape[1])
        ch = int(f.shape[2]) if f.dim() == 3 else 1
        if argmin is not None and tuple(argmin.shape) != tuple(p.shape):
            raise AssertionError("All arrays must have the same size.")
        bk = None
        if background is not None:
            bk = _need(background, torch.float64, "background")
            if tuple(bk.shape) != (cols, rows):
                raise AssertionError(f"background must have the frame's shape in the library layout {(cols, rows)}")
        req = _lib.ServeRequest(None, p.data_ptr(), argmin.data_ptr() if argmin is not None else None,
                                int(p.shape[1]), int(p.shape[0]), int(slices), float(z0), float(dz), float(wavlen),
                                float(dx), f.data_ptr(), rows, cols, int(f.stride(0)), ch, 1 if flip else 0,
                                bk.data_ptr() if bk is not None else None, float(background_offset))
        return self._submit(req, f, (f, p, argmin, bk))

    def _submit(self, req, on, keep) -> int:
        t = ctypes.c_int64()
        _, s = _ctx_stream(on)
        _lib.raise_for(_lib.lib().ph_serve_submit(self._handle, ctypes.byref(req), ctypes.byref(t), s),
                       self._ctx.handle)
        self._live[t.value] = keep   # keep the buffers alive while the request runs
        return t.value

    def stats(self) -> dict:
        """Requests queued and running, pool bytes in use and at peak, how many
        requests had to queue at submission, and how many were admitted in
        shared launches (same shape, slices and optics, queued together)."""
        q, r, w, g = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        used, peak = ctypes.c_size_t(), ctypes.c_size_t()
        _lib.raise_for(_lib.lib().ph_serve_stats(self._handle, ctypes.byref(q), ctypes.byref(r), ctypes.byref(used),
                                                 ctypes.byref(peak), ctypes.byref(w), ctypes.byref(g)),
                       self._ctx.handle)
        return {"queued": q.value, "running": r.value, "bytes_in_use": used.value, "bytes_peak": peak.value,
                "waited": w.value, "grouped": g.value}

    def poll(self, ticket: int, wait: bool = False) -> float | None:
        lat = ctypes.c_double()
        st = _lib.lib().ph_serve_poll(self._handle, int(ticket), 1 if wait else 0, ctypes.byref(lat))
        if st == _lib.PH_PENDING:
            return None
        _lib.raise_for(st, self._ctx.handle)
        self._live.pop(int(ticket), None)
        return lat.value

    def close(self) -> None:
        if getattr(self, "_handle", None):
            _lib.lib().ph_serve_destroy(self._handle)
            self._handle = None
            self._live.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
