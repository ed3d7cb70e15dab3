"""Serving: a request queue in front of ``cu_get_reconst_xyprojection``
(holofunc.jl:248-266) for a stream of holograms (``ph_serve_*``).  Requests run
asynchronously on the server's lanes; transfer functions for recurring optics
come from the server's cache.
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

    def __init__(self, max_shape, max_slices: int, lanes: int = 3, tf_cache: int = 16, device: int | None = None):
        dev = torch.cuda.current_device() if device is None else device
        self.device = dev
        self._ctx = _lib.default_context(dev)
        h = ctypes.c_void_p()
        ny, nx = int(max_shape[0]), int(max_shape[1])
        self._ctx.call("ph_serve_create", int(lanes), nx, ny, int(max_slices), int(tf_cache), ctypes.byref(h))
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
        t = ctypes.c_int64()
        _, s = _ctx_stream(h)
        _lib.raise_for(_lib.lib().ph_serve_submit(self._handle, ctypes.byref(req), ctypes.byref(t), s),
                       self._ctx.handle)
        self._live[t.value] = (h, p, argmin)   # keep the buffers alive while the request runs
        return t.value

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
