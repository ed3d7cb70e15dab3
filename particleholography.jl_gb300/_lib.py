"""ctypes binding of libphgb300.so (the C ABI declared in include/phgb300.h).

The library is built in-tree by ``build.py``.  Loading fails loudly when it is
missing: there is no CPU path behind any entry point.
"""
from __future__ import annotations

import ctypes
import threading
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libphgb300.so"

# status codes (phgb300.h)
PH_OK = 0
PH_ERR_SIZE = 1
PH_ERR_DTYPE = 2
PH_ERR_TOO_LARGE = 3
PH_ERR_OOM = 4
PH_ERR_CUDA = 5
PH_ERR_TIMEOUT = 6
PH_ERR_INVALID = 7
PH_ERR_UNSUPPORTED = 8

# element types
PH_N0F8, PH_F16, PH_F32, PH_F64, PH_C64, PH_BOOL = range(6)

# options
PH_OPT_SLICE_BATCH = 1
PH_OPT_USE_GRAPHS = 2
PH_OPT_LOOP_LIMIT = 3
PH_OPT_PROFILE = 4
PH_OPT_FORM = 5

# forms of the projection's row pass
PH_FORM_FP32, PH_FORM_BF16X3, PH_FORM_FP16X3, PH_FORM_FP16X2, PH_FORM_TUNED = range(5)

# identity of the packed-minimum merge (ph_reconst_xyproj_range)
PH_PACKED_EMPTY = 0x7FFFFFFFFFFFFFFF

_vp = ctypes.c_void_p
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_f64 = ctypes.c_double
_sz = ctypes.c_size_t

# name -> (restype, argtypes); every symbol include/phgb300.h declares.
SIGNATURES = {
    "ph_create": (_i32, [_i32, _sz, ctypes.POINTER(_vp)]),
    "ph_destroy": (None, [_vp]),
    "ph_last_error": (ctypes.c_char_p, [_vp]),
    "ph_version": (_i32, []),
    "ph_set_option": (_i32, [_vp, _i32, _i64]),
    "ph_scratch_bytes": (_sz, [_vp]),
    "ph_reserve": (_i32, [_vp, _i32, _i32, _i32, _vp]),
    "ph_kernel_launches": (_i64, [_vp]),
    "ph_profile_report": (_i64, [_vp, ctypes.c_char_p, _i64]),
    "ph_binarize_le": (_i32, [_vp, _vp, _vp, _i64, ctypes.c_float, _vp]),
    "ph_transfer_sqrt": (_i32, [_vp, _vp, _i32, _i32, _f64, _f64, _vp]),
    "ph_transfer": (_i32, [_vp, _vp, _vp, _i32, _i32, _f64, _f64, _vp]),
    "ph_transfer_fp64": (_i32, [_vp, _vp, _i32, _i32, _f64, _f64, _f64, _vp]),
    "ph_gabor_wavefront": (_i32, [_vp, _vp, _vp, _i32, _i32, _vp]),
    "ph_pad2d": (_i32, [_vp, _vp, _vp, _i32, _i32, _vp]),
    "ph_phase_retrieval": (_i32, [_vp, _vp, _vp, _vp, _vp, _vp, _i32, _i32, _i32, _vp, _vp]),
    "ph_asm_prop": (_i32, [_vp, _vp, _vp, _vp, _f64, _i32, _i32, _f64, _vp]),
    "ph_reconst_xyproj": (_i32, [_vp, _vp, _vp, _vp, _vp, _vp, _i32, _i32, _i32, _vp]),
    "ph_tc_selftest": (_i32, [_vp, _vp, _vp, _i32, _i32, _i32, _vp, _vp]),
    "ph_autotune": (_i32, [_vp, _i32, _i32, _i32, _i32, ctypes.c_char_p, _vp, ctypes.POINTER(_f64), _vp]),
    "ph_reconst_xyproj_range": (_i32, [_vp, _vp, _vp, _vp, _vp, _i32, _i32, _i32, _i32, _i32, _vp]),
    "ph_unpack_projection": (_i32, [_vp, _vp, _vp, _vp, _i32, _i32, _vp]),
    "ph_reconst_xyproj_lpf": (_i32, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _i32, _i32, _i32, _vp]),
    "ph_reconst_binary_vol": (_i32, [_vp, _vp, ctypes.c_float, _vp, _vp, _vp, _vp, _i32, _i32, _i32, _vp]),
    "ph_reconst_subvolumes": (_i32, [_vp, _vp, _vp, _vp, _i32, _vp, _vp, _vp, _i32, _i32, _i32, _vp]),
    "ph_reconst_vol": (_i32, [_vp, _vp, _i32, _vp, _vp, _vp, _vp, _i32, _i32, _i32, _vp]),
    "ph_reconst_vol_padded": (_i32, [_vp, _vp, _vp, _vp, _vp, _vp, _i32, _i32, _i32, _i32, _vp]),
    "ph_propagate": (_i32, [_vp, _vp, _vp, _vp, _i32, _i32, _vp]),
    "ph_lpf_rectangle": (_i32, [_vp, _vp, _i32, _f64, _f64, _f64, _vp]),
    "ph_lpf_super_gaussian": (_i32, [_vp, _vp, _i32, _f64, _f64, _f64, _vp]),
    "ph_apply_lpf": (_i32, [_vp, _vp, _vp, _vp, _i32, _i32, _vp]),
    "ph_synth_hologram": (_i32, [_vp, _vp, _i32, _i32, _vp, _i32, _f64, _f64, _f64, _vp, _vp]),
    "ph_ccl": (_i32, [_vp, _vp, _vp, _i32, _i64, _i64, _vp]),
    "ph_ccl_roots": (_i32, [_vp, _vp, _i64, ctypes.POINTER(_i64), _vp, _i64, _vp]),
    "ph_ccl_batch": (_i32, [_vp, _vp, _vp, _i32, _i64, _i64, _i64, _vp]),
    "ph_ccl_count_noalloc": (_i32, [_vp, _vp, _i64, _vp]),
    "ph_noalloc_last_error": (ctypes.c_char_p, []),
    "ph_ccl_boxes": (_i32, [_vp, _vp, _i64, ctypes.POINTER(_i64), _vp, _i64, _i64, _i64, _vp]),
    "ph_batch_plan": (_i32, [_vp, _vp, _i32, _i32, ctypes.POINTER(_vp)]),
    "ph_batch_run": (_i32, [_vp, _vp]),
    "ph_batch_scratch_bytes": (_sz, [_vp]),
    "ph_batch_destroy": (None, [_vp]),
    "ph_serve_create": (_i32, [_vp, _i32, _i32, _i32, _i32, _i32, _sz, ctypes.POINTER(_vp)]),
    "ph_serve_stats": (_i32, [_vp, ctypes.POINTER(_i64), ctypes.POINTER(_i64), ctypes.POINTER(_sz), ctypes.POINTER(_sz),
                              ctypes.POINTER(_i64), ctypes.POINTER(_i64)]),
    "ph_serve_submit": (_i32, [_vp, _vp, ctypes.POINTER(_i64), _vp]),
    "ph_serve_poll": (_i32, [_vp, _i64, _i32, ctypes.POINTER(_f64)]),
    "ph_serve_destroy": (None, [_vp]),
    "ph_background_mode": (_i32, [_vp, _vp, _vp, _i64, _i32, _i32, _vp]),
    "ph_background_mean": (_i32, [_vp, _vp, _vp, _i64, _i32, _i32, _vp]),
    "ph_pad_with_mean": (_i32, [_vp, _vp, _vp, _i32, _i32, _i32, _vp]),
}

PH_PENDING = 9


class ServeRequest(ctypes.Structure):
    """ph_serve_request (phgb300.h)."""
    _fields_ = [("hologram", _vp), ("proj", _vp), ("argmin", _vp), ("n_fast", _i32), ("n_slow", _i32),
                ("slices", _i32), ("z0", _f64), ("dz", _f64), ("wavlen", _f64), ("dx", _f64),
                ("frame", _vp), ("frame_n_fast", _i32), ("frame_n_slow", _i32), ("frame_pitch", _i32),
                ("frame_channels", _i32), ("frame_flip", _i32), ("background", _vp), ("background_offset", _f64)]


class ReconItem(ctypes.Structure):
    """ph_recon_item (phgb300.h)."""
    _fields_ = [("hologram", _vp), ("wavefront", _vp), ("tf_front", _vp), ("tf_dz", _vp), ("proj", _vp),
                ("argmin", _vp), ("n_fast", _i32), ("n_slow", _i32), ("slices", _i32)]

_lib = None
_lock = threading.Lock()            # guards loading the library
_ctx_lock = threading.Lock()        # guards the per-device context table


class PhError(RuntimeError):
    """A libphgb300 call failed (CUDA error, timeout of a bounded device loop ...)."""

    def __init__(self, status: int, message: str):
        super().__init__(f"[status {status}] {message}")
        self.status = status


def lib():
    """The loaded library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        with _lock:
            if _lib is None:
                if not LIB_PATH.exists():
                    raise ImportError(
                        f"{LIB_PATH} is missing: build it with __graft_entry__.build() "
                        "(or python particleholography.jl_gb300/build.py); there is no CPU fallback.")
                h = ctypes.CDLL(str(LIB_PATH))
                for name, (res, args) in SIGNATURES.items():
                    fn = getattr(h, name)
                    fn.restype = res
                    fn.argtypes = args
                _lib = h
    return _lib


def raise_for(status: int, ctx) -> None:
    """Maps a status to the exception the reference raises in the same case."""
    if status == PH_OK:
        return
    msg = lib().ph_last_error(ctx).decode("utf-8", "replace") if ctx else "no context"
    if status in (PH_ERR_SIZE, PH_ERR_TOO_LARGE):
        raise AssertionError(msg)              # the reference's @assert
    if status == PH_ERR_DTYPE:
        raise ValueError(msg)                  # the reference's ArgumentError
    if status == PH_ERR_OOM:
        raise MemoryError(msg)
    raise PhError(status, msg)


class Context:
    """One ph_ctx: scratch memory, twiddle tables and cached graphs on one device."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0):
        self.device = device
        h = _vp()
        st = lib().ph_create(device, hbm_budget_bytes, ctypes.byref(h))
        if st != PH_OK:
            raise PhError(st, f"ph_create(device={device}) failed")
        self.handle = h

    def __del__(self):
        h = getattr(self, "handle", None)
        if h and _lib is not None:
            _lib.ph_destroy(h)
            self.handle = None

    def call(self, name: str, *args) -> None:
        raise_for(getattr(lib(), name)(self.handle, *args), self.handle)

    def set_option(self, option: int, value: int) -> None:
        raise_for(lib().ph_set_option(self.handle, option, int(value)), self.handle)

    def profile_report(self) -> dict:
        """{kernel name: (launches, total ms)} of the profiled passes since the last report."""
        # one call: the report also clears the records
        buf = ctypes.create_string_buffer(1 << 16)
        need = int(lib().ph_profile_report(self.handle, buf, len(buf)))
        if need > len(buf):
            raise PhError(PH_ERR_INVALID, f"profile report truncated ({need} bytes)")
        out = {}
        for line in buf.value.decode().splitlines():
            name, cnt, ms = line.split(",")
            out[name] = (int(cnt), float(ms))
        return out

    @property
    def launches(self) -> int:
        return int(lib().ph_kernel_launches(self.handle))

    @property
    def scratch_bytes(self) -> int:
        return int(lib().ph_scratch_bytes(self.handle))


_contexts: dict[int, Context] = {}


def default_context(device: int) -> Context:
    """The process-wide context of a device (created on first use)."""
    ctx = _contexts.get(device)
    if ctx is None:
        lib()                       # load outside the table lock
        with _ctx_lock:
            ctx = _contexts.get(device)
            if ctx is None:
                ctx = _contexts[device] = Context(device)
    return ctx
