"""ctypes loader for the C restatement of the reference CCL (``ccl_ref.c``).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).  ``build()`` compiles
``ccl_ref.c`` with gcc into ``oracle/_build/libccl_oracle.so``; it is rebuilt
when the source is newer than the library.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
_SRC = _HERE / "ccl_ref.c"
_LIB = _HERE / "_build" / "libccl_oracle.so"
_handle = None


def build(force: bool = False) -> Path:
    """Compile the C oracle (gcc, -O2, portable: no -march flags)."""
    if force or not _LIB.exists() or _LIB.stat().st_mtime < _SRC.stat().st_mtime:
        _LIB.parent.mkdir(exist_ok=True)
        tmp = _LIB.with_suffix(f".{os.getpid()}.tmp")
        subprocess.run(["gcc", "-O2", "-std=c99", "-fPIC", "-shared", str(_SRC), "-o", str(tmp)], check=True)
        os.replace(tmp, _LIB)
    return _LIB


def _lib():
    global _handle
    if _handle is None:
        build()
        h = ctypes.CDLL(str(_LIB))
        h.oracle_ccl_f32.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64]
        h.oracle_ccl_f32.restype = None
        _handle = h
    return _handle


def connected_component_labeling(img: np.ndarray, rows: int | None = None, cols: int | None = None) -> np.ndarray:
    """``cu_connected_component_labeling`` (ccl.jl:186-211) on the CPU.

    ``img`` is any real or bool array; it is compared for equality as Float32.
    The buffer is labelled as a C-row-major ``rows x cols`` grid (default: the
    array's own 2-D shape).  Returns UInt32 labels of the same shape.
    """
    a = np.ascontiguousarray(np.asarray(img), dtype=np.float32)
    if a.size > 2**32 - 1:
        raise AssertionError("Image is too large. Maximum length is 2^32-1.")
    if rows is None or cols is None:
        rows, cols = a.shape
    assert rows * cols == a.size
    out = np.zeros(a.shape, dtype=np.uint32)
    _lib().oracle_ccl_f32(a.ctypes.data, out.ctypes.data, int(rows), int(cols))
    return out
