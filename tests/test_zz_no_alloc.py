"""The allocation-free component count (ph_ccl_count_noalloc).

Callers that may not allocate device memory -- a real-time acquisition loop
past start-up, a host that only lends the buffers it registered up front --
count labeling components with ph_ccl_count_noalloc: no context, no
cudaMalloc, scratch in a fixed device array of the library.  Its count must
equal the regular entry point's (ph_ccl_roots, i.e. count_labels) exactly, on
two calls in a row (the second one sees the first one's leftovers in the
shared array).  This file runs last, alone or after the other tests.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _noalloc(lib):
    fn = lib.ph_ccl_count_noalloc
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]
    return fn


def _count_regular(lib, ctx, labels, s):
    c = ctypes.c_int64(-1)
    st = lib.ph_ccl_roots(ctx.handle, None, 0, ctypes.byref(c), labels.data_ptr(), labels.numel(), s)
    assert st == 0
    return c.value


def test_noalloc_count_matches_regular_twice(ph, cuda):
    from ph_gb300 import _lib
    lib = _lib.lib()
    fn = _noalloc(lib)
    ctx = _lib.default_context(0)
    s = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(12)
    images = [(rng.random((1024, 1024)) < 0.45), (rng.random((512, 768)) < 0.6)]
    out = torch.full((1,), -1, dtype=torch.int64, device=cuda)
    for img in images:
        lab = ph.cu_connected_component_labeling(torch.from_numpy(img).to(cuda), reference_grid=False)
        want = _count_regular(lib, ctx, lab, s)
        assert want > 0
        for _ in range(2):                      # two calls in a row on the shared scratch
            out.fill_(-1)
            st = fn(out.data_ptr(), lab.data_ptr(), lab.numel(), s)
            assert st == 0, lib.ph_noalloc_last_error()
            torch.cuda.synchronize()
            assert int(out.item()) == want


def test_noalloc_rejects_oversize(ph, cuda):
    from ph_gb300 import _lib
    lib = _lib.lib()
    fn = _noalloc(lib)
    lib.ph_noalloc_last_error.restype = ctypes.c_char_p
    out = torch.zeros((1,), dtype=torch.int64, device=cuda)
    lab = torch.zeros((4,), dtype=torch.int32, device=cuda)
    st = fn(out.data_ptr(), lab.data_ptr(), (1 << 28) + 1, torch.cuda.current_stream().cuda_stream)
    assert st == _lib.PH_ERR_TOO_LARGE
    assert b"exceed" in lib.ph_noalloc_last_error()


def test_noalloc_empty_input_counts_zero(ph, cuda):
    """n = 0 writes a count of 0 (and launches nothing that reads labels)."""
    from ph_gb300 import _lib
    lib = _lib.lib()
    fn = _noalloc(lib)
    out = torch.full((1,), -1, dtype=torch.int64, device=cuda)
    lab = torch.zeros((1,), dtype=torch.int32, device=cuda)
    for _ in range(2):
        out.fill_(-1)
        assert fn(out.data_ptr(), lab.data_ptr(), 0, torch.cuda.current_stream().cuda_stream) == 0
        torch.cuda.synchronize()
        assert int(out.item()) == 0
