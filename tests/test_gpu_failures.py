"""Failure detection without a GPU fault: host-side refusals map to the
reference's exceptions, a context refuses scratch beyond its HBM budget, and
bad arguments never reach a kernel."""
import numpy as np
import pytest
import torch

from phtest import to_dev

pytestmark = pytest.mark.gpu
LAM, DX = 0.6328, 10.0


def test_hbm_budget_refusal(ph, cuda):
    from ph_gb300 import _lib
    ctx = _lib.Context(0, hbm_budget_bytes=1 << 20)      # 1 MiB: far too small for 256^2 x 8 slices
    n = 256
    wf = torch.ones((n, n), dtype=torch.complex64, device=cuda)
    proj = torch.empty((n, n), dtype=torch.float32, device=cuda)
    with pytest.raises(MemoryError, match="HBM budget"):
        ctx.call("ph_reconst_xyproj", proj.data_ptr(), None, wf.data_ptr(), wf.data_ptr(), wf.data_ptr(), n, n, 8,
                 torch.cuda.current_stream().cuda_stream)
    assert ctx.scratch_bytes == 0
    # the same context still serves a call that fits
    small = torch.ones((8, 8), dtype=torch.complex64, device=cuda)
    p8 = torch.empty((8, 8), dtype=torch.float32, device=cuda)
    ctx.call("ph_reconst_xyproj", p8.data_ptr(), None, small.data_ptr(), small.data_ptr(), small.data_ptr(), 8, 8, 2,
             torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert torch.isfinite(p8).all()


def test_argument_errors(ph, cuda):
    from ph_gb300 import _lib
    ctx = _lib.default_context(0)
    s = torch.cuda.current_stream().cuda_stream
    x = torch.ones((12, 12), dtype=torch.complex64, device=cuda)
    p = torch.empty((12, 12), dtype=torch.float32, device=cuda)
    with pytest.raises(_lib.PhError, match="not supported"):          # 10 is neither 2^a nor 3*2^a
        ctx.call("ph_reconst_xyproj", p.data_ptr(), None, x.data_ptr(), x.data_ptr(), x.data_ptr(), 10, 10, 2, s)
    with pytest.raises(_lib.PhError, match="must not be NULL"):
        ctx.call("ph_reconst_xyproj", p.data_ptr(), None, None, x.data_ptr(), x.data_ptr(), 8, 8, 2, s)
    with pytest.raises(AssertionError, match="slices must be >= 1"):
        ctx.call("ph_reconst_xyproj", p.data_ptr(), None, x.data_ptr(), x.data_ptr(), x.data_ptr(), 8, 8, 0, s)
    with pytest.raises(ValueError, match="return_type"):
        ctx.call("ph_reconst_vol", p.data_ptr(), 9, None, x.data_ptr(), x.data_ptr(), x.data_ptr(), 8, 8, 2, s)
    with pytest.raises(AssertionError, match="too large"):
        ctx.call("ph_ccl", p.data_ptr(), p.data_ptr(), _lib.PH_F32, 1 << 17, 1 << 16, s)
    # the context is still usable afterwards
    d = ph.cu_transfer_sqrt_arr(8, LAM, DX)
    assert torch.isfinite(d.data).all()


def test_two_streams_are_ordered(ph, cuda):
    """Calls of one context on different streams never overlap on its scratch."""
    n = 512
    rng = np.random.default_rng(3)
    holo = to_dev(rng.uniform(0.1, 1.0, (n, n)).astype(np.float32), cuda)
    d = ph.cu_transfer_sqrt_arr(n, LAM, DX)
    tf, tdz = ph.cu_transfer(-1000.0, n, LAM, d), ph.cu_transfer(-200.0, n, LAM, d)
    wf = ph.cu_gabor_wavefront(holo)
    want = ph.cu_get_reconst_xyprojection(wf, tf, tdz, 16)
    torch.cuda.synchronize()
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    outs = []
    for k in range(6):
        with torch.cuda.stream(s1 if k % 2 == 0 else s2):
            outs.append(ph.cu_get_reconst_xyprojection(wf, tf, tdz, 16))
    torch.cuda.synchronize()
    for o in outs:
        assert torch.equal(o, want)
