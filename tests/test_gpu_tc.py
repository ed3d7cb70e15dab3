"""The tensor-core building block of the split-precision passes: one tcgen05
MMA chain (swizzled K-major operand tiles, shared-memory descriptors, FP32
accumulators in tensor memory) against a host product of the same 16-bit
operands."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _bits(x: np.ndarray, fp16: bool) -> np.ndarray:
    if fp16:
        return x.astype(np.float16).view(np.uint16)
    u = x.astype(np.float32).view(np.uint32)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)     # round to nearest even


def _value(bits: np.ndarray, fp16: bool) -> np.ndarray:
    if fp16:
        return bits.view(np.float16).astype(np.float64)
    return (bits.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


@pytest.mark.parametrize("fp16", [0, 1])
@pytest.mark.parametrize("n,k", [(16, 64), (64, 64), (64, 128), (128, 128), (32, 128)])
def test_tc_product(ph, cuda, n, k, fp16):
    from ph_gb300 import _lib
    rng = np.random.default_rng(n * 1000 + k + fp16)
    a = _bits(rng.standard_normal((128, k)).astype(np.float32), fp16)
    b = _bits(rng.standard_normal((n, k)).astype(np.float32), fp16)
    want = _value(a, fp16) @ _value(b, fp16).T
    da = torch.from_numpy(a.view(np.int16)).to(cuda)
    db = torch.from_numpy(b.view(np.int16)).to(cuda)
    d = torch.full((128, n), float("nan"), dtype=torch.float32, device=cuda)
    err = torch.zeros(1, dtype=torch.int32, device=cuda)
    st = _lib.lib().ph_tc_selftest(d.data_ptr(), da.data_ptr(), db.data_ptr(), n, k, fp16, err.data_ptr(),
                                   torch.cuda.current_stream().cuda_stream)
    assert st == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    got = d.cpu().numpy().astype(np.float64)
    assert np.all(np.isfinite(got))
    assert np.max(np.abs(got - want)) <= 1e-5 * np.max(np.abs(want)) + 1e-6
