"""Depth shards through the library (ph_reconst_xyproj_range +
ph_unpack_projection): slice ranges with global indices, merged by a per-word
minimum, equal one reconstruction over all slices (holofunc.jl:248-266)."""
import numpy as np
import pytest
import torch

from oracle import ref_semantics as ref
from phtest import ARGMIN_AGREE, REL_L2, rel_l2, to_dev, to_np

pytestmark = pytest.mark.gpu
LAM, DX = 0.6328, 10.0


def _case(n, seed, slices_dz=-200.0):
    rng = np.random.default_rng(seed)
    holo = rng.uniform(0.1, 1.0, (n, n)).astype(np.float32)
    d = ref.transfer_sqrt_arr(n, LAM, DX)
    return holo, ref.transfer(-1000.0, n, LAM, d), ref.transfer(slices_dz, n, LAM, d)


def _tensors(ph, cuda, holo, hf, hdz):
    return (ph.cu_gabor_wavefront(to_dev(holo, cuda)), ph.CuTransfer(to_dev(hf, cuda)),
            ph.CuTransfer(to_dev(hdz, cuda)))


@pytest.mark.parametrize("n,cuts", [(256, (0, 7, 19)), (1024, (0, 1, 2, 40)), (96, (0, 13, 13, 30))])
def test_shards_bit_identical(ph, cuda, n, cuts):
    """Where every slice is evaluated directly from the spectrum state (no
    product chain), shards reproduce the single call bit for bit."""
    from ph_gb300 import parallel
    wf, tf, td = _tensors(ph, cuda, *_case(n, seed=n))
    slices = cuts[-1]
    p1, a1 = ph.cu_get_reconst_xyprojection(wf, tf, td, slices, return_argmin=True)
    # accumulate into one buffer, shard after shard
    packed = None
    for i, (k0, k1) in enumerate(zip(cuts[:-1], cuts[1:])):
        packed = parallel.reconst_xyprojection_range(wf, tf, td, k0, k1, packed=packed, accumulate=i > 0)
    p, a = parallel.unpack_projection(packed)
    assert np.array_equal(to_np(p), to_np(p1)) and np.array_equal(to_np(a), to_np(a1))
    # separate buffers merged by an int64 minimum (what an all-reduce MIN does)
    parts = [parallel.reconst_xyprojection_range(wf, tf, td, k0, k1) for k0, k1 in zip(cuts[:-1], cuts[1:])]
    merged = parts[0]
    for q in parts[1:]:
        merged = torch.minimum(merged, q)
    assert torch.equal(merged, packed)


def test_chain_length_shards(ph, cuda):
    """At 2048 pass A advances X by the Hdz product within a slice group, so
    shards agree with the single call to the chain's rounding, and both with
    the oracle's chain from slice 0."""
    from ph_gb300 import parallel
    n, slices = 2048, 96
    holo, hf, hdz = _case(n, seed=5, slices_dz=-100.0)
    wf, tf, td = _tensors(ph, cuda, holo, hf, hdz)
    p1, a1 = (to_np(t) for t in ph.cu_get_reconst_xyprojection(wf, tf, td, slices, return_argmin=True))
    packed = parallel.reconst_xyprojection_range(wf, tf, td, 0, 40)
    parallel.reconst_xyprojection_range(wf, tf, td, 40, slices, packed=packed, accumulate=True)
    p, a = (to_np(t) for t in parallel.unpack_projection(packed))
    p_ref, a_ref = ref.reconst_xyprojection(ref.gabor_wavefront(holo), hf, hdz, slices, with_argmin=True)
    assert rel_l2(p, p1) < 1e-5 and np.mean(a == a1) >= ARGMIN_AGREE
    assert rel_l2(p, p_ref) < REL_L2 and np.mean(a == a_ref) >= ARGMIN_AGREE


def test_chain_length_shards_4096(ph, cuda):
    """At 4096 pass A's tensor-map store form (full frames) also runs the
    product chain: shards (chains of 10 and 14 slices) agree with the single
    call (one chain of 24) to the chain's rounding."""
    from ph_gb300 import parallel
    n, slices, cut = 4096, 24, 10
    wf, tf, td = _tensors(ph, cuda, *_case(n, seed=7, slices_dz=-100.0))
    p1, a1 = (to_np(t) for t in ph.cu_get_reconst_xyprojection(wf, tf, td, slices, return_argmin=True))
    packed = parallel.reconst_xyprojection_range(wf, tf, td, 0, cut)
    parallel.reconst_xyprojection_range(wf, tf, td, cut, slices, packed=packed, accumulate=True)
    p, a = (to_np(t) for t in parallel.unpack_projection(packed))
    assert rel_l2(p, p1) < 1e-5 and np.mean(a == a1) >= ARGMIN_AGREE


def test_empty_shard_is_identity(ph, cuda):
    from ph_gb300 import parallel, _lib
    wf, tf, td = _tensors(ph, cuda, *_case(64, seed=3))
    packed = parallel.reconst_xyprojection_range(wf, tf, td, 5, 5)
    assert torch.all(packed == _lib.PH_PACKED_EMPTY)
    # merging the identity changes nothing
    real = parallel.reconst_xyprojection_range(wf, tf, td, 0, 5)
    before = real.clone()
    parallel.reconst_xyprojection_range(wf, tf, td, 5, 5, packed=real, accumulate=True)
    assert torch.equal(real, before)


def test_bad_range_rejected(ph, cuda):
    from ph_gb300 import parallel
    wf, tf, td = _tensors(ph, cuda, *_case(16, seed=1))
    with pytest.raises(AssertionError):
        parallel.reconst_xyprojection_range(wf, tf, td, 4, 2)
