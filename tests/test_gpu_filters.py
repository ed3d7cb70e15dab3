"""Low-pass filters (frequency_filters.jl) on the GPU against the oracle; the
reference's own tests (runtests.jl:519-576) are mirrored first."""
import numpy as np
import pytest
import torch

from oracle import ref_semantics as ref
from phtest import REL_L2, rel_l2, to_dev, to_np

pytestmark = pytest.mark.gpu


def test_reference_filter_tests(ph, cuda):
    # runtests.jl:520-541
    for build in (ph.cu_rectangle_filter, ph.cu_super_gaussian_filter):
        lpf = build(0.01, 5.3e-7, 128, 6.5e-6)
        assert isinstance(lpf, ph.CuLowPassFilter) and lpf.size() == (128, 128)
    # runtests.jl:543-575: all-pass filter on an (i+j, i-j) field changes the data only by FFT rounding
    i = np.arange(1, 129)
    jl = (i[:, None] + i[None, :]) + 1j * (i[:, None] - i[None, :])     # Julia [i, j]
    holo = ph.CuWavefront(to_dev(jl.T.astype(np.complex64), cuda))
    orig = holo.data.clone()
    ones = ph.CuLowPassFilter(torch.ones((128, 128), dtype=torch.float32, device=cuda))
    out = ph.cu_apply_low_pass_filter(holo, ones)
    assert out is not holo and tuple(out.data.shape) == (128, 128) and out.data.dtype == torch.complex64
    assert torch.equal(holo.data, orig)
    ph.cu_apply_low_pass_filter_(holo, ones)
    assert holo.data.dtype == torch.complex64
    assert rel_l2(to_np(holo.data), to_np(orig)) < 1e-6


@pytest.mark.parametrize("n,d,lam,p", [(128, 0.01, 5.3e-7, 6.5e-6), (1024, 80000.0, 0.6328, 10.0),
                                       (256, 5000.0, 0.6328, 10.0)])
def test_masks_match_oracle(ph, cuda, n, d, lam, p):
    assert np.array_equal(to_np(ph.cu_rectangle_filter(d, lam, n, p).data), ref.rectangle_filter(d, lam, n, p))
    g = to_np(ph.cu_super_gaussian_filter(d, lam, n, p).data)
    assert np.max(np.abs(g - ref.super_gaussian_filter(d, lam, n, p))) < 2e-7


def test_apply_matches_oracle(ph, cuda):
    n = 256
    rng = np.random.default_rng(2)
    u = (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))).astype(np.complex64)
    m = ref.super_gaussian_filter(20000.0, 0.6328, n, 10.0)
    got = ph.cu_apply_low_pass_filter(ph.CuWavefront(to_dev(u, cuda)), ph.CuLowPassFilter(to_dev(m, cuda)))
    assert rel_l2(to_np(got.data), ref.apply_low_pass_filter(u, m)) < REL_L2


@pytest.mark.parametrize("n,slices,build", [(256, 9, "super_gaussian"), (512, 5, "rectangle")])
def test_filtered_projection_matches_filter_then_reconstruct(ph, cuda, n, slices, build):
    """The low-pass filter folded into the reconstruction spectrum equals
    cu_apply_low_pass_filter followed by cu_get_reconst_xyprojection."""
    rng = np.random.default_rng(n)
    holo = rng.uniform(0.1, 1.0, (n, n)).astype(np.float32)
    d = ref.transfer_sqrt_arr(n, 0.6328, 10.0)
    hf, hdz = ref.transfer(-3000.0, n, 0.6328, d), ref.transfer(-150.0, n, 0.6328, d)
    mask = (ref.super_gaussian_filter if build == "super_gaussian" else ref.rectangle_filter)(60000.0, 0.6328, n, 10.0)
    wf = ref.gabor_wavefront(holo)
    want, want_arg = ref.reconst_xyprojection(ref.apply_low_pass_filter(wf, mask), hf, hdz, slices, with_argmin=True)
    got, arg = ph.cu_get_reconst_xyprojection_lpf(ph.CuWavefront(to_dev(wf, cuda)), ph.CuTransfer(to_dev(hf, cuda)),
                                                  ph.CuTransfer(to_dev(hdz, cuda)), to_dev(mask, cuda), slices,
                                                  return_argmin=True)
    assert rel_l2(to_np(got), want) < REL_L2
    assert np.mean(to_np(arg) == want_arg) >= 0.999
