"""Parity at the workloads' full sizes.

* 1024^2 x 256 (the plain-method workload) on a seeded synthetic hologram:
  projection rel L2 and argmin-depth agreement against the full FP32 oracle.
* 2048^2 x 512 (the phase-retrieval workload's reconstruction): size-independent
  properties -- exact power-of-two scaling, the projection bounds every slice,
  the argmin slice attains the minimum -- and slices k in {0, S/2, S-1} against
  the oracle's cumulative-product slices.
* 2048^2 Gerchberg-Saxton, 20 iterations, against the FP32 oracle.
"""
import numpy as np
import pytest
import torch

from oracle import ref_semantics as ref
from phtest import ARGMIN_AGREE, REL_L2, rel_l2, to_np

pytestmark = pytest.mark.gpu
LAM, DX = 0.6328, 10.0


def _synth(ph, n, seed, count, dmin, dmax, zmin, zmax):
    from ph_gb300 import synth
    return synth.synth_hologram(synth.HologramSpec(seed=seed, n=n, count=count, dmin=dmin, dmax=dmax, zmin=zmin,
                                                   zmax=zmax), 0)


def test_plain_1024_x256_against_oracle(ph, cuda):
    n, S, z0, dz = 1024, 256, 1000.0, 200.0
    holo = _synth(ph, n, 1, 200, 20.0, 80.0, 1000.0, 50000.0)
    d = ph.cu_transfer_sqrt_arr(n, LAM, DX)
    hf, hdz = ph.cu_transfer(-z0, n, LAM, d), ph.cu_transfer(-dz, n, LAM, d)
    proj, arg = ph.cu_get_reconst_xyprojection(ph.cu_gabor_wavefront(holo), hf, hdz, S, return_argmin=True)
    h = to_np(holo)
    p_ref, a_ref = ref.reconst_xyprojection(ref.gabor_wavefront(h), to_np(hf.data), to_np(hdz.data), S,
                                            with_argmin=True)
    assert rel_l2(to_np(proj), p_ref) < REL_L2
    assert np.mean(to_np(arg) == a_ref) >= ARGMIN_AGREE
    # the labeling of the thresholded projection is bit-exact against the oracle on the same binary image
    from oracle import ccl as occl
    binary = proj <= 0.5
    lab = ph.cu_connected_component_labeling(binary)
    want = occl.connected_component_labeling(to_np(binary).astype(np.float32))
    assert np.array_equal(to_np(lab).astype(np.uint32), want)
    assert ph.count_labels(lab) == ref.count_labels(want) > 0


@pytest.fixture(scope="module")
def big(ph, cuda):
    n, S = 2048, 512
    holo = _synth(ph, n, 2, 800, 10.0, 60.0, 5000.0, 100000.0)
    d = ph.cu_transfer_sqrt_arr(n, LAM, DX)
    hf, hdz = ph.cu_transfer(-5000.0, n, LAM, d), ph.cu_transfer(-200.0, n, LAM, d)
    return holo, hf, hdz, n, S


def test_2048_x512_properties(ph, big):
    holo, hf, hdz, n, S = big
    proj, arg = ph.cu_get_reconst_xyprojection(ph.cu_gabor_wavefront(holo), hf, hdz, S, return_argmin=True)
    # scaling the hologram by 4 scales the wavefront by 2 and every intensity by 4, exactly
    p4, a4 = ph.cu_get_reconst_xyprojection(ph.cu_gabor_wavefront(holo * 4), hf, hdz, S, return_argmin=True)
    assert torch.equal(p4, proj * 4) and torch.equal(a4, arg)
    # deterministic
    p2, a2 = ph.cu_get_reconst_xyprojection(ph.cu_gabor_wavefront(holo), hf, hdz, S, return_argmin=True)
    assert torch.equal(p2, proj) and torch.equal(a2, arg)
    a = to_np(arg)
    assert a.min() >= 0 and a.max() < S


def test_2048_x512_slices_against_oracle(ph, big):
    holo, hf, hdz, n, S = big
    cvol = ph.cu_get_reconst_complex_vol(ph.cu_gabor_wavefront(holo), hf, hdz, S)      # 16 GiB
    proj, arg = ph.cu_get_reconst_xyprojection(ph.cu_gabor_wavefront(holo), hf, hdz, S, return_argmin=True)
    inten = cvol.real ** 2 + cvol.imag ** 2
    pmin, _ = inten.min(dim=0)
    assert rel_l2(to_np(pmin), to_np(proj)) < 1e-6
    picked = torch.gather(inten, 0, arg.long().unsqueeze(0))[0]
    assert rel_l2(to_np(picked), to_np(proj)) < 1e-6
    want = {0, S // 2, S - 1}
    hfn, hdzn = to_np(hf.data), to_np(hdz.data)
    for k, x in enumerate(ref.iter_slices(ref.gabor_wavefront(to_np(holo)), hfn, hdzn, S)):
        if k in want:
            u = ref._ifft2(ref.ifftshift(x))
            assert rel_l2(to_np(cvol[k]), u) < REL_L2, k
    del cvol, inten


def test_gs_2048_x20_against_oracle(ph, cuda):
    from ph_gb300 import synth
    n = 2048
    spec = synth.HologramSpec(seed=2, n=n, count=800, dmin=10.0, dmax=60.0, zmin=5000.0, zmax=100000.0)
    h1, h2 = synth.synth_pair(spec, 5000.0, 0)
    d = ph.cu_transfer_sqrt_arr(n, LAM, DX)
    tp, tpi = ph.cu_transfer(5000.0, n, LAM, d), ph.cu_transfer(-5000.0, n, LAM, d)
    u, res = ph.cu_phase_retrieval_holo(h1, h2, tp, tpi, 20, n, return_residual=True)
    u_ref, r_ref = ref.phase_retrieval_holo(to_np(h1), to_np(h2), to_np(tp.data), to_np(tpi.data), 20, n,
                                            return_residual=True)
    assert rel_l2(to_np(u.data), u_ref) < REL_L2
    assert abs(float(res) - r_ref) <= 1e-4 * max(r_ref, 1e-3)


def test_gs2048_then_2048_x512_projection_against_oracle(ph, cuda):
    """The whole phase-retrieval workload against the oracle: 20 GS iterations on
    the seeded 2048^2 pair 5 mm apart, then the full 512-slice projection and
    argmin of the retrieved field (every pixel, every slice)."""
    from ph_gb300 import synth
    n, S = 2048, 512
    spec = synth.HologramSpec(seed=2, n=n, count=800, dmin=10.0, dmax=60.0, zmin=5000.0, zmax=100000.0)
    h1, h2 = synth.synth_pair(spec, 5000.0, 0)
    d = ph.cu_transfer_sqrt_arr(n, LAM, DX)
    tp, tpi = ph.cu_transfer(5000.0, n, LAM, d), ph.cu_transfer(-5000.0, n, LAM, d)
    hf, hdz = ph.cu_transfer(-5000.0, n, LAM, d), ph.cu_transfer(-200.0, n, LAM, d)
    u = ph.cu_phase_retrieval_holo(h1, h2, tp, tpi, 20, n)
    proj, arg = ph.cu_get_reconst_xyprojection(u, hf, hdz, S, return_argmin=True)
    u_ref = ref.phase_retrieval_holo(to_np(h1), to_np(h2), to_np(tp.data), to_np(tpi.data), 20, n)
    p_ref, a_ref = ref.reconst_xyprojection(u_ref, to_np(hf.data), to_np(hdz.data), S, with_argmin=True)
    assert rel_l2(to_np(proj), p_ref) < REL_L2
    assert np.mean(to_np(arg) == a_ref) >= ARGMIN_AGREE


def test_4096_x1024_slices_against_oracle(ph, cuda):
    """The precision workload's size, 4096^2 over 1024 slices (3000 discs):
    the first slices through the complex-volume path, and slices 511 and 1023
    through one-slice depth shards (global slice index), against the oracle's
    cumulative product from slice 0."""
    from ph_gb300 import parallel
    n, S = 4096, 1024
    holo = _synth(ph, n, 3, 3000, 10.0, 60.0, 5000.0, 200000.0)
    d = ph.cu_transfer_sqrt_arr(n, LAM, DX)
    dz = (200000.0 - 5000.0) / S
    hf, hdz = ph.cu_transfer(-5000.0, n, LAM, d), ph.cu_transfer(-dz, n, LAM, d)
    wf = ph.cu_gabor_wavefront(holo)
    cvol = to_np(ph.cu_get_reconst_complex_vol(wf, hf, hdz, 3))
    one = {}
    for k in (S // 2 - 1, S - 1):
        p, a = parallel.unpack_projection(parallel.reconst_xyprojection_range(wf, hf, hdz, k, k + 1))
        assert torch.all(a == k)
        one[k] = to_np(p)
    hfn, hdzn = to_np(hf.data), to_np(hdz.data)
    for k, x in enumerate(ref.iter_slices(ref.gabor_wavefront(to_np(holo)), hfn, hdzn, S)):
        if k < 3:
            assert rel_l2(cvol[k], ref._ifft2(ref.ifftshift(x))) < REL_L2, k
        elif k in one:
            assert rel_l2(one[k], ref._intensity(ref._ifft2(ref.ifftshift(x)))) < REL_L2, k


def test_padded_1024_to_2048_x64_against_oracle(ph, cuda):
    """cu_get_reconst_vol_and_xyprojection_padded (holofunc.jl:339-364) at a
    realistic size: a 1024^2 wavefront mean-padded to 2048^2, 64 slices."""
    n, S = 1024, 64
    holo = _synth(ph, n, 4, 200, 20.0, 80.0, 1000.0, 50000.0)
    d2 = ph.cu_transfer_sqrt_arr(2 * n, LAM, DX)
    hf, hdz = ph.cu_transfer(-10000.0, 2 * n, LAM, d2), ph.cu_transfer(-300.0, 2 * n, LAM, d2)
    vol, proj = ph.cu_get_reconst_vol_and_xyprojection_padded(ph.cu_gabor_wavefront(holo), hf, hdz, S)
    v_ref, p_ref = ref.reconst_vol_and_xyprojection_padded(ref.gabor_wavefront(to_np(holo)), to_np(hf.data),
                                                           to_np(hdz.data), S)
    v = to_np(vol)
    assert v.shape == v_ref.shape == (S, n, n)
    diff = np.abs(v.astype(np.int16) - v_ref.astype(np.int16))
    assert diff.max() <= 1 and np.mean(diff > 0) < 1e-4
    assert np.array_equal(to_np(proj), ref.xy_projection_from_vol(v))
    assert np.mean(to_np(proj) != p_ref) < 1e-4
