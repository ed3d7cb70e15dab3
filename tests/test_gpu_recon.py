"""Reconstruction parity on the GPU against the reference-semantics oracle
(holofunc.jl:184-364): projection + argmin, volumes of every return type,
complex volume, volume + projection, padded variant."""
import numpy as np
import pytest
import torch

from oracle import ref_semantics as ref
from phtest import ARGMIN_AGREE, REL_L2, rel_l2, to_dev, to_np

pytestmark = pytest.mark.gpu
LAM, DX = 0.6328, 10.0


def _case(n, seed=0, z0=-1000.0, dz=-200.0, n_slow=None):
    rng = np.random.default_rng(seed)
    ny = n if n_slow is None else n_slow
    holo = rng.uniform(0.1, 1.0, (ny, n)).astype(np.float32)
    d = ref.transfer_sqrt_arr(n, LAM, DX, n_slow=ny)
    return holo, ref.transfer(z0, n, LAM, d), ref.transfer(dz, n, LAM, d)


@pytest.mark.parametrize("n,slices", [(1, 2), (2, 3), (4, 3), (8, 5), (16, 7), (32, 9), (64, 12), (128, 10),
                                      (256, 6), (512, 4), (1024, 3), (2048, 2), (4096, 2), (8192, 2)])
def test_xyprojection_matches_oracle(ph, cuda, n, slices):
    holo, hf, hdz = _case(n, seed=n)
    wf = ph.cu_gabor_wavefront(to_dev(holo, cuda))
    proj, arg = ph.cu_get_reconst_xyprojection(wf, ph.CuTransfer(to_dev(hf, cuda)), ph.CuTransfer(to_dev(hdz, cuda)),
                                               slices, return_argmin=True)
    p_ref, a_ref = ref.reconst_xyprojection(ref.gabor_wavefront(holo), hf, hdz, slices, with_argmin=True)
    assert rel_l2(to_np(proj), p_ref) < REL_L2
    assert np.mean(to_np(arg) == a_ref) >= (ARGMIN_AGREE if n >= 16 else 1.0 - 1.0 / (n * n))


def test_xyprojection_golden(ph, cuda, golden):
    g = golden("oracle_small")
    wf = ph.cu_gabor_wavefront(to_dev(g["rec_holo"], cuda))
    proj, arg = ph.cu_get_reconst_xyprojection(wf, ph.CuTransfer(to_dev(g["rec_hf"], cuda)),
                                               ph.CuTransfer(to_dev(g["rec_hdz"], cuda)), 12, return_argmin=True)
    assert rel_l2(to_np(proj), g["rec_proj"]) < REL_L2
    assert np.mean(to_np(arg) == g["rec_argmin"]) >= ARGMIN_AGREE


# (6, 4096), (3, 8192), (24, 6144): pass A rows in clusters of 2 / 4 / 2 CTAs, the last
# cluster padded with CTAs that hold no valid row
@pytest.mark.parametrize("nx,ny", [(32, 16), (16, 64), (256, 128), (3, 6), (12, 24), (96, 48), (768, 384),
                                   (2048, 1536), (1536, 1536), (6, 4096), (3, 8192), (24, 6144), (4096, 32)])
def test_rectangular_projection(ph, cuda, nx, ny):
    holo, hf, hdz = _case(nx, seed=3, n_slow=ny)
    wf = ph.cu_gabor_wavefront(to_dev(holo, cuda))
    proj = ph.cu_get_reconst_xyprojection(wf, ph.CuTransfer(to_dev(hf, cuda)), ph.CuTransfer(to_dev(hdz, cuda)), 5)
    p_ref = ref.reconst_xyprojection(ref.gabor_wavefront(holo), hf, hdz, 5)
    assert rel_l2(to_np(proj), p_ref) < REL_L2


@pytest.mark.parametrize("rt,np_rt", [("N0f8", ref.N0f8), (torch.float16, np.float16), (torch.float32, np.float32),
                                      (torch.float64, np.float64)])
def test_vol_return_types(ph, cuda, rt, np_rt):
    holo, hf, hdz = _case(64, seed=5)
    rtype = ph.N0f8 if rt == "N0f8" else rt
    wf = ph.cu_gabor_wavefront(to_dev(holo, cuda))
    vol = ph.cu_get_reconst_vol(wf, ph.CuTransfer(to_dev(hf, cuda)), ph.CuTransfer(to_dev(hdz, cuda)), 6, rtype)
    v_ref = ref.reconst_vol(ref.gabor_wavefront(holo), hf, hdz, 6, np_rt)
    got = to_np(vol)
    assert got.shape == v_ref.shape
    if np_rt is ref.N0f8:
        diff = np.abs(got.astype(np.int32) - v_ref.astype(np.int32))
        assert diff.max() <= 1 and np.mean(diff > 0) < 1e-3      # rounding-boundary flips only
    else:
        assert rel_l2(got.astype(np.float64), v_ref.astype(np.float64)) < (2e-3 if np_rt is np.float16 else REL_L2)


def test_complex_vol(ph, cuda, golden):
    g = golden("oracle_small")
    wf = ph.cu_gabor_wavefront(to_dev(g["rec_holo"][:16, :16].copy(), cuda))
    cv = ph.cu_get_reconst_complex_vol(wf, ph.CuTransfer(to_dev(g["rec_hf"][:16, :16].copy(), cuda)),
                                       ph.CuTransfer(to_dev(g["rec_hdz"][:16, :16].copy(), cuda)), 4)
    assert rel_l2(to_np(cv), g["rec_cvol"]) < REL_L2


def test_vol_and_xyprojection(ph, cuda, golden):
    g = golden("oracle_small")
    wf = ph.cu_gabor_wavefront(to_dev(g["rec_holo"], cuda))
    vol, proj = ph.cu_get_reconst_vol_and_xyprojection(wf, ph.CuTransfer(to_dev(g["rec_hf"], cuda)),
                                                       ph.CuTransfer(to_dev(g["rec_hdz"], cuda)), 12)
    diff = np.abs(to_np(vol).astype(np.int32) - g["rec_vol_n0f8"].astype(np.int32))
    assert diff.max() <= 1
    # the projection is the strict-< minimum of the stored N0f8 volume
    assert np.array_equal(to_np(proj), ref.xy_projection_from_vol(to_np(vol)))
    assert np.mean(np.abs(to_np(proj) - g["rec_volproj_proj"]) > 0) < 1e-3


@pytest.mark.parametrize("m,slices", [(4, 2), (16, 4)])
def test_padded(ph, cuda, golden, m, slices):
    g = golden("oracle_small")
    wf = ph.cu_gabor_wavefront(to_dev(g[f"pad{m}_holo"], cuda))
    vol, proj = ph.cu_get_reconst_vol_and_xyprojection_padded(wf, ph.CuTransfer(to_dev(g[f"pad{m}_tf"], cuda)),
                                                              ph.CuTransfer(to_dev(g[f"pad{m}_tdz"], cuda)), slices)
    assert tuple(vol.shape) == (slices, m, m) and vol.dtype == torch.uint8     # runtests.jl:379-382
    assert tuple(proj.shape) == (m, m) and proj.dtype == torch.float32
    diff = np.abs(to_np(vol).astype(np.int32) - g[f"pad{m}_vol"].astype(np.int32))
    assert diff.max() <= 1 and np.mean(diff > 0) < 0.02
    assert np.array_equal(to_np(proj), ref.xy_projection_from_vol(to_np(vol)))


def test_size_assertions(ph, cuda):
    holo, hf, hdz = _case(16)
    wf = ph.cu_gabor_wavefront(to_dev(holo, cuda))
    bad = ph.CuTransfer(to_dev(np.ones((8, 8), np.complex64), cuda))
    with pytest.raises(AssertionError, match="All arrays must have the same size"):
        ph.cu_get_reconst_xyprojection(wf, bad, bad, 3)
    with pytest.raises(ValueError, match="return_type"):
        ph.cu_get_reconst_vol(wf, ph.CuTransfer(to_dev(hf, cuda)), ph.CuTransfer(to_dev(hdz, cuda)), 3, torch.int32)
    with pytest.raises(AssertionError, match="2\\*size"):
        ph.cu_get_reconst_vol_and_xyprojection_padded(wf, ph.CuTransfer(to_dev(hf, cuda)),
                                                      ph.CuTransfer(to_dev(hdz, cuda)), 2)


def test_graph_replay_matches_direct_launches(ph, cuda):
    """Repeated calls replay a cached CUDA graph; the results equal direct launches."""
    from ph_gb300 import _lib
    holo, hf, hdz = _case(256, seed=11)
    wf = ph.cu_gabor_wavefront(to_dev(holo, cuda))
    tfs = (ph.CuTransfer(to_dev(hf, cuda)), ph.CuTransfer(to_dev(hdz, cuda)))
    ctx = _lib.default_context(0)
    ctx.set_option(_lib.PH_OPT_USE_GRAPHS, 0)
    p0, a0 = (to_np(t) for t in ph.cu_get_reconst_xyprojection(wf, *tfs, 9, return_argmin=True))
    ctx.set_option(_lib.PH_OPT_USE_GRAPHS, 1)
    proj = torch.empty((256, 256), dtype=torch.float32, device=cuda)
    arg = torch.empty((256, 256), dtype=torch.int32, device=cuda)
    s = torch.cuda.current_stream().cuda_stream
    for _ in range(3):
        proj.zero_()
        ctx.call("ph_reconst_xyproj", proj.data_ptr(), arg.data_ptr(), wf.data.data_ptr(), tfs[0].data.data_ptr(),
                 tfs[1].data.data_ptr(), 256, 256, 9, s)
        assert np.array_equal(to_np(proj), p0) and np.array_equal(to_np(arg), a0)


def test_slice_batches_agree(ph, cuda):
    """The result does not depend on how slices are batched between the passes
    (at this size every slice group holds one slice: bit for bit)."""
    from ph_gb300 import _lib
    holo, hf, hdz = _case(128, seed=9)
    wf = ph.cu_gabor_wavefront(to_dev(holo, cuda))
    args = (wf, ph.CuTransfer(to_dev(hf, cuda)), ph.CuTransfer(to_dev(hdz, cuda)), 37)
    ctx = _lib.default_context(0)
    outs = []
    for b in (0, 1, 5, 37):
        ctx.set_option(_lib.PH_OPT_SLICE_BATCH, b)
        outs.append([to_np(t) for t in ph.cu_get_reconst_xyprojection(*args, return_argmin=True)])
    ctx.set_option(_lib.PH_OPT_SLICE_BATCH, 0)
    for p, a in outs[1:]:
        assert np.array_equal(p, outs[0][0]) and np.array_equal(a, outs[0][1])


def test_long_slice_groups(ph, cuda):
    """Slice groups of many slices at length 2048, where pass A advances X by
    the Hdz product chain within each group, against the oracle's chain from
    slice 0; batchings that split the groups differently agree to rounding."""
    from ph_gb300 import _lib
    n, slices = 2048, 64
    holo, hf, hdz = _case(n, seed=11, z0=-2000.0, dz=-100.0)
    p_ref, a_ref = ref.reconst_xyprojection(ref.gabor_wavefront(holo), hf, hdz, slices, with_argmin=True)
    wf = ph.cu_gabor_wavefront(to_dev(holo, cuda))
    args = (wf, ph.CuTransfer(to_dev(hf, cuda)), ph.CuTransfer(to_dev(hdz, cuda)), slices)
    ctx = _lib.default_context(0)
    outs = []
    try:
        for b in (0, 16, 40):
            ctx.set_option(_lib.PH_OPT_SLICE_BATCH, b)
            outs.append([to_np(t) for t in ph.cu_get_reconst_xyprojection(*args, return_argmin=True)])
    finally:
        ctx.set_option(_lib.PH_OPT_SLICE_BATCH, 0)
    for p, a in outs:
        assert rel_l2(p, p_ref) < REL_L2
        assert np.mean(a == a_ref) >= ARGMIN_AGREE
        assert rel_l2(p, outs[0][0]) < 1e-5


# Non-unit slice transfers: |Hdz|^k must be exact, not 1 + k(|Hdz| - 1).  Each
# length exercises one pass A form: 512 / 2048 the product chain, 256 / 1024
# the staged state, 1536 the staged X0 with the phase rate from L2, 4096 the
# cluster store.
@pytest.mark.parametrize("n,slices,mag", [(256, 512, 0.999), (512, 512, 0.999), (1024, 96, 1.001),
                                          (1536, 64, 0.99), (2048, 64, 0.99), (4096, 16, 0.95)])
def test_non_unit_slice_transfer(ph, cuda, n, slices, mag):
    holo, hf, hdz = _case(n, seed=n + 1, dz=-150.0)
    hdz = (hdz * np.float32(mag)).astype(np.complex64)
    wf = ph.cu_gabor_wavefront(to_dev(holo, cuda))
    proj, arg = ph.cu_get_reconst_xyprojection(wf, ph.CuTransfer(to_dev(hf, cuda)), ph.CuTransfer(to_dev(hdz, cuda)),
                                               slices, return_argmin=True)
    p_ref, a_ref = ref.reconst_xyprojection(ref.gabor_wavefront(holo), hf, hdz, slices, with_argmin=True)
    assert rel_l2(to_np(proj), p_ref) < REL_L2
    assert np.mean(to_np(arg) == a_ref) >= ARGMIN_AGREE


def test_non_unit_complex_slices(ph, cuda):
    """Every slice of the complex volume with |Hdz| = 0.99 over 64 slices (0.53
    at the last one) against the oracle's cumulative product."""
    n, slices = 512, 64
    holo, hf, hdz = _case(n, seed=21, dz=-150.0)
    hdz = (hdz * np.float32(0.99)).astype(np.complex64)
    wf = ph.cu_gabor_wavefront(to_dev(holo, cuda))
    cv = to_np(ph.cu_get_reconst_complex_vol(wf, ph.CuTransfer(to_dev(hf, cuda)), ph.CuTransfer(to_dev(hdz, cuda)),
                                             slices))
    cv_ref = ref.reconst_complex_vol(ref.gabor_wavefront(holo), hf, hdz, slices)
    for k in range(slices):
        assert rel_l2(cv[k], cv_ref[k]) < REL_L2, k
