"""The device side of particle_bounding_boxes (particle_detection.jl:58-96): the
binary volume from the reconstruction's own epilogue equals the thresholded
Float32 volume, and the per-slice boxes equal the oracle's labels and
get_bounding_rectangles slice by slice."""
import numpy as np
import pytest
import torch

from oracle import ccl as occl
from oracle import ref_semantics as ref
from phtest import to_dev, to_np

pytestmark = pytest.mark.gpu

LAM, DX = 0.6328, 10.0


def _case(cuda, n, seed):
    rng = np.random.default_rng(seed)
    holo = np.ones((n, n), np.float32)
    yy, xx = np.mgrid[:n, :n]
    for _ in range(12):   # dark discs give compact components in every slice
        cy, cx, r = rng.integers(8, n - 8), rng.integers(8, n - 8), rng.integers(2, 6)
        holo[(yy - cy) ** 2 + (xx - cx) ** 2 <= r * r] = 0.05
    holo += rng.normal(0, 0.01, holo.shape).astype(np.float32)
    holo = np.clip(holo, 0, None)
    d = ref.transfer_sqrt_arr(n, LAM, DX)
    wf = ref.gabor_wavefront(holo)
    return (ph_wave(cuda, wf), to_dev(ref.transfer(-400.0, n, LAM, d), cuda), to_dev(ref.transfer(-100.0, n, LAM, d), cuda),
            wf, ref.transfer(-400.0, n, LAM, d), ref.transfer(-100.0, n, LAM, d))


def ph_wave(cuda, wf):
    return to_dev(wf, cuda)


@pytest.mark.parametrize("n,slices,thr", [(128, 6, 0.3), (256, 9, 0.5)])
def test_binary_volume_is_thresholded_float_volume(ph, cuda, n, slices, thr):
    wf, hf, hdz, wf_np, hf_np, hdz_np = _case(cuda, n, seed=n)
    W, F, D = ph.CuWavefront(wf), ph.CuTransfer(hf), ph.CuTransfer(hdz)
    binv, proj = ph.cu_get_reconst_binary_vol(W, F, D, slices, thr, return_proj=True)
    volf, projf = ph.cu_get_reconst_vol_and_xyprojection(W, F, D, slices, torch.float32)
    assert binv.dtype == torch.bool and tuple(binv.shape) == (slices, n, n)
    assert torch.equal(binv, volf <= thr)
    assert torch.equal(proj, projf)
    want = ref.reconst_vol(wf_np, hf_np, hdz_np, slices, return_type=np.float32) <= thr
    assert np.mean(to_np(binv) == want) >= 0.999


def test_slice_boxes_match_oracle(ph, cuda):
    wf, hf, hdz, *_ = _case(cuda, 256, seed=3)
    binv = ph.cu_get_reconst_binary_vol(ph.CuWavefront(wf), ph.CuTransfer(hf), ph.CuTransfer(hdz), 7, 0.25)
    per = ph.slice_bounding_boxes(binv)
    vol = to_np(binv)
    assert len(per) == 7
    for k in range(7):
        lab = occl.connected_component_labeling(vol[k].astype(np.float32))
        valid = ref.find_valid_labels(lab)
        assert np.array_equal(per[k][:, 0], valid)
        assert [tuple(b) for b in per[k][:, 1:].tolist()] == ref.bounding_rectangles(lab, valid)
    assert sum(len(b) for b in per) > 0


def test_subvolumes_equal_volume_crops(ph, cuda):
    """ph_reconst_subvolumes: every box equals the same crop of the N0f8 volume,
    without the volume being formed (edge, overlapping and one-voxel boxes)."""
    n, S = 128, 10
    wf, hf, hdz, *_ = _case(cuda, n, seed=11)
    W, F, D = ph.CuWavefront(wf), ph.CuTransfer(hf), ph.CuTransfer(hdz)
    vol = to_np(ph.cu_get_reconst_vol(W, F, D, S, ph.N0f8))         # (z, slow, fast) raw levels
    boxes = np.array([[1, 1, 1, 10, 12, 3],            # corner
                      [5, 7, 2, 40, 30, 9],            # overlaps the next
                      [20, 20, 4, 60, 70, 10],
                      [128, 128, 10, 128, 128, 10],    # one voxel at the far corner
                      [64, 1, 5, 64, 128, 5],          # one full fast line
                      [1, 100, 1, 128, 101, 10]])      # full slow range
    subs = ph.cu_reconst_subvolumes(W, F, D, S, boxes)
    assert len(subs) == len(boxes)
    for (x0, y0, z0, x1, y1, z1), sv in zip(boxes.tolist(), subs):
        want = vol[z0 - 1:z1, x0 - 1:x1, y0 - 1:y1]
        assert tuple(sv.shape) == want.shape
        assert np.array_equal(to_np(sv), want.astype(np.uint8) if want.dtype != np.uint8 else want)
    with pytest.raises(AssertionError):
        ph.cu_reconst_subvolumes(W, F, D, S, [[0, 1, 1, 2, 2, 2]])   # outside the volume (1-based)
    coords = ph.particle_coordinates(boxes[:3], subs[:3])
    assert coords.shape == (3, 3)
    for (x0, y0, z0, x1, y1, z1), (x, y, z) in zip(boxes[:3].tolist(), coords.tolist()):
        assert x0 <= x <= x1 and y0 <= y <= y1 and z0 <= z <= z1
