"""Preprocessing of utils.jl on the device against the oracle: the per-pixel
background mode (cu_make_background_mode, exact, ties to the first maximum),
the background mean and pad_with_mean."""
import numpy as np
import pytest
import torch

from oracle import ref_semantics as ref
from phtest import to_dev, to_np

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("count,shape,levels", [(1, (16, 24), 256), (7, (64, 48), 4), (33, (128, 130), 256),
                                                (200, (256, 256), 8)])
def test_background_mode_matches_oracle(ph, cuda, count, shape, levels):
    rng = np.random.default_rng(count)
    imgs = rng.integers(0, levels, (count,) + shape).astype(np.uint8)   # few levels: many ties
    got = ph.cu_make_background_mode(list(imgs))
    assert got.dtype == np.float64 and got.shape == shape
    assert np.array_equal(got, ref.make_background_mode(imgs))


def test_background_from_float_images(ph, cuda):
    rng = np.random.default_rng(2)
    f = rng.random((9, 32, 32)).astype(np.float32)
    u8 = np.round(np.clip(f * 255, 0, 255)).astype(np.uint8)
    assert np.array_equal(ph.cu_make_background_mode(list(f)), ref.make_background_mode(u8))


def test_background_mean_matches_oracle(ph, cuda):
    imgs = np.random.default_rng(3).integers(0, 256, (25, 40, 56)).astype(np.uint8)
    got = ph.make_background(list(imgs), mode="mean")
    assert np.max(np.abs(got - ref.make_background_mean(imgs))) < 1e-12


@pytest.mark.parametrize("shape,pad", [((30, 20), 64), ((64, 64), 65), ((7, 100), 128)])
def test_pad_with_mean_matches_oracle(ph, cuda, shape, pad):
    img = np.random.default_rng(4).random(shape).astype(np.float32)
    got = to_np(ph.pad_with_mean(to_dev(img, cuda), pad))
    want = ref.pad_with_mean(img, pad)
    inner = want != want[0, 0]
    assert np.array_equal(got[inner], want[inner])                      # the image placement is exact
    assert abs(float(got[0, 0]) - float(want[0, 0])) <= 1e-6            # the mean (FP64 accumulation)


def test_pad_with_mean_asserts(ph, cuda):
    with pytest.raises(AssertionError):
        ph.pad_with_mean(torch.ones((10, 10), dtype=torch.float32, device=cuda), 10)
