"""Connected-component labeling on the GPU: bit-exact against the C oracle
(ccl.jl:13-238) and the reference's known answer (84 components)."""
import numpy as np
import pytest

from oracle import ccl as occl
from oracle import ref_semantics as ref
from phtest import to_dev, to_np

pytestmark = pytest.mark.gpu


def _labels(ph, img_np, cuda, **kw):
    return to_np(ph.cu_connected_component_labeling(to_dev(img_np, cuda), **kw)).astype(np.uint32)


def test_binaryparticles_84(ph, cuda, golden):
    g = golden("binaryparticles")
    img = np.unpackbits(g["fg_bits"])[: int(np.prod(g["shape"]))].reshape(g["shape"]).astype(np.float32)
    lab_t = ph.cu_connected_component_labeling(to_dev(img, cuda))
    assert tuple(lab_t.shape) == (1024, 1024)
    lab = to_np(lab_t).astype(np.uint32)
    assert np.array_equal(lab, occl.connected_component_labeling(img))
    assert ph.count_labels(lab_t) == 84                      # runtests.jl:217
    valid = ph.cu_find_valid_labels(lab_t)
    assert valid.dtype == np.int64 and len(valid) == 84       # runtests.jl:231
    assert np.array_equal(valid, ref.find_valid_labels(lab))
    # Bool input gives the same labels
    lab_b = to_np(ph.cu_connected_component_labeling(to_dev(img > 0, cuda))).astype(np.uint32)
    assert np.array_equal(lab_b, lab)


@pytest.mark.parametrize("shape,levels,p", [((1, 1), 2, 0.5), ((1, 37), 2, 0.5), ((37, 1), 2, 0.5),
                                            ((64, 64), 2, 0.45), ((64, 64), 4, 0.5), ((256, 256), 2, 0.6),
                                            ((1024, 1024), 2, 0.5), ((2048, 2048), 2, 0.3)])
def test_random_images_bit_exact(ph, cuda, shape, levels, p):
    rng = np.random.default_rng(shape[0] * 7 + levels)
    if levels == 2:
        img = (rng.random(shape) < p).astype(np.float32)
    else:
        img = rng.integers(0, levels, shape).astype(np.float32)
    assert np.array_equal(_labels(ph, img, cuda), occl.connected_component_labeling(img))


def test_golden_multivalued(ph, cuda, golden):
    g = golden("oracle_small")
    for k in range(3):
        # the golden labels are on each image's own 2-D grid (one of them is 12 x 20)
        assert np.array_equal(_labels(ph, g[f"ccl{k}_img"], cuda, reference_grid=False), g[f"ccl{k}_lab"])


@pytest.mark.parametrize("shape", [(24, 40), (40, 24)])
def test_rectangular_grids(ph, cuda, shape):
    rng = np.random.default_rng(5)
    img = (rng.random(shape) < 0.5).astype(np.float32)
    n_slow, n_fast = shape
    # the reference's grid: rows = size(img,1) = n_fast over the linear buffer
    want_ref = occl.connected_component_labeling(img, rows=n_fast, cols=n_slow)
    assert np.array_equal(_labels(ph, img, cuda).reshape(-1), want_ref.reshape(-1))
    # the true 2-D image
    want_2d = occl.connected_component_labeling(img)
    assert np.array_equal(_labels(ph, img, cuda, reference_grid=False), want_2d)


@pytest.mark.parametrize("case", ["near_full", "blocks_48", "partial_tiles"])
def test_uniform_tiles_bit_exact(ph, cuda, case):
    """Tiles of one foreground value take the tile-local fast path (one root,
    no hooks): near-total foreground (a projection thresholded high), blocks of
    three values 48 pixels wide (uniform tiles beside mixed ones), and a
    1000^2 image whose edge tiles are partial."""
    rng = np.random.default_rng(len(case))
    if case == "blocks_48":
        img = np.kron(rng.integers(0, 3, (11, 11)), np.ones((48, 48)))[:512, :512].astype(np.float32)
    else:
        n = 1024 if case == "near_full" else 1000
        img = np.ones((n, n), np.float32)
        img.flat[rng.integers(0, n * n, 60)] = 0.0
    lab = _labels(ph, img, cuda)
    assert np.array_equal(lab, occl.connected_component_labeling(img))


def test_uniform_tiles_across_slices(ph, cuda):
    """Batched slices 48 rows high: a tile of one value that straddles a slice
    boundary is two components, one per slice."""
    rng = np.random.default_rng(11)
    vol = np.ones((3, 48, 96), np.float32)
    vol[1, 20, 40] = 0.0
    vol[2] = (rng.random((48, 96)) < 0.9).astype(np.float32)
    lab = to_np(ph.cu_connected_component_labeling_batch(to_dev(vol, cuda))).astype(np.uint32)
    for k in range(3):
        assert np.array_equal(lab[k], occl.connected_component_labeling(vol[k]))


def test_snake_long_chains(ph, cuda):
    """A single serpentine component exercises long union chains."""
    n = 512
    img = np.zeros((n, n), np.float32)
    img[::2, :] = 1
    img[1::4, -1] = 1
    img[3::4, 0] = 1
    lab = _labels(ph, img, cuda)
    assert np.array_equal(lab, occl.connected_component_labeling(img))
    assert ref.count_labels(lab) == 1


def test_loop_limit_reports_timeout(ph, cuda):
    """With an iteration limit of 1 the bounded chase gives up and the host sees PH_ERR_TIMEOUT."""
    from ph_gb300 import _lib
    ctx = _lib.default_context(0)
    n = 256
    img = np.zeros((n, n), np.float32)
    img[::2, :] = 1
    img[1::4, -1] = 1
    img[3::4, 0] = 1
    try:
        ctx.set_option(_lib.PH_OPT_LOOP_LIMIT, 1)
        lab = ph.cu_connected_component_labeling(to_dev(img, cuda))
        with pytest.raises(_lib.PhError, match="iteration limit"):
            ph.count_labels(lab)
    finally:
        ctx.set_option(_lib.PH_OPT_LOOP_LIMIT, 1 << 20)
    lab = ph.cu_connected_component_labeling(to_dev(img, cuda))
    assert ph.count_labels(lab) == 1


def test_bounding_rectangles(ph, cuda, golden):
    g = golden("binaryparticles")
    img = np.unpackbits(g["fg_bits"])[: int(np.prod(g["shape"]))].reshape(g["shape"]).astype(np.float32)
    lab_t = ph.cu_connected_component_labeling(to_dev(img, cuda))
    boxes = ph.cu_bounding_rectangles(lab_t)
    lab = to_np(lab_t).astype(np.uint32)
    valid = ref.find_valid_labels(lab)
    assert boxes.shape == (84, 5) and np.array_equal(boxes[:, 0], valid)
    want = ref.bounding_rectangles(lab, valid)
    assert [tuple(b) for b in boxes[:, 1:].tolist()] == want


def test_batched_slices_match_per_slice(ph, cuda):
    """One labeling launch set over a binary volume equals labeling each slice alone."""
    rng = np.random.default_rng(8)
    vol = rng.random((6, 96, 80)) < 0.45
    vol[2] = False                                   # an empty slice
    lab = to_np(ph.cu_connected_component_labeling_batch(to_dev(vol, cuda))).astype(np.uint32)
    total = 0
    for k in range(vol.shape[0]):
        want = occl.connected_component_labeling(vol[k].astype(np.float32))
        assert np.array_equal(lab[k], want)
        total += ref.count_labels(want)
    boxes = ph.cu_bounding_rectangles(ph.cu_connected_component_labeling_batch(to_dev(vol, cuda)))
    assert len(boxes) == total
    n = 96 * 80
    for root, x0, y0, x1, y1 in boxes[:50]:
        k, local = divmod(int(root) - 1, n)
        sl = lab[k]
        xs, ys = np.nonzero(sl == local + 1)
        assert (x0, y0, x1, y1) == (xs.min() + 1, ys.min() + 1, xs.max() + 1, ys.max() + 1)


def test_deterministic(ph, cuda):
    rng = np.random.default_rng(0)
    img = (rng.random((512, 512)) < 0.55).astype(np.float32)
    t = to_dev(img, cuda)
    first = to_np(ph.cu_connected_component_labeling(t))
    for _ in range(20):
        assert np.array_equal(to_np(ph.cu_connected_component_labeling(t)), first)
