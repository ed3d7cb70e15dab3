"""The oracle itself, pinned against the reference's own known answers and the
committed golden vectors (no GPU)."""
import numpy as np
import pytest
import scipy.ndimage as ndi

from oracle import ccl as occl
from oracle import fp64 as o64
from oracle import ref_semantics as ref

LAM, DX = 0.6328, 10.0


def _canonical_labels(img):
    """Independent CCL: scipy 8-connectivity per value, label = 1 + min linear index."""
    out = np.zeros(img.shape, np.uint32)
    idx = np.arange(img.size).reshape(img.shape)
    for v in np.unique(img):
        if v <= 0:
            continue
        lab, n = ndi.label(img == v, structure=np.ones((3, 3)))
        if n == 0:
            continue
        mins = np.asarray(ndi.minimum(idx, lab, index=np.arange(1, n + 1)), np.int64)
        m = lab > 0
        out[m] = mins[lab[m] - 1] + 1
    return out


def test_ccl_oracle_known_answer_84(golden):
    g = golden("binaryparticles")
    img = np.unpackbits(g["fg_bits"])[: int(np.prod(g["shape"]))].reshape(g["shape"]).astype(np.float32)
    lab = occl.connected_component_labeling(img)
    assert lab.dtype == np.uint32 and lab.shape == (1024, 1024)
    assert ref.count_labels(lab) == 84                      # runtests.jl:217
    assert len(ref.find_valid_labels(lab)) == 84            # runtests.jl:231
    assert np.array_equal(lab, _canonical_labels(img))


@pytest.mark.parametrize("seed", range(12))
def test_ccl_oracle_vs_scipy(seed):
    rng = np.random.default_rng(seed)
    shape = tuple(rng.integers(1, 48, 2))
    img = (rng.random(shape) < rng.uniform(0.2, 0.8)).astype(np.float32)
    if seed % 3 == 0:
        img = rng.integers(-1, 3, shape).astype(np.float32)
    assert np.array_equal(occl.connected_component_labeling(img), _canonical_labels(img))


def test_ccl_golden(golden):
    g = golden("oracle_small")
    for k in range(3):
        assert np.array_equal(occl.connected_component_labeling(g[f"ccl{k}_img"]), g[f"ccl{k}_lab"])


def test_transfer_sqrt_formula():
    d = ref.transfer_sqrt_arr(8, LAM, DX)
    # holofunc.jl:12 at x = y = datLen/2 + 1 (1-based) is exactly 1
    assert d[4, 4] == np.float32(1.0)
    assert d.dtype == np.float32 and d.shape == (8, 8)
    assert np.array_equal(d, d.T)
    x = 1
    t = (x - 8 / 2 - 1.0) * LAM / 8 / DX
    assert d[4, 0] == np.float32(1.0 - t * t)


def test_golden_vectors_reproduce(golden):
    g = golden("oracle_small")
    d = ref.transfer_sqrt_arr(64, LAM, DX)
    assert np.array_equal(d, g["sqr_64"])
    assert np.array_equal(ref.transfer(-100.0, 64, LAM, d), g["tf_64_-100"])
    assert np.array_equal(ref.gabor_wavefront(g["gabor_in"]), g["gabor_out"])
    p, a = ref.reconst_xyprojection(ref.gabor_wavefront(g["rec_holo"]), g["rec_hf"], g["rec_hdz"], 12, True)
    assert np.allclose(p, g["rec_proj"], rtol=1e-5, atol=1e-7)
    assert np.mean(a == g["rec_argmin"]) > 0.999


def test_reference_shapes():
    """Output sizes and types the reference's tests pin (runtests.jl:362-383)."""
    arr = np.array([[1 + 1j, 2 + 1j], [3 + 1j, 4 + 1j]], np.complex64)
    pad = ref.pad2d(arr)
    assert pad.shape == (4, 4) and np.array_equal(pad[1:3, 1:3], arr)
    rng = np.random.default_rng(0)
    d = ref.transfer_sqrt_arr(8, LAM, DX)
    vol, proj = ref.reconst_vol_and_xyprojection_padded(ref.gabor_wavefront(rng.random((4, 4), np.float32)),
                                                        ref.transfer(-100.0, 8, LAM, d), ref.transfer(-10.0, 8, LAM, d), 2)
    assert vol.shape == (2, 4, 4) and vol.dtype == np.uint8 and proj.shape == (4, 4) and proj.dtype == np.float32
    out = ref.asm_prop(np.ones((4, 4), np.complex64), ref.transfer_sqrt_arr(4, LAM, DX), 100.0, 4, LAM)
    assert out.shape == (4, 4) and np.sum(np.abs(out)) > 0


def test_n0f8_rounding_half_even():
    v = np.array([0.5 / 255, 1.5 / 255, 2.5 / 255, -1.0, 2.0, 1.0], np.float32)
    q = ref.normedfloat_to_n0f8(v)
    assert list(q) == list(np.rint(np.clip(v, 0, 1) * np.float32(255)).astype(np.uint8))
    assert q[3] == 0 and q[4] == 255 and q[5] == 255


def test_size_asserts():
    with pytest.raises(AssertionError, match="All arrays must have the same size"):
        ref.reconst_xyprojection(np.zeros((4, 4), np.complex64), np.zeros((8, 8), np.complex64),
                                 np.zeros((4, 4), np.complex64), 2)
    with pytest.raises(ValueError, match="return_type"):
        ref.ifft_and_abs(np.zeros((4, 4), np.complex64), np.int32)


def test_reference_tf_vs_exact_phase_gap():
    """The reference's Float32 sqrt term puts its transfer phase ~0.02-0.09 rad
    off the exact physics at 52-200 mm (a property of the reference itself)."""
    n = 1024
    d = ref.transfer_sqrt_arr(n, LAM, DX)
    for z, lo, hi in ((52000.0, 0.005, 0.05), (200000.0, 0.02, 0.2)):
        gap = np.max(np.abs(np.angle(ref.transfer(z, n, LAM, d) * np.conj(o64.transfer_exact(z, n, LAM, DX)))))
        assert lo < gap < hi


def test_fp32_oracle_vs_fp64_physics():
    """The FP32 reference-semantics projection agrees with the FP64 physics at small size."""
    n, s, z0, dz = 64, 8, 1000.0, 200.0
    rng = np.random.default_rng(3)
    holo = rng.uniform(0.2, 1.0, (n, n)).astype(np.float32)
    d = ref.transfer_sqrt_arr(n, LAM, DX)
    p32 = ref.reconst_xyprojection(ref.gabor_wavefront(holo), ref.transfer(-z0, n, LAM, d),
                                   ref.transfer(-dz, n, LAM, d), s)
    p64 = o64.reconst_xyprojection_fp64(np.sqrt(holo.astype(np.float64)), z0, dz, s, LAM, DX)
    assert np.linalg.norm(p32 - p64) / np.linalg.norm(p64) < 1e-3


def test_generator_golden(golden):
    g = golden("oracle_small")
    discs = o64.draw_discs(11, 64, 5, 40.0, 80.0, 2000.0, 20000.0, DX)
    inten = np.abs(o64.synth_field(discs, 64, 64, LAM, DX)) ** 2
    assert np.allclose(inten, g["synth64_intensity"], rtol=1e-12, atol=1e-12)


def test_gs_residual_decreases():
    n = 32
    rng = np.random.default_rng(0)
    discs = o64.draw_discs(5, n, 3, 30.0, 60.0, 2000.0, 4000.0, DX)
    f1 = o64.synth_field(discs, n, n, LAM, DX)
    f2 = o64.propagate_natural(f1, 2000.0, LAM, DX)
    h1, h2 = (np.abs(f1) ** 2).astype(np.float32), (np.abs(f2) ** 2).astype(np.float32)
    d = ref.transfer_sqrt_arr(n, LAM, DX)
    tp, tpi = ref.transfer(2000.0, n, LAM, d), ref.transfer(-2000.0, n, LAM, d)
    _, r1 = ref.phase_retrieval_holo(h1, h2, tp, tpi, 1, n, return_residual=True)
    _, r10 = ref.phase_retrieval_holo(h1, h2, tp, tpi, 10, n, return_residual=True)
    assert r10 < r1


def test_background_mode_first_maximum():
    """cu_make_background_mode (utils.jl:279-317): the argmax loop keeps the first
    (smallest) value among equally frequent ones."""
    imgs = np.array([[[3, 1]], [[1, 1]], [[3, 2]], [[1, 2]]], dtype=np.uint8)   # pixel 0: 1 and 3 twice each
    got = ref.make_background_mode(imgs)
    assert got[0, 0] == 1 / 255.0 and got[0, 1] == 1 / 255.0
    rng = np.random.default_rng(0)
    st = rng.integers(0, 5, (11, 6, 7)).astype(np.uint8)
    m = ref.make_background_mode(st)
    for y in range(6):
        for x in range(7):
            assert m[y, x] == np.argmax(np.bincount(st[:, y, x], minlength=256)) / 255.0


def test_pad_with_mean_placement():
    """pad_with_mean (utils.jl:319-325) places a Julia (h, w) image at rows
    div(p,2)-div(h,2)+1.. and columns div(p,2)-div(w,2)+1..; here (w, h) order."""
    img = np.arange(15, dtype=np.float32).reshape(3, 5)        # Julia (h=5, w=3)
    out = ref.pad_with_mean(img, 9)
    assert out.shape == (9, 9)
    o_fast, o_slow = 9 // 2 - 5 // 2, 9 // 2 - 3 // 2
    assert np.array_equal(out[o_slow:o_slow + 3, o_fast:o_fast + 5], img)
    assert np.all(out[0] == np.float32(7.0))
