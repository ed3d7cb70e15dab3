"""Batches of projections (ph_batch_plan / ph_batch_run): every item equals its
own single cu_get_reconst_xyprojection call bit for bit, the plan replays with
new input contents, and bad items are rejected before anything runs."""
import numpy as np
import pytest
import torch

from oracle import ref_semantics as ref
from phtest import REL_L2, rel_l2, to_dev, to_np

pytestmark = pytest.mark.gpu

LAM, DX = 0.6328, 10.0


def _item(cuda, nx, ny, slices, seed, as_hologram, z0=-1500.0, dz=-150.0):
    rng = np.random.default_rng(seed)
    holo = rng.uniform(0.1, 1.0, (ny, nx)).astype(np.float32)
    d = ref.transfer_sqrt_arr(nx, LAM, DX, n_slow=ny)
    hf, hdz = ref.transfer(z0, nx, LAM, d), ref.transfer(dz - seed, nx, LAM, d)
    it = {"transfer_front": to_dev(hf, cuda), "transfer_dz": to_dev(hdz, cuda), "slices": slices}
    if as_hologram:
        it["hologram"] = to_dev(holo, cuda)
    else:
        it["wavefront"] = to_dev(ref.gabor_wavefront(holo), cuda)
    return it, holo, hf, hdz


def _single(ph, it):
    wf = it["wavefront"] if "wavefront" in it else ph.cu_gabor_wavefront(it["hologram"]).data
    return ph.cu_get_reconst_xyprojection(ph.CuWavefront(wf), ph.CuTransfer(it["transfer_front"]),
                                          ph.CuTransfer(it["transfer_dz"]), it["slices"], return_argmin=True)


SHAPES = [(64, 64, 5), (128, 256, 9), (96, 48, 3), (512, 512, 17), (3, 6, 2), (256, 128, 33), (1024, 1024, 4),
          (32, 32, 1)]


@pytest.mark.parametrize("lanes", [1, 3, 8])
def test_batch_equals_single_calls(ph, cuda, lanes):
    items = [_item(cuda, nx, ny, s, seed=i, as_hologram=(i % 2 == 0))[0] for i, (nx, ny, s) in enumerate(SHAPES)]
    batch = ph.ReconBatch(items, lanes=lanes)
    proj, arg = batch.run()
    torch.cuda.synchronize()
    assert batch.scratch_bytes > 0
    for it, p, a in zip(items, proj, arg):
        p1, a1 = _single(ph, it)
        assert torch.equal(p, p1)
        assert torch.equal(a, a1)
    batch.close()


def test_grouped_items_equal_single_calls(ph, cuda):
    """Items of one shape whose own launches are small share one launch of each
    pass (grid z = item, up to 8 per group): own inputs, transfer functions and
    slice counts, including the 2048 product-chain form and more items than
    one group holds.  Each equals
    its single call bit for bit (both with 64-slice batches of intermediates,
    so the product chains restart at the same slices)."""
    from ph_gb300 import _lib
    spec = [(256, 256, sl, True) for sl in (1, 5, 33, 64, 100, 7, 2, 200, 50, 3)]
    spec += [(2048, 2048, sl, True) for sl in (96, 40)]           # large launches: each alone
    spec += [(512, 512, sl, True) for sl in (96, 40, 200, 3)]     # grouped, with pass A's product chain
    spec += [(1024, 512, sl, False) for sl in (12, 70, 1)]
    items = [_item(cuda, nx, ny, sl, seed=20 + i, as_hologram=h)[0] for i, (nx, ny, sl, h) in enumerate(spec)]
    ctx = _lib.default_context(0)
    ctx.set_option(_lib.PH_OPT_SLICE_BATCH, 64)
    try:
        batch = ph.ReconBatch(items, lanes=3)
        proj, arg = batch.run()
        torch.cuda.synchronize()
        for it, p, a in zip(items, proj, arg):
            p1, a1 = _single(ph, it)
            assert torch.equal(p, p1), it["slices"]
            assert torch.equal(a, a1), it["slices"]
        batch.close()
    finally:
        ctx.set_option(_lib.PH_OPT_SLICE_BATCH, 0)


def test_batch_against_oracle_and_replay(ph, cuda):
    it0, holo0, hf0, hdz0 = _item(cuda, 256, 256, 12, seed=5, as_hologram=True)
    it1, holo1, hf1, hdz1 = _item(cuda, 128, 64, 7, seed=6, as_hologram=False)
    batch = ph.ReconBatch([it0, it1], lanes=2)
    proj, _ = batch.run()
    want0 = ref.reconst_xyprojection(ref.gabor_wavefront(holo0), hf0, hdz0, 12)
    want1 = ref.reconst_xyprojection(ref.gabor_wavefront(holo1), hf1, hdz1, 7)
    assert rel_l2(to_np(proj[0]), want0) < REL_L2
    assert rel_l2(to_np(proj[1]), want1) < REL_L2
    # replay with new hologram contents in the same buffer
    new = np.random.default_rng(99).uniform(0.1, 1.0, holo0.shape).astype(np.float32)
    it0["hologram"].copy_(torch.from_numpy(new))
    proj, _ = batch.run()
    want0 = ref.reconst_xyprojection(ref.gabor_wavefront(new), hf0, hdz0, 12)
    assert rel_l2(to_np(proj[0]), want0) < REL_L2
    batch.close()


def test_batch_rejects_bad_items(ph, cuda):
    good = _item(cuda, 64, 64, 3, seed=1, as_hologram=True)[0]
    bad = dict(good, slices=0)
    with pytest.raises(AssertionError):
        ph.ReconBatch([good, bad])
    odd = _item(cuda, 10, 10, 3, seed=2, as_hologram=True)[0]
    with pytest.raises(ph._lib.PhError):   # length 10 is not 2^a or 3 * 2^a
        ph.ReconBatch([good, odd])
    mismatched = dict(good, transfer_dz=torch.zeros((32, 64), dtype=torch.complex64, device=good["hologram"].device))
    with pytest.raises(AssertionError):
        ph.ReconBatch([mismatched])


def test_autotune_choice_cached_and_used(ph, cuda, tmp_path):
    """The autotuner times the knobs of a shape once, writes its choice to the
    JSON cache keyed by device and shape, reads it back without timing again,
    and reconstructions under the chosen knobs still match the oracle."""
    import json
    from oracle import ref_semantics as ref
    from phtest import ARGMIN_AGREE, REL_L2, rel_l2, to_dev, to_np
    from ph_gb300 import _lib
    cache = tmp_path / "tune.json"
    n, slices = 256, 96
    first = ph.autotune(n, n, slices, allow_forms=False, cache=str(cache))
    assert first["ms"] > 0 and first["form"] == 0 and first["group_cap"] in (0, 16, 32, 64)
    data = json.loads(cache.read_text())
    (dev, shapes), = data.items()
    assert "GB300" in dev and shapes[f"{n}x{n}"]["slices"] == slices
    again = ph.autotune(n, n, slices, cache=str(cache))
    # read back, not timed again (the file keeps the time to 9 significant digits)
    assert {k: again[k] for k in ("form", "group_cap", "batch_slices")} == \
        {k: first[k] for k in ("form", "group_cap", "batch_slices")}
    assert abs(again["ms"] - first["ms"]) <= 1e-6 * first["ms"]
    rng = np.random.default_rng(5)
    holo = rng.uniform(0.1, 1.0, (n, n)).astype(np.float32)
    d = ref.transfer_sqrt_arr(n, 0.6328, 10.0)
    hf, hdz = ref.transfer(-1000.0, n, 0.6328, d), ref.transfer(-200.0, n, 0.6328, d)
    ctx = _lib.default_context(0)
    ctx.set_option(_lib.PH_OPT_FORM, _lib.PH_FORM_TUNED)
    try:
        p, a = ph.cu_get_reconst_xyprojection(ph.cu_gabor_wavefront(to_dev(holo, cuda)),
                                              ph.CuTransfer(to_dev(hf, cuda)), ph.CuTransfer(to_dev(hdz, cuda)),
                                              slices, return_argmin=True)
    finally:
        ctx.set_option(_lib.PH_OPT_FORM, 0)
    p_ref, a_ref = ref.reconst_xyprojection(ref.gabor_wavefront(holo), hf, hdz, slices, with_argmin=True)
    assert rel_l2(to_np(p), p_ref) < REL_L2 and np.mean(to_np(a) == a_ref) >= ARGMIN_AGREE


def test_autotune_with_forms_at_2048(ph, cuda, tmp_path):
    """With the split-precision forms allowed, the tuner times them too and
    records whichever is fastest (the choice is a measurement, not a rule)."""
    r = ph.autotune(2048, 2048, 64, allow_forms=True, cache=str(tmp_path / "t.json"))
    assert r["form"] in (0, 1, 2) and r["ms"] > 0
