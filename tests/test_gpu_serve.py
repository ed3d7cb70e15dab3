"""Serving (ph_serve_*): requests of mixed sizes and optics on several lanes give
exactly the projections of single calls with the same transfer functions, the
transfer cache evicts safely, and bad requests are rejected."""
import numpy as np
import pytest
import torch

from phtest import to_dev

pytestmark = pytest.mark.gpu

LAM, DX = 0.6328, 10.0


def _single(ph, holo, slices, z0, dz):
    ny, nx = holo.shape
    d = ph.cu_transfer_sqrt_arr(nx, LAM, DX, device=holo.device.index, n_slow=ny)
    hf, hdz = ph.cu_transfer(-z0, nx, LAM, d), ph.cu_transfer(-dz, nx, LAM, d)
    return ph.cu_get_reconst_xyprojection(ph.cu_gabor_wavefront(holo), hf, hdz, slices, return_argmin=True)


def test_requests_equal_single_calls(ph, cuda):
    rng = np.random.default_rng(7)
    shapes = [(64, 64), (128, 256), (256, 256), (48, 96), (512, 512)]
    srv = ph.Server(max_shape=(512, 512), max_slices=40, lanes=3, tf_cache=4)   # small cache: forces evictions
    reqs = []
    for i in range(14):
        ny, nx = shapes[i % len(shapes)]
        holo = to_dev(rng.uniform(0.1, 1.0, (ny, nx)).astype(np.float32), cuda)
        slices, z0, dz = int(rng.integers(1, 41)), float(rng.choice([800.0, 1500.0])), float(rng.choice([100.0, 200.0]))
        proj = torch.empty_like(holo)
        arg = torch.empty(holo.shape, dtype=torch.int32, device=holo.device)
        t = srv.submit(holo, proj, slices, z0, dz, LAM, DX, argmin=arg)
        reqs.append((t, holo, proj, arg, slices, z0, dz))
    for t, holo, proj, arg, slices, z0, dz in reqs:
        lat = srv.poll(t, wait=True)
        assert lat is not None and lat >= 0.0
        p1, a1 = _single(ph, holo, slices, z0, dz)
        assert torch.equal(proj, p1)
        assert torch.equal(arg, a1)
    srv.close()


def test_poll_pending_then_done(ph, cuda):
    srv = ph.Server(max_shape=(1024, 1024), max_slices=64, lanes=1)
    holo = to_dev(np.random.default_rng(1).uniform(0.1, 1.0, (1024, 1024)).astype(np.float32), cuda)
    proj = torch.empty_like(holo)
    t = srv.submit(holo, proj, 64, 1000.0, 200.0)
    first = srv.poll(t)                 # usually still running; either answer is valid
    lat = first if first is not None else srv.poll(t, wait=True)
    assert lat > 0.0
    with pytest.raises(ph._lib.PhError):
        srv.poll(t)                     # the ticket was released
    srv.close()


def test_rejects_oversize_and_bad_requests(ph, cuda):
    srv = ph.Server(max_shape=(128, 128), max_slices=8, lanes=2)
    big = torch.ones((256, 256), dtype=torch.float32, device=cuda)
    with pytest.raises(AssertionError):
        srv.submit(big, torch.empty_like(big), 4, 1000.0, 100.0)
    small = torch.ones((64, 64), dtype=torch.float32, device=cuda)
    with pytest.raises(AssertionError):
        srv.submit(small, torch.empty_like(small), 0, 1000.0, 100.0)
    with pytest.raises(AssertionError):
        srv.submit(small, torch.empty((32, 64), dtype=torch.float32, device=cuda), 4, 1000.0, 100.0)
    srv.close()


def _block_bytes(ph, cuda, n, slices):
    """Pool bytes one n x n x slices request takes (the server's peak after it alone)."""
    srv = ph.Server(max_shape=(n, n), max_slices=slices, lanes=1)
    holo = torch.full((n, n), 0.5, dtype=torch.float32, device=cuda)
    srv.poll(srv.submit(holo, torch.empty_like(holo), slices, 1000.0, 200.0), wait=True)
    b = srv.stats()["bytes_peak"]
    srv.close()
    return b


def test_requests_wait_for_budget_then_complete(ph, cuda):
    """Admission against the HBM budget: with room for one request's scratch, the
    later ones queue at submission and run as the earlier ones finish; every
    result equals the single call."""
    n, slices = 1024, 512       # ~3 ms each: the later submissions arrive while the first runs
    block = _block_bytes(ph, cuda, n, slices)
    srv = ph.Server(max_shape=(n, n), max_slices=slices, lanes=4, budget_bytes=int(block * 1.5))
    rng = np.random.default_rng(3)
    holos = [to_dev(rng.uniform(0.1, 1.0, (n, n)).astype(np.float32), cuda) for _ in range(3)]
    outs = [(torch.empty_like(h), torch.empty(h.shape, dtype=torch.int32, device=cuda)) for h in holos]
    torch.cuda.synchronize()
    reqs = []
    for i, (holo, (proj, arg)) in enumerate(zip(holos, outs)):
        reqs.append((srv.submit(holo, proj, slices, 1000.0 + 100 * i, 200.0, argmin=arg), holo, proj, arg, i))
    st = srv.stats()
    assert st["waited"] == 2 and st["running"] + st["queued"] <= 3
    for t, holo, proj, arg, i in reqs:
        assert srv.poll(t, wait=True) > 0.0
        p1, a1 = _single(ph, holo, slices, 1000.0 + 100 * i, 200.0)
        assert torch.equal(proj, p1) and torch.equal(arg, a1)
    st = srv.stats()
    assert st["queued"] == 0 and st["running"] == 0 and st["bytes_in_use"] == 0
    assert block <= st["bytes_peak"] <= block * 1.5
    srv.close()


def test_budget_below_one_request_is_rejected(ph, cuda):
    with pytest.raises(MemoryError):
        ph.Server(max_shape=(1024, 1024), max_slices=64, lanes=2, budget_bytes=1 << 20)


@pytest.mark.parametrize("channels,flip", [(1, False), (3, True)])
def test_frame_ingest_equals_host_preprocessing(ph, cuda, channels, flip):
    """An 8-bit camera frame decoded, background-corrected and mean-padded on the
    device in the serving loop gives the projection of the same steps done
    beforehand (load_gray2float, img .- bkg .+ 64/255, pad_with_mean)."""
    rows, cols, n, slices = 200, 180, 256, 12
    rng = np.random.default_rng(11)
    img = rng.integers(40, 220, (rows, cols), dtype=np.uint8)          # row-major camera frame
    # Float64, library layout; small enough that img - bkg + offset stays positive (sqrt of it is the field)
    bkg = rng.uniform(0.1, 0.3, (cols, rows))
    off = 64 / 255
    # host-side steps, in the library layout (image row = fast index)
    holo_small = ((img.T.astype(np.float32) / np.float32(255.0)).astype(np.float64) - bkg + off).astype(np.float32)
    holo = ph.pad_with_mean(to_dev(holo_small, cuda), n)
    p_ref, a_ref = _single(ph, holo, slices, 1000.0, 200.0)
    frame = np.repeat(img[:, :, None], channels, axis=2) if channels == 3 else img
    if flip:
        frame = frame[::-1]
    srv = ph.Server(max_shape=(n, n), max_slices=slices, lanes=2)
    proj, arg = torch.empty((n, n), dtype=torch.float32, device=cuda), torch.empty((n, n), dtype=torch.int32,
                                                                                   device=cuda)
    t = srv.submit_frame(to_dev(np.ascontiguousarray(frame), cuda), proj, slices, 1000.0, 200.0, argmin=arg,
                         background=to_dev(bkg, cuda), background_offset=off, flip=flip)
    srv.poll(t, wait=True)
    srv.close()
    from phtest import rel_l2, to_np
    assert rel_l2(to_np(proj), to_np(p_ref)) < 1e-6
    assert np.mean(to_np(arg) == to_np(a_ref)) > 0.999


def test_same_shape_requests_share_launches(ph, cuda):
    """Requests of one shape, slice count and optics that queue together are
    admitted as a group on one slot and share one launch of each pass; every
    result still equals its single call bit for bit."""
    n, slices = 1024, 256
    block = _block_bytes(ph, cuda, n, slices)
    # one slot, and a budget with room for several requests (the default pool holds one)
    srv = ph.Server(max_shape=(n, n), max_slices=slices, lanes=1, budget_bytes=6 * block)
    rng = np.random.default_rng(21)
    holos = [to_dev(rng.uniform(0.1, 1.0, (n, n)).astype(np.float32), cuda) for _ in range(5)]
    outs = [(torch.empty_like(h), torch.empty(h.shape, dtype=torch.int32, device=cuda)) for h in holos]
    torch.cuda.synchronize()
    tickets = [srv.submit(h, p, slices, 1500.0, 200.0, argmin=a) for h, (p, a) in zip(holos, outs)]
    for t in tickets:
        assert srv.poll(t, wait=True) > 0.0
    st = srv.stats()
    assert st["grouped"] >= 2, st                    # the ones queued behind the first ran as a group
    for h, (p, a) in zip(holos, outs):
        p1, a1 = _single(ph, h, slices, 1500.0, 200.0)
        assert torch.equal(p, p1) and torch.equal(a, a1)
    srv.close()
