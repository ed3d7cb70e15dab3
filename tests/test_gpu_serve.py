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
