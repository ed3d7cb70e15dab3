"""The seeded synthetic-hologram generator and the propagation primitive it
uses, against the FP64 oracle."""
import numpy as np
import pytest
import torch

from oracle import fp64 as o64
from phtest import rel_l2, to_dev, to_np

pytestmark = pytest.mark.gpu
LAM, DX = 0.6328, 10.0


@pytest.mark.parametrize("n,z", [(64, 2500.0), (256, 40000.0), (2048, 95000.0)])
def test_propagate_fp64_transfer(ph, cuda, n, z):
    from ph_gb300 import _lib
    rng = np.random.default_rng(n)
    u = (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))).astype(np.complex64)
    tf = ph.cu_transfer_fp64(z, n, LAM, DX)
    t = to_dev(u, cuda)
    out = torch.empty_like(t)
    _lib.default_context(0).call("ph_propagate", out.data_ptr(), t.data_ptr(), tf.data.data_ptr(), n, n,
                                 torch.cuda.current_stream().cuda_stream)
    want = o64.propagate_natural(u.astype(np.complex128), z, LAM, DX)
    assert rel_l2(to_np(out), want) < 1e-5


def test_generator_matches_fp64_oracle(ph, cuda):
    from ph_gb300 import synth
    spec = synth.HologramSpec(seed=11, n=64, count=5, dmin=40.0, dmax=80.0, zmin=2000.0, zmax=20000.0, sigma=0.0)
    got = to_np(synth.synth_hologram(spec, 0, noise=False))
    discs = o64.draw_discs(11, 64, 5, 40.0, 80.0, 2000.0, 20000.0, DX)
    inten = np.abs(o64.synth_field(discs, 64, 64, LAM, DX)) ** 2
    want = (inten - inten.min()) / (inten.max() - inten.min())
    assert np.isfinite(got).all()
    assert np.max(np.abs(got - want)) < 1e-4


def test_generator_disc_draws_match_oracle(ph):
    from ph_gb300 import synth
    spec = synth.HologramSpec(seed=7, n=2048, count=800, dmin=10.0, dmax=60.0, zmin=5000.0, zmax=100000.0)
    d = synth.draw_discs(spec)
    o = o64.draw_discs(7, 2048, 800, 10.0, 60.0, 5000.0, 100000.0, DX)
    assert np.array_equal(d, np.stack([o.x, o.y, o.d, o.z], axis=1))


def test_generator_full_size_is_finite(ph, cuda):
    from ph_gb300 import synth
    spec = synth.HologramSpec(seed=2, n=2048, count=800, dmin=10.0, dmax=60.0, zmin=5000.0, zmax=100000.0)
    h = synth.synth_hologram(spec, 0)
    assert torch.isfinite(h).all()
    assert -0.1 < float(h.min()) < 0.1 and 0.9 < float(h.max()) < 1.1
