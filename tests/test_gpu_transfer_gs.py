"""Transfer functions, Gabor wavefront, padding, propagation and
Gerchberg-Saxton on the GPU against the oracle (holofunc.jl:8-149, 383-388)."""
import numpy as np
import pytest
import torch

from oracle import fp64 as o64
from oracle import ref_semantics as ref
from phtest import REL_L2, rel_l2, to_dev, to_np

pytestmark = pytest.mark.gpu
LAM, DX = 0.6328, 10.0


@pytest.mark.parametrize("n", [1, 4, 8, 64, 1024])
def test_transfer_sqrt_bit_exact(ph, cuda, n):
    got = to_np(ph.cu_transfer_sqrt_arr(n, LAM, DX).data)
    assert got.shape == (n, n) and got.dtype == np.float32
    assert np.array_equal(got, ref.transfer_sqrt_arr(n, LAM, DX))


@pytest.mark.parametrize("n,z", [(64, 80000.0), (64, -80000.0), (64, -100.0), (1024, 80000.0), (1024, -1000.0)])
def test_transfer(ph, cuda, n, z):
    d = ph.cu_transfer_sqrt_arr(n, LAM, DX)
    got = to_np(ph.cu_transfer(z, n, LAM, d).data)
    want = ref.transfer(z, n, LAM, ref.transfer_sqrt_arr(n, LAM, DX))
    assert got.dtype == np.complex64
    # FP64 sin/cos on both sides, rounded to Float32: at most one ulp apart
    assert np.max(np.abs(got - want)) <= 1.2e-7


def test_transfer_golden(ph, cuda, golden):
    g = golden("oracle_small")
    d = ph.cu_transfer_sqrt_arr(64, LAM, DX)
    assert np.array_equal(to_np(d.data), g["sqr_64"])
    for z in (80000, -80000, -100):
        assert np.max(np.abs(to_np(ph.cu_transfer(float(z), 64, LAM, d).data) - g[f"tf_64_{z}"])) <= 1.2e-7


def test_transfer_fp64(ph, cuda):
    n = 256
    got = to_np(ph.cu_transfer_fp64(-52000.0, n, LAM, DX).data)
    want = o64.transfer_exact(-52000.0, n, LAM, DX)
    assert np.max(np.abs(got - want)) < 2e-7
    # the reference-compatible transfer differs from the exact phase (Float32 sqrt term)
    d = ph.cu_transfer_sqrt_arr(n, LAM, DX)
    ref_tf = to_np(ph.cu_transfer(-52000.0, n, LAM, d).data)
    assert np.max(np.abs(np.angle(ref_tf * np.conj(want)))) > 1e-3


def test_gabor_wavefront(ph, cuda, golden):
    g = golden("oracle_small")
    got = to_np(ph.cu_gabor_wavefront(to_dev(g["gabor_in"], cuda)).data)
    assert np.array_equal(got, g["gabor_out"])


def test_2d_pad(ph, cuda, golden):
    g = golden("oracle_small")
    out = to_np(ph.cu_2d_pad(to_dev(g["pad2d_in"], cuda)))
    assert out.shape == (4, 4)
    assert np.array_equal(out[1:3, 1:3], g["pad2d_in"])       # runtests.jl:367
    assert np.allclose(out, g["pad2d_out"], atol=1e-6)


def test_asm_prop(ph, cuda, golden):
    g = golden("oracle_small")
    # runtests.jl:385-394: ones 4x4, z = 100
    inh = ph.CuWavefront(torch.ones((4, 4), dtype=torch.complex64, device=cuda))
    outh = ph.CuWavefront(torch.zeros((4, 4), dtype=torch.complex64, device=cuda))
    ph.cu_asm_prop_(outh, inh, ph.cu_transfer_sqrt_arr(4, LAM, DX), 100.0, 4, LAM)
    o = to_np(outh.data)
    assert o.shape == (4, 4) and np.sum(np.abs(o)) > 0
    assert rel_l2(o, g["asm_ones_out"]) < REL_L2
    inh = ph.CuWavefront(to_dev(g["asm_in"], cuda))
    outh = ph.CuWavefront(torch.empty((16, 16), dtype=torch.complex64, device=cuda))
    ph.cu_asm_prop_(outh, inh, ph.CuTransferSqrtPart(to_dev(g["asm_sqr"], cuda)), 2500.0, 16, LAM)
    assert rel_l2(to_np(outh.data), g["asm_out"]) < REL_L2


@pytest.mark.parametrize("n", [256, 1024])
def test_asm_prop_in_place(ph, cuda, n):
    rng = np.random.default_rng(n)
    u = (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))).astype(np.complex64)
    d = ref.transfer_sqrt_arr(n, LAM, DX)
    want = ref.asm_prop(u, d, -3000.0, n, LAM)
    t = to_dev(u, cuda)
    w = ph.CuWavefront(t)
    ph.cu_asm_prop_(w, w, ph.CuTransferSqrtPart(to_dev(d, cuda)), -3000.0, n, LAM)
    assert rel_l2(to_np(t), want) < REL_L2


def test_gs_golden(ph, cuda, golden):
    g = golden("oracle_small")
    u, res = ph.cu_phase_retrieval_holo(to_dev(g["gs_h1"], cuda), to_dev(g["gs_h2"], cuda),
                                        ph.CuTransfer(to_dev(g["gs_tp"], cuda)),
                                        ph.CuTransfer(to_dev(g["gs_tpi"], cuda)), 5, 64, return_residual=True)
    assert rel_l2(to_np(u.data), g["gs_out"]) < REL_L2
    assert abs(float(res) - float(g["gs_resid"])) < 1e-4 * max(1.0, float(g["gs_resid"]))


@pytest.mark.parametrize("n,iters", [(1, 2), (8, 3), (128, 4), (512, 3), (96, 3), (768, 2), (1024, 3)])
def test_gs_matches_oracle(ph, cuda, n, iters):
    rng = np.random.default_rng(n)
    h1 = rng.uniform(0.1, 1.0, (n, n)).astype(np.float32)
    h2 = rng.uniform(0.1, 1.0, (n, n)).astype(np.float32)
    d = ref.transfer_sqrt_arr(n, LAM, DX)
    tp, tpi = ref.transfer(5000.0, n, LAM, d), ref.transfer(-5000.0, n, LAM, d)
    u = ph.cu_phase_retrieval_holo(to_dev(h1, cuda), to_dev(h2, cuda), ph.CuTransfer(to_dev(tp, cuda)),
                                   ph.CuTransfer(to_dev(tpi, cuda)), iters, n)
    assert rel_l2(to_np(u.data), ref.phase_retrieval_holo(h1, h2, tp, tpi, iters, n)) < REL_L2


def test_gs_real_holograms(ph, cuda, golden):
    """The reference test's real holograms (runtests.jl:318-333), 256^2 crops, z = 80 mm."""
    g = golden("holo_crops")
    h1 = (g["holo1"].astype(np.float32) / np.float32(255.0)).astype(np.float32)
    h2 = (g["holo2"].astype(np.float32) / np.float32(255.0)).astype(np.float32)
    n = 256
    d = ref.transfer_sqrt_arr(n, LAM, DX)
    tp, tpi = ref.transfer(80000.0, n, LAM, d), ref.transfer(-80000.0, n, LAM, d)
    u = ph.cu_phase_retrieval_holo(to_dev(h1, cuda), to_dev(h2, cuda), ph.CuTransfer(to_dev(tp, cuda)),
                                   ph.CuTransfer(to_dev(tpi, cuda)), 20, n)
    assert tuple(u.data.shape) == (n, n) and u.data.dtype == torch.complex64
    assert rel_l2(to_np(u.data), ref.phase_retrieval_holo(h1, h2, tp, tpi, 20, n)) < REL_L2


@pytest.mark.parametrize("n", [64, 1024])
def test_gs_zero_field(ph, cuda, n):
    """A zero transfer makes every propagated field exactly zero; angle(0) == 0
    (holofunc.jl:115-125), so each amplitude replacement gives sqrt(I) + 0i."""
    h1 = torch.rand((n, n), device=cuda) + 0.1
    h2 = torch.rand((n, n), device=cuda) + 0.1
    z = ph.CuTransfer(torch.zeros((n, n), dtype=torch.complex64, device=cuda))
    u = ph.cu_phase_retrieval_holo(h1, h2, z, z, 3, n)
    assert torch.equal(u.data, torch.complex(torch.sqrt(h1), torch.zeros_like(h1)))


@pytest.mark.parametrize("n", [64, 1024])
def test_gs_tiny_field(ph, cuda, n):
    """Transfers scaled by 1e-20 make |u|^2 ~ 1e-40 (subnormal), so every
    amplitude replacement takes its scaled path; the phases, and so the
    result, still match the oracle."""
    rng = np.random.default_rng(5)
    h1 = rng.uniform(0.1, 1.0, (n, n)).astype(np.float32)
    h2 = rng.uniform(0.1, 1.0, (n, n)).astype(np.float32)
    d = ref.transfer_sqrt_arr(n, LAM, DX)
    tp = (ref.transfer(5000.0, n, LAM, d) * np.float32(1e-20)).astype(np.complex64)
    tpi = (ref.transfer(-5000.0, n, LAM, d) * np.float32(1e-20)).astype(np.complex64)
    u = ph.cu_phase_retrieval_holo(to_dev(h1, cuda), to_dev(h2, cuda), ph.CuTransfer(to_dev(tp, cuda)),
                                   ph.CuTransfer(to_dev(tpi, cuda)), 3, n)
    assert rel_l2(to_np(u.data), ref.phase_retrieval_holo(h1, h2, tp, tpi, 3, n)) < REL_L2


# (2048, 768) / (768, 2048): the 4-row passes at 2048 walk 192 blocks, a second
# round on 40 CTAs; (2048, 6) / (2048, 3): fewer blocks than CTAs, the one
# block of the row pass partial.
@pytest.mark.parametrize("n_fast,n_slow", [(2048, 1024), (1024, 2048), (2048, 768), (768, 2048), (2048, 6),
                                           (2048, 3)])
def test_gs_rectangular_through_abi(ph, cuda, n_fast, n_slow):
    """Rectangular frames through the C ABI (the Python mirror keeps the
    reference's square assertion): the staged column and row passes run at
    different lengths, each storing through a tensor map whose inner extent is
    the other length.  Random unit-modulus centred transfers, 2 iterations,
    against the oracle's propagation and amplitude steps."""
    from ph_gb300 import _lib
    rng = np.random.default_rng(n_fast + 3 * n_slow)
    shape = (n_slow, n_fast)
    h1 = rng.uniform(0.1, 1.0, shape).astype(np.float32)
    h2 = rng.uniform(0.1, 1.0, shape).astype(np.float32)
    tp = np.exp(1j * rng.uniform(-np.pi, np.pi, shape)).astype(np.complex64)
    tpi = np.conj(tp).astype(np.complex64)
    iters = 2
    d1, d2, dtp, dtpi = to_dev(h1, cuda), to_dev(h2, cuda), to_dev(tp, cuda), to_dev(tpi, cuda)
    out = torch.empty(shape, dtype=torch.complex64, device=cuda)
    ctx = _lib.default_context(cuda.index or 0)
    ctx.call("ph_phase_retrieval", out.data_ptr(), d1.data_ptr(), d2.data_ptr(), dtp.data_ptr(), dtpi.data_ptr(),
             n_fast, n_slow, iters, None, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    s1, s2 = np.sqrt(h1), np.sqrt(h2)
    u = s1.astype(np.complex64)
    for _ in range(iters):
        u = ref._amplitude_replace(s1, ref._propagate(ref._amplitude_replace(s2, ref._propagate(u, tp)), tpi))
    assert rel_l2(to_np(out), u) < REL_L2


def test_gs_zero_iterations_and_sizes(ph, cuda):
    n = 16
    h = torch.rand((n, n), device=cuda)
    tf = ph.cu_transfer(10.0, n, LAM, ph.cu_transfer_sqrt_arr(n, LAM, DX))
    u = ph.cu_phase_retrieval_holo(h, h, tf, tf, 0, n)
    assert torch.equal(u.data, torch.complex(torch.sqrt(h), torch.zeros_like(h)))
    with pytest.raises(AssertionError, match="All arrays must have the same size"):
        ph.cu_phase_retrieval_holo(h, h, tf, tf, 1, 8)


def test_lpf_all_pass_identity(ph, cuda):
    """An all-ones mask leaves the wavefront unchanged up to FFT rounding."""
    from ph_gb300 import _lib
    n = 128
    rng = np.random.default_rng(1)
    u = (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))).astype(np.complex64)
    t = to_dev(u, cuda)
    out = torch.empty_like(t)
    mask = torch.ones((n, n), dtype=torch.float32, device=cuda)
    _lib.default_context(0).call("ph_apply_lpf", out.data_ptr(), t.data_ptr(), mask.data_ptr(), n, n,
                                 torch.cuda.current_stream().cuda_stream)
    assert rel_l2(to_np(out), u) < 1e-6
