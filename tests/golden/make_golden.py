"""Regenerates the golden fixtures of this directory.

Two kinds of fixtures:

* Reference data, read here from the reference checkout's ``test/data`` and
  stored small: the binary particle image of the CCL known answer (84
  components, ``test/runtests.jl:213-231``) as packed bits, and 256 x 256 centre
  crops of the real holograms ``holo1.bmp`` / ``holo2_corrected.png``.
* Oracle vectors: inputs and outputs of ``oracle/ref_semantics.py`` (and the
  FP64 oracle) at small sizes, covering every function of the hot path.

All arrays are stored in the C order of the Julia buffer: a Julia array of size
``(n_fast, n_slow)`` is a numpy array of shape ``(n_slow, n_fast)``; an image
as displayed (row, col) is therefore stored transposed.

Usage: ``python tests/golden/make_golden.py <path-to-reference-checkout>``.
"""
from __future__ import annotations

import struct
import sys
import zlib
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from oracle import ccl as occl          # noqa: E402
from oracle import fp64 as o64          # noqa: E402
from oracle import ref_semantics as ref  # noqa: E402

LAM, DX = 0.6328, 10.0


# ------------------------------------------------------------------ image readers

def read_png(path: Path):
    """Minimal PNG decoder: 8-bit gray / RGB / palette, non-interlaced."""
    d = path.read_bytes()
    assert d[:8] == b"\x89PNG\r\n\x1a\n"
    i, idat, pal = 8, b"", None
    while i < len(d):
        n, = struct.unpack(">I", d[i:i + 4])
        t, body = d[i + 4:i + 8], d[i + 8:i + 8 + n]
        if t == b"IHDR":
            w, h, bd, ct, _, _, il = struct.unpack(">IIBBBBB", body)
            assert bd == 8 and il == 0
        elif t == b"PLTE":
            pal = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif t == b"IDAT":
            idat += body
        i += 12 + n
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ct]
    stride = w * ch
    raw = np.frombuffer(zlib.decompress(idat), np.uint8)
    out = np.zeros((h, stride), np.int32)
    prev = np.zeros(stride, np.int32)
    p = 0
    for y in range(h):
        f = raw[p]
        line = raw[p + 1:p + 1 + stride].astype(np.int32)
        p += 1 + stride
        cur = np.zeros(stride, np.int32)
        if f == 0:
            cur = line.copy()
        elif f == 2:
            cur = (line + prev) & 255
        else:
            for x in range(stride):
                a = cur[x - ch] if x >= ch else 0
                b = prev[x]
                c = prev[x - ch] if x >= ch else 0
                if f == 1:
                    pr = a
                elif f == 3:
                    pr = (a + b) // 2
                else:
                    pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                    pr = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cur[x] = (line[x] + pr) & 255
        out[y] = cur
        prev = cur
    img = out.astype(np.uint8).reshape(h, w, ch)
    if ct == 3:
        img = pal[img[..., 0]]
    return img


def read_bmp(path: Path):
    d = path.read_bytes()
    off, = struct.unpack("<I", d[10:14])
    w, h = struct.unpack("<ii", d[18:26])
    bpp, = struct.unpack("<H", d[28:30])
    assert bpp == 24
    stride = (w * 3 + 3) // 4 * 4
    rows = np.frombuffer(d[off:off + stride * abs(h)], np.uint8).reshape(abs(h), stride)[:, :w * 3]
    img = rows.reshape(abs(h), w, 3)[:, :, ::-1]
    return img[::-1] if h > 0 else img       # bottom-up storage


def gray_u8(img: np.ndarray) -> np.ndarray:
    if img.ndim == 2:
        return img
    if img.shape[-1] == 1:
        return img[..., 0]
    assert np.array_equal(img[..., 0], img[..., 1]) and np.array_equal(img[..., 1], img[..., 2])
    return img[..., 0]


# ------------------------------------------------------------------ fixtures

def reference_data(refroot: Path):
    data = refroot / "test" / "data"
    g = gray_u8(read_png(data / "binaryparticles.png"))
    fg = (1.0 - g.astype(np.float32) / 255.0)          # runtests.jl:204 `1.0f0 .- img`
    buf = fg.T.copy()                                   # Julia buffer order
    assert set(np.unique(buf)) <= {0.0, 1.0}
    assert ref.count_labels(occl.connected_component_labeling(buf)) == 84
    np.savez_compressed(HERE / "binaryparticles.npz", fg_bits=np.packbits(buf.astype(bool).reshape(-1)),
                        shape=np.array(buf.shape), count=np.array(84))
    h1 = gray_u8(read_bmp(data / "holo1.bmp")).T
    h2 = gray_u8(read_png(data / "holo2_corrected.png")).T
    c = slice(384, 640)
    np.savez_compressed(HERE / "holo_crops.npz", holo1=h1[c, c].copy(), holo2=h2[c, c].copy())
    pipeline_data(refroot)


def pipeline_data(refroot: Path):
    """Inputs and output of the reference's end-to-end detection test
    (``test/runtests.jl:153-193``): the full 1024^2 holograms ``holo1.bmp`` /
    ``holo2.bmp`` as 8-bit levels in Julia buffer order, and the 22 particle
    coordinates ``[x, y, z_slice]`` the reference wrote to
    ``test/data/particles.json`` (UUID keys dropped: they are time-based)."""
    import json
    data = refroot / "test" / "data"
    h1 = gray_u8(read_bmp(data / "holo1.bmp")).T.copy()
    h2 = gray_u8(read_bmp(data / "holo2.bmp")).T.copy()
    coords = json.loads((data / "particles.json").read_text())
    rows = np.array(sorted(coords.values()), dtype=np.float32).reshape(-1, 3)
    np.savez_compressed(HERE / "holo_pair.npz", holo1=h1, holo2=h2)
    np.savez_compressed(HERE / "particles_ref.npz", coords=rows)


def oracle_vectors():
    rng = np.random.default_rng(20241203)
    out = {}
    # transfer functions
    for n in (4, 8, 64):
        d = ref.transfer_sqrt_arr(n, LAM, DX)
        out[f"sqr_{n}"] = d
        for z in (80000.0, -80000.0, -100.0):
            out[f"tf_{n}_{int(z)}"] = ref.transfer(z, n, LAM, d)
    out["sqr_rect_16x32"] = ref.transfer_sqrt_arr(32, LAM, DX, n_slow=16)
    # gabor
    h = rng.uniform(0.0, 1.0, (64, 64)).astype(np.float32)
    out["gabor_in"] = h
    out["gabor_out"] = ref.gabor_wavefront(h)
    # reconstruction, 64^2 x 12 slices
    n, s = 64, 12
    d = out["sqr_64"]
    hf = ref.transfer(-1000.0, n, LAM, d)
    hdz = ref.transfer(-200.0, n, LAM, d)
    holo = rng.uniform(0.1, 1.0, (n, n)).astype(np.float32)
    wf = ref.gabor_wavefront(holo)
    out.update(rec_holo=holo, rec_hf=hf, rec_hdz=hdz)
    p, a = ref.reconst_xyprojection(wf, hf, hdz, s, with_argmin=True)
    out.update(rec_proj=p, rec_argmin=a)
    out["rec_vol_n0f8"] = ref.reconst_vol(wf, hf, hdz, s)
    out["rec_vol_f32"] = ref.reconst_vol(wf, hf, hdz, s, np.float32)
    v, pv = ref.reconst_vol_and_xyprojection(wf, hf, hdz, s)
    out["rec_volproj_proj"] = pv
    out["rec_cvol"] = ref.reconst_complex_vol(wf[:16, :16], hf[:16, :16], hdz[:16, :16], 4)
    # padded (the reference test's shapes: 4x4 input, 8x8 transfers, 2 slices) and 16 -> 32
    for m, sl in ((4, 2), (16, 4)):
        d2 = ref.transfer_sqrt_arr(2 * m, LAM, DX)
        tf2 = ref.transfer(-100.0, 2 * m, LAM, d2)
        tdz2 = ref.transfer(-10.0, 2 * m, LAM, d2)
        hm = rng.uniform(0.0, 1.0, (m, m)).astype(np.float32)
        vol, pj = ref.reconst_vol_and_xyprojection_padded(ref.gabor_wavefront(hm), tf2, tdz2, sl)
        out.update({f"pad{m}_holo": hm, f"pad{m}_tf": tf2, f"pad{m}_tdz": tdz2, f"pad{m}_vol": vol,
                    f"pad{m}_proj": pj})
    # cu_2d_pad example of runtests.jl:362-368 (Julia [1+1im 2+1im; 3+1im 4+1im] -> buffer order)
    jl = np.array([[1 + 1j, 2 + 1j], [3 + 1j, 4 + 1j]], dtype=np.complex64)
    out["pad2d_in"] = jl.T.copy()
    out["pad2d_out"] = ref.pad2d(jl.T.copy())
    # asm propagation: the reference test's 4x4 ones and a random 16^2 field
    d4 = out["sqr_4"]
    out["asm_ones_out"] = ref.asm_prop(np.ones((4, 4), np.complex64), d4, 100.0, 4, LAM)
    u = (rng.normal(size=(16, 16)) + 1j * rng.normal(size=(16, 16))).astype(np.complex64)
    d16 = ref.transfer_sqrt_arr(16, LAM, DX)
    out.update(asm_in=u, asm_sqr=d16, asm_out=ref.asm_prop(u, d16, 2500.0, 16, LAM))
    # Gerchberg-Saxton 64^2, 5 iterations
    g1 = rng.uniform(0.2, 1.0, (n, n)).astype(np.float32)
    g2 = rng.uniform(0.2, 1.0, (n, n)).astype(np.float32)
    tp = ref.transfer(5000.0, n, LAM, d)
    tpi = ref.transfer(-5000.0, n, LAM, d)
    gu, gr = ref.phase_retrieval_holo(g1, g2, tp, tpi, 5, n, return_residual=True)
    out.update(gs_h1=g1, gs_h2=g2, gs_tp=tp, gs_tpi=tpi, gs_out=gu, gs_resid=np.float64(gr))
    # labeling: a few small images with several values, and their labels
    for k, (r_, c_) in enumerate(((7, 7), (16, 16), (12, 20))):
        img = rng.integers(0, 3, (r_, c_)).astype(np.float32)
        out[f"ccl{k}_img"] = img
        out[f"ccl{k}_lab"] = occl.connected_component_labeling(img)
    # FP64 generator, 64^2 with 5 discs
    discs = o64.draw_discs(11, 64, 5, 40.0, 80.0, 2000.0, 20000.0, DX)
    field = o64.synth_field(discs, 64, 64, LAM, DX)
    out["synth64_intensity"] = (np.abs(field) ** 2).astype(np.float64)
    np.savez_compressed(HERE / "oracle_small.npz", **out)


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0] if __doc__ else None)
    ap.add_argument("reference", type=Path, help="checkout of ParticleHolography.jl (its test/data fixtures)")
    refroot = ap.parse_args().reference
    if not (refroot / "test" / "data").exists():
        sys.exit(f"{refroot} holds no test/data: give the path of a ParticleHolography.jl checkout")
    reference_data(refroot)
    oracle_vectors()
    for f in sorted(HERE.glob("*.npz")):
        print(f"{f.name}: {f.stat().st_size} bytes")
