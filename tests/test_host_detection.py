"""The host side of particle_coordinates (particle_detection.jl:113-160) on
sub-volumes with a known answer, without a GPU: the Tamura depth profile's
peak picks the slice, the centre of mass of that slice gives x and y."""
import numpy as np
import torch


def _reference_coords(box, sv):
    """Plain-loop restatement of particle_detection.jl:146-160 for one box:
    Float32 levels / 255, tamura = std / mean per slice, Gaussian(5) smoothing
    with replicated ends, first maximum, getcenterfromslice (:117-130)."""
    x0, y0, z0 = box[:3]
    v = sv.astype(np.float32) / np.float32(255.0)                  # (z, x, y)
    prof = []
    for sl in v:
        prof.append(float(np.std(sl, ddof=1) / np.mean(sl)))
    sigma = 5.0
    h = 2 * int(np.ceil(sigma))
    taps = [np.exp(-(t * t) / (2 * sigma * sigma)) for t in range(-h, h + 1)]
    taps = [t / sum(taps) for t in taps]
    sm = []
    for i in range(len(prof)):
        acc = 0.0
        for t in range(-h, h + 1):
            acc += taps[t + h] * prof[min(max(i + t, 0), len(prof) - 1)]
        sm.append(acc)
    z = max(range(len(sm)), key=lambda i: (sm[i], -i))              # first maximum
    arr = v[z].T                                                   # (y rows i, x columns j), 1-based below
    sx = sy = tot = 0.0
    for i in range(arr.shape[0]):
        for j in range(arr.shape[1]):
            sy += (i + 1) * float(arr[i, j])
            sx += (j + 1) * float(arr[i, j])
            tot += float(arr[i, j])
    return (sx / tot + x0 - 1, sy / tot + y0 - 1, z + 1 + z0 - 1)


def test_particle_coordinates_known_answer(ph):
    rng = np.random.default_rng(4)
    boxes, subs, want = [], [], []
    for b, (nz, nx, ny, zpk) in enumerate([(9, 12, 10, 4), (5, 7, 9, 0), (13, 20, 16, 11)]):
        sv = np.full((nz, nx, ny), 26, dtype=np.uint8)
        sv += rng.integers(0, 3, sv.shape, dtype=np.uint8)         # faint texture on every slice
        xa, ya = rng.integers(0, nx - 3), rng.integers(0, ny - 3)
        sv[zpk, xa:xa + 3, ya:ya + 3] = 255                        # the particle, sharp at slice zpk
        x0, y0, z0 = 10 + 5 * b, 3 + b, 2 + 7 * b
        box = (x0, y0, z0, x0 + nx - 1, y0 + ny - 1, z0 + nz - 1)
        boxes.append(box)
        subs.append(torch.from_numpy(sv))
        want.append(_reference_coords(box, sv))
        assert want[-1][2] == z0 + zpk                            # the peak slice wins
    got = ph.particle_coordinates(np.array(boxes), subs)
    np.testing.assert_allclose(got, np.array(want), rtol=0, atol=1e-4)
