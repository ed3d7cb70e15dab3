"""Restatement of the reference's 3-D particle detection -- TEST INFRASTRUCTURE ONLY.

Imported by tests only, as the checker of the end-to-end detection pipeline
that ``test/runtests.jl:153-193`` runs (phase retrieval, N0f8 volume,
threshold, ``particle_bounding_boxes``, ``particle_coordinates``) and whose
output the reference ships as ``test/data/particles.json``.

Functions follow, step by step:

* ``slice_rectangles``        -- ``cu_connected_component_labeling`` + ``cu_find_valid_labels``
  + ``get_bounding_rectangles`` (ccl.jl:186-264) for one binary slice.  The
  labeling of a Bool image is 8-connected components of the true pixels
  (``resolve_background``, ccl.jl:159-172, zeroes the false ones); components
  are listed in the order of their root, the minimum linear index, which is
  the order in which a raster scan first meets them (scipy's label order).
* ``gen_particle_neighborhoods``, ``update_particle_neighborhoods``,
  ``finalize_particle_neighborhoods``, ``delete_duplicates``, the overlap tests
  (ccl.jl:266-360, 424-467).
* ``particle_bounding_boxes`` (particle_detection.jl:58-76).
* ``particle_coordinates`` with ``tamura``, ``depth_profile``,
  ``getcenterfromslice`` and ``Kernel.gaussian((5,))`` smoothing with
  ImageFiltering's default replicated border (particle_detection.jl:109-157).

Dictionary order.  The reference keys its neighbourhoods by time-based UUIDs
(``uuid1``) in a ``Dict``, so it visits them in hash order, which differs run
to run.  The merge rules above depend on that order only when several boxes
overlap one another; here the neighbourhoods are visited in insertion order.

Coordinates.  A Julia slice of size ``(n_fast, n_slow)`` is held as a numpy
array ``(n_slow, n_fast)``.  The reference's rectangle ``(x, y)`` is
(second index, first index) = (slow + 1, fast + 1), 1-based.
"""
from __future__ import annotations

import itertools

import numpy as np
from scipy import ndimage

_EIGHT = np.ones((3, 3), dtype=bool)


# ---------------------------------------------------------------- per-slice rectangles

def slice_rectangles(binary: np.ndarray) -> list[tuple[int, int, int, int]]:
    """``get_bounding_rectangles(labels, cu_find_valid_labels(labels))`` of one
    binary slice ``(n_slow, n_fast)``: ``(x_min, y_min, x_max, y_max)`` per
    component, 1-based inclusive, in root order (ccl.jl:234-264)."""
    lab, n = ndimage.label(np.asarray(binary, dtype=bool), structure=_EIGHT)
    out = []
    for sl in ndimage.find_objects(lab, max_label=n):
        out.append((sl[0].start + 1, sl[1].start + 1, sl[0].stop, sl[1].stop))
    return out


# ---------------------------------------------------------------- neighbourhoods (ccl.jl:266-467)

def judge_overlap2d(r1, r2) -> bool:
    """ccl.jl:279-288: strict overlap of two (x_min, y_min, x_max, y_max)."""
    return r1[0] < r2[2] and r1[2] > r2[0] and r1[1] < r2[3] and r1[3] > r2[1]


def judge_overlap3d(r1, r2) -> bool:
    """ccl.jl:290-299: strict overlap of two (x_min, y_min, z_min, x_max, y_max, z_max)."""
    return (r1[0] < r2[3] and r1[3] > r2[0] and r1[1] < r2[4] and r1[4] > r2[1]
            and r1[2] < r2[5] and r1[5] > r2[2])


def new_rect(r1, r2) -> list[int]:
    """ccl.jl:301-311: the union box of two (x_min, y_min, x_max, y_max)."""
    return [min(r1[0], r2[0]), min(r1[1], r2[1]), max(r1[2], r2[2]), max(r1[3], r2[3])]


class _Keys:
    """Stand-in for ``uuid1(rng)``: distinct keys in creation order."""

    def __init__(self):
        self._c = itertools.count()

    def __call__(self) -> int:
        return next(self._c)


def gen_particle_neighborhoods(rects, slicenum: int, keys: _Keys) -> dict:
    """ccl.jl:266-277: one neighbourhood [x_min, y_min, z, x_max, y_max, z] per rectangle."""
    return {keys(): [r[0], r[1], slicenum, r[2], r[3], slicenum] for r in rects}


def update_particle_neighborhoods(pn: dict, rects, slicenum: int, keys: _Keys) -> None:
    """ccl.jl:325-360: every rectangle grows each neighbourhood it overlaps in x-y
    (and extends its z range), or starts a new one; then 1 x 1 x 1 spans go."""
    for br in rects:
        overlap = False
        for v in pn.values():
            if judge_overlap2d(br, (v[0], v[1], v[3], v[4])):
                nb = new_rect(br, (v[0], v[1], v[3], v[4]))
                v[0], v[1], v[3], v[4] = nb
                if slicenum < v[2]:
                    v[2] = slicenum
                elif slicenum > v[5]:
                    v[5] = slicenum
                overlap = True
        if not overlap:
            pn[keys()] = [br[0], br[1], slicenum, br[2], br[3], slicenum]
    for k in list(pn):
        v = pn[k]
        if abs(v[0] - v[3]) == 1 and abs(v[1] - v[4]) == 1 and abs(v[2] - v[5]) == 1:
            del pn[k]


def delete_duplicates(pn: dict) -> None:
    """ccl.jl:441-467: a neighbourhood absorbs the first other one it overlaps in
    3-D (which is deleted); repeated until nothing changes.  Entries deleted
    during the pass are not visited again."""
    while True:
        changed = False
        for k in list(pn):
            if k not in pn:
                continue
            v = pn[k]
            for k2 in list(pn):
                if k2 == k:
                    continue
                v2 = pn[k2]
                if judge_overlap3d(v, v2):
                    nb = new_rect((v[0], v[1], v[3], v[4]), (v2[0], v2[1], v2[3], v2[4]))
                    v[0], v[1], v[3], v[4] = nb
                    v[2] = min(v[2], v2[2])
                    v[5] = max(v[5], v2[5])
                    del pn[k2]
                    changed = True
                    break
        if not changed:
            return


def _ratio(num: int, den: int) -> float:
    """Julia's Int / Int: Float64 division with x/0 = Inf and 0/0 = NaN."""
    if den == 0:
        return float("nan") if num == 0 else float("inf")
    return num / den


def finalize_particle_neighborhoods(pn: dict) -> None:
    """ccl.jl:424-439: drop neighbourhoods one slice deep, with an x-y aspect
    ratio above 3 or below 1/3, or an x-y area below 10."""
    delete_duplicates(pn)
    for k in list(pn):
        v = pn[k]
        r = _ratio(abs(v[0] - v[3]), abs(v[1] - v[4]))
        if abs(v[2] - v[5]) == 1 or r > 3 or r < 1 / 3 or abs(v[0] - v[3]) * abs(v[1] - v[4]) < 10:
            del pn[k]


def neighborhoods_from_rectangles(rects_per_slice) -> list[list[int]]:
    """The bookkeeping of particle_bounding_boxes (particle_detection.jl:59-75)
    over per-slice rectangle lists (slice 1 first, each in root order): the
    surviving neighbourhoods [x_min, y_min, z_min, x_max, y_max, z_max]
    (1-based, z the slice number)."""
    keys = _Keys()
    rects = iter(rects_per_slice)
    pn = gen_particle_neighborhoods(next(rects), 1, keys)
    for idx, r in enumerate(rects, start=2):
        update_particle_neighborhoods(pn, r, idx, keys)
    finalize_particle_neighborhoods(pn)
    return [list(v) for v in pn.values()]


def particle_bounding_boxes(bin_vol: np.ndarray) -> list[list[int]]:
    """particle_detection.jl:58-76 on a Bool volume ``(slices, n_slow, n_fast)``."""
    return neighborhoods_from_rectangles(slice_rectangles(s) for s in bin_vol)


# ---------------------------------------------------------------- coordinates (particle_detection.jl:109-157)

def gaussian_kernel(sigma: float = 5.0) -> np.ndarray:
    """ImageFiltering ``Kernel.gaussian((sigma,))``: 4 ceil(sigma) + 1 taps of
    exp(-x^2 / (2 sigma^2)), normalised to sum 1."""
    h = 2 * int(np.ceil(sigma))
    x = np.arange(-h, h + 1, dtype=np.float64)
    k = np.exp(-x * x / (2.0 * sigma * sigma))
    return k / k.sum()


def particle_coordinates(boxes, vol_n0f8: np.ndarray, sigma: float = 5.0) -> np.ndarray:
    """particle_detection.jl:146-157 on an N0f8 volume ``(slices, n_slow, n_fast)``
    (raw levels): per box the Tamura profile (std / mean, corrected std) of the
    Float32 sub-volume's slices, smoothed (replicated border), its first
    maximum z, and the intensity-weighted centre of that slice.  Rows
    ``(x, y, z)`` in the reference's 1-based coordinates, rounded to Float32
    as the reference stores them."""
    k = gaussian_kernel(sigma)
    h = len(k) // 2
    out = []
    for x0, y0, z0, x1, y1, z1 in boxes:
        sub = vol_n0f8[z0 - 1:z1, x0 - 1:x1, y0 - 1:y1].astype(np.float32) / np.float32(255.0)   # (z, x, y)
        flat = sub.reshape(sub.shape[0], -1).astype(np.float64)
        prof = flat.std(axis=1, ddof=1) / flat.mean(axis=1)
        pad = np.concatenate([np.full(h, prof[0]), prof, np.full(h, prof[-1])])
        smooth = np.correlate(pad, k, mode="valid")
        z = int(np.argmax(smooth))                   # first maximum
        sl = sub[z].astype(np.float64)               # [x][y]: x = Julia's second index j, y its first i
        tot = sl.sum()
        x = (np.arange(1, sl.shape[0] + 1)[:, None] * sl).sum() / tot
        y = (np.arange(1, sl.shape[1] + 1)[None, :] * sl).sum() / tot
        out.append((x + x0 - 1, y + y0 - 1, z + 1 + z0 - 1))
    return np.array(out, dtype=np.float32).reshape(-1, 3)


# ---------------------------------------------------------------- matching against particles.json

def match_particles(got: np.ndarray, want: np.ndarray, tol_xy: float, tol_z: float):
    """Greedy one-to-one nearest matching of particle rows (x, y, z): pairs whose
    |dx|, |dy| <= tol_xy and |dz| <= tol_z, closest (in x-y, then z) first.
    Returns (pairs [(i_got, i_want)], unmatched got indices, unmatched want indices)."""
    got = np.asarray(got, dtype=np.float64).reshape(-1, 3)
    want = np.asarray(want, dtype=np.float64).reshape(-1, 3)
    cand = []
    for i, g in enumerate(got):
        for j, w in enumerate(want):
            d = np.abs(g - w)
            if d[0] <= tol_xy and d[1] <= tol_xy and d[2] <= tol_z:
                cand.append((float(np.hypot(d[0], d[1])), float(d[2]), i, j))
    cand.sort()
    used_g, used_w, pairs = set(), set(), []
    for _, _, i, j in cand:
        if i not in used_g and j not in used_w:
            used_g.add(i)
            used_w.add(j)
            pairs.append((i, j))
    return (pairs, [i for i in range(len(got)) if i not in used_g], [j for j in range(len(want)) if j not in used_w])
