"""The oracle pinned to the reference's own output: the CPU restatement runs the
reference's end-to-end detection test (test/runtests.jl:153-193) and must
reproduce the 22 particles of test/data/particles.json.  This pins transfer
functions, Gerchberg-Saxton, the N0f8 volume, labeling and the detection
bookkeeping of the oracle, whose FFT is scipy's pocketfft where the
reference's is cuFFT.  (About 30 s on 8 cores.)"""
import numpy as np

import pipeline_case as pc
from oracle import detect_ref as dr
from oracle import ref_semantics as ref


def test_oracle_reproduces_reference_particles():
    h1, h2 = pc.holograms()
    n = pc.DATLEN
    d = ref.transfer_sqrt_arr(n, pc.LAM, pc.DX)
    u = ref.phase_retrieval_holo(h1, h2, ref.transfer(pc.PR_DIST, n, pc.LAM, d),
                                 ref.transfer(-pc.PR_DIST, n, pc.LAM, d), pc.PR_ITER, n)
    vol = np.empty((pc.SLICES, n, n), np.uint8)
    for k, x in enumerate(ref.iter_slices(u, ref.transfer(-pc.Z0, n, pc.LAM, d), ref.transfer(-pc.DZ, n, pc.LAM, d),
                                          pc.SLICES)):
        vol[k] = ref.ifft_and_abs(x, ref.N0f8)
    boxes = dr.particle_bounding_boxes(vol <= pc.THRESHOLD_LEVEL)
    got = dr.particle_coordinates(boxes, vol)
    want = pc.reference_particles()
    pairs, extra, missing = dr.match_particles(got, want, tol_xy=1e-3, tol_z=0.0)
    assert not extra and not missing, (got[extra], want[missing])
    assert len(pairs) == len(want) == 22
