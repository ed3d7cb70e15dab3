"""The reference's end-to-end detection case (test/runtests.jl:153-193) shared
by the CPU oracle test and the GPU library test: phase retrieval of
holo1.bmp / holo2.bmp (80 mm apart, 9 iterations), 1000 N0f8 slices every
100 um from 80 mm, threshold 10/255, particle_bounding_boxes,
particle_coordinates.  Its output, test/data/particles.json, is the fixture
tests/golden/particles_ref.npz."""
from __future__ import annotations

from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"

LAM = 0.6328            # wavelength [um]
DX = 10.0               # pixel pitch [um]
Z0 = 80000.0            # hologram to the front of the volume [um]
DZ = 100.0              # slice spacing [um]
DATLEN = 1024
SLICES = 1000
PR_DIST = 80000.0       # between the two holograms [um]
PR_ITER = 9
THRESHOLD_LEVEL = 10    # d_vol .<= 10/255 on N0f8 levels: level <= 10


def holograms() -> tuple[np.ndarray, np.ndarray]:
    """load_gray2float (utils.jl:23-25): 8-bit levels / 255 as Float32."""
    with np.load(GOLDEN / "holo_pair.npz") as z:
        return (z["holo1"].astype(np.float32) / np.float32(255.0),
                z["holo2"].astype(np.float32) / np.float32(255.0))


def reference_particles() -> np.ndarray:
    with np.load(GOLDEN / "particles_ref.npz") as z:
        return z["coords"].astype(np.float64)
