"""GB300 (sm_103a) implementation of ParticleHolography.jl's reconstruction hot path.

The compute lives in ``libphgb300.so`` (hand-written CUDA kernels behind the C
ABI of ``include/phgb300.h``); this package is its host side, mirroring the
reference's Julia API (src/holofunc.jl, src/ccl.jl, src/types.jl) with torch
CUDA tensors standing in for CuArrays.

The directory name is not a Python identifier; load the package with
``__graft_entry__.load_package()`` (it registers it as ``ph_gb300``).
"""
from . import _lib
from .batch import ReconBatch, autotune
from .detection import (cu_get_reconst_binary_vol, cu_reconst_subvolumes, particle_coordinates,
                        slice_bounding_boxes)
from .serve import Server
from .ccl import (count_labels, cu_bounding_rectangles, cu_connected_component_labeling,
                  cu_connected_component_labeling_batch, cu_find_valid_labels)
from .frequency_filters import (cu_apply_low_pass_filter, cu_apply_low_pass_filter_, cu_rectangle_filter,
                                cu_super_gaussian_filter)
from .holofunc import (cu_2d_pad, cu_asm_prop_, cu_gabor_wavefront, cu_get_reconst_complex_vol,
                       cu_get_reconst_vol, cu_get_reconst_vol_and_xyprojection,
                       cu_get_reconst_vol_and_xyprojection_padded, cu_get_reconst_xyprojection, cu_get_reconst_xyprojection_lpf,
                       cu_phase_retrieval_holo, cu_transfer, cu_transfer_fp64, cu_transfer_sqrt_arr)
from .utils import cu_make_background_mode, make_background, pad_with_mean
from .types import CuLowPassFilter, CuTransfer, CuTransferSqrtPart, CuWavefront, N0f8

LIB_PATH = _lib.LIB_PATH


def library_loaded() -> bool:
    """True once libphgb300.so has been loaded into this process."""
    return _lib._lib is not None
