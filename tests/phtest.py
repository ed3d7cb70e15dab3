"""Helpers shared by the tests: tolerances, error metrics, device transfers."""
from __future__ import annotations

import numpy as np

# Tolerances (relative L2 unless noted) of the FP32 path against the
# reference-semantics FP32 oracle.
REL_L2 = 1e-4          # slices / projections / fields
ARGMIN_AGREE = 0.999   # fraction of pixels whose argmin depth matches


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.complex128 if np.iscomplexobj(a) or np.iscomplexobj(b) else np.float64)
    b = np.asarray(b, dtype=a.dtype)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


def to_dev(x, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).to(dev)


def to_np(t):
    return t.detach().cpu().numpy()


def argmin_agreement(got, want, proj_ref, slices_ref=None) -> float:
    """Fraction of pixels whose argmin matches."""
    return float(np.mean(np.asarray(got) == np.asarray(want)))
