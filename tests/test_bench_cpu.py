"""The CPU legs of bench.py (the oracle sample behind `cpu_baseline`, its
accuracy against the exact-physics FP64 oracle, and the `--impl reference`
line) on small frames, without a GPU."""
import io
import json
import math
from contextlib import redirect_stdout
from types import SimpleNamespace

import numpy as np

import bench


def _small(name: str, n: int = 64, slices: int = 8) -> dict:
    cfg = dict(bench.CONFIGS[name])
    cfg.update(n=n, slices=slices)
    return cfg


def test_cpu_sample_and_fp64_accuracy():
    cfg = _small("c2")
    rng = np.random.default_rng(3)
    h1 = rng.uniform(0.2, 1.0, (cfg["n"], cfg["n"])).astype(np.float32)
    h2 = rng.uniform(0.2, 1.0, (cfg["n"], cfg["n"])).astype(np.float32)
    outs = {}
    t_it, t_slice, t_ccl = bench.cpu_frame_sample(cfg, h1, h2, 2, 4, outs)
    assert min(t_it, t_slice, t_ccl) > 0
    assert bench.cpu_mvoxel_per_s(cfg, t_it, t_slice, t_ccl) > 0
    acc = bench.fp64_accuracy(cfg, h1, h2, outs["wf"], outs["proj"], outs["arg"], 2, 4)
    for key in ("field_rel_l2", "projection_rel_l2", "argmin_agreement", "phase_rms_rad", "gs_residual_fp64"):
        assert math.isfinite(acc[key]), key
    # the FP32 reference semantics against the physics: close, not equal
    assert acc["field_rel_l2"] < 1e-2 and acc["projection_rel_l2"] < 1e-2
    assert acc["argmin_agreement"] > 0.9


def test_reference_arm_line():
    cfg = _small("c1", n=128, slices=256)
    args = SimpleNamespace(steps=1, warmup=0, gpus=1)
    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.reference_arm(args, cfg, 0, 1)
    line = json.loads(buf.getvalue().strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "Mvoxel/s"
    assert line["cpu_baseline"]["value"] == line["value"] and line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
