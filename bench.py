"""Benchmark of the reconstruction hot path on GB300 (one JSON line on stdout).

Workload (default, ``--config c2``): a seeded pair of 2048 x 2048 Float32
holograms (800 opaque discs, diameter 10-60 um, z in [5, 100] mm, recorded
5 mm apart, lambda = 0.6328 um, pitch 10 um).  One step is one frame:
Gerchberg-Saxton phase retrieval (20 iterations) -> angular-spectrum
reconstruction of 512 slices at dz = 0.2 mm from z0 = 5 mm reduced on the fly to
the xy min-projection and argmin-depth map -> threshold -> connected-component
labeling.  Metric: reconstructed Mvoxel/s (voxel = one pixel of one slice),
with p50/p99 frame latency.

``value``  device-resident inputs, CUDA events per step on the launching stream,
          L2 flushed (a 512 MiB write) before every timed step, outside the events.
``e2e``    the same frame through the public API from pinned host buffers: the
          hologram pair copied in, projection + argmin copied out and the
          component count read back, every step.
``roofline`` the dominant kernel's algorithmic bytes per launch over its
          CUDA-event duration (library profiler, on the launching stream,
          during the timed steps).
``cpu_baseline`` the oracle (numpy / scipy.fft on all host cores, FP32) timed
          on a bounded sample of the frame and scaled to Mvoxel/s.
``--impl reference`` times that CPU path as the reference arm.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

LAM, DX = 0.6328, 10.0
CONFIGS = {
    # name: (n, slices, dz, z0, discs, dmin, dmax, zmin, zmax, gs_iters, gs_sep, threshold, seed)
    "c1": dict(n=1024, slices=256, dz=200.0, z0=1000.0, discs=200, dmin=20.0, dmax=80.0, zmin=1000.0,
               zmax=50000.0, gs_iters=0, gs_sep=0.0, threshold=0.5, seed=1,
               workload="gabor1024_recon256_ccl"),
    "c2": dict(n=2048, slices=512, dz=200.0, z0=5000.0, discs=800, dmin=10.0, dmax=60.0, zmin=5000.0,
               zmax=100000.0, gs_iters=20, gs_sep=5000.0, threshold=0.1, seed=2,
               workload="gs2048_pr20_recon512_proj_argmin_ccl"),
    "c3": dict(n=4096, slices=1024, dz=(200000.0 - 5000.0) / 1024, z0=5000.0, discs=3000, dmin=10.0, dmax=60.0,
               zmin=5000.0, zmax=200000.0, gs_iters=0, gs_sep=0.0, threshold=0.1, seed=3,
               workload="gabor4096_recon1024_ccl"),
    # the 2048^2 frame cut to 64 slices and 2 GS iterations, sized for ncu captures (~3 GB on the
    # device): GS launches have their c2 size, reconstruction launches an eighth of it (64 of 512 slices)
    "p2": dict(n=2048, slices=64, dz=200.0, z0=5000.0, discs=800, dmin=10.0, dmax=60.0, zmin=5000.0,
               zmax=100000.0, gs_iters=2, gs_sep=5000.0, threshold=0.1, seed=2,
               workload="gs2048_pr2_recon64_profile"),
    # the 4096^2 workload cut to one 16-slice batch, for kernel captures of pass A in clusters
    "p3": dict(n=4096, slices=16, dz=(200000.0 - 5000.0) / 1024, z0=5000.0, discs=3000, dmin=10.0, dmax=60.0,
               zmin=5000.0, zmax=200000.0, gs_iters=0, gs_sep=0.0, threshold=0.1, seed=3,
               workload="gabor4096_recon16_profile"),
}
# Mixed batch: (n_fast, n_slow, count) size classes; per item slices ~ U{32..512} and
# dz ~ U(0.1, 0.5) mm drawn from numpy PCG64(1000 + i); reconstructed from z0 = 5 mm.
C4_CLASSES = [(512, 512, 32), (1024, 1024, 32), (2048, 1536, 16), (2048, 2048, 16)]
CONFIGS["c4"] = dict(n=2048, slices=0, dz=0.0, z0=5000.0, discs=200, dmin=10.0, dmax=60.0, zmin=5000.0,
                     zmax=100000.0, gs_iters=0, gs_sep=0.0, threshold=0.1, seed=4, kind="batch",
                     workload="batch96_mixed_512_1024_1536x2048_2048_proj_argmin")
# Serving: Poisson arrivals at fractions of the measured capacity; 60 % 1024^2 x 256
# slices (z0 1 mm), 40 % 2048^2 x 512 slices (z0 5 mm), dz 0.2 mm: recurring optics.
C5_MIX = [(1024, 256, 1000.0, 200.0, 0.6), (2048, 512, 5000.0, 200.0, 0.4)]
C5_LOADS = [0.25, 0.5, 0.75, 0.9, 1.1]
CONFIGS["c5"] = dict(n=2048, slices=0, dz=200.0, z0=5000.0, discs=400, dmin=10.0, dmax=60.0, zmin=1000.0,
                     zmax=100000.0, gs_iters=0, gs_sep=0.0, threshold=0.1, seed=5, kind="serve",
                     workload="serve_mix60_1024x256_40_2048x512_poisson")
L2_FLUSH_BYTES = 512 << 20


def c4_items():
    """(n_fast, n_slow, slices, dz_um) of the 96 items of the mixed batch."""
    out = []
    for nx, ny, count in C4_CLASSES:
        for _ in range(count):
            rng = np.random.default_rng(1000 + len(out))
            out.append((nx, ny, int(rng.integers(32, 513)), float(rng.uniform(100.0, 500.0))))
    return out


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------- algorithmic bytes per launch

def algorithmic_bytes(name: str, cfg: dict, launches: int, slices_per_frame: int) -> float | None:
    """Bytes one launch of `name` must move through DRAM by design, per launch.

    recon_a  writes the slice intermediate T: 8 B per voxel (the spectrum state it
             reads, 16 B per pixel, stays resident in L2 across the batch).
    recon_b  reads T: 8 B per voxel.
    gs_col   reads and writes the field: 16 B per pixel.
    gs_row_* reads and writes the field (16 B) and reads the hologram (4 B).
    fwd_rows / spectrum: 8 + 8 B and 8 + 16 (+16 transfer reads) B per pixel.
    """
    n2 = cfg["n"] ** 2
    per_frame = {
        "recon_a": 8.0 * n2 * slices_per_frame,
        "recon_b": 8.0 * n2 * slices_per_frame,
        "recon_b_tc": 8.0 * n2 * slices_per_frame,
    }
    if name in per_frame:
        return per_frame[name] / max(1, launches)
    per_launch = {"gs_col": 16.0 * n2 + 16.0 * n2, "gs_row_mid": 20.0 * n2, "gs_row_final": 20.0 * n2,
                  "fwd_rows": 16.0 * n2, "spectrum": 8.0 * n2 + 16.0 * n2 + 16.0 * n2}
    return per_launch.get(name)


# ---------------------------------------------------------------- clocks

class ClockSampler:
    """nvidia-smi samples (every 50 ms) of the SM clock and the throttle reasons;
    only the samples taken between mark_start() and mark_end() count."""
    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.t0 = self.t1 = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"ph_clocks_{os.getpid()}.csv"

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        deadline = time.time() + 5.0          # wait for the first sample before the timed region
        while time.time() < deadline and self.path.stat().st_size == 0:
            time.sleep(0.02)

    def mark_start(self):
        self.t0 = time.time()

    def mark_end(self):
        self.t1 = time.time()

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.1)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        from datetime import datetime
        rows = []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 10:
                continue
            try:
                ts = datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                rows.append((ts, float(parts[2]), float(parts[3]),
                             {nm for nm, v in zip(names, parts[6:10]) if v.lower() == "active"}))
            except ValueError:
                continue
        self.path.unlink(missing_ok=True)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        inside = [r for r in rows if self.t0 is not None and self.t1 is not None and self.t0 <= r[0] <= self.t1]
        use = inside or [min(rows, key=lambda r: abs(r[0] - (self.t0 or r[0])))]
        reasons = set().union(*(r[3] for r in use))
        return {"sm_mhz": statistics.median(r[1] for r in use), "sm_max_mhz": max(r[2] for r in use),
                "reasons": sorted(reasons), "samples": len(use), "interval_ms": 50}


# ---------------------------------------------------------------- CPU (oracle) frame sample

def cpu_frame_sample(cfg: dict, h1: np.ndarray, h2: np.ndarray, gs_iters: int, slices: int, outputs=None):
    """Times the oracle on `gs_iters` GS iterations, `slices` slices and one labeling;
    returns (seconds per GS iteration, seconds per slice, seconds per labeling).
    With a dict `outputs`, also stores the oracle's field, projection and argmin there."""
    from oracle import ccl as occl
    from oracle import ref_semantics as ref
    n = cfg["n"]
    d = ref.transfer_sqrt_arr(n, LAM, DX)
    hf, hdz = ref.transfer(-cfg["z0"], n, LAM, d), ref.transfer(-cfg["dz"], n, LAM, d)
    t_it = 0.0
    if cfg["gs_iters"] > 0 and gs_iters > 0:
        tp, tpi = ref.transfer(cfg["gs_sep"], n, LAM, d), ref.transfer(-cfg["gs_sep"], n, LAM, d)
        t = time.perf_counter()
        wf = ref.phase_retrieval_holo(h1, h2, tp, tpi, gs_iters, n)
        t_it = (time.perf_counter() - t) / gs_iters
    else:
        wf = ref.gabor_wavefront(h1)
    t = time.perf_counter()
    proj, arg = ref.reconst_xyprojection(wf, hf, hdz, slices, with_argmin=True)
    t_slice = (time.perf_counter() - t) / slices
    if outputs is not None:
        outputs.update(wf=wf, proj=proj, arg=arg)
    t = time.perf_counter()
    occl.connected_component_labeling((proj <= cfg["threshold"]).astype(np.float32))
    t_ccl = time.perf_counter() - t
    return t_it, t_slice, t_ccl


def cufft_standin(cfg: dict, h1, h2, hf, hdz, hp, hpi, frames: int) -> dict:
    """The reference's kernel sequence re-enacted with torch.fft (cuFFT) and
    one broadcast per step, on the same device buffers: GS as holofunc.jl:100-129
    (fft, fftshift, multiply, ifftshift, ifft, angle, polar per half iteration)
    and the projection as holofunc.jl:248-266 (cumulative X .*= Hdz, ifftshift,
    ifft, x*conj(x), abs, min per slice, host loop).  Not the reference: a
    stand-in for its structure on this GPU.  Labeling is left out (< 0.1 ms)."""
    import torch
    n, S = cfg["n"], cfg["slices"]
    H, Hi, Hf, Hdz = (t.reshape(n, n) for t in (hp, hpi, hf, hdz))
    s1, s2 = torch.sqrt(h1), torch.sqrt(h2)
    fft2, ifft2, fsh, ifsh = torch.fft.fft2, torch.fft.ifft2, torch.fft.fftshift, torch.fft.ifftshift

    def frame():
        if cfg["gs_iters"] > 0:
            u1 = torch.complex(s1, torch.zeros_like(s1))
            for _ in range(cfg["gs_iters"]):
                u2 = ifft2(ifsh(fsh(fft2(u1)) * H))
                u2 = torch.polar(s2, torch.angle(u2))
                u1 = ifft2(ifsh(fsh(fft2(u2)) * Hi))
                u1 = torch.polar(s1, torch.angle(u1))
        else:
            u1 = torch.complex(s1, torch.zeros_like(s1))
        x = fsh(fft2(u1)) * Hf
        proj = torch.full((n, n), float("inf"), device=h1.device)
        for k in range(S):
            if k > 0:
                x = x * Hdz
            img = ifft2(ifsh(x))
            img = torch.abs(img * torch.conj(img)).float()
            proj = torch.minimum(proj, img)
        return proj

    frame()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(frames):
        frame()
    ev1.record()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / frames
    return {"value": round(n * n * S / (ms / 1e3) / 1e6, 2), "unit": "Mvoxel/s", "ms_per_frame": round(ms, 3),
            "frames": frames, "dtype": "c64",
            "what": "cuFFT stand-in of the reference's kernel sequence (torch.fft + one broadcast per step, "
                    "per-slice host loop; GS + projection, labeling excluded), same GPU and inputs"}


def sample_accuracy(ctx, cfg, h1, h2, hp, hpi, hf, hdz, outs, gs_iters, slices, s, form: int = 0) -> dict:
    """Our device path on the CPU baseline's sample (same holograms, GS
    iterations and slices), compared with the oracle outputs of that sample;
    `form` selects the arithmetic of the projection's row pass (PH_FORM_*)."""
    import torch
    from ph_gb300 import _lib
    n = cfg["n"]
    dev = h1.device
    wf = torch.empty((n, n), dtype=torch.complex64, device=dev)
    res = torch.zeros((), dtype=torch.float64, device=dev)
    if gs_iters > 0:
        ctx.call("ph_phase_retrieval", wf.data_ptr(), h1.data_ptr(), h2.data_ptr(), hp.data.data_ptr(),
                 hpi.data.data_ptr(), n, n, gs_iters, res.data_ptr(), s)
    else:
        ctx.call("ph_gabor_wavefront", wf.data_ptr(), h1.data_ptr(), n, n, s)
    proj = torch.empty((n, n), dtype=torch.float32, device=dev)
    arg = torch.empty((n, n), dtype=torch.int32, device=dev)
    ctx.set_option(_lib.PH_OPT_FORM, form)
    try:
        ctx.call("ph_reconst_xyproj", proj.data_ptr(), arg.data_ptr(), wf.data_ptr(), hf.data.data_ptr(),
                 hdz.data.data_ptr(), n, n, slices, s)
        torch.cuda.synchronize()
    finally:
        ctx.set_option(_lib.PH_OPT_FORM, 0)

    w, p, a = wf.cpu().numpy(), proj.cpu().numpy(), arg.cpu().numpy()
    acc = {"against": "oracle FP32 (reference semantics) on the same sample",
           "field_rel_l2": rel_l2(w, outs["wf"]),
           "projection_rel_l2": rel_l2(p, outs["proj"]),
           "argmin_agreement": float(np.mean(a == outs["arg"])),
           "tolerance": {"rel_l2": 1e-4, "argmin_agreement": 0.999}}
    acc["vs_fp64"] = fp64_accuracy(cfg, h1.cpu().numpy(), h2.cpu().numpy(), w, p, a, gs_iters, slices)
    if gs_iters > 0:
        acc["vs_fp64"]["gs_residual"] = float(res.item())   # this path's, FP64-accumulated on the device
    return acc


def rel_l2(a, b) -> float:
    a, b = np.asarray(a, dtype=np.complex128), np.asarray(b, dtype=np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def fp64_accuracy(cfg, h1: np.ndarray, h2: np.ndarray, wf, proj, arg, gs_iters: int, slices: int) -> dict:
    """The same sample against the exact-physics FP64 oracle (complex128, the
    transfer's square root in FP64): what the FP32 path, with the reference's
    own Float32 transfer arithmetic, gives up against the physics."""
    from oracle import fp64 as o64
    out = {}
    if gs_iters > 0:
        wf64, out["gs_residual_fp64"] = o64.phase_retrieval_fp64(h1, h2, cfg["gs_sep"], gs_iters, LAM, DX,
                                                                return_residual=True)
    else:
        wf64 = np.sqrt(np.asarray(h1, dtype=np.float64)).astype(np.complex128)
    p64, a64 = o64.reconst_xyprojection_fp64(wf64, cfg["z0"], cfg["dz"], slices, LAM, DX, with_argmin=True)
    lit = np.abs(wf64) > 0.05   # phases where the field has amplitude
    ph = np.abs(np.exp(1j * np.angle(wf)) - np.exp(1j * np.angle(wf64)))[lit]
    out.update({"against": "oracle FP64 (exact physics) on the same sample",
                "field_rel_l2": rel_l2(wf, wf64),
                "projection_rel_l2": rel_l2(proj, p64),
                "argmin_agreement": float(np.mean(arg == a64)),
                "phase_rms_rad": float(np.sqrt(np.mean(ph ** 2))) if ph.size else 0.0})
    return out


def cpu_mvoxel_per_s(cfg, t_it, t_slice, t_ccl) -> float:
    frame = cfg["gs_iters"] * t_it + cfg["slices"] * t_slice + t_ccl
    return cfg["n"] ** 2 * cfg["slices"] / frame / 1e6


# ---------------------------------------------------------------- main

def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)   # ~0.8 s timed: enough 50 ms clock samples
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c2", choices=sorted(CONFIGS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-profile", action="store_true")
    ap.add_argument("--no-standin", action="store_true", help="skip the cuFFT stand-in of the reference sequence")
    ap.add_argument("--no-forms", action="store_true", help="skip the tensor-core forms of the row pass")
    ap.add_argument("--no-extras", action="store_true", help="skip the brief batch (C4) and serving (C5) runs")
    ap.add_argument("--shard", default="replica", choices=["replica", "depth"],
                    help="replica: one frame per GPU; depth: one frame's slices split over the GPUs")
    ap.add_argument("--form", default="fp32", choices=["fp32", "bf16x3", "fp16x3", "fp16x2"],
                    help="arithmetic of the projection's row pass in the timed frames")
    args = ap.parse_args()
    cfg = CONFIGS[args.config]

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        return reference_arm(args, cfg, rank, world)
    if cfg.get("kind") == "batch":
        return batch_main(args, cfg, rank, world, local)
    if cfg.get("kind") == "serve":
        return serve_main(args, cfg, rank, world, local)

    import torch
    import torch.distributed as dist
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device(f"cuda:{local}")

    import __graft_entry__ as g
    ph = g.load_package()
    from ph_gb300 import _lib, synth

    n, S = cfg["n"], cfg["slices"]
    ctx = _lib.default_context(local)
    # ---- inputs (seeded, synthesised on the device, then kept on the host too)
    spec = synth.HologramSpec(seed=cfg["seed"] + 1000 * rank, n=n, count=cfg["discs"], dmin=cfg["dmin"],
                              dmax=cfg["dmax"], zmin=cfg["zmin"], zmax=cfg["zmax"], wavlen=LAM, dx=DX)
    if cfg["gs_iters"] > 0:
        h1, h2 = synth.synth_pair(spec, cfg["gs_sep"], local)
    else:
        h1 = synth.synth_hologram(spec, local)
        h2 = h1
    d_sqr = ph.cu_transfer_sqrt_arr(n, LAM, DX, device=local)
    hf = ph.cu_transfer(-cfg["z0"], n, LAM, d_sqr)
    hdz = ph.cu_transfer(-cfg["dz"], n, LAM, d_sqr)
    hp = ph.cu_transfer(cfg["gs_sep"], n, LAM, d_sqr)
    hpi = ph.cu_transfer(-cfg["gs_sep"], n, LAM, d_sqr)
    h1_host = torch.empty(h1.shape, dtype=torch.float32, pin_memory=True)
    h2_host = torch.empty(h2.shape, dtype=torch.float32, pin_memory=True)
    h1_host.copy_(h1)
    h2_host.copy_(h2)
    proj_host = torch.empty((n, n), dtype=torch.float32, pin_memory=True)
    arg_host = torch.empty((n, n), dtype=torch.int32, pin_memory=True)
    wf = torch.empty((n, n), dtype=torch.complex64, device=dev)
    proj = torch.empty((n, n), dtype=torch.float32, device=dev)
    arg = torch.empty((n, n), dtype=torch.int32, device=dev)
    binary = torch.empty((n, n), dtype=torch.uint8, device=dev)
    labels = torch.empty((n, n), dtype=torch.int32, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    s = stream.cuda_stream

    depth = args.shard == "depth"
    if depth:
        # one frame over the ranks: GS replicated (each rank needs the whole field), the
        # slices split into contiguous ranges with global indices, packed words merged
        from ph_gb300 import parallel
        k0, k1 = parallel.shard_range(S, rank, world)
        packed = torch.empty((n, n), dtype=torch.int64, device=dev)

    def frame(in1, in2):
        if cfg["gs_iters"] > 0:
            ctx.call("ph_phase_retrieval", wf.data_ptr(), in1.data_ptr(), in2.data_ptr(), hp.data.data_ptr(),
                     hpi.data.data_ptr(), n, n, cfg["gs_iters"], None, s)
        else:
            ctx.call("ph_gabor_wavefront", wf.data_ptr(), in1.data_ptr(), n, n, s)
        if depth:
            ctx.call("ph_reconst_xyproj_range", packed.data_ptr(), wf.data_ptr(), hf.data.data_ptr(),
                     hdz.data.data_ptr(), n, n, k0, k1, 0, s)
            if world > 1:
                dist.all_reduce(packed, op=dist.ReduceOp.MIN)
            ctx.call("ph_unpack_projection", proj.data_ptr(), arg.data_ptr(), packed.data_ptr(), n, n, s)
        else:
            ctx.call("ph_reconst_xyproj", proj.data_ptr(), arg.data_ptr(), wf.data_ptr(), hf.data.data_ptr(),
                     hdz.data.data_ptr(), n, n, S, s)
        ctx.call("ph_binarize_le", binary.data_ptr(), proj.data_ptr(), n * n, float(cfg["threshold"]), s)
        ctx.call("ph_ccl", labels.data_ptr(), binary.data_ptr(), _lib.PH_BOOL, n, n, s)

    form_code = {"fp32": 0, "bf16x3": 1, "fp16x3": 2, "fp16x2": 3}[args.form]
    ctx.set_option(_lib.PH_OPT_FORM, form_code)

    # ---- device-resident timing
    for _ in range(args.warmup):
        frame(h1, h2)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    clocks.start()
    l0 = ctx.launches
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStart()      # ncu --profile-from-start off captures the timed steps only
    clocks.mark_start()
    for i in range(args.steps):
        flush.zero_()                     # L2 flush, outside the step's events
        ev[i][0].record(stream)
        frame(h1, h2)
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    clocks.mark_end()
    torch.cuda.cudart().cudaProfilerStop()
    launches = ctx.launches - l0
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    # Per-kernel times: the same steps again with the library's per-pass CUDA events
    # (on the launching stream; graph replay is off while they are recorded, so the
    # frame time above is taken without them).
    prof = {}
    prof_steps = min(args.steps, 10)
    if not args.no_profile:
        ctx.set_option(_lib.PH_OPT_PROFILE, 1)
        ctx.profile_report()
        for _ in range(prof_steps):
            flush.zero_()
            frame(h1, h2)
        torch.cuda.synchronize()
        prof = ctx.profile_report()
        ctx.set_option(_lib.PH_OPT_PROFILE, 0)
    total_ms = float(sum(step_ms))
    t = torch.tensor([total_ms], device=dev)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    total_ms = float(t.item())
    voxels = n * n * S
    # replicas: every rank reconstructs its own frame; depth shards: the ranks share one frame
    value = voxels * args.steps * (1 if depth else world) / (total_ms / 1e3) / 1e6

    # ---- end to end through the public API, host buffers
    e2e = None
    if not args.no_e2e:
        d1 = torch.empty_like(h1)
        d2 = torch.empty_like(h2)

        def e2e_frame():
            d1.copy_(h1_host, non_blocking=True)
            d2.copy_(h2_host, non_blocking=True)
            if cfg["gs_iters"] > 0:
                u = ph.cu_phase_retrieval_holo(d1, d2, hp, hpi, cfg["gs_iters"], n)
            else:
                u = ph.cu_gabor_wavefront(d1)
            if depth:
                pk = parallel.reconst_xyprojection_range(u, hf, hdz, k0, k1)
                if world > 1:
                    dist.all_reduce(pk, op=dist.ReduceOp.MIN)
                p, a = parallel.unpack_projection(pk)
            else:
                p, a = ph.cu_get_reconst_xyprojection(u, hf, hdz, S, return_argmin=True)
            ctx.call("ph_binarize_le", binary.data_ptr(), p.data_ptr(), n * n, float(cfg["threshold"]), s)
            lab = ph.cu_connected_component_labeling(binary)
            proj_host.copy_(p, non_blocking=True)
            arg_host.copy_(a, non_blocking=True)
            return ph.count_labels(lab)       # reads the count back (synchronises)

        for _ in range(max(1, args.warmup)):
            e2e_frame()
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        e_ms = []
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ncomp = e2e_frame()
            torch.cuda.synchronize()
            e_ms.append((time.perf_counter() - t0) * 1e3)
        te = torch.tensor([sum(e_ms)], device=dev)
        if world > 1:
            dist.all_reduce(te, op=dist.ReduceOp.MAX)
        e2e = {"value": round(voxels * args.steps * (1 if depth else world) / (float(te.item()) / 1e3) / 1e6, 2),
               "unit": "Mvoxel/s",
               "h2d_bytes_per_step": int(h1.numel() * 4 * (2 if cfg["gs_iters"] > 0 else 1)),
               "d2h_bytes_per_step": int(proj.numel() * 4 + arg.numel() * 4 + 8),
               "p50_frame_ms": round(statistics.median(e_ms), 3),
               "p99_frame_ms": round(float(np.percentile(e_ms, 99)), 3), "components": int(ncomp)}

    standin = None
    if not args.no_standin:
        standin = cufft_standin(cfg, h1, h2, hf.data, hdz.data, hp.data, hpi.data, frames=2)

    if rank != 0:
        if world > 1:
            dist.barrier()
            dist.destroy_process_group()
        return

    # ---- roofline of the dominant kernel (library profiler, live)
    hbm, peak_kind = _peaks()
    kernels = {}
    for name, (cnt, ms) in prof.items():
        b = algorithmic_bytes(name, cfg, cnt, S * prof_steps) if name in ("recon_a", "recon_b", "recon_b_tc") else \
            algorithmic_bytes(name, cfg, cnt, S)
        per_launch_ms = ms / cnt
        gbs = (b / (per_launch_ms / 1e3) / 1e9) if b else None
        kernels[name] = {"launches": cnt, "total_ms": round(ms, 3),
                         "share": round(ms / max(total_ms * prof_steps / args.steps, 1e-9), 4),
                         "ms_per_launch": round(per_launch_ms, 4),
                         "achieved_gbs": round(gbs, 1) if gbs else None,
                         "bytes_per_launch": int(b) if b else None}
    roofline = None
    if kernels:
        dom = max(kernels, key=lambda k: kernels[k]["total_ms"])
        kd = kernels[dom]
        traffic, traffic_src = _traffic_from_profiles(dom, args.config)
        roofline = {"kernel": dom, "bound": "hbm", "achieved": kd["achieved_gbs"], "peak": hbm, "unit": "GB/s",
                    "frac": round(kd["achieved_gbs"] / hbm, 4) if kd["achieved_gbs"] else None,
                    "peak_kind": peak_kind, "traffic": traffic, "bytes_per_launch": kd["bytes_per_launch"],
                    "traffic_source": (f"not measured in this run: ncu DRAM bytes of a smaller launch, scaled to "
                                       f"this launch by the slices it processes ({traffic_src})")
                                      if traffic is not None else None}

    # ---- CPU baseline (oracle, all host cores)
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        h1n, h2n = h1.cpu().numpy(), h2.cpu().numpy()
        outs = {}
        t_it, t_slice, t_ccl = cpu_frame_sample(cfg, h1n, h2n, 2 if cfg["gs_iters"] else 0, 16, outs)
        cpu = {"value": round(cpu_mvoxel_per_s(cfg, t_it, t_slice, t_ccl), 3), "unit": "Mvoxel/s",
               "cores": len(os.sched_getaffinity(0)), "kind": "port",
               "sample": f"oracle FP32 (numpy/scipy.fft workers=all): {2 if cfg['gs_iters'] else 0} GS iterations, "
                         f"16 slices and one labeling at {n}^2, scaled to {cfg['gs_iters']} iterations + {S} slices",
               "accuracy": sample_accuracy(ctx, cfg, h1, h2, hp, hpi, hf, hdz, outs, 2 if cfg["gs_iters"] else 0,
                                           16, s)}

    # ---- the split-precision tensor-core forms of the projection's row pass, same frame
    forms = None
    if not args.no_forms and world == 1 and form_code == 0:
        forms = {"fp32": {"ms_per_frame": round(total_ms / args.steps, 3), "mvoxel_s": round(value, 2),
                          "p99_frame_ms": round(float(np.percentile(step_ms, 99)), 3),
                          "recon_b_ms": kernels.get("recon_b", {}).get("ms_per_launch") if kernels else None}}
        if cpu is not None:
            forms["fp32"]["accuracy"] = _form_accuracy(cpu["accuracy"])
        for name, code in (("bf16x3", _lib.PH_FORM_BF16X3), ("fp16x3", _lib.PH_FORM_FP16X3),
                           ("fp16x2", _lib.PH_FORM_FP16X2)):
            ctx.set_option(_lib.PH_OPT_FORM, code)
            try:
                for _ in range(2):
                    frame(h1, h2)
                torch.cuda.synchronize()
                nf = min(args.steps, 20)
                fev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nf)]
                for i in range(nf):
                    flush.zero_()
                    fev[i][0].record(stream)
                    frame(h1, h2)
                    fev[i][1].record(stream)
                torch.cuda.synchronize()
                fms = [a.elapsed_time(b) for a, b in fev]
                ctx.set_option(_lib.PH_OPT_PROFILE, 1)
                ctx.profile_report()
                for _ in range(3):
                    flush.zero_()
                    frame(h1, h2)
                torch.cuda.synchronize()
                fprof = ctx.profile_report()
                ctx.set_option(_lib.PH_OPT_PROFILE, 0)
            finally:
                ctx.set_option(_lib.PH_OPT_FORM, 0)
            tcb = fprof.get("recon_b_tc")
            forms[name] = {"ms_per_frame": round(statistics.mean(fms), 3),
                           "mvoxel_s": round(voxels / (statistics.mean(fms) / 1e3) / 1e6, 2),
                           "p99_frame_ms": round(float(np.percentile(fms, 99)), 3), "frames": nf,
                           "recon_b_ms": round(tcb[1] / tcb[0], 4) if tcb else None}
            if cpu is not None:
                acc = sample_accuracy(ctx, cfg, h1, h2, hp, hpi, hf, hdz, outs, 2 if cfg["gs_iters"] else 0, 16, s,
                                      form=code)
                forms[name]["accuracy"] = _form_accuracy(acc)
        forms["note"] = ("tensor-core forms replace the projection's row pass (pass B) by two complex DFT GEMMs "
                         "on tcgen05 (FP32 accumulation, hi + lo operands); pass A, GS and labeling stay FP32. "
                         "accuracy: the CPU sample (2 GS iterations, 16 slices) against the FP32 and FP64 oracles")

    # ---- the batch (C4) and serving (C5) workloads, briefly, beside the frame
    c4 = c5 = None
    if not args.no_extras and world == 1 and args.config == "c2":
        ctx.set_option(_lib.PH_OPT_FORM, 0)
        c4 = quick_c4(ph, ctx, local, cfg)
        c5 = quick_c5(ph, ctx, local)

    line = {
        "metric": "reconstructed Mvoxel/s + p99 frame latency, chosen vs plain FP32 form, 1 GB300",
        "value": round(value, 2), "unit": "Mvoxel/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(total_ms / args.steps, 3), "higher_is_better": True,
        "scaling": "strong" if depth else "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded disc holograms generated on the device)",
        "config": {"workload": cfg["workload"], "n": n, "slices": S, "dz_um": cfg["dz"], "z0_um": cfg["z0"],
                   "gs_iterations": cfg["gs_iters"], "discs": cfg["discs"],
                   "form": "fp32-stockham" if form_code == 0 else f"{args.form}-tcgen05 row pass",
                   "l2": "flushed (512 MiB write) before every timed step",
                   "kernel_timing": f"{prof_steps} further steps with per-pass CUDA events on the launching stream "
                                    "(graph replay off); the frame time is taken without them",
                   "parallelism": (f"depth shards x{world} (slice ranges, int64 MIN all-reduce of packed words)"
                                   if depth else f"replicas x{world}" if world > 1 else "single GPU")},
        "p50_frame_ms": round(statistics.median(step_ms), 3),
        "p99_frame_ms": round(float(np.percentile(step_ms, 99)), 3),
        "gpu_launches": int(launches),
        "roofline": roofline,
        "kernels": kernels,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "cufft_standin": standin,
        "forms": forms,
        "c4": c4,
        "c5": c5,
        "clocks": clk,
    }
    print(json.dumps(line))
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


def quick_c4(ph, ctx, local: int, cfg: dict, steps: int = 3) -> dict:
    """The mixed batch (96 holograms of four shapes, own slices and dz each) as a
    planned batch against the plain per-hologram path looped on the host."""
    import torch
    from ph_gb300 import synth
    c4 = CONFIGS["c4"]
    holos, sqr = {}, {}
    for ci, (nx, ny, _) in enumerate(C4_CLASSES):
        spec = synth.HologramSpec(seed=c4["seed"] + 100 * ci, n=nx, n_slow=ny, count=c4["discs"], dmin=c4["dmin"],
                                  dmax=c4["dmax"], zmin=c4["zmin"], zmax=c4["zmax"], wavlen=LAM, dx=DX)
        holos[(nx, ny)] = synth.synth_hologram(spec, local)
        sqr[(nx, ny)] = ph.cu_transfer_sqrt_arr(nx, LAM, DX, device=local, n_slow=ny)
    spec_items = c4_items()
    items = []
    for nx, ny, S, dz in spec_items:
        items.append({"hologram": holos[(nx, ny)], "transfer_front": ph.cu_transfer(-c4["z0"], nx, LAM, sqr[(nx, ny)]),
                      "transfer_dz": ph.cu_transfer(-dz, nx, LAM, sqr[(nx, ny)]), "slices": S})
    voxels = sum(nx * ny * S for nx, ny, S, _ in spec_items)
    batch = ph.ReconBatch(items, lanes=4)
    batch.run()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        batch.run()
    e1.record()
    torch.cuda.synchronize()
    bms = e0.elapsed_time(e1) / steps
    wfs = {k: ph.cu_gabor_wavefront(h) for k, h in holos.items()}

    def looped():
        for it, (nx, ny, S, _) in zip(items, spec_items):
            ph.cu_get_reconst_xyprojection(wfs[(nx, ny)], it["transfer_front"], it["transfer_dz"], S,
                                           return_argmin=True)
    looped()
    torch.cuda.synchronize()
    e0.record()
    looped()
    e1.record()
    torch.cuda.synchronize()
    lms = e0.elapsed_time(e1)
    batch.close()
    return {"workload": c4["workload"], "items": len(items), "voxels": voxels, "batch_ms": round(bms, 3),
            "mvoxel_s": round(voxels / (bms / 1e3) / 1e6, 2), "looped_plain_ms": round(lms, 3),
            "looped_plain_mvoxel_s": round(voxels / (lms / 1e3) / 1e6, 2), "speedup_vs_looped": round(lms / bms, 3),
            "what": "ph_batch_plan graph over 4 lanes vs a host loop of single ph_reconst_xyproj calls (each "
                    "with its own wavefront); device-resident, CUDA events, L2 not flushed between items"}


def quick_c5(ph, ctx, local: int, loads=(0.5, 0.9, 1.1), nreq: int = 30) -> dict:
    """Serving under an HBM budget: capacity from a saturated queue, then
    Poisson arrivals at fractions of it; latency = submission to completion."""
    import torch
    from ph_gb300 import synth
    c5 = CONFIGS["c5"]
    dev = torch.device(f"cuda:{local}")
    holos, ring = {}, {}
    for n, S, *_ in C5_MIX:
        spec = synth.HologramSpec(seed=c5["seed"] + n, n=n, count=c5["discs"], dmin=c5["dmin"], dmax=c5["dmax"],
                                  zmin=c5["zmin"], zmax=c5["zmax"], wavlen=LAM, dx=DX)
        holos[n] = synth.synth_hologram(spec, local)
        ring[n] = [(torch.empty((n, n), dtype=torch.float32, device=dev),
                    torch.empty((n, n), dtype=torch.int32, device=dev)) for _ in range(8)]
    budget = 60 << 30
    srv = ph.Server(max_shape=(2048, 2048), max_slices=512, lanes=8, budget_bytes=budget)
    pick = [0]

    def submit(kind):
        n, S, z0, dz, _ = C5_MIX[kind]
        p, a = ring[n][pick[0] % 8]
        pick[0] += 1
        return srv.submit(holos[n], p, S, z0, dz, LAM, DX, argmin=a), n * n * S

    def mix(i):
        return 0 if np.random.default_rng(5000 + i).random() < C5_MIX[0][4] else 1

    for i in range(4):
        srv.poll(submit(i % 2)[0], wait=True)
    alone = {}
    for kind in (0, 1):
        lat = [srv.poll(submit(kind)[0], wait=True) for _ in range(5)]
        alone[f"{C5_MIX[kind][0]}x{C5_MIX[kind][1]}"] = round(float(np.median(lat)), 3)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    clocks.mark_start()
    t0 = time.perf_counter()
    tk, vox = [], 0
    for i in range(3 * nreq):
        t, v = submit(mix(i))
        tk.append(t)
        vox += v
    for t in tk:
        srv.poll(t, wait=True)
    sat = time.perf_counter() - t0
    capacity = 3 * nreq / sat
    rows = []
    for load in loads:
        rng = np.random.default_rng(6000 + int(load * 100))
        arrivals = np.cumsum(rng.exponential(1.0 / (load * capacity), nreq))
        start = time.perf_counter()
        tickets = []
        for i, at in enumerate(arrivals):
            while time.perf_counter() - start < at:
                pass
            tickets.append(submit(mix(10000 + i))[0])
        lat = [srv.poll(t, wait=True) for t in tickets]
        rows.append({"load": load, "offered_req_s": round(load * capacity, 2),
                     "p50_ms": round(float(np.percentile(lat, 50)), 3), "p99_ms": round(float(np.percentile(lat, 99)), 3),
                     "requests": nreq})
    clocks.mark_end()
    clk = clocks.stop()
    st = srv.stats()
    srv.close()
    return {"workload": c5["workload"], "capacity_req_s": round(capacity, 2),
            "capacity_mvoxel_s": round(vox / sat / 1e6, 2), "loads": rows, "alone_p50_ms": alone,
            "budget_bytes": budget, "peak_scratch_bytes": st["bytes_peak"], "requests_queued_at_submit": st["waited"],
            "slots": 8, "clocks": clk,
            "what": "ph_serve_* with admission against a 60 GiB scratch budget, 8 slots; 60 % 1024^2 x 256 / 40 % "
                    "2048^2 x 512 requests, recurring optics (cached transfer functions)"}


def _form_accuracy(acc: dict) -> dict:
    """The figures of one form's sample accuracy that the forms table reports."""
    f64 = acc.get("vs_fp64", {})
    return {"projection_rel_l2_vs_fp32_oracle": acc["projection_rel_l2"],
            "argmin_agreement_vs_fp32_oracle": acc["argmin_agreement"],
            "projection_rel_l2_vs_fp64": f64.get("projection_rel_l2"),
            "argmin_agreement_vs_fp64": f64.get("argmin_agreement")}


def _traffic_from_profiles(kernel: str, config: str):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, if any
    (lines ``traffic <kernel> <config> <bytes_per_launch>`` in profiles/*.md),
    and the summary's file name."""
    for f in sorted((ROOT / "profiles").glob("*.md")):
        for line in f.read_text().splitlines():
            parts = line.strip().strip("`").split()
            if len(parts) == 4 and parts[0] == "traffic" and parts[1] == kernel and parts[2] == config:
                try:
                    return float(parts[3]), f"profiles/{f.name}"
                except ValueError:
                    pass
    return None, None


def batch_main(args, cfg, rank, world, local):
    """The mixed batch (C4) through ph_batch_plan / ph_batch_run: 96 holograms of
    four sizes, each with its own slice count and dz, as one graph launch per step."""
    import torch
    import torch.distributed as dist
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device(f"cuda:{local}")
    import __graft_entry__ as g
    ph = g.load_package()
    from ph_gb300 import _lib, synth
    ctx = _lib.default_context(local)
    items_spec = c4_items()
    holos, sqr, host = {}, {}, {}
    for ci, (nx, ny, _) in enumerate(C4_CLASSES):
        spec = synth.HologramSpec(seed=cfg["seed"] + 100 * ci + 1000 * rank, n=nx, n_slow=ny, count=cfg["discs"],
                                  dmin=cfg["dmin"], dmax=cfg["dmax"], zmin=cfg["zmin"], zmax=cfg["zmax"],
                                  wavlen=LAM, dx=DX)
        holos[(nx, ny)] = synth.synth_hologram(spec, local)
        host[(nx, ny)] = torch.empty((ny, nx), dtype=torch.float32, pin_memory=True)
        host[(nx, ny)].copy_(holos[(nx, ny)])
        sqr[(nx, ny)] = ph.cu_transfer_sqrt_arr(nx, LAM, DX, device=local, n_slow=ny)
    items = []
    for nx, ny, S, dz in items_spec:
        hf, hdz = ph.cu_transfer(-cfg["z0"], nx, LAM, sqr[(nx, ny)]), ph.cu_transfer(-dz, nx, LAM, sqr[(nx, ny)])
        items.append({"hologram": holos[(nx, ny)], "transfer_front": hf, "transfer_dz": hdz, "slices": S})
    voxels = sum(nx * ny * S for nx, ny, S, _ in items_spec)
    batch = ph.ReconBatch(items, lanes=4)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    for _ in range(args.warmup):
        batch.run()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    clocks.start()
    l0 = ctx.launches
    clocks.mark_start()
    for i in range(args.steps):
        flush.zero_()
        ev[i][0].record(stream)
        batch.run()
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    clocks.mark_end()
    launches = ctx.launches - l0
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    t = torch.tensor([sum(step_ms)], device=dev)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    total_ms = float(t.item())
    value = voxels * args.steps * world / (total_ms / 1e3) / 1e6

    e2e = None
    if not args.no_e2e:
        outs_host = [torch.empty(p.shape, dtype=torch.float32, pin_memory=True) for p in batch.proj]

        def e2e_step():
            for k in holos:
                holos[k].copy_(host[k], non_blocking=True)
            proj, _ = batch.run()
            for o, p in zip(outs_host, proj):
                o.copy_(p, non_blocking=True)
            torch.cuda.synchronize()

        e2e_step()
        e_ms = []
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            e2e_step()
            e_ms.append((time.perf_counter() - t0) * 1e3)
        e2e = {"value": round(voxels * args.steps / (sum(e_ms) / 1e3) / 1e6, 2), "unit": "Mvoxel/s",
               "h2d_bytes_per_step": int(sum(h.numel() * 4 for h in host.values())),
               "d2h_bytes_per_step": int(sum(o.numel() * 4 for o in outs_host)),
               "p50_batch_ms": round(statistics.median(e_ms), 3), "p99_batch_ms": round(float(np.percentile(e_ms, 99)), 3)}

    standin = None
    if not args.no_standin:
        fft2, ifft2, fsh, ifsh = torch.fft.fft2, torch.fft.ifft2, torch.fft.fftshift, torch.fft.ifftshift

        def standin_step():
            for it in items:
                h = it["hologram"]
                x = fsh(fft2(torch.complex(torch.sqrt(h), torch.zeros_like(h)))) * it["transfer_front"].data
                proj = torch.full(h.shape, float("inf"), device=dev)
                for k in range(it["slices"]):
                    if k > 0:
                        x = x * it["transfer_dz"].data
                    img = ifft2(ifsh(x))
                    proj = torch.minimum(proj, torch.abs(img * torch.conj(img)).float())
        standin_step()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        standin_step()
        b.record()
        torch.cuda.synchronize()
        sms = a.elapsed_time(b)
        standin = {"value": round(voxels / (sms / 1e3) / 1e6, 2), "unit": "Mvoxel/s", "ms_per_step": round(sms, 3),
                   "what": "cuFFT stand-in of the reference's kernel sequence, one item after another (host loop)"}

    cpu = None
    if not args.no_cpu_baseline and world == 1:
        from oracle import ref_semantics as ref
        secs = 0.0
        for (nx, ny, _) in C4_CLASSES:
            hn = holos[(nx, ny)].cpu().numpy()
            d = ref.transfer_sqrt_arr(nx, LAM, DX, n_slow=ny)
            hf, hdz = ref.transfer(-cfg["z0"], nx, LAM, d), ref.transfer(-200.0, nx, LAM, d)
            t0 = time.perf_counter()
            ref.reconst_xyprojection(ref.gabor_wavefront(hn), hf, hdz, 2)
            per_slice = (time.perf_counter() - t0) / 2
            secs += per_slice * sum(S for x, y, S, _ in items_spec if (x, y) == (nx, ny))
        cpu = {"value": round(voxels / secs / 1e6, 3), "unit": "Mvoxel/s", "cores": len(os.sched_getaffinity(0)),
               "kind": "port", "sample": "oracle FP32 (numpy/scipy.fft workers=all): 2 slices per size class, "
                                         "scaled by each class's total slices"}
    if rank != 0:
        if world > 1:
            dist.barrier()
            dist.destroy_process_group()
        return
    line = {
        "metric": "reconstructed Mvoxel/s + p99 frame latency, chosen vs plain FP32 form, 1 GB300",
        "value": round(value, 2), "unit": "Mvoxel/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(total_ms / args.steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (one seeded disc hologram per size class, shared by the class's items)",
        "config": {"workload": cfg["workload"], "items": len(items_spec), "voxels_per_step": voxels,
                   "lanes": 4, "form": "fp32-stockham", "l2": "flushed (512 MiB write) before every timed step",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
        "p50_frame_ms": round(statistics.median(step_ms), 3),
        "p99_frame_ms": round(float(np.percentile(step_ms, 99)), 3),
        "gpu_launches": int(launches), "roofline": None, "cpu_baseline": cpu, "e2e": e2e,
        "cufft_standin": standin, "clocks": clk,
        "batch_scratch_bytes": batch.scratch_bytes,
    }
    print(json.dumps(line))
    batch.close()
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


def serve_main(args, cfg, rank, world, local):
    """Serving (C5) through ph_serve_*: capacity from a saturated queue, then
    Poisson arrivals at fractions of it; latency = submission to completion."""
    import torch
    torch.cuda.set_device(local)
    dev = torch.device(f"cuda:{local}")
    import __graft_entry__ as g
    ph = g.load_package()
    from ph_gb300 import _lib, synth
    ctx = _lib.default_context(local)
    holos, ring = {}, {}
    for n, S, *_ in C5_MIX:
        spec = synth.HologramSpec(seed=cfg["seed"] + n + 1000 * rank, n=n, count=cfg["discs"], dmin=cfg["dmin"],
                                  dmax=cfg["dmax"], zmin=cfg["zmin"], zmax=cfg["zmax"], wavlen=LAM, dx=DX)
        holos[n] = synth.synth_hologram(spec, local)
        ring[n] = [(torch.empty((n, n), dtype=torch.float32, device=dev),
                    torch.empty((n, n), dtype=torch.int32, device=dev)) for _ in range(16)]
    srv = ph.Server(max_shape=(2048, 2048), max_slices=512, lanes=3)
    pick = [0]

    def submit(kind):
        n, S, z0, dz, _ = C5_MIX[kind]
        p, a = ring[n][pick[0] % 16]
        pick[0] += 1
        return srv.submit(holos[n], p, S, z0, dz, LAM, DX, argmin=a), n * n * S

    def mix(i):
        r = np.random.default_rng(5000 + i).random()
        return 0 if r < C5_MIX[0][4] else 1

    # warm-up (builds the transfer cache and twiddles), then capacity from a saturated queue
    for i in range(max(3, args.warmup) * 2):
        srv.poll(submit(i % 2)[0], wait=True)
    torch.cuda.synchronize()
    nsat = max(20, 4 * args.steps)
    l0 = ctx.launches
    clocks = ClockSampler(local)
    clocks.start()
    clocks.mark_start()
    t0 = time.perf_counter()
    tk, vox = [], 0
    for i in range(nsat):
        t, v = submit(mix(i))
        tk.append(t)
        vox += v
    for t in tk:
        srv.poll(t, wait=True)
    sat_s = time.perf_counter() - t0
    launches = ctx.launches - l0
    capacity = nsat / sat_s
    mean_vox = vox / nsat
    rows = []
    nreq = max(40, 8 * args.steps)
    for load in C5_LOADS:
        rate = load * capacity
        rng = np.random.default_rng(6000 + int(load * 100))
        arrivals = np.cumsum(rng.exponential(1.0 / rate, nreq))
        start = time.perf_counter()
        tickets = []
        for i, at in enumerate(arrivals):
            while time.perf_counter() - start < at:
                pass
            tickets.append(submit(mix(10000 + i))[0])
        lat = [srv.poll(t, wait=True) for t in tickets]
        span = time.perf_counter() - start
        rows.append({"load": load, "offered_req_s": round(rate, 2), "achieved_req_s": round(nreq / span, 2),
                     "p50_ms": round(float(np.percentile(lat, 50)), 3), "p99_ms": round(float(np.percentile(lat, 99)), 3),
                     "requests": nreq})
    clocks.mark_end()
    clk = clocks.stop()
    srv.close()
    p99_09 = next(r["p99_ms"] for r in rows if r["load"] == 0.9)
    line = {
        "metric": "reconstructed Mvoxel/s + p99 frame latency, chosen vs plain FP32 form, 1 GB300",
        "value": round(capacity * mean_vox / 1e6, 2), "unit": "Mvoxel/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1e3 / capacity, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (one seeded disc hologram per size, shared by its requests)",
        "config": {"workload": cfg["workload"], "lanes": 3, "capacity_req_s": round(capacity, 2),
                   "saturated_requests": nsat, "form": "fp32-stockham",
                   "l2": "inputs larger than L2 per request (2048^2 x 512: 16 GiB of slice intermediates, in 2 GiB lane batches)",
                   "parallelism": "single GPU"},
        "p99_frame_ms": p99_09, "serving": rows, "gpu_launches": int(launches), "roofline": None,
        "cpu_baseline": None, "e2e": None, "clocks": clk,
    }
    print(json.dumps(line))


def reference_arm(args, cfg, rank, world):
    """The reference's CPU path (the oracle port, all host cores) on a bounded
    sample of the same frame; only rank 0 runs."""
    if rank != 0:
        return
    n = cfg["n"]
    from oracle import fp64 as o64
    h1 = o64.synth_hologram(cfg["seed"], min(n, 256), 20, cfg["dmin"], cfg["dmax"], cfg["zmin"], cfg["zmax"])
    # the sample runs at the full frame size on a tiled stand-in hologram of the same statistics
    reps = n // h1.shape[0]
    h1 = np.tile(h1, (reps, reps)).astype(np.float32)
    h2 = np.roll(h1, 3, axis=1)
    gs_it = 1 if cfg["gs_iters"] else 0
    vals, step_ms = [], []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        t_it, t_slice, t_ccl = cpu_frame_sample(cfg, h1, h2, gs_it, 2)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            vals.append(cpu_mvoxel_per_s(cfg, t_it, t_slice, t_ccl))
            step_ms.append(dt * 1e3)
    v = float(statistics.mean(vals))
    frame_ms = cfg["n"] ** 2 * cfg["slices"] / (v * 1e6) * 1e3
    cores = len(os.sched_getaffinity(0))
    sample = (f"per step: {gs_it} GS iteration(s), 2 slices and one labeling at {n}^2 "
              f"(oracle FP32, scipy.fft workers={cores}); value = full-frame Mvoxel/s from those timed costs "
              f"({cfg['gs_iters']} iterations + {cfg['slices']} slices + one labeling)")
    line = {
        "metric": "reconstructed Mvoxel/s + p99 frame latency, chosen vs plain FP32 form, 1 GB300",
        "value": round(v, 3), "unit": "Mvoxel/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        # the wall time of one timed sample step (what ran), not of a whole frame
        "ms_per_step": round(statistics.mean(step_ms), 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
        "config": {"workload": cfg["workload"], "n": n, "slices": cfg["slices"], "gs_iterations": cfg["gs_iters"],
                   "step": "a bounded sample of the frame (see cpu_baseline.sample)",
                   "frame_ms_extrapolated": round(frame_ms, 1)},
        "cpu_baseline": {"value": round(v, 3), "unit": "Mvoxel/s", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(v, 3), "unit": "Mvoxel/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
