#!/usr/bin/env python3
"""Benchmark of the enblend/enfuse multiresolution path on GB300.

Default workload: enblend's two-image pyramid blend of 2 x 4096x3072 RGBA
uint16 images offset by 2867 px (union canvas 6963x3072, 10 levels) under a
random-walk seam mask, synthetic and seeded.  Metric: Mpx*exposures/s, the
input pixels blended per second (2 x 4096 x 3072 = 25.17 Mpx per step).

  value  device-resident inputs, one enb_enblend call per step (CUDA events
         on the library's stream, which is torch's current stream)
  e2e    the same call with pinned host buffers: host->device copies of both
         images and the mask, the blend, device->host copies of the image
         and its alpha, every step
  roofline  the dominant kernel from the library's per-launch CUDA-event
         profile: algorithmic bytes / device time, against the measured HBM
         copy bandwidth
  cpu_baseline  the CPU oracle (a port of the reference's algorithm: serial
         pyramids, OpenMP pointwise steps) on a quarter of the rows

  adjoint  one step of the differentiable fuse (8 x 2048x2048 FP32):
         forward, loss and all gradients through enb_fuse_grad
  batched_fuse  the batched uneven-stack workload (64 FP32 stacks of
         uneven sizes and exposure counts): enb_fuse_stacks replayed as one
         CUDA graph against the plain per-stack path on the same GPU
  enfuse_small / enfuse_large  enfuse of 3 x 1024x768 RGB u8 and of
         9 x 6000x4000 RGB u16 (contrast and entropy 5x5 windows) through the
         fused integer driver: value, e2e, roofline, kernels, CPU oracle

--impl reference times that CPU implementation alone on the same metric.
Multi-GPU runs are independent replicas (the path does not shard): each rank
blends its own copy, value = total Mpx / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

REPO = Path(__file__).resolve().parent
for _p in (REPO, REPO / "enblend-enfuse_gb300"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

import numpy as np  # noqa: E402

WORKLOAD = "enblend 2x4096x3072 RGBA u16, offset 2867 (union 6963x3072), 10 levels"
H, W, OFFSET = 3072, 4096, 2867
UNITS = 2 * W * H / 1e6              # Mpx*exposures per step
CPU_ROWS = 768                       # bounded CPU sample: a quarter of the rows
METRIC = "Mpx*exposures/s"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-only", action="store_true",
                    help="run warmup + steps on device inputs only (for ncu launch lists)")
    ap.add_argument("--rows", type=int, default=H,
                    help="with --profile-only: scene height (a smaller case of the same workload for ncu)")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the batched uneven-stack measurement (batched_fuse object)")
    ap.add_argument("--batched-stacks", type=int, default=64)
    ap.add_argument("--no-adjoint", action="store_true", help="skip the differentiable-fuse step (adjoint object)")
    ap.add_argument("--no-enfuse", action="store_true",
                    help="skip the enfuse workloads (enfuse_small: 3x1024x768 u8, enfuse_large: 9x6000x4000 u16)")
    ap.add_argument("--profile-batched", action="store_true",
                    help="run only a small batched fuse (4 stacks of 5 FP32 1024x768 exposures, every level above 0 "
                         "in the coarse kernel, no graph): the case of the batched kernels' ncu capture")
    ap.add_argument("--profile-adjoint", action="store_true",
                    help="one differentiable-fuse step on 8 x 1536x1536 (an ncu capture case)")
    ap.add_argument("--profile-enfuse", action="store_true",
                    help="run only two fused enfuse calls on 9 x 1500x1000 RGB u16 with the 9 x 6000x4000 "
                         "workload's generator and weights: the case of the fused enfuse kernels' ncu captures")
    ap.add_argument("--plain", action="store_true",
                    help="with --profile-only: the reference's pass structure instead of the fused passes")
    return ap.parse_args()


# --------------------------------------------------------------------------
# clocks sampled during the timed region
# --------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu, self.rows, self.proc, self.thread = gpu, [], None, None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "50", "-i", str(self.gpu)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except OSError:
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append((time.time(), [x.strip() for x in line.split(",")]))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)

    def summary(self, t0: float, t1: float) -> dict:
        inside = [r for t, r in self.rows if t0 <= t <= t1 + 0.05]
        note = "sampled during the timed region"
        if not inside:
            # the region is shorter than the sampling interval: nearest samples
            inside = [r for t, r in self.rows if t0 - 0.5 <= t <= t1 + 0.5]
            note = "timed region shorter than the 50 ms sampling interval; samples within 0.5 s of it"
        if not inside:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "note": "nvidia-smi unavailable"}
        sm = [float(r[2]) for r in inside if r[2].replace(".", "").isdigit()]
        mx = [float(r[3]) for r in inside if r[3].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in inside:
            for n, v in zip(names, r[6:10]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(inside), "note": note}


# --------------------------------------------------------------------------
# helpers
# --------------------------------------------------------------------------

def measured_peaks() -> dict:
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d.get("hbm_gbs"), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def ncu_traffic() -> dict:
    """Per-launch DRAM bytes of each kernel from the committed ncu summary, if any."""
    p = REPO / "profiles" / "traffic_enblend_2x4096x3072_u16.txt"
    out = {}
    if p.exists():
        for line in p.read_text().splitlines():
            parts = line.split()
            if len(parts) == 2 and not line.startswith("#"):
                try:
                    out[parts[0]] = float(parts[1])
                except ValueError:
                    pass
    return out


def make_inputs(seed: int, rows: int = H):
    from enbgpu import synthetic
    return synthetic.panorama_pair(rows, W, OFFSET, np.uint16, seed)


def cpu_oracle_rate(seed: int, repeats: int = 3) -> dict:
    """Time the CPU oracle on the bounded sample (rows 0..CPU_ROWS of the scene)."""
    from oracle import oracle
    white, black, mask = make_inputs(seed, CPU_ROWS)
    oracle.enblend(white, black, mask)  # warm (builds, pages in)
    times = []
    for _ in range(repeats):
        t = time.perf_counter()
        oracle.enblend(white, black, mask)
        times.append(time.perf_counter() - t)
    units = 2 * W * CPU_ROWS / 1e6
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": units / statistics.median(times), "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"2 x 4096x{CPU_ROWS} RGBA u16 (quarter of the rows of the workload), median of {repeats}; "
                      f"serial pyramid passes and OpenMP pointwise passes as in the reference"}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(ms: float, ws: int, device: str = "cuda") -> float:
    """The job's time: the slowest rank's (all_reduce MAX over the process group)."""
    if ws <= 1:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_value(units_per_rank: float, ws: int, steps: int, ms: float) -> float:
    """Whole-job throughput of ws independent replicas (weak scaling): every
    rank's units over the slowest rank's time."""
    return ws * units_per_rank * steps / (ms / 1e3)


# --------------------------------------------------------------------------
# arms
# --------------------------------------------------------------------------

def workload_config(levels: int, ws: int) -> dict:
    """The `config` of both arms' lines: the enblend workload (the reference
    arm times a bounded sample of it, named in its cpu_baseline)."""
    return {"workload": WORKLOAD, "levels": levels, "pixel": "RGBA u16",
            "pyramid": "int32 17.7 fixed point, mask int32 9.15", "parallelism": f"replicas x{ws}",
            "l2": "inputs larger than L2 (each image 171 MB)",
            "device_layout": "rows padded to 128-byte boundaries (enbgpu.pitched), as the host-buffer "
                             "path stages them"}


def run_reference(args) -> None:
    ws, rank, _ = dist_setup()
    if rank != 0:
        return
    from oracle import oracle
    white, black, mask = make_inputs(args.seed, CPU_ROWS)
    units = 2 * W * CPU_ROWS / 1e6
    for _ in range(args.warmup):
        oracle.enblend(white, black, mask)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.enblend(white, black, mask)
    dt = time.perf_counter() - t0
    value = units * args.steps / dt
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": workload_config(oracle.num_levels(W + OFFSET, H), ws),
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
                         "sample": f"each step: 2 x 4096x{CPU_ROWS} RGBA u16 (a quarter of the rows)"},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def batched_fuse(ctx, stream, n_stacks: int, reps: int = 3) -> dict:
    """The batched uneven-stack workload: n FP32 RGB stacks, width and height
    log-uniform in [512, 4096], 3..7 exposures, EVs evenly spaced over
    +-(count - 1) stops, weights exposure 1.0 / saturation 0.2 / contrast 0.5
    (5x5) / entropy 0.3 (5x5) in normalised-float mode; enb_fuse_stacks (one
    CUDA graph, level schedule from enb_fuse_stacks_tune) against the plain
    per-stack path (enb_enfuse per stack) on the same GPU, device-resident
    inputs."""
    import torch
    import enbgpu
    from enbgpu import synthetic
    specs = synthetic.uneven_stack_specs(n_stacks)
    stacks = synthetic.uneven_stacks_torch(specs)
    outs = [st[0].new_zeros(st[0].shape) for st in stacks]
    units = sum(len(st) * st[0].shape[0] * st[0].shape[1] for st in stacks) / 1e6
    prm = enbgpu.enfuse_params(saturation_weight=0.2, contrast_weight=0.5, entropy_weight=0.3,
                               contrast_window_size=5, entropy_window_size=5, float_range=1.0)

    def timed(fn, n):
        fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(n):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / n

    # the level schedule (coarse threshold) from measured times; the timed
    # calls below use it (coarse_pixels=0)
    tune = ctx.tune_stacks(stacks, params=prm, outs=outs, reps=2)
    l0 = ctx.launches
    batched_ms = timed(lambda: ctx.fuse_stacks(stacks, params=prm, outs=outs), reps)
    launches = (ctx.launches - l0) // (reps + 1)
    ref = [o.clone() for o in outs]
    plain_ms = timed(lambda: ctx.fuse_stacks(stacks, params=prm, outs=outs, plain=True), max(1, reps - 1))
    max_rel = max(float(((o - r).abs() / (r.abs() + 1e-6)).max()) for o, r in zip(outs, ref))
    ctx.profile(True)
    ctx.fuse_stacks(stacks, params=prm, outs=outs, graph=False)
    kb = ctx.profile_report()
    ctx.profile(False)
    ctx.profile(True)
    ctx.fuse_stacks(stacks, params=prm, outs=outs, plain=True)
    kp = ctx.profile_report()
    ctx.profile(False)
    weights_b, weights_p = kb["batch_weights"]["ms"], kp["f_enfuse_mask"]["ms"]
    return {
        "workload": f"{n_stacks} FP32 RGB stacks, W,H log-uniform [512,4096], 3..7 exposures, "
                    "weights exposure 1.0 / saturation 0.2 / contrast 0.5 (5x5) / entropy 0.3 (5x5), "
                    "normalised-float mode (float_range 1.0)",
        "units": units, "metric": METRIC,
        "batched": {"value": units / (batched_ms / 1e3), "ms_per_step": batched_ms, "graph": True,
                    "launches_per_step": launches, "coarse_pixels": tune["best"],
                    "tuned_ms": {str(k): round(v, 3) for k, v in tune["ms"].items()}},
        "plain": {"value": units / (plain_ms / 1e3), "ms_per_step": plain_ms,
                  "what": "enb_enfuse stack by stack (the per-stack path)"},
        "speedup": plain_ms / batched_ms,
        "weights_ms": {"batched": weights_b, "plain": weights_p},
        "excluding_weights_ms": {"batched": batched_ms - weights_b, "plain": plain_ms - weights_p,
                                 "speedup": (plain_ms - weights_p) / max(batched_ms - weights_b, 1e-9)},
        "batched_kernels": {k: {"launches": v["launches"], "ms": v["ms"],
                                "GBps": v["bytes"] / (v["ms"] / 1e3) / 1e9 if v["ms"] > 0 and v["bytes"] else None}
                            for k, v in kb.items()},
        "max_rel_diff_vs_plain": max_rel,
    }


# The enfuse workloads: 3 x 1024x768 RGB u8 (EV -2, 0, +2; exposure 1.0,
# saturation 0.2) and 9 x 6000x4000 RGB u16 (EV -4..+4, 12-stop scene, sensor
# noise N(0, 2^-12) before quantisation; exposure 1.0, saturation 0.2,
# contrast 0.5 in 5x5 windows, entropy 0.3 in 5x5 windows).
ENFUSE_WORKLOADS = {
    "enfuse_3x1024x768_u8": dict(h=768, w=1024, evs=[-2.0, 0.0, 2.0], dtype=np.uint8, stops=8.0, noise=0.0,
                                 kw=dict(saturation_weight=0.2), seed=1, cpu_rows=768, flush=True),
    "enfuse_9x6000x4000_u16": dict(h=4000, w=6000, evs=[float(e) for e in range(-4, 5)], dtype=np.uint16,
                                   stops=12.0, noise=2.0 ** -12,
                                   kw=dict(saturation_weight=0.2, contrast_weight=0.5, entropy_weight=0.3,
                                           contrast_window_size=5, entropy_window_size=5),
                                   seed=3, cpu_rows=96, flush=False),
}


def enfuse_workload(ctx, stream, name: str, steps: int, cpu: bool) -> dict:
    """One enfuse workload through enb_enfuse (the fused integer driver):
    device-resident value with per-step CUDA events (the L2 flushed between
    steps when the inputs fit in it), e2e through the host-buffer entry point
    with pinned memory, the per-kernel profile with the dominant kernel's
    roofline, and the CPU oracle on a bounded sample of the rows."""
    import torch
    import enbgpu
    from enbgpu import synthetic
    sp = ENFUSE_WORKLOADS[name]
    h, w, K = sp["h"], sp["w"], len(sp["evs"])
    imgs = synthetic.exposure_stack_torch(h, w, sp["evs"], sp["dtype"], sp["stops"], sp["seed"], sp["noise"])
    prm = enbgpu.enfuse_params(**sp["kw"])
    out = torch.empty_like(imgs[0])
    oa = torch.empty((h, w), dtype=torch.uint8, device="cuda")
    units = K * h * w / 1e6
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda") if sp["flush"] else None

    def call():
        ctx.enfuse(imgs, params=prm, out=out, out_alpha=oa)

    for _ in range(3):
        call()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    l0 = ctx.launches
    for a, b in ev:
        if flush is not None:
            flush.zero_()   # L2 (129 MB) flushed outside the timed interval
        a.record(stream)
        call()
        b.record(stream)
    torch.cuda.synchronize()
    launches = (ctx.launches - l0) // steps
    ms = sum(a.elapsed_time(b) for a, b in ev) / steps
    # e2e: pinned host buffers, copies inside the call
    pin = lambda t: t.cpu().pin_memory().numpy()  # noqa: E731
    himgs = [pin(x) for x in imgs]
    hout = torch.empty(tuple(out.shape), dtype=out.dtype).pin_memory().numpy()
    hoa = torch.empty((h, w), dtype=torch.uint8).pin_memory().numpy()
    for _ in range(2):
        ctx.enfuse(himgs, params=prm, out=hout, out_alpha=hoa)
    e2e_steps = max(2, min(steps, 5))
    torch.cuda.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(e2e_steps):
        ctx.enfuse(himgs, params=prm, out=hout, out_alpha=hoa)
    f1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = f0.elapsed_time(f1) / e2e_steps
    same = bool(np.array_equal(hout, out.cpu().numpy()))
    # per-kernel profile
    ctx.profile(True)
    for _ in range(2):
        call()
    rep = ctx.profile_report()
    ctx.profile(False)
    total = sum(v["ms"] for v in rep.values())
    dom = max(rep, key=lambda k: rep[k]["ms"])
    d = rep[dom]
    peaks = measured_peaks()
    achieved = d["bytes"] / (d["ms"] / 1e3) / 1e9
    res = {
        "workload": name.replace("enfuse_", "enfuse ").replace("_", " ") + ", weights " +
                    ", ".join(f"{k}={v}" for k, v in sorted(dict(exposure_weight=1.0, **sp["kw"]).items())),
        "units": units, "metric": METRIC, "value": units / (ms / 1e3), "ms_per_step": ms, "steps": steps,
        "l2": "flushed between steps (256 MB write)" if flush is not None else "inputs larger than L2",
        "gpu_launches": launches,
        "e2e": {"value": units / (e2e_ms / 1e3), "unit": METRIC, "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": int(sum(x.nbytes for x in himgs)),
                "d2h_bytes_per_step": int(hout.nbytes + hoa.nbytes), "same_pixels_as_device_run": same},
        "roofline": {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"], "peak_source": peaks["source"],
                     "algorithmic_bytes_per_launch": d["bytes"] / d["launches"],
                     "share_of_device_time": d["ms"] / total if total else None},
        "kernels": {k: {"launches_per_step": v["launches"] / 2, "ms_per_step": v["ms"] / 2,
                        "GBps": v["bytes"] / (v["ms"] / 1e3) / 1e9 if v["ms"] > 0 else None}
                    for k, v in sorted(rep.items(), key=lambda kv: -kv[1]["ms"])},
    }
    if cpu:
        from oracle import oracle
        rows = sp["cpu_rows"]
        sample = [x[:rows].copy() for x in himgs]
        orc_prm = oracle.params(**sp["kw"])
        oracle.enfuse([x[:16].copy() for x in sample], None, orc_prm)  # warm (build, page-in)
        t = time.perf_counter()
        oracle.enfuse(sample, None, orc_prm)
        dt = time.perf_counter() - t
        res["cpu_baseline"] = {"value": K * w * rows / 1e6 / dt, "unit": METRIC,
                               "cores": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1)), "kind": "port",
                               "sample": f"{K} x {w}x{rows} (the first {rows} rows of the workload), one run; serial "
                                         "pyramid passes and OpenMP pointwise passes as in the reference"}
    del imgs, out, oa, flush
    torch.cuda.empty_cache()
    return res


def seam_mask_step(ctx, stream, white, black, reps: int = 5) -> dict:
    """enblend's nearest-feature seam mask (enb_nft_mask) of the benchmark
    pair's footprints on the 6963x3072 canvas, device-resident, CUDA events
    (the call synchronises, so each rep is timed on its own)."""
    import torch
    wa = torch.from_numpy(np.where(white[..., 3] >= 32767, 255, 0).astype(np.uint8)).cuda()
    ba = torch.from_numpy(np.where(black[..., 3] >= 32767, 255, 0).astype(np.uint8)).cuda()
    mask = torch.empty_like(wa)
    ctx.nft_mask(wa, ba, mask=mask)
    times = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ctx.nft_mask(wa, ba, mask=mask)
        b.record(stream)
        torch.cuda.synchronize()
        times.append(a.elapsed_time(b))
    ctx.profile(True)
    ctx.nft_mask(wa, ba, mask=mask)
    rep = ctx.profile_report()
    ctx.profile(False)
    h, w = mask.shape
    return {"workload": f"nearest-feature seam mask of the benchmark pair's footprints, {w}x{h}",
            "ms_per_call": statistics.median(times), "Mpx_per_s": w * h / 1e6 / (statistics.median(times) / 1e3),
            "kernels_ms": {k: round(v["ms"], 3) for k, v in rep.items()}}


def adjoint_step(ctx, stream, reps: int = 3) -> dict:
    """The differentiable fuse: 8 exposures of 2048x2048 FP32 RGB (EV -3.5..+3.5
    in 1-stop steps), loss = mean squared difference to the scene's tone-mapped
    radiance (radiance / (1 + radiance))^(1/2.2); one step = the forward fuse,
    the loss and all gradients (exposure optimum and width, exposure /
    saturation / contrast coefficients, a per-exposure logit map) through
    enb_fuse_grad."""
    import torch
    import enbgpu
    from enbgpu import synthetic
    h = w = 2048
    lr = synthetic.log_radiance_torch(h, w, 8.0, seed=5)
    imgs = [synthetic.expose_torch(lr, ev) for ev in np.arange(-3.5, 3.6, 1.0)]
    rad = torch.exp2(lr)
    target = ((rad / (1.0 + rad)) ** (1.0 / 2.2)).float().contiguous()
    del lr, rad
    logits = [torch.zeros((h, w), device="cuda") for _ in imgs]
    grads = [torch.zeros_like(x) for x in logits]
    prm = enbgpu.enfuse_params(exposure_optimum=0.5, exposure_width=0.2, saturation_weight=0.2, contrast_weight=0.5,
                               contrast_window_size=5, float_range=1.0)
    for _ in range(2):
        r = ctx.fuse_grad(imgs, target, params=prm, logits=logits, grad_logits=grads)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.time()
    a.record(stream)
    for _ in range(reps):
        r = ctx.fuse_grad(imgs, target, params=prm, logits=logits, grad_logits=grads)
    b.record(stream)
    torch.cuda.synchronize()
    host_ms = (time.time() - t0) / reps * 1e3
    ms = a.elapsed_time(b) / reps
    ctx.profile(True)
    ctx.fuse_grad(imgs, target, params=prm, logits=logits, grad_logits=grads)
    rep = ctx.profile_report()
    ctx.profile(False)
    # the dominant kernel against the copy bandwidth, and the step's algorithmic
    # bytes (each launcher's own count) against its time
    dom = max(rep, key=lambda k: rep[k]["ms"])
    d = rep[dom]
    peaks = measured_peaks()
    achieved = d["bytes"] / (d["ms"] / 1e3) / 1e9
    total_bytes = sum(v["bytes"] for v in rep.values())
    return {"workload": "8 x 2048x2048 FP32 RGB, EV -3.5..+3.5, weights exposure 1.0 / saturation 0.2 / "
                        "contrast 0.5 (5x5), per-exposure logit maps", "ms_per_step": ms,
            "host_ms_per_step": host_ms,
            "what": "forward + loss + all gradients (enb_fuse_grad; CUDA events on the call's stream, the call "
                    "reads the loss back each step)",
            "loss": r["loss"], "units": 8 * h * w / 1e6,
            "roofline": {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"],
                         "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"], "peak_source": peaks["source"],
                         "algorithmic_bytes_per_launch": d["bytes"] / d["launches"],
                         "share_of_device_time": d["ms"] / sum(v["ms"] for v in rep.values())},
            "pipeline": {"algorithmic_bytes_per_step": total_bytes, "GBps": total_bytes / (ms / 1e3) / 1e9},
            "kernels": {k: {"launches": v["launches"], "ms": round(v["ms"], 3),
                            "GBps": round(v["bytes"] / (v["ms"] / 1e3) / 1e9, 1) if v["ms"] > 0 else None}
                        for k, v in sorted(rep.items(), key=lambda kv: -kv[1]["ms"])}}


def profile_adjoint() -> None:
    """One differentiable-fuse step on 8 x 1536x1536 FP32 RGB (inputs 226 MB,
    larger than L2), parameters as the adjoint workload's."""
    import torch
    import enbgpu
    from enbgpu import synthetic
    ctx = enbgpu.Context(0)
    h = w = 1536
    lr = synthetic.log_radiance_torch(h, w, 8.0, seed=5)
    imgs = [synthetic.expose_torch(lr, ev) for ev in np.arange(-3.5, 3.6, 1.0)]
    rad = torch.exp2(lr)
    target = ((rad / (1.0 + rad)) ** (1.0 / 2.2)).float().contiguous()
    logits = [torch.zeros((h, w), device="cuda") for _ in imgs]
    grads = [torch.zeros_like(x) for x in logits]
    prm = enbgpu.enfuse_params(exposure_optimum=0.5, exposure_width=0.2, saturation_weight=0.2, contrast_weight=0.5,
                               contrast_window_size=5, float_range=1.0)
    r = ctx.fuse_grad(imgs, target, params=prm, logits=logits, grad_logits=grads)
    torch.cuda.synchronize()
    print("adjoint profile case ok", r["loss"])
    ctx.close()


def run_ours(args) -> None:
    import torch
    import enbgpu

    ws, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    ctx = enbgpu.Context(local)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)

    white, black, mask = make_inputs(args.seed, args.rows if args.profile_only else H)
    # device-resident inputs in the layout the host-buffer path stages into:
    # rows on 128-byte boundaries (the 6963-pixel rows are 55,704 bytes)
    dw, db, dm = (enbgpu.pitched(x) for x in (white, black, mask))
    out = torch.empty(black.shape, dtype=torch.uint16, device="cuda")
    oa = torch.empty(mask.shape, dtype=torch.uint8, device="cuda")

    def step(plain=False, inputs=None):
        w_, b_, m_ = inputs if inputs is not None else (dw, db, dm)
        ctx.enblend(w_, b_, m_, out=out, out_alpha=oa, plain=plain)

    if args.profile_only:
        for _ in range(args.warmup + args.steps):
            step(args.plain)
        torch.cuda.synchronize()
        return
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # ---- device-resident timed region ----
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    launches0 = ctx.launches
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.time()
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    barrier()
    t1 = time.time()
    sampler.stop()
    launches = ctx.launches - launches0
    ms = max_over_ranks(e0.elapsed_time(e1), ws)
    value = replica_value(UNITS, ws, args.steps, ms)

    # ---- the reference's pass structure on the same GPU, for comparison ----
    plain_steps = max(3, min(args.steps, 20))
    step(plain=True)
    barrier()
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    for _ in range(plain_steps):
        step(plain=True)
    p1.record(stream)
    barrier()
    plain_ms = p0.elapsed_time(p1) / plain_steps

    # ---- the same call on dense device rows (55,704-byte pitch, rows not on
    # 16-byte boundaries: level 0 takes the per-thread copy feed) ----
    dense = tuple(torch.from_numpy(x).cuda() for x in (white, black, mask))
    step(inputs=dense)
    barrier()
    q0, q1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    q0.record(stream)
    for _ in range(plain_steps):
        step(inputs=dense)
    q1.record(stream)
    barrier()
    dense_ms = q0.elapsed_time(q1) / plain_steps
    del dense

    # ---- end to end through the host-buffer entry point (pinned memory) ----
    pin = lambda a: torch.from_numpy(a).pin_memory().numpy()  # noqa: E731
    hw, hb, hm = pin(white), pin(black), pin(mask)
    ho = torch.empty(black.shape, dtype=torch.uint16).pin_memory().numpy()
    hoa = torch.empty(mask.shape, dtype=torch.uint8).pin_memory().numpy()
    e2e_steps = max(3, min(args.steps, 20))
    for _ in range(2):
        ctx.enblend(hw, hb, hm, out=ho, out_alpha=hoa)
    barrier()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(e2e_steps):
        ctx.enblend(hw, hb, hm, out=ho, out_alpha=hoa)
    f1.record(stream)
    barrier()
    e2e_ms = max_over_ranks(f0.elapsed_time(f1), ws)
    e2e_value = replica_value(UNITS, ws, e2e_steps, e2e_ms)
    h2d = hw.nbytes + hb.nbytes + hm.nbytes
    d2h = ho.nbytes + hoa.nbytes

    # ---- per-kernel profile (CUDA events per launch) ----
    ctx.profile(True)
    prof_steps = max(3, min(args.steps, 20))
    for _ in range(prof_steps):
        step()
    report = ctx.profile_report()
    ctx.profile(False)
    total_ms = sum(v["ms"] for v in report.values())
    dom = max(report, key=lambda k: report[k]["ms"])
    d = report[dom]
    peaks = measured_peaks()
    achieved = d["bytes"] / (d["ms"] / 1e3) / 1e9
    traffic = ncu_traffic().get(dom)
    per_launch_bytes = d["bytes"] / d["launches"]
    roofline = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"] if peaks["hbm_gbs"] else None,
                "peak_source": peaks["source"], "algorithmic_bytes_per_launch": per_launch_bytes,
                "traffic": traffic, "share_of_device_time": d["ms"] / total_ms if total_ms else None}
    kernels = {k: {"launches_per_step": v["launches"] / prof_steps, "ms_per_step": v["ms"] / prof_steps,
                   "GBps": v["bytes"] / (v["ms"] / 1e3) / 1e9 if v["ms"] > 0 else None}
               for k, v in sorted(report.items(), key=lambda kv: -kv[1]["ms"])}
    pipeline_bytes = sum(v["bytes"] for v in report.values()) / prof_steps

    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": workload_config(enbgpu.num_levels(W + OFFSET, H), ws),
        "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_ms / e2e_steps},
        "plain_passes": {"value": UNITS / (plain_ms / 1e3), "unit": METRIC, "ms_per_step": plain_ms,
                         "what": "same call with one kernel per reference operation (enb_fuse_options.plain)"},
        "dense_rows": {"value": UNITS / (dense_ms / 1e3), "unit": METRIC, "ms_per_step": dense_ms,
                       "what": "same call on unpadded device images (rows not 16-byte aligned)"},
        "gpu_launches": launches,
        "roofline": roofline,
        "kernels": kernels,
        "pipeline": {"algorithmic_bytes_per_step": pipeline_bytes,
                     "GBps": pipeline_bytes / (ms / args.steps / 1e3) / 1e9},
        "clocks": sampler.summary(t0, t1),
    }
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_oracle_rate(args.seed)
    if rank == 0 and ws == 1:
        line["seam_mask"] = seam_mask_step(ctx, stream, white, black)
    if rank == 0 and ws == 1 and not args.no_enfuse:
        del dw, db, dm, out, oa
        torch.cuda.empty_cache()
        line["enfuse_small"] = enfuse_workload(ctx, stream, "enfuse_3x1024x768_u8", 20, not args.no_cpu_baseline)
        line["enfuse_large"] = enfuse_workload(ctx, stream, "enfuse_9x6000x4000_u16", 5, not args.no_cpu_baseline)
    if rank == 0 and ws == 1 and not args.no_batched:
        line["batched_fuse"] = batched_fuse(ctx, stream, args.batched_stacks)
    if rank == 0 and ws == 1 and not args.no_adjoint:
        line["adjoint"] = adjoint_step(ctx, stream)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


def profile_batched() -> None:
    import torch
    import enbgpu
    from enbgpu import synthetic
    ctx = enbgpu.Context(0)
    specs = [(768, 1024, list(np.linspace(-4, 4, 5)), 100 + i) for i in range(4)]
    stacks = synthetic.uneven_stacks_torch(specs)
    prm = enbgpu.enfuse_params(saturation_weight=0.2, contrast_weight=0.5, entropy_weight=0.3,
                               contrast_window_size=5, entropy_window_size=5, float_range=1.0)
    outs = ctx.fuse_stacks(stacks, params=prm, graph=False, coarse_pixels=1 << 30)
    torch.cuda.synchronize()
    print("batched profile case ok", float(outs[0].mean()))
    ctx.close()


def profile_enfuse() -> None:
    """Two fused enfuse calls on 9 x 1500x1000 RGB u16 (EV -4..+4, 12-stop
    scene, noise 2^-12; exposure 1.0, saturation 0.2, contrast 0.5 and
    entropy 0.3 in 5x5 windows): 13.5 Mpx*exposures, inputs 81 MB."""
    import torch
    import enbgpu
    from enbgpu import synthetic
    ctx = enbgpu.Context(0)
    sp = ENFUSE_WORKLOADS["enfuse_9x6000x4000_u16"]
    imgs = synthetic.exposure_stack_torch(1000, 1500, sp["evs"], sp["dtype"], sp["stops"], sp["seed"], sp["noise"])
    prm = enbgpu.enfuse_params(**sp["kw"])
    for _ in range(2):
        out, _ = ctx.enfuse(imgs, params=prm)
    torch.cuda.synchronize()
    print("enfuse profile case ok", float(out.float().mean()))
    ctx.close()


def main():
    args = parse_args()
    if args.profile_batched:
        profile_batched()
        return
    if args.profile_enfuse:
        profile_enfuse()
        return
    if args.profile_adjoint:
        profile_adjoint()
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
