#!/usr/bin/env python
"""Throughput of the projector pair A / A^T on GB300.

Workload (the configuration the headline metric is quoted on): a 512^3
float32 volume x ~ N(0,1) in z_order 0 (SY, SX, H), 192 angles
linspace(0, pi), detector width 512 (the reference's default max(SY, SX)).
One step = y += A x, then x' += A^T y, on device-resident tensors.
Unit of work: one voxel x angle update (VU); a step is 2 * 512^3 * 192 VU.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference operator's CPU evaluation (the FP32
OpenMP restatement in oracle/, all host threads) on a bounded sample of the
same workload.  The reference package has no CPU implementation of its own.

Under torchrun (N > 1) every rank runs its own replica on its own GPU (the
problem does not need a collective); the value is the sum over ranks with
the time taken as the maximum over ranks.

Prints one JSON line.
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
import torch

ROOT = Path(__file__).resolve().parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

METRIC = "GVU/s (voxel×angle) for A and Aᵀ at 512³/192 ang"


def metric_name(args) -> str:
    """The headline metric's name for the headline workload; other sizes and
    angle counts carry their own in the same form."""
    if (args.size, args.angles, heights(args)) == (512, 192, 512):
        return METRIC
    if heights(args) == args.size:
        return f"GVU/s (voxel×angle) for A and Aᵀ at {args.size}³/{args.angles} ang"
    return (f"GVU/s (voxel×angle) for A and Aᵀ at {args.size}²×{heights(args)}/{args.angles} "
            f"ang")
UNIT = "GVU/s"
# The reference's published timing (its README.md:58-59, RTX 3060, z_order 0,
# 512^3, 192 angles, units taken as ms):
# A 516 ms, A^T 397 ms -> 2 * 512^3 * 192 VU / 0.913 s.
PUBLISHED_GVU_S = 2 * 512**3 * 192 / 0.913 / 1e9
L2_BYTES = 129 * 2**20
# The default kernels of each direction at the benchmark sizes.  z_order 2
# with 32 heights or more runs the z_order 0 kernels between two tiled
# transposes (transpose_kernel).
KERNELS = {("A", 0): "fp_z0_kernel", ("AT", 0): "bp_z0_runs_kernel",
           ("A", 2): "fp_z0_kernel", ("AT", 2): "bp_z0_runs_kernel"}


def parse_args():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawTextHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--size", type=int, default=512)
    ap.add_argument("--height", type=int, default=0,
                    help="volume heights (0: as --size, a cube)")
    ap.add_argument("--angles", type=int, default=192)
    ap.add_argument("--z-order", type=int, default=0, choices=[0, 2])
    ap.add_argument("--trig", choices=["reference", "precise"], default="reference")
    ap.add_argument("--variant-fwd", type=int, default=0,
                    help="kernel variant for A (0 = library default)")
    ap.add_argument("--variant-bwd", type=int, default=0,
                    help="kernel variant for A^T (0 = library default)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0,
                    help="target CPU work for the CPU-baseline sample")
    return ap.parse_args()


# ----------------------------------------------------------------- helpers --

def dist_info():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(value: float, world: int, device) -> float:
    """The largest per-rank value over all ranks: a job's time is its slowest
    rank's.  Needs the default process group when world > 1."""
    if world <= 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def whole_job_gvu_s(world: int, steps: int, vu_step: float, total_ms: float) -> float:
    """Voxel-angle updates of all ranks / the slowest rank's time, in GVU/s.
    Replicas: every rank runs its own problem of vu_step updates per step."""
    return world * steps * vu_step / (total_ms / 1e3) / 1e9


def heights(args) -> int:
    return getattr(args, "height", 0) or args.size


def shapes(S, n, z, H=None):
    """x and y shapes of an S x S volume of H heights (a cube by default)."""
    H = S if H is None else H
    xs = (S, S, H) if z == 0 else (H, S, S)
    ys = (n, S, H) if z == 0 else (H, n, S)
    return xs, ys


def algorithmic_bytes(S, n, PX, H=None):
    H = S if H is None else H
    vol = S * S * H * 4
    sino = n * PX * H * 4
    return {"A": vol + 2 * sino, "AT": sino + 2 * vol}


def weights_nnz(S, n, PX, angles):
    """Exact number of nonzero (voxel, angle, bin) weights that land on the
    detector (FP64), i.e. the algorithmic multiply-adds per height."""
    c0 = 0.5 * (S - 1)
    pc = 0.5 * (PX - 1)
    t = np.arange(S, dtype=np.float64) - c0
    total = 0
    for phi in np.asarray(angles, np.float32):
        c, s = np.cos(np.float64(phi)), np.sin(np.float64(phi))
        cms, cps = abs(0.5 * (c - s)), abs(0.5 * (c + s))
        a, b = min(cms, cps), max(cms, cps)
        xp = t[None, :] * c + t[:, None] * s + pc
        r = np.rint(xp)
        # bin r+k (k=-1,0,1) has positive weight iff the footprint [xp-b, xp+b]
        # overlaps the open bin (r+k-1/2, r+k+1/2)
        for k in (-1, 0, 1):
            lo, hi = r + k - 0.5, r + k + 0.5
            ov = (np.minimum(hi, xp + b) - np.maximum(lo, xp - b)) > 0
            onb = (r + k >= 0) & (r + k < PX)
            total += int(np.count_nonzero(ov & onb))
    return total


def read_json(path):
    try:
        return json.loads(Path(path).read_text())
    except Exception:
        return None


class ClockSampler:
    """Samples nvidia-smi clocks / throttle reasons while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    NAMES = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, device_index: int):
        self.proc = None
        self.gpu_id = None
        try:
            uuid = getattr(torch.cuda.get_device_properties(device_index), "uuid", None)
            if uuid is not None:
                u = str(uuid)
                self.gpu_id = u if u.startswith("GPU-") else "GPU-" + u
        except Exception:
            pass

    def start(self):
        cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
               "-lms", "100"]
        if self.gpu_id:
            cmd.insert(1, f"--id={self.gpu_id}")
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                         text=True)
        except (FileNotFoundError, OSError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, reasons = [], [], set()
        for line in out.strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for name, val in zip(self.NAMES, parts[4:8]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


# --------------------------------------------------------------- CPU legs --

def cpu_sample(S, n, z, target_s, x_np=None, H=None):
    """Times the FP32 OpenMP CPU evaluation of A then A^T on a prefix of the
    angles, sized to take about target_s seconds; returns (GVU/s, cores,
    description)."""
    from oracle import oracle

    H = S if H is None else H
    xs, ys = shapes(S, n, z, H)
    rng = np.random.default_rng(0)
    x = x_np if x_np is not None else rng.standard_normal(xs, dtype=np.float32)
    ang = np.linspace(0, np.pi, n).astype(np.float32)
    y = np.zeros(ys, np.float32)
    xb = np.zeros(xs, np.float32)

    def run(k):
        t0 = time.perf_counter()
        oracle.forward_f32_(x, y, ang, z, 0, k)
        oracle.backward_f32_(y, xb, ang, z, 0, k)
        return time.perf_counter() - t0

    k = min(n, 2)
    dt = run(k)
    k = int(max(1, min(n, k * target_s / max(dt, 1e-3))))
    dt = run(k)
    vu = 2 * S * S * H * k
    vol = f"{S}³" if H == S else f"{S}²×{H}"
    desc = (f"A then Aᵀ on the full {vol} volume for the first {k} of {n} angles, "
            f"FP32 CPU restatement (oracle/vp_oracle.c), OpenMP")
    return vu / dt / 1e9, oracle.max_threads(), desc, k


def run_reference_arm(args, world, rank):
    """--impl reference: the operator evaluated on the host cores."""
    if rank != 0:
        return
    from oracle import oracle

    S, n, z, H = args.size, args.angles, args.z_order, heights(args)
    xs, ys = shapes(S, n, z, H)
    rng = np.random.default_rng(0)
    x = rng.standard_normal(xs, dtype=np.float32)
    ang = np.linspace(0, np.pi, n).astype(np.float32)
    y = np.zeros(ys, np.float32)
    xb = np.zeros(xs, np.float32)
    # size one step to ~3 s of CPU work so steps + warmup end within minutes
    _, _, _, k = cpu_sample(S, n, z, 3.0, x, H)

    def step():
        oracle.forward_f32_(x, y, ang, z, 0, k)
        oracle.backward_f32_(y, xb, ang, z, 0, k)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t0
    vu = 2 * S * S * H * k * args.steps
    val = vu / dt / 1e9
    vol = f"{S}³" if H == S else f"{S}²×{H}"
    sample = (f"each step: A then Aᵀ on the full {vol} volume for the first {k} of {n} angles "
              f"(FP32 CPU restatement, oracle/vp_oracle.c, OpenMP; the reference package has "
              f"no CPU implementation)")
    line = {
        "impl": "reference",
        "metric": metric_name(args), "value": round(val, 4), "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(dt / args.steps * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(args),
        "cpu_baseline": {"value": round(val, 4), "unit": UNIT, "cores": oracle.max_threads(),
                         "kind": "port", "sample": sample},
        "e2e": {"value": round(val, 4), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }
    print(json.dumps(line), flush=True)


def l2_note(x_bytes: int, y_bytes: int) -> str:
    """How the timed steps stand to the L2 rule: the steps are not separated
    by an L2 flush, so only inputs larger than L2 keep DRAM in the loop."""
    mb = (x_bytes // 2**20, y_bytes // 2**20, L2_BYTES // 2**20)
    if min(x_bytes, y_bytes) > L2_BYTES:
        return "inputs larger than L2 (x %d MB, y %d MB > %d MB L2)" % mb
    return ("inputs not all larger than L2 (x %d MB, y %d MB; %d MB L2) and L2 not flushed "
            "between steps: warm-L2 figure" % mb)


def workload_config(args):
    S, n, H = args.size, args.angles, heights(args)
    vol = f"{S}³" if H == S else f"{S}²×{H}"
    return {
        "workload": (f"A then Aᵀ, z_order {args.z_order}, {vol} float32 volume N(0,1), {n} "
                     f"angles linspace(0,π), detector width {S}"),
        "volume": [S, S, H] if args.z_order == 0 else [H, S, S], "n_angles": n,
        "detector_width": S, "z_order": args.z_order,
        "trig": args.trig,
        "l2": l2_note(S * S * H * 4, n * S * H * 4),
        "parallelism": "replicas (one independent problem per GPU)",
        "kernel_variants": {"A": args.variant_fwd or "default", "AT": args.variant_bwd or "default"},
    }


# ---------------------------------------------------------------- our arm --

def run_ours(args, world, rank, local):
    import voxelproj_gb300 as vp
    from voxelproj_gb300 import _lib

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    if world > 1:
        torch.distributed.init_process_group("nccl", device_id=dev)
    vp.set_trig_mode(args.trig)
    # z_order 2 with 32 heights or more runs the z_order 0 kernels between
    # transposes: the variants apply to those too
    for op_f, op_b in ((0, 1), (2, 3)) if args.z_order == 2 else ((0, 1),):
        _lib.LIB.vp_set_kernel_variant(op_f, args.variant_fwd)
        _lib.LIB.vp_set_kernel_variant(op_b, args.variant_bwd)
    S, n, z, H = args.size, args.angles, args.z_order, heights(args)
    PX = S
    xs, ys = shapes(S, n, z, H)
    fwd = vp._CU.forward_z0 if z == 0 else vp._CU.forward_z2
    bwd = vp._CU.backward_z0 if z == 0 else vp._CU.backward_z2

    gen = torch.Generator(device=dev).manual_seed(1234 + rank)
    x = torch.randn(xs, device=dev, generator=gen)
    ang_np = np.linspace(0, np.pi, n).astype(np.float32)
    ang = torch.tensor(ang_np, device=dev)
    y = torch.zeros(ys, device=dev)
    xb = torch.zeros(xs, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step(ev=None):
        if ev is not None:
            ev[0].record(stream)
        fwd(x, y, ang)
        if ev is not None:
            ev[1].record(stream)
        bwd(y, xb, ang)
        if ev is not None:
            ev[2].record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)

    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    sampler = ClockSampler(local) if rank == 0 else None
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    if sampler:
        sampler.start()
        time.sleep(0.3)  # let the sampler start before the timed region
    launches0 = _lib.LIB.vp_launch_count()
    start.record(stream)
    for k in range(args.steps):
        step(evs[k])
    end.record(stream)
    torch.cuda.synchronize(dev)
    launches = _lib.LIB.vp_launch_count() - launches0
    clocks = sampler.stop() if sampler else None
    if world > 1:
        torch.distributed.barrier()
    total_ms = start.elapsed_time(end)
    t_fwd = [e[0].elapsed_time(e[1]) for e in evs]
    t_bwd = [e[1].elapsed_time(e[2]) for e in evs]
    total_ms = max_over_ranks(total_ms, world, dev)
    vu_step = 2 * S * S * H * n
    value = whole_job_gvu_s(world, args.steps, vu_step, total_ms)
    fwd_ms = statistics.mean(t_fwd)
    bwd_ms = statistics.mean(t_bwd)

    result = None
    if rank == 0:
        peaks = read_json(ROOT / "MEASURED_PEAKS.json") or {}
        hbm_peak = peaks.get("hbm_gbs")
        peak_note = "measured" if hbm_peak else "fallback"
        hbm_peak = hbm_peak or 6800.0
        alg = algorithmic_bytes(S, n, PX, H)
        kern = "A" if fwd_ms >= bwd_ms else "AT"
        kname = KERNELS[(kern, z)]
        dur_s = (fwd_ms if kern == "A" else bwd_ms) / 1e3
        achieved = alg[kern] / dur_s / 1e9
        # traffic per call of the operator (its slab / class launches together),
        # the same unit as `achieved`, from the committed ncu capture
        traffic, launches_per_call = None, None
        tr = read_json(ROOT / "profiles" / "traffic.json")
        wl = (tr or {}).get("workload", {})
        if (wl.get("size"), wl.get("n_angles"), wl.get("z_order", 0)) == (S, n, z):
            kt = tr.get("kernels", {}).get(kname, {})
            traffic = kt.get("dram_bytes_per_call")
            launches_per_call = kt.get("launches_per_call")
        nnz = weights_nnz(S, n, PX, ang_np)
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        clk = peaks.get("sm_max_mhz", 2070.0)
        fp32_peak = sms * 128 * 2 * clk * 1e6 / 1e12
        flops = 2.0 * nnz * H  # one multiply-add per nonzero weight per height
        # the reference publishes A and A^T times for 512^3 / 192 angles, z_order 0
        published = (S, n, args.z_order, H) == (512, 192, 0, 512)
        result = {
            "metric": metric_name(args), "value": round(value, 3), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(total_ms / args.steps, 4), "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": round(value / PUBLISHED_GVU_S, 3) if published else None,
            "vs_baseline_basis": ("RTX 3060, README.md:58-59 of the reference (A 516 ms + Aᵀ "
                                  "397 ms at 512³/192, z_order 0, units assumed ms) -> %.1f GVU/s"
                                  % PUBLISHED_GVU_S) if published else
                                 "no published figure for this configuration",
            "dtype": "f32", "data": "synthetic", "config": workload_config(args),
            "parts": {
                "A": {"ms": round(fwd_ms, 4), "gvu_s": round(S * S * H * n / fwd_ms / 1e6, 2),
                      "kernel": KERNELS[("A", z)]},
                "AT": {"ms": round(bwd_ms, 4), "gvu_s": round(S * S * H * n / bwd_ms / 1e6, 2),
                       "kernel": KERNELS[("AT", z)]},
            },
            "roofline": {"bound": "hbm", "kernel": kname, "achieved": round(achieved, 2),
                         "peak": hbm_peak, "peak_source": peak_note, "unit": "GB/s",
                         "frac": round(achieved / hbm_peak, 4), "traffic": traffic,
                         "algorithmic_bytes": alg[kern],
                         "per": "one %s call (%s kernel launches), CUDA events on its stream"
                                % (kern, launches_per_call or "its")},
            "fma_roofline": {
                "kernel": kname, "nonzero_weights": nnz,
                "achieved": round(flops / dur_s / 1e12, 3), "unit": "TFLOP/s",
                "peak": round(fp32_peak, 2),
                "peak_basis": f"{sms} SMs x 128 FP32 lanes x 2 x {clk:.0f} MHz",
                "frac": round(flops / dur_s / 1e12 / fp32_peak, 4),
            },
            "gpu_launches": int(launches),
            "clocks": clocks,
        }
    if world > 1:
        torch.distributed.barrier()

    # ---- end to end through the public API with host buffers (pinned) ----
    if rank == 0 and result is not None and not args.no_e2e:
        result["e2e"] = e2e_leg(args, vp, x, ang_np, dev)
    if rank == 0 and result is not None and world == 1 and not args.no_cpu_baseline:
        val, cores, desc, _ = cpu_sample(S, n, z, args.cpu_seconds, None, H)
        result["cpu_baseline"] = {"value": round(val, 4), "unit": UNIT, "cores": cores,
                                  "kind": "port", "sample": desc}
    if rank == 0 and result is not None:
        print(json.dumps(result), flush=True)
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


def e2e_leg(args, vp, x_dev, ang_np, dev):
    """Same step through voxelproj_gb300.forward/backward with pinned CPU
    tensors: every step copies x, the output containers and the sinogram to
    the device and reads both results back."""
    S, n, z, H = args.size, args.angles, args.z_order, heights(args)
    xs, ys = shapes(S, n, z, H)
    x_h = x_dev.cpu().pin_memory()
    y_h = torch.zeros(ys).pin_memory()
    xb_h = torch.zeros(xs).pin_memory()

    def step():
        vp.forward(x_h, ang_np, y_h, z_order=z)
        vp.backward(y_h, ang_np, xb_h, z_order=z)

    for _ in range(min(args.warmup, 2)):
        step()
    torch.cuda.synchronize(dev)
    # each step timed on its own (a step ends with its results in host
    # memory); the median is reported, so that a stretch of host-side
    # contention on a shared machine (seen to double single steps) does not
    # decide the figure; mean and slowest step are reported beside it
    k = max(5, min(args.steps, 10))
    ts = []
    for _ in range(k):
        t0 = time.perf_counter()
        step()
        torch.cuda.synchronize(dev)
        ts.append(time.perf_counter() - t0)
    dt = float(np.median(ts))
    vol, sino, a = 4 * S * S * H, 4 * n * S * H, 4 * n
    return {"value": round(2 * S * S * H * n / dt / 1e9, 3), "unit": UNIT,
            "ms_per_step": round(dt * 1e3, 3), "steps_timed": k,
            "stat": "median of individually timed steps",
            "ms_per_step_mean": round(float(np.mean(ts)) * 1e3, 3),
            "ms_per_step_max": round(float(np.max(ts)) * 1e3, 3),
            "h2d_bytes_per_step": vol + sino + a + sino + vol + a,
            "d2h_bytes_per_step": sino + vol,
            "path": "voxelproj_gb300.forward(x, angles, y) then backward(y, angles, x') with "
                    "pinned CPU tensors (inputs and accumulate-into containers copied in, "
                    "results copied out, every step; z_order 0 host arrays go through "
                    "vp_forward_z0_host / vp_backward_z0_host, which overlap the copies "
                    "with the kernels)"}


def main():
    args = parse_args()
    world, rank, local = dist_info()
    if args.impl == "reference":
        run_reference_arm(args, world, rank)
        return
    run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
