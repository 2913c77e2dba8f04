"""Benchmark: simulated audio-seconds per wall-second of the cochlear solver
path on one GB300 (one process per GPU under torchrun; weak scaling).

Workload (default "tone_sweep"): 64 pure tones log-spaced 125 Hz-8 kHz x
{20,40,60,80,100} dB SPL = 320 signals of 80 ms at 100 kHz, each split into
Decouple_Filter=8 blocks of 10 ms with the 5 ms overlap warm-up -- 2,560 BM
units per step, 25.6 s of audio.  A step is one pass of the path over the
whole batch with inputs resident in HBM: BM/OHC solver (FP32).

Arms:
  default            the GB300 kernels (value: device time; e2e: host buffers
                     in, results back to host, through the C ABI)
  --impl reference   the reference algorithm on the host cores (the CPU
                     restatement of kernel 17; the reference ships no
                     runnable CPU path of its own), bounded sample per step
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "simulated audio-s/sec on 1 GB300: batched+learned vs plain, equal max error"
UNIT = "audio-s/s"


# ----------------------------------------------------------------------------
# workload
# ----------------------------------------------------------------------------
def tone_sweep(mv, n_freq=64, levels=(20, 40, 60, 80, 100)):
    """n_freq=64 is the full workload; smaller values give profiling cases."""
    from cochlearmodel_gb300 import model, native
    cfg = model.RunConfig(Time_Block_Length=0.01, Decouple_Filter=8, Overlap_Time=0.005)
    n_sig = n_freq * len(levels)
    cfg.Time_Blocks = n_sig * cfg.Decouple_Filter
    sc = model.bm_scalars(cfg, mv)
    units = model.reference_units(cfg)
    N = cfg.calc_time_block_nodes()
    L = N * cfg.Decouple_Filter
    n_in = cfg.total_time_nodes_p1() + 4
    freqs = 125.0 * 64.0 ** (np.arange(n_freq) / (n_freq - 1))
    two_pi = float(np.float32(2 * np.float32(math.pi)))
    t = np.arange(L, dtype=np.float64) / float(np.float32(cfg.Fs))
    x = np.zeros(n_in, np.float32)
    k = 0
    for db in levels:  # profile order: noise > power > frequency (src/params.cpp:697-740)
        amp = model.spl_to_amplitude(float(db))
        for f in freqs:
            x[k * L:(k + 1) * L] = (amp * np.cos(two_pi * f * t)).astype(np.float32)
            k += 1
    audio_s = n_sig * L / cfg.Fs
    return dict(cfg=cfg, sc=sc, units=units, x=x, rows=n_in, gamma=cfg.gamma()[None],
                audio_s=audio_s, n_sig=n_sig, name="tone_sweep")


# ----------------------------------------------------------------------------
# clocks sampling during the timed region
# ----------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


# FP32 operations per section, counted from the kernel's source (FMA = 2):
# every outer iteration ~44 (predictor, G, Y, acceleration, psi', partial
# reductions), the OHC/TM update on the first two iterations of a step ~50,
# each Jacobi sweep 3 (one add + one fma).
FLOP_PER_SECTION_ITER = 44
FLOP_PER_SECTION_TM = 50
FLOP_PER_SECTION_SWEEP = 3


def bm_flops(stats) -> float:
    it = float(stats["iterations"].sum())
    sub = float(stats["substeps"].sum())
    sw = float(stats["sweeps"].sum())
    return 256.0 * (FLOP_PER_SECTION_ITER * it + FLOP_PER_SECTION_TM * 2 * sub +
                    FLOP_PER_SECTION_SWEEP * sw)


# ----------------------------------------------------------------------------
# CPU baseline (oracle restatement on the host cores)
# ----------------------------------------------------------------------------
def cpu_sample(wl, mv, target_s=15.0):
    from oracle import oracle as orc
    cores = os.cpu_count() or 1
    units = wl["units"]
    secp = mv.section_params()
    # calibrate on one unit per core
    n = min(len(units), cores)
    t0 = time.perf_counter()
    _, _, st = orc.bm_run(secp, wl["gamma"], wl["sc"], units[:n], wl["x"], wl["rows"],
                          threads=cores)
    dt = time.perf_counter() - t0
    reps = max(1, int(target_s / max(dt, 1e-3)))
    n2 = min(len(units), n * reps)
    sel = units[:n2]
    t0 = time.perf_counter()
    _, _, st = orc.bm_run(secp, wl["gamma"], wl["sc"], sel, wl["x"], wl["rows"], threads=cores)
    dt = time.perf_counter() - t0
    audio = float((sel["end"] - sel["out_first"]).sum()) / wl["cfg"].Fs
    return audio / dt, cores, f"{n2} of {len(units)} BM units of {wl['name']} " \
                              f"({audio:.3f} audio-s), FP32 oracle, {cores} threads, {dt:.1f} s"


# ----------------------------------------------------------------------------
# arms
# ----------------------------------------------------------------------------
def run_reference(args, rank, world):
    from cochlearmodel_gb300 import model
    if rank != 0:
        return None
    mv = model.ModelVectors.build()
    wl = tone_sweep(mv)
    vals = []
    for i in range(args.warmup + args.steps):
        v, cores, sample = cpu_sample(wl, mv, target_s=args.cpu_seconds / max(1, args.steps))
        if i >= args.warmup:
            vals.append(v)
    value = float(np.mean(vals))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": wl["audio_s"] / value * 1000.0, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": wl["name"], "signals": wl["n_sig"], "units": len(wl["units"]),
                       "audio_s_per_step": wl["audio_s"], "sample": "bounded"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    return line


def run_ours(args, rank, world, device):
    import torch
    from cochlearmodel_gb300 import model, native
    from cochlearmodel_gb300.solver import BMSolver, units_to_device

    mv = model.ModelVectors.build()
    wl = tone_sweep(mv, n_freq=args.n_freq)
    solver = BMSolver(device, mv)
    native.check(native.load().cgb_bm_set_launch_shape(args.shape), "launch shape")
    units = wl["units"]
    solver.check_units(units, 1, wl["x"].size, wl["rows"])
    d_units = units_to_device(units, device)
    d_gamma = torch.from_numpy(wl["gamma"]).to(device)
    d_in = torch.from_numpy(wl["x"]).to(device)
    d_out = torch.empty((wl["rows"], 256), dtype=torch.float32, device=device)
    d_failed = torch.zeros(wl["rows"], dtype=torch.int32, device=device)
    d_stats = torch.zeros((len(units), native.STATS_DTYPE.itemsize), dtype=torch.uint8,
                          device=device)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)
    stream = torch.cuda.current_stream(device)

    def step():
        solver.run_dev(wl["sc"], d_gamma, d_units, len(units), d_in, d_out, d_failed, d_stats)

    launches0 = native.load().cgb_kernel_launch_count()
    for _ in range(args.warmup):
        step()
        flush.fill_(1.0)
    torch.cuda.synchronize(device)
    stats = d_stats.cpu().numpy().view(native.STATS_DTYPE).reshape(-1)
    flops = bm_flops(stats)

    clocks = ClockSampler(torch.cuda.current_device() if world == 1 else rank)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(device)
    clocks.start()
    launches_a = native.load().cgb_kernel_launch_count()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    for i in range(args.steps):
        ev[i][0].record(stream)
        step()
        ev[i][1].record(stream)
        flush.fill_(float(i))  # L2 flush between timed steps (256 MB > 129 MB L2)
    torch.cuda.synchronize(device)
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    launches = native.load().cgb_kernel_launch_count() - launches_a
    ms = [a.elapsed_time(b) for a, b in ev]
    t_total = sum(ms) / 1000.0
    if world > 1:
        tt = torch.tensor([t_total], device=device)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_total = float(tt.item())
    value = wl["audio_s"] * args.steps * world / t_total

    # e2e: host input -> device -> solver -> host velocity, through the ABI
    h_in = torch.from_numpy(wl["x"]).pin_memory()
    h_out = torch.empty((wl["rows"], 256), dtype=torch.float32).pin_memory()
    torch.cuda.synchronize(device)
    e_start, e_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e_ms = 0.0
    for i in range(max(1, args.steps // 2)):
        e_start.record(stream)
        d_in.copy_(h_in, non_blocking=True)
        step()
        h_out.copy_(d_out, non_blocking=True)
        e_end.record(stream)
        torch.cuda.synchronize(device)
        e_ms += e_start.elapsed_time(e_end)
        flush.fill_(float(i))
    e_steps = max(1, args.steps // 2)
    e2e = wl["audio_s"] * e_steps * world / (e_ms / 1000.0)

    peaks, peak_kind = measured_peaks()
    clock_mhz = peaks.get("sm_max_mhz", 2070.0)
    n_sm = torch.cuda.get_device_properties(device).multi_processor_count
    fp32_peak = 2.0 * 128 * n_sm * clock_mhz * 1e6 / 1e12
    achieved = flops / (t_total / args.steps * world) / 1e12 if world == 1 else \
        flops / (t_total / args.steps) / 1e12
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_total / args.steps * 1000.0,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": wl["name"], "signals": wl["n_sig"], "units": len(units),
                   "audio_s_per_step": wl["audio_s"], "fs": wl["cfg"].Fs,
                   "l2": "flushed between timed steps (256 MB write)",
                   "path": "BM/OHC solver (reference semantics, 20/2 Jacobi sweeps)",
                   "launch_shape": args.shape},
        "gpu_launches": int(launches),
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(wl["x"].nbytes),
                "d2h_bytes_per_step": int(h_out.numel() * 4)},
        "roofline": {"bound": "fp32", "kernel": "bm_warp_kernel", "achieved": achieved,
                     "peak": fp32_peak, "unit": "TFLOP/s", "frac": achieved / fp32_peak,
                     "traffic": None,
                     "peak_source": f"2 x 128 FP32 lanes x {n_sm} SMs x sm_max_mhz "
                                    f"({peak_kind} MEASURED_PEAKS.json)"},
        "clocks": clk,
    }
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--shape", type=int, default=0, help="BM kernel launch shape")
    ap.add_argument("--n-freq", type=int, default=64,
                    help="tones per level (64 = the full tone sweep; less for profiling)")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        line = run_reference(args, rank, world)
        if line is not None:
            print(json.dumps(line))
        return

    import torch
    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    if world > 1:
        torch.distributed.init_process_group("nccl", device_id=device)
    line = run_ours(args, rank, world, device)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from cochlearmodel_gb300 import model
        mv = model.ModelVectors.build()
        v, cores, sample = cpu_sample(tone_sweep(mv), mv, target_s=args.cpu_seconds)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": sample}
    if world > 1:
        torch.distributed.destroy_process_group()
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
