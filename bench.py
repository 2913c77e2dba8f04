"""Benchmark: simulated audio-seconds per wall-second of the cochlear solver
path on one GB300 (one process per GPU under torchrun; weak scaling).

Workload (default "tone_sweep", config 2): 64 pure tones log-spaced
125 Hz-8 kHz x {20,40,60,80,100} dB SPL = 320 signals of 80 ms at 100 kHz,
each split into Decouple_Filter=8 blocks of 10 ms with the 5 ms overlap
warm-up -- 2,560 BM units per step, 25.6 s of audio.  A step is one pass of
the path over the whole batch with its inputs resident in HBM: input
generation, BM/OHC solver (FP32), IHC + lambda for the three fibre groups.

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
def tone_sweep_config(n_freq=64, levels=(20, 40, 60, 80, 100)):
    """Config 2: n_freq log-spaced tones 125 Hz-8 kHz x levels, 10 ms blocks x
    Decouple_Filter 8, 5 ms overlap, healthy profiles, outputs v + lambda.
    n_freq=64 is the full workload; smaller values give profiling cases."""
    from cochlearmodel_gb300 import model
    from cochlearmodel_gb300.pipeline import ProfileSweep
    cfg = model.RunConfig(Time_Block_Length=0.01, Decouple_Filter=8, Overlap_Time=0.005)
    freqs = list(125.0 * 64.0 ** (np.arange(n_freq) / max(1, n_freq - 1)))
    sweep = ProfileSweep(frequencies=freqs, powers=list(levels), calculate_jnd=False)
    return cfg, sweep


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
def cpu_sample(run, target_s=15.0, threads=None):
    """The path (BM + IHC/lambda in the reference's arithmetic) on the first K
    signals of the sweep, all host threads; returns audio-s per wall-second."""
    from cochlearmodel_gb300 import ihc as ihcmod
    from oracle import oracle as orc
    cores = threads or os.cpu_count() or 1
    D = run.cfg.Decouple_Filter
    ov = run.cfg.calc_overlap_nodes()
    x = run.d_in.cpu().numpy()
    secp = run.mv.section_params()
    gamma = run.cfg.gamma()[None]
    st = run.ihc

    def sample(k):
        units = run.units[:k * D]
        t0 = time.perf_counter()
        v, _, _ = orc.bm_run(secp, gamma, run.sc, units, x, run.rows, threads=cores)
        rows = k * run.L + ov
        orc.ihc_lambda(v[:rows], run.L, k * run.L, ihcmod.round64(rows), k * run.L,
                       st.ac.astype(np.float64), st.dc.astype(np.float64), 1.0, 1.0, 100.0,
                       st.dmg_host[0].astype(np.float64), st.nerve.aihc(),
                       np.asarray(st.nerve.spontRate, np.float32), 500.0, mode=0)
        return time.perf_counter() - t0

    k = max(1, min(run.n_int, cores // D))
    dt = sample(k)
    k2 = max(1, min(run.n_int, int(k * target_s / max(dt, 1e-3))))
    if k2 > k:
        k, dt = k2, sample(k2)
    audio = k * run.L / run.cfg.Fs
    return audio / dt, cores, (f"{k} of {run.n_int} signals of the tone sweep ({audio:.3f} "
                               f"audio-s): BM (FP32 oracle) + IHC/lambda (reference mixed "
                               f"precision), {cores} threads, {dt:.1f} s")


# ----------------------------------------------------------------------------
# arms
# ----------------------------------------------------------------------------
def make_run(device, n_freq):
    from cochlearmodel_gb300.pipeline import ProfileRun
    cfg, sweep = tone_sweep_config(n_freq)
    return ProfileRun(device, cfg, sweep)


def run_reference(args, rank, world):
    """The path's CPU implementation on the host cores.  The input of the sweep
    is produced by the GPU input kernel when a GPU is present, else by the
    oracle's restatement of it; the timed work is CPU only."""
    if rank != 0:
        return None
    import torch
    dev = "cuda:0" if torch.cuda.is_available() else None
    if dev is None:
        print(json.dumps({"impl": "reference", "unavailable": "needs the input of the sweep"}))
        return None
    run = make_run(dev, args.n_freq)
    run.generate_input()
    torch.cuda.synchronize()
    vals = []
    for i in range(args.warmup + args.steps):
        v, cores, sample = cpu_sample(run, target_s=args.cpu_seconds / max(1, args.steps))
        if i >= args.warmup:
            vals.append(v)
    value = float(np.mean(vals))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": run.audio_seconds / value * 1000.0, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "tone_sweep", "signals": run.n_int, "units": len(run.units),
                       "audio_s_per_step": run.audio_seconds, "sample": "bounded"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    return line


def run_ours(args, rank, world, device):
    import torch
    from cochlearmodel_gb300 import native

    run = make_run(device, args.n_freq)
    native.check(native.load().cgb_bm_set_launch_shape(args.shape), "launch shape")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)
    stream = torch.cuda.current_stream(device)

    # warm-up, with per-stage device times on the last warm-up step
    stage_ms = {}
    for w in range(args.warmup):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        ev[0].record(stream)
        run.generate_input()
        ev[1].record(stream)
        run.solve_bm()
        ev[2].record(stream)
        run.ihc_lambda()
        ev[3].record(stream)
        flush.fill_(1.0)
        torch.cuda.synchronize(device)
        stage_ms = {"input_gen": ev[0].elapsed_time(ev[1]), "bm_solver": ev[1].elapsed_time(ev[2]),
                    "ihc_lambda": ev[2].elapsed_time(ev[3])}
    stats = run.d_stats.cpu().numpy().view(native.STATS_DTYPE).reshape(-1)
    flops = bm_flops(stats)

    clocks = ClockSampler(device.index if device.index is not None else 0)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(device)
    clocks.start()
    launches_a = native.load().cgb_kernel_launch_count()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    for i in range(args.steps):
        ev[i][0].record(stream)
        run.step()
        ev[i][1].record(stream)
        flush.fill_(float(i))  # L2 flush between timed steps (256 MB > 129 MB L2)
    torch.cuda.synchronize(device)
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    launches = native.load().cgb_kernel_launch_count() - launches_a
    t_total = sum(a.elapsed_time(b) for a, b in ev) / 1000.0
    if world > 1:
        tt = torch.tensor([t_total], device=device)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_total = float(tt.item())
    value = run.audio_seconds * args.steps * world / t_total

    # e2e: the sweep's profile table in from pinned host memory, the path,
    # velocity and the three lambda planes back to pinned host memory
    h_prof = torch.from_numpy(run.prof.view(np.uint8).copy()).pin_memory()
    h_v = torch.empty(run.d_v.shape, dtype=torch.float32).pin_memory()
    h_lam = torch.empty(run.d_lam.shape, dtype=torch.float32).pin_memory()
    e_steps = max(1, args.steps // 2)
    e_ms = 0.0
    for i in range(e_steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(device)
        a.record(stream)
        run.d_prof.copy_(h_prof, non_blocking=True)
        run.step()
        h_v.copy_(run.d_v, non_blocking=True)
        h_lam.copy_(run.d_lam, non_blocking=True)
        b.record(stream)
        torch.cuda.synchronize(device)
        e_ms += a.elapsed_time(b)
        flush.fill_(float(i))
    e2e = run.audio_seconds * e_steps * world / (e_ms / 1000.0)

    peaks, peak_kind = measured_peaks()
    clock_mhz = peaks.get("sm_max_mhz", 2070.0)
    n_sm = torch.cuda.get_device_properties(device).multi_processor_count
    fp32_peak = 2.0 * 128 * n_sm * clock_mhz * 1e6 / 1e12
    bm_s = stage_ms["bm_solver"] / 1000.0
    achieved = flops / bm_s / 1e12
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_total / args.steps * 1000.0,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "tone_sweep", "signals": run.n_int, "units": len(run.units),
                   "audio_s_per_step": run.audio_seconds, "fs": run.cfg.Fs,
                   "l2": "flushed between timed steps (256 MB write)",
                   "path": "input generation -> BM/OHC solver (20/2 Jacobi sweeps) -> "
                           "IHC/lambda (3 fibre groups)",
                   "launch_shape": args.shape, "stage_ms": stage_ms},
        "gpu_launches": int(launches),
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(h_prof.numel()),
                "d2h_bytes_per_step": int(h_v.numel() * 4 + h_lam.numel() * 4)},
        "roofline": {"bound": "fp32", "kernel": "bm_warp_kernel", "achieved": achieved,
                     "peak": fp32_peak, "unit": "TFLOP/s", "frac": achieved / fp32_peak,
                     "traffic": None,
                     "peak_source": f"2 x 128 FP32 lanes x {n_sm} SMs x sm_max_mhz "
                                    f"({peak_kind} MEASURED_PEAKS.json)"},
        "clocks": clk,
    }
    return line, run


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
    line, run = run_ours(args, rank, world, device)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, cores, sample = cpu_sample(run, target_s=args.cpu_seconds)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": sample}
    if world > 1:
        torch.distributed.destroy_process_group()
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
