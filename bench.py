"""Benchmark: simulated audio-seconds per wall-second of the cochlear solver
path on one GB300 (one process per GPU under torchrun; weak scaling).

Workloads (--workload):
  jnd_sweep (default, configuration 3): a 1 kHz tone at 10..100 dB SPL x noise
      levels {none, 0, 10, 20, 30, 40} dB SPL plus one noise-only reference per
      noise level, 4 noise seeds -> 264 signals; interval lengths drawn per
      (seed, noise) group uniformly in 20-200 ms; hearing-loss OHC/IHC
      profiles; ~10 ms blocks with the 5 ms overlap warm-up.  A step is the
      whole path -- input generation, BM/OHC solver, IHC + lambda, JND Fisher
      sums -- for all 264 signals, replayed from one CUDA graph.
  tone_sweep (configuration 2): 64 log-spaced tones 125 Hz-8 kHz x {20..100}
      dB SPL = 320 signals of 80 ms, Decouple_Filter 8 blocks of 10 ms; input,
      BM, IHC + lambda.
  mixed_batch (configuration 5): 1,024 signals of lengths log-uniform
      10 ms - 1 s, a seeded mix of tones, harmonic complexes and tones in
      white noise, each with its own smooth random OHC (0-0.5) and IHC (5-8)
      profile; BM, IHC + lambda and JND (tone in noise against the noise
      alone, the others against silence) in one graph; the value counts the
      1,024 test signals only.  Its e2e copies the input samples in and the
      Fisher sums and failure flags out (the 120 GB of velocity and lambda
      stay in HBM).

--jacobi selects the pressure solve: reference (the reference's fixed
20/2 sweep schedule, default), or the tolerance mode (|dp| <= 1e-6 |p|)
started from the previous pressure, its extrapolation, or the learned guess.
--bm-kernel 0 runs the reference's default BM kernel (BMOHC_NEW_kernel's
fault-count controller in the reference's operation order, bit-exact with its
compiled kernel) in place of kernel 17's semantics.

Every step recomputes everything from the profile table in HBM.  Reported
beside the batched value: the same kernels run one signal at a time ("plain
single-signal"), the CPU restatement on the host cores, and (JND sweep,
reference schedule) max_rel_vs_fp64: the step's velocity, lambda and JND error
against the FP64 oracle on the shortest group, after the timed region.

Arms:
  default            the GB300 kernels (value: device time; e2e: host tables in,
                     velocity + lambda back to host, through the C ABI)
  --impl reference   the path on the host cores through the CPU oracle alone
                     (input generation, BM, IHC/lambda, JND; the reference ships
                     no runnable CPU path of its own, and its IHC/lambda
                     restatement equals the reference's kernels bit for bit);
                     each step a bounded sample of the sweep; no part of the
                     GPU library is loaded
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
# one process per GPU: every rank runs the whole workload (replicas, weak
# scaling, no collective on the data path); the job's time is the slowest rank


def max_over_ranks(x: float, world: int) -> float:
    """The maximum of a per-rank scalar (a time) over the ranks of the job
    (one all-reduce on the process group's own device: the GPU under NCCL,
    the CPU under gloo)."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(audio_s_per_step: float, steps: int, world: int, t_max_s: float) -> float:
    """Whole-job throughput: the audio-seconds all ranks processed over the
    slowest rank's time."""
    return audio_s_per_step * steps * world / t_max_s


# ----------------------------------------------------------------------------
# workloads
# ----------------------------------------------------------------------------
def make_workload(name, device, n_freq=64, n_seeds=4, n_signals=1024):
    from cochlearmodel_gb300 import batch, mixed, model
    from cochlearmodel_gb300.pipeline import ProfileRun, ProfileSweep
    if name == "tone_sweep":
        cfg = model.RunConfig(Time_Block_Length=0.01, Decouple_Filter=8, Overlap_Time=0.005)
        freqs = list(125.0 * 64.0 ** (np.arange(n_freq) / max(1, n_freq - 1)))
        sweep = ProfileSweep(frequencies=freqs, powers=[20.0, 40.0, 60.0, 80.0, 100.0])
        run = ProfileRun(device, cfg, sweep)
        run.kind = "tone_sweep"
        return run
    if name == "jnd_sweep":
        run = batch.BatchSweep(device, batch.jnd_sweep_spec(n_seeds=n_seeds))
        run.kind = "jnd_sweep"
        return run
    if name == "mixed_batch":
        run = mixed.MixedBatch(device, mixed.mixed_batch_spec(n_signals=n_signals))
        run.kind = "mixed_batch"
        return run
    raise ValueError(name)


JACOBI = {"reference": None, "previous": 0, "extrapolated": 1, "learned": 2}


def set_jacobi(run, mode, device):
    """Switches the workload's BM scalars to the chosen pressure solve."""
    from cochlearmodel_gb300 import model
    guess = JACOBI[mode]
    if guess is None:
        return None
    run.sc = model.tolerance_mode(run.sc, guess=guess)
    if guess == 2:
        from cochlearmodel_gb300 import warmstart
        run.net = warmstart.WarmStartNet.load(warmstart.WEIGHTS, device)
        run.extras = run.net.extras()
    return guess


def stages(run):
    s = [] if run.kind == "mixed_batch" else [("input_gen", run.generate_input)]
    s += [("bm_solver", run.solve_bm), ("ihc_lambda", run.ihc_lambda)]
    if run.kind in ("jnd_sweep", "mixed_batch"):
        s.append(("jnd", run.jnd_sums))
    return s


def n_signals(run):
    return run.n_signals if run.kind in ("jnd_sweep", "mixed_batch") else run.n_int


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


# DRAM bytes per BM launch, from ncu (dram__bytes_read.sum + dram__bytes_write.sum)
# on the 40-signal tone sweep (278.9 MB for 320 units), scaled by the units a
# launch processes: the traffic is the velocity rows written, in proportion.
BM_TRAFFIC_PER_UNIT = 278.9e6 / 320


# ----------------------------------------------------------------------------
# CPU restatement on the host cores (bounded sample)
# ----------------------------------------------------------------------------
def cpu_sample(run, target_s=15.0, threads=None):
    """The path (BM in FP32 + IHC/lambda in the reference's mixed precision)
    on the first K signals (tone sweep) or groups (JND sweep), all host
    threads; returns (audio-s per wall-second, cores, description)."""
    from cochlearmodel_gb300 import ihc as ihcmod
    from oracle import oracle as orc
    cores = threads or os.cpu_count() or 1
    x = run.d_in.cpu().numpy()
    secp = run.mv.section_params()
    st = run.ihc

    def ihc_frame(v, fr):
        r0 = int(fr["v_row0"])
        orc.ihc_lambda(v[r0:r0 + int(fr["rows"])], int(fr["seg"]), int(fr["frdp"]),
                       int(fr["total"]), int(fr["lam_rows"]), st.ac.astype(np.float64),
                       st.dc.astype(np.float64), 1.0, 1.0, 100.0,
                       st.dmg_host[0].astype(np.float64), st.nerve.aihc(),
                       np.asarray(st.nerve.spontRate, np.float32), 500.0, mode=0)

    if run.kind == "tone_sweep":
        D = run.cfg.Decouple_Filter
        ov = run.cfg.calc_overlap_nodes()
        gamma = run.cfg.gamma()[None]

        def sample(k):
            units = run.units[:k * D]
            t0 = time.perf_counter()
            v, _, _ = orc.bm_run(secp, gamma, run.sc, units, x, run.rows, threads=cores)
            rows = k * run.L + ov
            fr = np.zeros(1, ihcmod.FRAME_DTYPE)[0]
            fr["v_row0"], fr["rows"], fr["lam_rows"] = 0, rows, k * run.L
            fr["seg"], fr["frdp"], fr["total"] = run.L, k * run.L, ihcmod.round64(rows)
            ihc_frame(v, fr)
            return time.perf_counter() - t0, k * run.L / run.cfg.Fs

        k, limit, what = max(1, min(run.n_int, cores // D)), run.n_int, "signals of the tone sweep"
    else:
        gamma = run.d_gamma.cpu().numpy()

        def sample(k):
            groups = run.groups[:k]
            units = np.concatenate([run.units[run.units["out_base"] == g.v_row0] for g in groups])
            t0 = time.perf_counter()
            v, _, _ = orc.bm_run(secp, gamma, run.sc, units, x, run.v_rows, threads=cores)
            for gi in range(k):
                ihc_frame(v, run.frames[gi])
            return time.perf_counter() - t0, sum(len(g.prof) * g.L for g in groups) / run.Fs

        k, limit, what = 1, len(run.groups), "groups of the JND sweep"
    dt, audio = sample(k)
    k2 = max(1, min(limit, int(k * target_s / max(dt, 1e-3))))
    if k2 > k:
        k = k2
        dt, audio = sample(k)
    return audio / dt, cores, (f"{k} {what} ({audio:.3f} audio-s): BM (FP32 restatement) + "
                               f"IHC/lambda (reference mixed precision), {cores} threads, "
                               f"{dt:.1f} s")


class RefSweepCPU:
    """The JND sweep (configuration 3) on the host cores through the oracle
    alone: input generation (orc.input_gen), BM in FP32 with the reference
    schedule (orc.bm_run), IHC/lambda in the reference's mixed precision
    (orc.ihc_lambda mode 0, which equals the reference's own kernels bit for
    bit) and the JND Fisher sums in the reference's float arithmetic
    (orc.jnd).  The signals, lengths, partitions and filters are those of the
    GPU arm's workload, built from the same seeded description; no part of
    the product library is loaded (the model, unit tables and section
    parameters come from the oracle).  A step runs one group's reference
    interval plus its first m tested intervals; step() returns the audio
    seconds it simulated."""

    def __init__(self, n_seeds=4, Fs=100000, overlap_time=0.005, block_target=1000):
        from cochlearmodel_gb300 import batch, ihc
        from cochlearmodel_gb300.pipeline import JNDWindow
        from oracle import oracle as orc
        self.orc = orc
        self.batch = batch
        self.Fs, self.overlap_time, self.block_target = Fs, overlap_time, block_target
        self.specs = batch.jnd_sweep_spec(n_seeds=n_seeds)
        f = np.float32
        md = orc.model_setup()
        self.secp = np.stack([f(1.0) / md["M"].astype(f), f(1.0) / md["diag_m"].astype(f),
                              md["R"].astype(f), md["S"].astype(f), md["Q"].astype(f),
                              md["S_ohc"].astype(f), md["S_tm"].astype(f),
                              md["R_tm"].astype(f)]).astype(f)
        self.scal = md["scal"]
        self.gamma = batch.hearing_loss_ohc()[None]
        self.nerve = ihc.NerveConfig()
        self.dmg = ihc.ihc_damage(batch.hearing_loss_ihc()).astype(np.float64)
        self.ac = ihc.design_ac_lowpass().astype(np.float64)
        self.dc = self.nerve.dc_taps(Fs).astype(np.float64)
        self.win = JNDWindow()
        self.ihc = ihc
        self.n_groups = len(self.specs)
        self.group_audio = []
        self.units_total = 0
        for sp in self.specs:
            N, D = batch.block_nodes_for(sp["length"], block_target, Fs)
            n_int = len(sp["sweep"].powers) + 1
            self.group_audio.append(n_int * N * D / Fs)
            self.units_total += n_int * D
        self.audio_seconds = float(sum(self.group_audio))

    def scalars(self, cfg):
        orc = self.orc
        s = orc.OrcScalars()
        F32 = np.float32
        for name, i in (("w_ohc", 0), ("delta_x", 1), ("alpha_r", 2), ("alpha_l", 3),
                        ("alpha_s", 4), ("Gme", 5), ("a0", 6), ("a1", 7), ("a2", 8),
                        ("sigma_ow", 9), ("eta_1", 10), ("eta_2", 11)):
            setattr(s, name, float(F32(self.scal[i])))
        s.time_step, s.time_step_out = float(cfg.time_step()), float(cfg.time_step_out())
        s.Ts = float(cfg.Ts())
        s.dt_min, s.dt_max = float(F32(cfg.cuda_min_time_step)), float(F32(cfg.cuda_max_time_step))
        s.jacobi_fast, s.jacobi_slow, s.max_outer = 2, 20, 10
        s.red_lanes, s.jacobi_mode, s.max_substeps_per_sample = 32, 0, 1 << 20
        s.learned_every = 1
        return s

    def step(self, gi: int, cores: int) -> float:
        """One bounded sample: group gi's noise-only reference interval and its
        first m tested intervals, m the fewest that give every host thread a
        BM block (at most the group's 10).  Input generation, BM (threads
        across blocks), IHC/lambda and the JNDs of the m intervals; returns
        the audio seconds simulated."""
        from cochlearmodel_gb300.model import RunConfig
        from cochlearmodel_gb300.pipeline import ProfileSweep
        orc = self.orc
        sp = self.specs[gi]
        full = sp["sweep"]
        N, D = self.batch.block_nodes_for(sp["length"], self.block_target, self.Fs)
        m = max(1, min(len(full.powers), -(-cores // D) - 1))
        sweep = ProfileSweep(frequencies=full.frequencies, powers=list(full.powers[:m]),
                             noises=full.noises, calculate_jnd=True)
        prof, _, ref_of = sweep.build()
        n_int, L = len(prof), N * D
        cfg = RunConfig(Fs=self.Fs, Time_Block_Length=N / self.Fs, Decouple_Filter=D,
                        Time_Blocks=n_int * D, Overlap_Time=self.overlap_time)
        noise = np.zeros(L, np.float32)
        nz = np.asarray(sp["noise"], np.float32)[:L]
        noise[:len(nz)] = nz
        p1 = cfg.total_time_nodes_p1()
        rows = p1 + 4
        # input generation (CudaGenerateInputFromProfile restated)
        pt = np.stack([prof["dA"], prof["Wn"], prof["frequency"]], 1)
        x = np.zeros(rows, np.float32)
        x[:n_int * L] = orc.input_gen(pt, noise, L, 0, float(self.Fs), 0.0, 1.0, 1.0).ravel()
        # BM over the reference block partition
        st, of, en = orc.block_partition(cfg.Time_Blocks, p1, cfg.calc_overlap_nodes(), D)
        units = np.zeros(cfg.Time_Blocks, orc.UNIT_DTYPE)
        units["start"], units["out_first"], units["end"] = st, of, en
        units["mtt"], units["mmspt"] = np.float32(1e-10), np.float32(1e-15)
        v, _, _ = orc.bm_run(self.secp, self.gamma, self.scalars(cfg), units, x, rows,
                             threads=cores)
        # IHC / lambda in the reference's mixed precision
        fr = self.ihc.reference_frame(cfg)[0]
        nv = self.nerve
        _, lam = orc.ihc_lambda(v[:int(fr["rows"])], int(fr["seg"]), int(fr["frdp"]),
                                int(fr["total"]), int(fr["lam_rows"]), self.ac, self.dc,
                                nv.scale, nv.eta_AC, nv.eta_DC, self.dmg, nv.aihc(),
                                np.asarray(nv.spontRate, np.float32), nv.Lambda_SAT, mode=0)
        # JND Fisher sums in the reference's float arithmetic, then dB
        head, length = self.win.nodes(self.Fs, L)
        ra, ai = orc.jnd(lam, n_int, L, head, length, prof["dA"], ref_of, nv.nihc(),
                         np.asarray(nv.W, np.float32), float(self.Fs), 0.2 * self.Fs,
                         fp64=False)
        for k in range(n_int):
            if ref_of[k] != k:
                orc.jnd_db(ra[:, k].sum())
                orc.jnd_db(ai[:, k].sum())
        return n_int * L / self.Fs


def ref_cpu_timed(ref, steps, warmup, cores):
    """Times `steps` bounded sample steps of the CPU sweep after `warmup`
    (RefSweepCPU.step), the groups taken in turn.  Returns (audio-s/s, mean
    step ms, description)."""
    t_sum = a_sum = 0.0
    for i in range(warmup + steps):
        t0 = time.perf_counter()
        audio = ref.step(i % ref.n_groups, cores)
        dt = time.perf_counter() - t0
        if i >= warmup:
            t_sum += dt
            a_sum += audio
    value = a_sum / t_sum
    desc = (f"{steps} steps, each one JND-sweep group's noise-only reference interval and "
            f"its first tested intervals (enough for a BM block per thread), groups in "
            f"turn ({a_sum:.3f} audio-s in all): input generation, BM (FP32, reference "
            f"schedule), IHC/lambda (reference mixed precision), JND (reference float "
            f"arithmetic); {cores} threads, {t_sum:.1f} s")
    return value, t_sum / steps * 1000.0, desc


# ----------------------------------------------------------------------------
# plain single-signal arm (the same kernels, one signal per launch)
# ----------------------------------------------------------------------------
def plain_single_signal(run, device, n_sample=12):
    """Each sampled signal is solved alone -- its blocks as one BM launch, then
    its IHC/lambda -- as a single-signal solver does; audio-s/s over the sample."""
    import torch
    from cochlearmodel_gb300 import batch
    from cochlearmodel_gb300.pipeline import ProfileSweep
    if run.kind != "jnd_sweep":
        return None
    rng = np.random.default_rng(1)
    picks = rng.choice(len(run.groups), size=min(n_sample, len(run.groups)), replace=False)
    tot_ms = tot_audio = 0.0
    stream = torch.cuda.current_stream(device)
    for gi in picks:
        g = run.groups[gi]
        p = g.prof[0]
        noise_db = 1111.0 if p["Wn"] == 0 else 20 * math.log10(p["Wn"] / (10 * 2e-5))
        spec = [dict(length=g.L, noise=g.noise,
                     sweep=ProfileSweep(frequencies=[float(p["frequency"])],
                                        powers=[20 * math.log10(p["dA"] / (10 * 2e-5))],
                                        noises=[noise_db]))]
        one = batch.BatchSweep(device, spec, mv=run.mv)
        one.sc.controller, one.sc.arith = run.sc.controller, run.sc.arith
        for _ in range(2):
            one.generate_input()
            one.solve_bm()
            one.ihc_lambda()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(device)
        a.record(stream)
        one.generate_input()
        one.solve_bm()
        one.ihc_lambda()
        b.record(stream)
        torch.cuda.synchronize(device)
        tot_ms += a.elapsed_time(b)
        tot_audio += one.audio_seconds
        del one
    return {"value": tot_audio / (tot_ms / 1000.0), "unit": UNIT,
            "sample": f"{len(picks)} signals, each solved alone (its blocks in one launch)"}


# ----------------------------------------------------------------------------
# arms
# ----------------------------------------------------------------------------
def run_reference(args, rank, world):
    """The path on the host cores through the oracle only (RefSweepCPU): the
    reference ships no runnable CPU path of its own.  Rank 0 alone runs it."""
    if rank != 0:
        return None
    if args.workload != "jnd_sweep":
        return {"impl": "reference", "unavailable": "the host-core arm is built for the "
                                                    "default workload (jnd_sweep)"}
    if args.bm_kernel != 17:
        return {"impl": "reference", "unavailable": "the host-core arm evaluates kernel 17's "
                                                    "semantics (--bm-kernel 17)"}
    cores = os.cpu_count() or 1
    ref = RefSweepCPU(n_seeds=args.n_seeds)
    value, ms, desc = ref_cpu_timed(ref, args.steps, args.warmup, cores)
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": base_config("jnd_sweep", 66 * args.n_seeds, ref.units_total,
                                  ref.audio_seconds, args.jacobi),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": desc},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def base_config(kind, signals, units, audio, jacobi, bm_kernel=17):
    """The workload description both arms print (the GPU arm adds its details)."""
    if bm_kernel == 0:
        sem = ("BMOHC_NEW_kernel (the reference default, Run_Fast_BM_Calculation 0) in the "
               "reference's operation order, reference schedule (20/2 Jacobi sweeps)")
    elif jacobi == "reference":
        sem = "kernel 17, reference schedule (20/2 Jacobi sweeps)"
    else:
        sem = f"tolerance mode 1e-6, {jacobi} guess"
    return {"workload": kind, "signals": signals, "units": units, "audio_s_per_step": audio,
            "fs": 100000, "bm_semantics": sem}


def run_ours(args, rank, world, device):
    import torch
    from cochlearmodel_gb300 import native

    run = make_workload(args.workload, device, args.n_freq, args.n_seeds, args.n_signals)
    set_jacobi(run, args.jacobi, device)
    if args.bm_kernel == 0:
        # BMOHC_NEW_kernel's fault-count controller in the reference's operation
        # order (as model.bm_scalars sets it for Run_Fast_BM_Calculation 0); it
        # runs one launch shape of its own
        run.sc.controller = run.sc.arith = 1
    tuning = None
    if (args.tune != "off" and hasattr(run, "tune") and args.jacobi == "reference"
            and args.bm_kernel == 17):
        choice, source = run.tune(use_cache=args.tune == "cache")
        tuning = {"bm_shape": choice.bm_shape, "ihc_run": choice.ihc_run, "source": source}
        args.shape = choice.bm_shape
    else:
        native.check(native.load().cgb_bm_set_launch_shape(args.shape), "launch shape")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)
    stream = torch.cuda.current_stream(device)

    # warm-up with per-stage device times (eager), then capture the step
    stage_ms = {}
    for _ in range(args.warmup):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(len(stages(run)) + 1)]
        ev[0].record(stream)
        for i, (_, fn) in enumerate(stages(run)):
            fn()
            ev[i + 1].record(stream)
        flush.fill_(1.0)
        torch.cuda.synchronize(device)
        stage_ms = {nm: ev[i].elapsed_time(ev[i + 1]) for i, (nm, _) in enumerate(stages(run))}
    stats = run.d_stats.cpu().numpy().view(native.STATS_DTYPE).reshape(-1)
    flops = bm_flops(stats)
    lib = native.load()
    a0 = lib.cgb_kernel_launch_count()
    run.step()
    torch.cuda.synchronize(device)
    per_step_launches = lib.cgb_kernel_launch_count() - a0
    use_graph = not args.no_graph and hasattr(run, "capture")
    if use_graph:
        run.capture()
        torch.cuda.synchronize(device)
    step = run.replay if use_graph else run.step

    clocks = ClockSampler(device.index if device.index is not None else 0)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(device)
    clocks.start()
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
    t_total = max_over_ranks(sum(a.elapsed_time(b) for a, b in ev) / 1000.0, world)
    value = job_rate(run.audio_seconds, args.steps, world, t_total)

    # e2e: inputs in from pinned host memory (profile tables, or the samples of
    # the mixed batch), the path, results back to pinned host memory (velocity
    # and the three lambda planes; for the mixed batch the Fisher sums and
    # failure flags), through the C ABI
    if run.kind == "mixed_batch":
        tables, h_tables = [run.d_in], [run.h_in]
        outs = [run.d_FRA, run.d_FAI, run.d_failed]
    else:
        tables = [pg["d_prof"] for pg in run.per_group] if run.kind == "jnd_sweep" \
            else [run.d_prof]
        h_tables = [t.cpu().pin_memory() for t in tables]
        outs = [run.d_v, run.d_lam]
    h_outs = [torch.empty(o.shape, dtype=o.dtype).pin_memory() for o in outs]
    e_steps = max(1, args.steps // 2)
    e_ms = 0.0
    overlapped = hasattr(run, "step_host")
    if overlapped:  # the JND sweep overlaps the result copies with compute
        run.step_host(h_tables, h_outs[0], h_outs[1])  # uploads its chunk tables
    for i in range(e_steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(device)
        a.record(stream)
        if overlapped:
            run.step_host(h_tables, h_outs[0], h_outs[1])
        else:
            for d_t, h_t in zip(tables, h_tables):
                d_t.copy_(h_t, non_blocking=True)
            run.step()
            for h_o, d_o in zip(h_outs, outs):
                h_o.copy_(d_o, non_blocking=True)
        b.record(stream)
        torch.cuda.synchronize(device)
        e_ms += a.elapsed_time(b)
        flush.fill_(float(i))
    e2e = job_rate(run.audio_seconds, e_steps, world, max_over_ranks(e_ms / 1000.0, world))

    plain = plain_single_signal(run, device) \
        if rank == 0 and not args.no_plain and run.kind != "mixed_batch" else None
    accuracy = None
    if rank == 0 and run.kind == "jnd_sweep" and args.jacobi == "reference" \
            and not args.no_accuracy:
        t_acc = time.perf_counter()
        run.step()
        torch.cuda.synchronize(device)
        accuracy = accuracy_record(run)
        accuracy["seconds"] = time.perf_counter() - t_acc

    peaks, peak_kind = measured_peaks()
    clock_mhz = peaks.get("sm_max_mhz", 2070.0)
    n_sm = torch.cuda.get_device_properties(device).multi_processor_count
    fp32_peak = 2.0 * 128 * n_sm * clock_mhz * 1e6 / 1e12
    achieved = flops / (stage_ms["bm_solver"] / 1000.0) / 1e12
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_total / args.steps * 1000.0,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": base_config(run.kind, n_signals(run), len(run.units), run.audio_seconds,
                              args.jacobi, args.bm_kernel),
        "details": {"l2": "flushed between timed steps (256 MB write)",
                    "path": " -> ".join(nm for nm, _ in stages(run)),
                    "cuda_graph": use_graph, "launch_shape": args.shape, "stage_ms": stage_ms,
                    "autotune": tuning,
                    "value_is": "the batched solver with the reference's fixed Jacobi "
                                "schedule; the learned warm start is measured in 'learned'"
                    if args.jacobi == "reference" else f"--jacobi {args.jacobi}"},
        "gpu_launches": int(per_step_launches * args.steps),
        "e2e": {"value": e2e, "unit": UNIT,
                "h2d_bytes_per_step": int(sum(t.numel() * t.element_size() for t in h_tables)),
                "d2h_bytes_per_step": int(sum(o.numel() * o.element_size() for o in h_outs))},
        "roofline": {"bound": "fp32", "kernel": "bm_warp_kernel", "achieved": achieved,
                     "peak": fp32_peak, "unit": "TFLOP/s", "frac": achieved / fp32_peak,
                     "traffic": BM_TRAFFIC_PER_UNIT * len(run.units),
                     "peak_source": f"2 x 128 FP32 lanes x {n_sm} SMs x sm_max_mhz "
                                    f"({peak_kind} MEASURED_PEAKS.json)"},
        "clocks": clk,
    }
    if plain is not None:
        line["plain_single_signal"] = plain
        line["speedup_vs_plain"] = value / plain["value"]
    if accuracy is not None:
        line["max_rel_vs_fp64"] = accuracy
    if (rank == 0 and run.kind == "jnd_sweep" and args.jacobi == "reference"
            and args.bm_kernel == 17 and not args.no_learned):
        line["learned"] = learned_record(device, run.mv)
    return line, run


def accuracy_record(run):
    """The step's error against the FP64 method on a bounded sample: the
    shortest group of a batched JND sweep (a noise-only reference interval and
    ten tones, all its blocks), from the run's device results of its last step.
    Per interval:
    - velocity against the FP64 oracle with the same step controller and
      Jacobi schedule, and against the FP64 oracle with an exact tridiagonal
      solve (the Jacobi schedule's truncation added);
    - lambda (the worst of the three planes) against the FP64 IHC/lambda of
      the FP64 velocity, the whole chain up to lambda;
    - JND: |dB difference| of rate and all-info against the FP64 Fisher sums
      of that lambda (tested intervals).
    Errors are max |a - b| / max |b| over the interval's rows, and the
    relative L2 norm |a - b|_2 / |b|_2.  The max measure of lambda is set by
    the few rows where the IHC pre-potential crosses zero: the IHC stage
    takes log10 of the rectified value plus 1e-20, so a small velocity
    difference there moves the log between -20 and a finite value.  The
    oracle runs on the host cores."""
    from oracle import oracle as orc
    gi = int(np.argmin([g.L for g in run.groups]))
    g, fr = run.groups[gi], run.frames[gi]
    rows = g.cfg.total_time_nodes_p1() + 4
    units = run.units[run.units["out_base"] == g.v_row0].copy()
    units["in_base"] -= g.in_base
    units["out_base"] -= g.v_row0
    x = run.d_in[g.in_base:g.in_base + rows].cpu().numpy()
    v = run.d_v[g.v_row0:g.v_row0 + rows].cpu().numpy()
    n_lam = int(fr["lam_rows"])
    lam = run.d_lam[:, g.lam_row0:g.lam_row0 + n_lam].cpu().numpy()
    rate_db, ai_db = run.jnd_db()[gi][:2]
    gamma = run.d_gamma.cpu().numpy()
    secp = run.mv.section_params()
    cores = os.cpu_count() or 1

    def max_rel(a, b):
        return float(np.abs(np.asarray(a, np.float64) - b).max() / max(np.abs(b).max(), 1e-300))

    def rel_l2(a, b):
        b = np.asarray(b, np.float64)
        return float(np.linalg.norm(np.asarray(a, np.float64) - b) /
                     max(np.linalg.norm(b), 1e-300))

    v64, _, _ = orc.bm_run(secp, gamma, run.sc, units, x, rows, fp64=True, threads=cores)
    vex, _, _ = orc.bm_run(secp, gamma, run.sc, units, x, rows, fp64=True, threads=cores,
                           jacobi_mode=1)
    st, nv = run.ihc, run.nerve
    _, lam64 = orc.ihc_lambda(v64[:int(fr["rows"])], int(fr["seg"]), int(fr["frdp"]),
                              int(fr["total"]), n_lam, st.ac.astype(np.float64),
                              st.dc.astype(np.float64), nv.scale, nv.eta_AC, nv.eta_DC,
                              st.dmg_host[int(fr["ihc_profile"])].astype(np.float64), nv.aihc(),
                              np.asarray(nv.spontRate, np.float32), nv.Lambda_SAT, mode=1)
    n_int = len(g.prof)
    head, length = run.jnd_win.nodes(g.cfg.Fs, g.L)
    ra, ai = orc.jnd(lam64, n_int, g.L, head, length, g.prof["dA"], g.ref_of, nv.nihc(),
                     np.asarray(nv.W, np.float32), float(g.cfg.Fs),
                     run.jnd_win.delta_alpha_time_factor * g.cfg.Fs, fp64=True)
    tested = g.ref_of != np.arange(n_int)
    jnd_err = np.zeros(n_int)
    for got, ref in ((rate_db, ra), (ai_db, ai)):
        want = np.array([orc.jnd_db(ref[:, i].sum()) for i in range(n_int)])
        jnd_err[tested] = np.maximum(jnd_err[tested], np.abs(got[tested] - want[tested]))
    per = []
    for k in range(n_int):
        r = slice(k * g.L, (k + 1) * g.L)
        dA = float(g.prof["dA"][k])
        per.append({"signal": f"{20 * math.log10(dA / (10 * 2e-5)):.0f} dB tone"
                    if tested[k] else "noise only",
                    "velocity": max_rel(v[r], v64[r]), "velocity_rel_l2": rel_l2(v[r], v64[r]),
                    "velocity_vs_exact_solve": max_rel(v[r], vex[r]),
                    "lambda": max(max_rel(lam[j, r], lam64[j, r]) for j in range(3)),
                    "lambda_rel_l2": max(rel_l2(lam[j, r], lam64[j, r]) for j in range(3)),
                    "jnd_db_abs": float(jnd_err[k]) if tested[k] else None})
    worst = {k: max(p[k] for p in per)
             for k in ("velocity", "velocity_rel_l2", "velocity_vs_exact_solve", "lambda",
                       "lambda_rel_l2")}
    return {"sample": f"the shortest JND-sweep group ({n_int} intervals of {g.L} samples, "
                      f"{len(units)} blocks), the run's own results; per interval "
                      f"max |a - b| / max |b| and |a - b|_2 / |b|_2 over its rows "
                      f"(lambda: the worst plane); the top level is the worst interval",
            **worst, "jnd_db_abs": float(jnd_err.max()), "per_interval": per,
            "oracle_threads": cores}


def learned_record(device, mv, n_groups=3):
    """The learned warm start measured in the same run: the first n_groups
    groups of the JND sweep, batched, with the reference's fixed Jacobi
    schedule and with the tolerance-mode solve started from the network's
    guess; audio-s/s of the whole path, Jacobi sweeps per time step, and the
    learned velocity's max-rel from the fixed schedule's (max |a-b| / max |b|
    over each signal's rows, worst signal)."""
    import torch
    from cochlearmodel_gb300 import batch, model, native, warmstart
    spec = batch.jnd_sweep_spec(n_seeds=4)[:n_groups]
    out = {}
    runs = {}
    for name in ("reference_schedule", "learned"):
        b = batch.BatchSweep(device, spec, mv=mv)
        if name == "learned":
            b.sc = model.tolerance_mode(b.sc, guess=2)
            net = warmstart.WarmStartNet.load(warmstart.WEIGHTS, device)
            b.extras = net.extras()
        b.step()
        torch.cuda.synchronize(device)
        a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        b.step()
        e.record()
        torch.cuda.synchronize(device)
        st = b.d_stats.cpu().numpy().view(native.STATS_DTYPE).reshape(-1)
        out[name] = {"value": b.audio_seconds / (a.elapsed_time(e) / 1000.0), "unit": UNIT,
                     "sweeps_per_step": float(st["sweeps"].sum() / max(1, st["substeps"].sum()))}
        runs[name] = b
    v0 = runs["reference_schedule"].d_v.cpu().numpy()
    v1 = runs["learned"].d_v.cpu().numpy()
    worst = 0.0
    for g in runs["learned"].groups:
        n_int, L = len(g.prof), g.L
        for k in range(n_int):
            r = slice(g.v_row0 + k * L, g.v_row0 + (k + 1) * L)
            den = np.abs(v0[r]).max()
            if den > 0:
                worst = max(worst, float(np.abs(v1[r].astype(np.float64) - v0[r]).max() / den))
    out["learned"]["max_rel_vs_reference_schedule"] = worst
    out["sample"] = (f"the first {n_groups} groups of the JND sweep "
                     f"({runs['learned'].audio_seconds:.3f} audio-s), batched, one step each "
                     f"after a warm-up step")
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="jnd_sweep",
                    choices=["jnd_sweep", "tone_sweep", "mixed_batch"])
    ap.add_argument("--n-signals", type=int, default=1024, help="mixed_batch signals")
    ap.add_argument("--jacobi", default="reference", choices=list(JACOBI),
                    help="pressure solve: reference schedule or tolerance-mode guess")
    ap.add_argument("--bm-kernel", type=int, default=17, choices=[17, 0],
                    help="BM semantics (Run_Fast_BM_Calculation): 17 kernel 17 in the own "
                         "order (default), 0 the reference default BMOHC_NEW_kernel in the "
                         "reference's operation order")
    ap.add_argument("--cpu-seconds", type=float, default=20.0,
                    help="tone_sweep: seconds of the CPU baseline sample")
    ap.add_argument("--cpu-steps", type=int, default=4,
                    help="jnd_sweep: sample steps of the CPU baseline")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the max_rel_vs_fp64 record (FP64 oracle on one group)")
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--shape", type=int, default=0, help="BM kernel launch shape (--tune off)")
    ap.add_argument("--tune", default="cache", choices=["cache", "search", "off"],
                    help="launch choices: cached autotuner result (searched when absent), "
                         "a fresh search, or --shape with the automatic IHC run length")
    ap.add_argument("--n-freq", type=int, default=64,
                    help="tone_sweep: tones per level (64 = configuration 2)")
    ap.add_argument("--n-seeds", type=int, default=4,
                    help="jnd_sweep: noise seeds (4 = 264 signals)")
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
    if rank == 0 and world == 1 and not args.no_cpu_baseline and run.kind != "mixed_batch":
        if run.kind == "jnd_sweep":
            cores = os.cpu_count() or 1
            v, _, sample = ref_cpu_timed(RefSweepCPU(n_seeds=args.n_seeds), args.cpu_steps,
                                         1, cores)
        else:
            v, cores, sample = cpu_sample(run, target_s=args.cpu_seconds)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": sample}
    if world > 1:
        torch.distributed.destroy_process_group()
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
