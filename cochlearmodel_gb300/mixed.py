"""Large mixed batch: many signals of different lengths, types and hearing
profiles through the whole path in one step.

Each signal is its own group (one reference Run_Cuda profile run,
src/solver.cpp:234-962): its test interval and, for a tone in noise, the
noise alone as its reference interval, partitioned into Decouple_Filter
blocks of ~10 ms with the reference's default 5 ms overlap.  Every signal
carries its own OHC profile (a row of the gamma table, the unit's profile)
and IHC profile (the frame's damage row).  Pure tones and harmonic complexes
are referenced to silence: a silent input leaves the velocity at zero (every
forcing term of the BM/OHC equations vanishes from the zero state) and
lambda at the spontaneous rates whatever the profiles, so one silent group
as long as the longest signal serves all of them; its velocity rows are
left at zero rather than solved, and its lambda comes from the IHC kernel.

The BM units of all groups go into one table drained by the persistent
kernel (longest first), the IHC frames into one launch, the JND intervals
into one launch; the step can be captured in a CUDA graph.  The input
samples are produced on the host (harmonic complexes and noise are not
profile tones) and uploaded each step.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import native
from .batch import block_nodes_for
from .ihc import IHCStage, NerveConfig, reference_frame
from .model import ModelVectors, RunConfig, bm_scalars, reference_units, spl_to_amplitude
from .pipeline import JNDWindow

KINDS = ("tone", "complex", "tone_in_noise")


def smooth_walk(rng: np.random.Generator, lo: float, hi: float, n: int = 256,
                win: int = 16) -> np.ndarray:
    """A smooth random walk over the sections mapped onto [lo, hi]."""
    w = np.cumsum(rng.normal(size=n + win - 1))
    w = np.convolve(w, np.ones(win) / win, mode="valid")[:n]
    w = (w - w.min()) / max(float(w.max() - w.min()), 1e-12)
    return (lo + (hi - lo) * w).astype(np.float32)


@dataclass
class MixedSignal:
    kind: str
    test: np.ndarray            # float32[L]
    reference: np.ndarray | None  # noise alone (tone in noise) or None (silence)
    dA: float                   # amplitude the JND is taken against
    ohc: np.ndarray             # float32[256] in [0, 0.5]
    ihc: np.ndarray             # float32[256] in [5, 8]
    meta: dict


def mixed_signal(rng: np.random.Generator, n: int, fs: float) -> MixedSignal:
    """One seeded signal: a tone (125 Hz - 8 kHz), a 3-10-harmonic complex
    (f0 80-400 Hz, random phases, 4-16 Hz AM) or a tone in white Gaussian
    noise (0-40 dB SPL), at 20-100 dB SPL."""
    t = np.arange(n) / fs
    kind = KINDS[int(rng.integers(0, 3))]
    db = float(rng.uniform(20.0, 100.0))
    amp = spl_to_amplitude(db)
    ref = None
    if kind == "complex":
        h = int(rng.integers(3, 11))
        f0 = float(80.0 * 5.0 ** rng.uniform())
        ph = rng.uniform(0, 2 * np.pi, h)
        x = sum(np.sin(2 * np.pi * f0 * (k + 1) * t + ph[k]) for k in range(h))
        fm = float(rng.uniform(4.0, 16.0))
        x = x * (1.0 - 0.5 * (1.0 - np.cos(2 * np.pi * fm * t + rng.uniform(0, 2 * np.pi))))
        x = x * (amp / np.sqrt(2.0)) / max(float(np.sqrt(np.mean(x * x))), 1e-30)
        meta = {"f0": f0, "harmonics": h, "am_hz": fm, "db": db}
    else:
        f = float(125.0 * 64.0 ** rng.uniform())
        x = amp * np.sin(2 * np.pi * f * t + rng.uniform(0, 2 * np.pi))
        meta = {"f": f, "db": db}
        if kind == "tone_in_noise":
            ndb = float(rng.uniform(0.0, 40.0))
            ref = (rng.normal(size=n) * spl_to_amplitude(ndb) / np.sqrt(2.0)).astype(np.float32)
            x = x + ref
            meta["noise_db"] = ndb
    return MixedSignal(kind, x.astype(np.float32), ref, amp, smooth_walk(rng, 0.0, 0.5),
                       smooth_walk(rng, 5.0, 8.0), meta)


def mixed_batch_spec(n_signals: int = 1024, seed: int = 0, min_ms: float = 10.0,
                     max_ms: float = 1000.0, fs: int = 100000, block_target: int = 1000):
    """Signals with lengths log-uniform in [min_ms, max_ms] (whole blocks of
    ~block_target samples)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_signals):
        ms = float(np.exp(rng.uniform(np.log(min_ms), np.log(max_ms))))
        N, D = block_nodes_for(int(round(ms * fs / 1000.0)), block_target, fs)
        out.append((N, D, mixed_signal(rng, N * D, fs)))
    return out


class MixedBatch:
    """Device buffers and launches of a mixed batch (see the module text)."""

    def __init__(self, device, spec, mv=None, nerve=None, jnd=None, ac_taps=None,
                 overlap_time=0.005, Fs=100000):
        import torch
        from .solver import BMSolver, units_to_device
        self.torch = torch
        self.device = torch.device(device)
        self.lib = native.load()
        self.mv = mv or ModelVectors.build()
        self.nerve = nerve or NerveConfig()
        self.jnd_win = jnd or JNDWindow()
        self.Fs = Fs
        self.signals = [s for _, _, s in spec]
        n = len(spec)
        max_len = max(N * D for N, D, _ in spec)
        # the silent reference group: one block, as long as the longest signal
        groups = [(N, D, [s.test] + ([s.reference] if s.reference is not None else []), i)
                  for i, (N, D, s) in enumerate(spec)]
        Ns, Ds = block_nodes_for(max_len, 1000, Fs)
        groups.append((Ns, Ds, [np.zeros(Ns * Ds, np.float32)], n))
        ohc = np.stack([s.ohc for s in self.signals] + [self.signals[0].ohc])
        ihc_vec = np.stack([s.ihc for s in self.signals] + [self.signals[0].ihc])
        units, frames, inputs = [], [], []
        self.group_rows = []  # (lam_row0, L, n_int) per group
        in_base = v_row0 = lam_row0 = 0
        for N, D, intervals, prof in groups:
            L = N * D
            cfg = RunConfig(Fs=Fs, Time_Block_Length=N / Fs, Decouple_Filter=D,
                            Time_Blocks=len(intervals) * D, Overlap_Time=overlap_time)
            assert cfg.calc_time_block_nodes() == N
            rows = cfg.total_time_nodes_p1() + 4
            x = np.zeros(rows, np.float32)
            for k, iv in enumerate(intervals):
                x[k * L:(k + 1) * L] = iv
            inputs.append(x)
            if prof < n:  # the silent group is not solved: its velocity is zero
                units.append(reference_units(cfg, in_base=in_base, out_base=v_row0,
                                             profile=prof))
            frames.append(reference_frame(cfg, v_row0=v_row0, lam_row0=lam_row0,
                                          ihc_profile=prof))
            self.group_rows.append((lam_row0, L, len(intervals)))
            in_base += rows
            v_row0 += rows
            lam_row0 += int(frames[-1]["lam_rows"][0])
        self.cfg0 = RunConfig(Fs=Fs, Overlap_Time=overlap_time)
        self.sc = bm_scalars(self.cfg0, self.mv)
        units = np.concatenate(units)
        order = np.argsort(-(units["end"] - units["start"]), kind="stable")
        self.units = units[order]
        self.frames = np.concatenate(frames)
        self.h_in = torch.from_numpy(np.concatenate(inputs)).pin_memory()
        self.in_len, self.v_rows, self.lam_rows = int(self.h_in.numel()), v_row0, lam_row0
        self.bm = BMSolver(self.device, self.mv)
        self.bm.check_units(self.units, len(ohc), self.in_len, self.v_rows)
        d = self.device
        self.d_units = units_to_device(self.units, d)
        self.d_gamma = torch.from_numpy(np.ascontiguousarray(ohc, np.float32)).to(d)
        self.d_in = self.h_in.to(d)
        self.d_v = torch.zeros((self.v_rows, 256), dtype=torch.float32, device=d)
        self.d_failed = torch.zeros(self.v_rows, dtype=torch.int32, device=d)
        self.d_stats = torch.zeros((len(self.units), native.STATS_DTYPE.itemsize),
                                   dtype=torch.uint8, device=d)
        self.d_lam = torch.zeros((3, self.lam_rows, 256), dtype=torch.float32, device=d)
        self.ihc = IHCStage(d, self.nerve, ihc_vec, ac_taps, Fs)
        sc = self.ihc.scratch(len(self.frames))
        native.check(self.lib.cgb_ihc_lambda_upload_dev(
            native.ptr(self.frames), len(self.frames), native.ptr(self.ihc.ac), len(self.ihc.ac),
            native.ptr(self.ihc.dc), len(self.ihc.dc), C.byref(self.ihc.prm), self.v_rows,
            self.lam_rows, len(ihc_vec), native.ptr(sc), int(sc.numel()), self._stream(None)),
            "cgb_ihc_lambda_upload_dev")
        # JND: every test interval with a non-empty window
        sil_row0 = self.group_rows[-1][0]
        ivs, self.jnd_of = [], np.full(n, -1, np.int64)
        for i, s in enumerate(self.signals):
            r0, L, n_int = self.group_rows[i]
            head, length = self.jnd_win.nodes(Fs, L)
            if length <= 0:
                continue
            ref_row = r0 + L + head if n_int == 2 else sil_row0 + head
            self.jnd_of[i] = len(ivs)
            ivs.append((r0 + head, ref_row, s.dA, length, len(ivs)))
        # longest windows first (each keeps its output slot): the kernel issues
        # the table in order, so the long intervals do not trail the launch
        iv = np.array(ivs, dtype=native.JND_INTERVAL_DTYPE)
        self.jnd_iv = iv[np.argsort(-iv["len"], kind="stable")]
        self.d_jnd_iv = torch.from_numpy(self.jnd_iv.view(np.uint8).copy()).to(d)
        m = max(1, len(ivs))
        self.d_FRA = torch.zeros((3, m), dtype=torch.float64, device=d)
        self.d_FAI = torch.zeros((3, m), dtype=torch.float64, device=d)
        self.W = np.asarray(self.nerve.W, np.float32)
        self.d_nihc = torch.from_numpy(self.nerve.nihc()).to(d)
        self.graph = None
        self.extras = None  # tolerance-mode extras (network weights), see solver.run_dev

    # ---------------------------------------------------------------------------
    @property
    def n_signals(self) -> int:
        return len(self.signals)

    @property
    def audio_seconds(self) -> float:
        """Duration of the test signals (references and silence excluded)."""
        return sum(len(s.test) for s in self.signals) / self.Fs

    @property
    def simulated_seconds(self) -> float:
        """Everything the BM solver simulates: tests and noise references."""
        return sum(L * k for _, L, k in self.group_rows[:-1]) / self.Fs

    def _stream(self, stream):
        s = stream if stream is not None else self.torch.cuda.current_stream(self.device)
        return C.c_void_p(s.cuda_stream)

    def solve_bm(self, stream=None):
        self.bm.run_dev(self.sc, self.d_gamma, self.d_units, len(self.units), self.d_in,
                        self.d_v, self.d_failed, self.d_stats, stream, extras=self.extras)

    def ihc_lambda(self, stream=None):
        sc = self.ihc.scratch(len(self.frames))
        native.check(self.lib.cgb_ihc_lambda_launch_dev(
            native.ptr(self.d_v), self.v_rows, native.ptr(self.frames), len(self.frames),
            native.ptr(self.ihc.ac), len(self.ihc.ac), native.ptr(self.ihc.dc), len(self.ihc.dc),
            C.byref(self.ihc.prm), native.ptr(self.ihc.dmg), int(self.ihc.dmg.shape[0]),
            native.ptr(self.ihc.aihc), native.ptr(self.d_lam), self.lam_rows, None,
            native.ptr(sc), int(sc.numel()), native.ptr(self.ihc.status), self._stream(stream)),
            "cgb_ihc_lambda_launch_dev")

    def jnd_sums(self, stream=None):
        if len(self.jnd_iv) == 0:
            return
        native.check(self.lib.cgb_jnd_batch_dev(
            native.ptr(self.d_lam), self.lam_rows, native.ptr(self.d_jnd_iv), len(self.jnd_iv),
            len(self.jnd_iv), native.ptr(self.d_nihc), native.ptr(self.W), float(self.Fs),
            self.jnd_win.delta_alpha_time_factor * self.Fs, native.ptr(self.d_FRA),
            native.ptr(self.d_FAI), None, self._stream(stream)), "cgb_jnd_batch_dev")

    def step(self, stream=None):
        self.solve_bm(stream)
        self.ihc_lambda(stream)
        self.jnd_sums(stream)

    def capture(self):
        torch = self.torch
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            self.step(s)
        torch.cuda.current_stream(self.device).wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            self.step(s)
        self.graph = g
        return g

    def replay(self):
        self.graph.replay()

    def jnd_db(self):
        """(rate dB, AI dB) per signal; NaN where the signal is shorter than
        the JND window."""
        n = len(self.jnd_iv)
        rate = np.full(self.n_signals, np.nan)
        ai = np.full(self.n_signals, np.nan)
        if n == 0:
            return rate, ai
        F_RA = np.ascontiguousarray(self.d_FRA.cpu().numpy()[:, :n])
        F_AI = np.ascontiguousarray(self.d_FAI.cpu().numpy()[:, :n])
        r, a = np.zeros(n), np.zeros(n)
        no_ref = np.full(n, -1, np.int32)  # ref_of[i] == i would mark a reference
        native.check(self.lib.cgb_jnd_final(native.ptr(F_RA), native.ptr(F_AI), n,
                                            native.ptr(no_ref), self.cfg0.SPLRef,
                                            self.jnd_win.max_db, native.ptr(r), native.ptr(a)),
                     "cgb_jnd_final")
        sel = self.jnd_of >= 0
        rate[sel] = r[self.jnd_of[sel]]
        ai[sel] = a[self.jnd_of[sel]]
        return rate, ai

