"""Seeded BM test cases shared by the CPU and GPU tests.

Each case returns (cfg, sc, gamma[P,256], units, input, out_rows)."""
from __future__ import annotations

import math

import numpy as np

from cochlearmodel_gb300 import model, native


def tone(n, f, amp, Fs, head=0):
    """A pure tone sampled like CudaGenerateInputFromProfile (float-pi phase)."""
    two_pi = float(np.float32(2 * np.float32(math.pi)))
    t = (np.arange(n, dtype=np.float64) - head) / float(np.float32(Fs))
    return (amp * np.cos(two_pi * f * t)).astype(np.float32)


def cfg1_slice(mv, ms=5.0, db=60.0, freq=1000.0):
    """Config 1 (1 kHz, 60 dB SPL, healthy, one block) truncated to `ms`."""
    cfg = model.RunConfig(Time_Block_Length=ms / 1000.0, Time_Blocks=1, Decouple_Filter=1)
    sc = model.bm_scalars(cfg, mv)
    units = model.reference_units(cfg)
    n = cfg.total_time_nodes_p1() + 4
    x = model.sine_input(n, freq, model.spl_to_amplitude(db), cfg.Fs)
    return cfg, sc, cfg.gamma()[None], units, x, n


def decoupled_sweep(mv, n_signals=2, decouple=2, block_ms=2.0, overlap_ms=1.0, seed=0):
    """A profile-style run: n_signals tones back to back, each Decouple_Filter
    blocks long, partitioned like BMOHCNewKernel."""
    rng = np.random.default_rng(seed)
    cfg = model.RunConfig(Time_Block_Length=block_ms / 1000.0, Time_Blocks=n_signals * decouple,
                          Decouple_Filter=decouple, Overlap_Time=overlap_ms / 1000.0)
    sc = model.bm_scalars(cfg, mv)
    units = model.reference_units(cfg)
    N = cfg.calc_time_block_nodes()
    L = N * decouple
    n = cfg.total_time_nodes_p1() + 4
    x = np.zeros(n, np.float32)
    for i in range(n_signals):
        f = float(125.0 * 64 ** rng.uniform())
        db = float(rng.choice([20, 40, 60, 80, 100]))
        x[i * L:(i + 1) * L] = tone(L, f, model.spl_to_amplitude(db), cfg.Fs)
    return cfg, sc, cfg.gamma()[None], units, x, n


def hearing_loss_gamma():
    """OHC profile 0.5 on sections 0-127 ramping linearly to 0.05 at 255."""
    g = np.full(256, 0.5, np.float32)
    g[128:] = np.linspace(0.5, 0.05, 129, dtype=np.float64)[1:].astype(np.float32)
    return g


def framed_batch(mv, lengths_ms, seed=0, block_ms=None, overlap_ms=2.0, profiles=None):
    """Independent signals in separate frames (one frame per signal), each
    split into blocks like a Decouple_Filter run of its own; per-signal OHC
    profiles.  Returns the input with 4 samples of zero padding per frame."""
    rng = np.random.default_rng(seed)
    cfg = model.RunConfig()
    sc = model.bm_scalars(cfg, mv)
    Fs = cfg.Fs
    ov = int(round(overlap_ms * Fs / 1000))
    units, xs, in_base, out_base = [], [], 0, 0
    P = profiles if profiles is not None else np.stack([cfg.gamma(), hearing_loss_gamma()])
    for i, ms in enumerate(lengths_ms):
        L = int(round(ms * Fs / 1000))
        bl = L if block_ms is None else int(round(block_ms * Fs / 1000))
        nb = max(1, L // bl)
        bl = L // nb
        frame_len = L + ov + 4
        f = float(125.0 * 64 ** rng.uniform())
        db = float(rng.choice([20, 40, 60, 80, 100]))
        x = np.zeros(frame_len, np.float32)
        x[:L] = tone(L, f, model.spl_to_amplitude(db), Fs)
        for b in range(nb):
            # block b owns [b*bl, (b+1)*bl) and warms up from zero state over
            # the `ov` samples before it
            s = b * bl
            e = L if b == nb - 1 else (b + 1) * bl
            rec = np.zeros(1, native.UNIT_DTYPE)
            rec["in_base"], rec["out_base"] = in_base, out_base
            rec["start"] = max(0, s - ov)
            rec["out_first"] = s
            rec["end"] = e
            rec["profile"] = i % len(P)
            rec["mtt"], rec["mmspt"] = np.float32(1e-10), np.float32(1e-15)
            units.append(rec)
        xs.append(x)
        in_base += frame_len
        out_base += frame_len
    units = np.concatenate(units)
    return cfg, sc, np.ascontiguousarray(P, np.float32), units, np.concatenate(xs), out_base
