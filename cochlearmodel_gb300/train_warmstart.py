"""Trains the learned Jacobi warm start on the GPU and evaluates it.

    python -m cochlearmodel_gb300.train_warmstart --out weights.npz

1. Logs (state, pressure) records from the solver running the training
   signals (tones 125 Hz - 8 kHz and 3-10-harmonic AM complexes, 20-100 dB
   SPL; seeded) in tolerance mode with the extrapolated guess.
2. Prepares features and exact-pressure targets (FP64 tridiagonal solve).
3. Trains with the library's forward / backward / Adam kernels.
4. Evaluates on held-out seeds: Jacobi sweeps and outer iterations per step
   and simulated audio-s/s of the previous-step (0), extrapolated (1) and
   learned (2) guesses at the same tolerance, plus the reference schedule
   (fixed sweep counts), and the velocity difference between them.
Prints one JSON object.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np
import torch

from . import model
from . import warmstart as W
from .solver import BMSolver, units_to_device


def main(argv=None) -> dict:
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(W.WEIGHTS))
    ap.add_argument("--n-train", type=int, default=2000)
    ap.add_argument("--train-ms", type=float, default=20.0)
    ap.add_argument("--records", type=int, default=80000)
    ap.add_argument("--log-every", type=int, default=499)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=256)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--n-eval", type=int, default=64)
    ap.add_argument("--eval-ms", type=float, default=20.0)
    ap.add_argument("--seed", type=int, default=1234)
    ap.add_argument("--learned-every", type=int, nargs="*", default=[1, 4])
    a = ap.parse_args(argv)

    dev = torch.device("cuda:0")
    solver = BMSolver(dev)
    res: dict = {"n_train": a.n_train, "train_ms": a.train_ms, "tol": model.JACOBI_TOL}
    t0 = time.time()
    train_batch = W.signal_batch(a.n_train, a.train_ms, seed=a.seed)
    rec = W.log_records(solver, train_batch, cap=a.records, every=a.log_every)
    torch.cuda.synchronize()
    res["records"] = int(rec.shape[0])
    res["log_s"] = round(time.time() - t0, 2)

    net = W.WarmStartNet(dev, seed=a.seed)
    feat, target, nr = net.prepare(rec)
    net.s_out = W.fit_output_scale(target)
    net.pack()
    # hold out 5 % of the records to report the fit
    n = feat.shape[0]
    n_val = max(1, n // 20)
    t1 = time.time()
    hist = W.train(net, feat[n_val:], target[n_val:], a.steps, a.batch, a.lr, seed=a.seed,
                   log_every=max(1, a.steps // 10))
    torch.cuda.synchronize()
    res["train_s"] = round(time.time() - t1, 2)
    res["loss_history"] = [(s, round(l, 6)) for s, l in hist]
    with torch.no_grad():
        o = net.forward(feat[:n_val].contiguous())
        t = target[:n_val]
        res["val_mse"] = float(((net.s_out * o - t) ** 2).mean().item())
        res["val_mse_zero_guess"] = float((t ** 2).mean().item())
    res["s_out"] = net.s_out
    net.save(a.out)
    res["weights"] = str(a.out)

    ev = W.signal_batch(a.n_eval, a.eval_ms, seed=a.seed + 1)
    ref, ref_v = _reference(solver, ev)
    res["eval"] = {"signals": a.n_eval, "ms": a.eval_ms, "reference_schedule": ref}
    runs = {"previous": W.evaluate(solver, ev, 0, repeats=2),
            "extrapolated": W.evaluate(solver, ev, 1, repeats=2)}
    for k in a.learned_every:
        runs[f"learned_every_{k}"] = W.evaluate(solver, ev, 2, net=net, learned_every=k,
                                                repeats=2)
    base = runs["extrapolated"]["velocity"]
    for name, r in runs.items():
        res["eval"][name] = {
            "sweeps_per_step": round(r["sweeps_per_step"], 3),
            "iterations_per_step": round(r["iterations_per_step"], 3),
            "audio_s_per_s": round(r["audio_s_per_s"], 3),
            "ms": round(r["ms"], 3),
            "failed_samples": int(r["failed"].sum()),
            "max_rel_vs_extrapolated": W.max_rel(r["velocity"], base),
            "max_rel_vs_reference_schedule": W.max_rel(r["velocity"], ref_v),
        }
    print(json.dumps(res))
    return res


def _reference(solver: BMSolver, ev: W.SignalBatch):
    """The reference schedule (fixed sweep counts) on the same signals:
    (summary, velocity)."""
    sc = model.bm_scalars(ev.cfg, solver.mv)
    gamma = ev.cfg.gamma()[None]
    v, f, st = solver.run(sc, gamma, ev.units, ev.inp, ev.out_rows)
    d = solver.device
    g = torch.from_numpy(np.ascontiguousarray(gamma, np.float32)).to(d)
    u = units_to_device(ev.units, d)
    x = torch.from_numpy(ev.inp).to(d)
    out = torch.zeros((ev.out_rows, 256), dtype=torch.float32, device=d)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(2):
        solver.run_dev(sc, g, u, len(ev.units), x, out)
    e1.record()
    torch.cuda.synchronize(d)
    ms = e0.elapsed_time(e1) / 2
    sub = int(st["substeps"].sum())
    return {"sweeps_per_step": round(float(st["sweeps"].sum()) / sub, 3),
            "iterations_per_step": round(float(st["iterations"].sum()) / sub, 3),
            "audio_s_per_s": round(ev.audio_seconds / (ms / 1000.0), 3), "ms": round(ms, 3),
            "failed_samples": int(f.sum())}, v


if __name__ == "__main__":
    main()
