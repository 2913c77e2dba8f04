"""Autotuner for the launch choices that change speed but not results.

The reference hand-picks occupancy variants of its BM kernel
(TripleAggKernelLauncher<Occ>, include/cochlea.cuh:187-1011, dispatched at
src/cochlea.cu:1258-1435).  This module searches the equivalent choices of
this library on the workload and GPU at hand, and caches the winner:

- the BM launch shape (cgb_bm_set_launch_shape: warps per CTA, register bound,
  previous-step state in registers or shared memory);
- the IHC/lambda run length (cgb_ihc_set_run_length: consecutive tiles per CTA).

Every candidate gives the same results bit for bit (the search checks it); the
tile rows of the IHC kernel are fixed by the filters (the largest tile that fits
shared memory and holds the DC look-back), and the JND kernel's row groups set
its summation order, so neither is searched.

The cache is a JSON file (CGB_TUNE_CACHE, default cochlearmodel_gb300/_tune/
tuning.json) keyed by the device name, a hash of the library and a description
of the workload.
"""
from __future__ import annotations

import hashlib
import json
import os
from dataclasses import asdict, dataclass
from pathlib import Path
from typing import Callable, Sequence

from . import build, native

IHC_RUNS = (0, 8, 16, 32)  # 0: the automatic rule


@dataclass
class Choice:
    bm_shape: int = 0
    ihc_run: int = 0


def cache_path() -> Path:
    env = os.environ.get("CGB_TUNE_CACHE")
    return Path(env) if env else Path(__file__).resolve().parent / "_tune" / "tuning.json"


def library_hash() -> str:
    """First 16 hex digits of the SHA-256 of the built library."""
    h = hashlib.sha256()
    with open(build.lib_path(), "rb") as f:
        for chunk in iter(lambda: f.read(1 << 20), b""):
            h.update(chunk)
    return h.hexdigest()[:16]


def cache_key(device_name: str, workload: str, lib_hash: str | None = None) -> str:
    return f"{device_name}|{lib_hash or library_hash()}|{workload}"


def load_cache(path: Path | None = None) -> dict:
    p = path or cache_path()
    if not p.exists():
        return {}
    try:
        return json.loads(p.read_text())
    except (OSError, ValueError):
        return {}


def store(key: str, choice: Choice, timings: dict, path: Path | None = None) -> None:
    p = path or cache_path()
    p.parent.mkdir(parents=True, exist_ok=True)
    data = load_cache(p)
    data[key] = {"choice": asdict(choice), "timings_ms": timings}
    tmp = p.with_suffix(".tmp")
    tmp.write_text(json.dumps(data, indent=1, sort_keys=True))
    os.replace(tmp, p)


def lookup(key: str, path: Path | None = None) -> Choice | None:
    e = load_cache(path).get(key)
    return Choice(**e["choice"]) if e else None


MARGIN = 0.02  # a candidate replaces the default only when this much faster


def pick(timings: dict, margin: float = MARGIN) -> object:
    """The candidate with the smallest time (ties: the first listed), unless
    it beats the first listed candidate, the default, by less than `margin`
    (a fraction of the default's time): then the default.  Stage times on a
    shared GPU vary by a few percent from call to call, so a smaller gap is
    not a reason to leave the default."""
    items = list(timings.items())
    default, t0 = items[0]
    best, best_t = default, t0
    for cand, t in items[1:]:
        if t < best_t:
            best, best_t = cand, t
    return best if best_t < (1.0 - margin) * t0 else default


def apply(choice: Choice) -> None:
    lib = native.load()
    native.check(lib.cgb_bm_set_launch_shape(choice.bm_shape), "cgb_bm_set_launch_shape")
    native.check(lib.cgb_ihc_set_run_length(choice.ihc_run), "cgb_ihc_set_run_length")


def _rounds(stage: Callable[[], None], timer, cands, set_cand, prepare, output, what: str,
            changed: str, rounds: int, warmup: int) -> dict:
    """Best time of each candidate over `rounds` round-robin rounds, after
    `warmup` untimed calls of the stage (so that the first candidate is not
    timed while clocks and caches settle); the outputs of every candidate are
    checked against the first's in the first round."""
    for _ in range(warmup):
        stage()
    best = {c: float("inf") for c in cands}
    ref = None
    for r in range(rounds):
        for c in cands:
            set_cand(c)
            prepare()
            best[c] = min(best[c], timer(stage))
            if r == 0:
                out = output()
                if ref is None:
                    ref = out
                elif out != ref:
                    raise native.CGBError(f"{what} {c} changed the {changed}")
    return best


def search(stage_bm: Callable[[], None], stage_ihc: Callable[[], None],
           timer: Callable[[Callable[[], None]], float], outputs: Callable[[], tuple],
           shapes: Sequence[int] | None = None, runs: Sequence[int] = IHC_RUNS,
           prepare_bm: Callable[[], None] = lambda: None,
           prepare_ihc: Callable[[], None] = lambda: None, rounds: int = 3, warmup: int = 3,
           margin: float = MARGIN):
    """Times every candidate of each stage (timer(fn) -> ms), round-robin over
    `rounds` rounds after `warmup` untimed calls, and checks that its outputs
    (outputs() -> (velocity bytes, lambda bytes)) equal the first candidate's.
    prepare_bm / prepare_ihc run after a candidate is set and before it is
    timed: they must clear the stage's outputs (so that a candidate that leaves
    rows unwritten is caught) and re-upload anything the setting applies to.
    The first candidate of each list is the default, kept unless another is
    faster by `margin` (pick).  Returns (Choice, timings)."""
    lib = native.load()
    shapes = list(range(lib.cgb_bm_launch_shape_count())) if shapes is None else list(shapes)
    timings = {}
    timings["bm_shape"] = _rounds(
        stage_bm, timer, shapes,
        lambda sh: native.check(lib.cgb_bm_set_launch_shape(sh), "cgb_bm_set_launch_shape"),
        prepare_bm, lambda: outputs()[0], "BM launch shape", "velocity", rounds, warmup)
    best_shape = pick(timings["bm_shape"], margin)
    native.check(lib.cgb_bm_set_launch_shape(best_shape), "cgb_bm_set_launch_shape")
    stage_bm()
    timings["ihc_run"] = _rounds(
        stage_ihc, timer, list(runs),
        lambda r: native.check(lib.cgb_ihc_set_run_length(r), "cgb_ihc_set_run_length"),
        prepare_ihc, lambda: outputs()[1], "IHC run length", "lambda", rounds, warmup)
    choice = Choice(bm_shape=int(best_shape), ihc_run=int(pick(timings["ihc_run"], margin)))
    apply(choice)
    prepare_ihc()
    return choice, {k: {str(c): t for c, t in v.items()} for k, v in timings.items()}


def tune_sweep(run, device, rounds: int = 3, use_cache: bool = True):
    """Tunes a BatchSweep or ProfileRun on `device` (or takes the cached
    choice) and applies it; returns (Choice, source) with source 'cache' or
    'search'."""
    import torch
    name = torch.cuda.get_device_name(device)
    workload = (f"{type(run).__name__}:units={len(run.units)}:"
                f"frames={len(run.frames)}:lam_rows={int(run.d_lam.shape[1])}")
    key = cache_key(name, workload)
    if use_cache:
        hit = lookup(key)
        if hit is not None:
            apply(hit)
            if hasattr(run, "upload_ihc_tables"):
                run.upload_ihc_tables()
            return hit, "cache"
    stream = torch.cuda.current_stream(device)
    if hasattr(run, "generate_input"):
        run.generate_input()

    def timer(fn):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        torch.cuda.synchronize(device)
        return a.elapsed_time(b)

    def outputs():
        torch.cuda.synchronize(device)
        return (run.d_v.cpu().numpy().tobytes(), run.d_lam.cpu().numpy().tobytes())

    def prepare_bm():
        run.d_v.fill_(float("nan"))

    def prepare_ihc():
        if hasattr(run, "upload_ihc_tables"):
            run.upload_ihc_tables()
        run.d_lam.fill_(float("nan"))

    choice, timings = search(run.solve_bm, run.ihc_lambda, timer, outputs,
                             prepare_bm=prepare_bm, prepare_ihc=prepare_ihc, rounds=rounds)
    run.solve_bm()
    run.ihc_lambda()
    store(key, choice, timings)
    return choice, "search"


def occupancy_profile(run, shapes: Sequence[int], prefixes: Sequence[int], reps: int = 3):
    """BM stage time (ms, best of reps) of the first n units of `run`'s unit
    table (longest first) for each launch shape and n in `prefixes`.  With
    n below one wave the time is that of the longest units at n / (SMs x 4)
    warps per scheduler, so the table separates per-warp speed, throughput
    per scheduler and the last wave's fill."""
    import torch
    lib = native.load()
    dev = run.d_v.device
    stream = torch.cuda.current_stream(dev)
    if hasattr(run, "generate_input"):
        run.generate_input()

    def solve(n):
        run.bm.run_dev(run.sc, run.d_gamma, run.d_units, n, run.d_in, run.d_v, run.d_failed,
                       run.d_stats, stream, extras=getattr(run, "extras", None))

    out = {}
    try:
        for sh in shapes:
            native.check(lib.cgb_bm_set_launch_shape(sh), "cgb_bm_set_launch_shape")
            row = {}
            for n in prefixes:
                n = min(int(n), len(run.units))
                solve(n)
                best = None
                for _ in range(reps):
                    a = torch.cuda.Event(enable_timing=True)
                    b = torch.cuda.Event(enable_timing=True)
                    a.record(stream)
                    solve(n)
                    b.record(stream)
                    torch.cuda.synchronize(dev)
                    ms = a.elapsed_time(b)
                    best = ms if best is None else min(best, ms)
                row[n] = best
            out[sh] = row
    finally:
        native.check(lib.cgb_bm_set_launch_shape(0), "cgb_bm_set_launch_shape")
    solve(len(run.units))  # the per-unit statistics of the whole table
    stats = run.d_stats.cpu().numpy().view(native.STATS_DTYPE).reshape(-1)
    return out, stats


def _main(argv=None) -> None:
    import argparse
    import json as _json
    ap = argparse.ArgumentParser(description="BM launch-shape occupancy profile on the JND sweep")
    ap.add_argument("--shapes", default="0,3")
    ap.add_argument("--prefixes", default="152,608,912,1216,1824,2432,100000")
    ap.add_argument("--n-seeds", type=int, default=4)
    a = ap.parse_args(argv)
    from . import batch
    run = batch.BatchSweep("cuda:0", batch.jnd_sweep_spec(n_seeds=a.n_seeds))
    prof, stats = occupancy_profile(run, [int(s) for s in a.shapes.split(",")],
                                    [int(n) for n in a.prefixes.split(",")])
    ss = stats["substeps"]
    print(_json.dumps({"units": len(run.units), "substeps_total": int(ss.sum()),
                       "substeps_longest": int(ss.max()),
                       "ms": {str(k): {str(n): t for n, t in v.items()} for k, v in prof.items()}}))


if __name__ == "__main__":
    _main()
