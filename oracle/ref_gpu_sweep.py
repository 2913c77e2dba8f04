"""The reference's own compiled BMOHC_NEW_kernel (Run_Fast_BM_Calculation 0,
the reference default; include/cochlea.cuh:3486-4324) on the JND sweep,
against the product's BM stage in the same semantics (controller 1, arith 1).

Test infrastructure: it launches the reference cubin (oracle/build_ref_gpu.sh)
through oracle/ref_gpu.cpp.  Each group of the sweep (one signal length: a
noise-only reference interval and ten tone intervals) runs as the reference's
Run_Cuda runs it: one launch with one 256-thread block per time block
(src/cochlea.cu:2298-2330).  For every group:
- the product's BM runs first on the generated input (ProfileRun, one warp per
  block), and its per-unit status must show no substep-guard stop; a group
  that fails this is not given to the reference kernel, which has no guard;
- the reference kernel runs on the same input, timed by CUDA events around its
  launch;
- the velocity rows each block owns are compared bit for bit.
Then the product's batched BM stage (all groups in one launch, the JND sweep's
3,025 units) is timed in the same semantics.  Prints one JSON line.

    python -m oracle.ref_gpu_sweep [--seeds 4]
"""
import argparse
import json

import numpy as np


def _owned(units, rows):
    """Rows each block alone writes: [out_first, end), minus row out_first - 1
    of every later block (BMOHC_NEW_kernel writes it too)."""
    mask = np.zeros(rows, bool)
    for u in units:
        mask[u["out_first"]:u["end"]] = True
    mask[[int(u["out_first"]) - 1 for u in units[1:]]] = False
    return mask


def _events_ms(torch, fn, reps=1):
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    s.record()
    for _ in range(reps):
        fn()
    e.record()
    torch.cuda.synchronize()
    return s.elapsed_time(e) / reps


def compare_group(sp, mv, md, dev="cuda:0", Fs=100000):
    """One JND-sweep group (a jnd_sweep_spec entry) through the product's BM
    (controller 1, arith 1) and, when no unit stopped on the substep guard,
    through the reference's BMOHC_NEW_kernel on the same input.  Returns the
    group's record: blocks, audio seconds, substeps, the product's ms, and the
    reference's ms and bit-exactness on the owned rows (or why it was
    skipped)."""
    import torch
    from cochlearmodel_gb300 import batch, model, native
    from cochlearmodel_gb300.pipeline import ProfileRun
    from oracle import ref_gpu

    N, D = batch.block_nodes_for(sp["length"], 1000, Fs)
    cfg = model.RunConfig(Fs=Fs, Time_Block_Length=N / Fs, Decouple_Filter=D,
                          Overlap_Time=0.005, OHC_Vector=batch.hearing_loss_ohc(),
                          IHC_Vector=batch.hearing_loss_ihc(), Run_Fast_BM_Calculation=0)
    run = ProfileRun(dev, cfg, sp["sweep"], noise=sp["noise"], mv=mv, want_lambda=False)
    assert run.sc.controller == 1 and run.sc.arith == 1
    run.generate_input()
    run.solve_bm()  # warm-up
    ours_ms = _events_ms(torch, run.solve_bm)
    st = run.d_stats.cpu().numpy().view(native.STATS_DTYPE).ravel()
    g = {"length": int(sp["length"]), "blocks": len(run.units), "audio_s": run.audio_seconds,
         "substeps": int(st["substeps"].sum()), "ours_ms": ours_ms}
    if (st["status"] != 0).any():
        g["reference"] = "skipped: a unit stopped on the substep guard"
        return g
    x = run.d_in.cpu().numpy()
    v = run.d_v.cpu().numpy()
    p = ref_gpu.params_from(run.cfg, run.sc)
    secs = ref_gpu.sections_from(md, run.cfg.gamma())
    mtt = np.full(run.cfg.Time_Blocks, run.cfg.Max_Tolerance, np.float32)
    mmspt = np.full(run.cfg.Time_Blocks, run.cfg.Max_M1_SP_Error, np.float32)
    r_v, _, _ = ref_gpu.bm_run(0, p, secs, mtt, mmspt, x, run.rows)
    g["reference_ms"] = ref_gpu.last_bm_ms()
    mask = _owned(run.units, run.rows)
    g["owned_rows"] = int(mask.sum())
    g["bit_exact"] = bool(np.array_equal(v[mask].view(np.uint32), r_v[mask].view(np.uint32)))
    return g


def main():
    import torch
    from cochlearmodel_gb300 import batch, model
    from oracle import oracle as orc

    ap = argparse.ArgumentParser()
    ap.add_argument("--seeds", type=int, default=4)
    args = ap.parse_args()
    dev = "cuda:0"
    mv = model.ModelVectors.build()
    specs = batch.jnd_sweep_spec(n_seeds=args.seeds)
    md = orc.model_setup()
    groups = []
    for gi, sp in enumerate(specs):
        if gi == 0:
            compare_group(sp, mv, md, dev)  # module and kernel warm-up
        g = compare_group(sp, mv, md, dev)
        g["group"] = gi
        groups.append(g)
        torch.cuda.empty_cache()

    sweep = batch.BatchSweep(dev, specs, mv=mv)
    sweep.sc.controller = sweep.sc.arith = 1
    sweep.generate_input()
    sweep.solve_bm()
    batched_ms = min(_events_ms(torch, sweep.solve_bm) for _ in range(3))
    done = [g for g in groups if "reference_ms" in g]
    out = {
        "what": "BMOHC_NEW_kernel semantics on the JND sweep: the reference's compiled kernel "
                "(one launch per group, one 256-thread block per time block) against the "
                "product's warp kernel (controller 1, arith 1)",
        "groups": len(groups), "groups_run_on_reference": len(done),
        "groups_bit_exact": sum(g["bit_exact"] for g in done),
        "units": sum(g["blocks"] for g in groups),
        "audio_s": sum(g["audio_s"] for g in groups),
        "substeps": sum(g["substeps"] for g in groups),
        "reference_ms_sum": sum(g["reference_ms"] for g in done),
        "ours_per_group_ms_sum": sum(g["ours_ms"] for g in done),
        "ours_batched_ms": batched_ms,
        "per_group": groups,
    }
    print(json.dumps(out))


if __name__ == "__main__":
    main()
