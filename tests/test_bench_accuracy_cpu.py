"""bench.py's max_rel_vs_fp64 record (accuracy_record) on the CPU.

A stand-in for the batched run holds one short group laid out as BatchSweep
lays out a group, with the FP32 oracle's results in place of the device's:
velocity from orc.bm_run (bit-exact with the BM kernel), lambda from oracle
mode 2 (the IHC kernel's FP32 order, bit-exact) and the JNDs from the float
Fisher sums.  The record must measure those results against the FP64 chain:
the FP32 velocity of a quiet tone sits near 1e-4 of the FP64 method, and a
velocity error planted in the stand-in's results shows up in that figure."""
import sys
from types import SimpleNamespace

import numpy as np
import torch

from cochlearmodel_gb300 import batch, ihc, model
from cochlearmodel_gb300.pipeline import JNDWindow, ProfileSweep
from oracle import oracle as orc

ROOT = __file__.rsplit("/tests/", 1)[0]


def _stand_in(plant=0.0):
    Fs, N, D = 100000, 1000, 2  # 20 ms intervals, the sweep's shortest
    mv = model.ModelVectors.build()
    sweep = ProfileSweep(frequencies=[1000.0], powers=[30.0, 60.0], noises=[1111.0],
                         calculate_jnd=True)
    prof, _, ref_of = sweep.build()
    n_int, L = len(prof), N * D
    ohc, ihc_vec = batch.hearing_loss_ohc(), batch.hearing_loss_ihc()
    cfg = model.RunConfig(Fs=Fs, Time_Block_Length=N / Fs, Decouple_Filter=D,
                          Time_Blocks=n_int * D, Overlap_Time=0.005, OHC_Vector=ohc,
                          IHC_Vector=ihc_vec)
    assert cfg.calc_time_block_nodes() == N
    rows = cfg.total_time_nodes_p1() + 4
    g = batch.Group(cfg, prof, ref_of, None, N, L, 0, 0, 0)
    units = model.reference_units(cfg, in_base=0, out_base=0)
    frames = ihc.reference_frame(cfg, v_row0=0, lam_row0=0)
    sc = model.bm_scalars(cfg, mv)
    x = np.zeros(rows, np.float32)
    pt = np.stack([prof["dA"], prof["Wn"], prof["frequency"]], 1)
    x[:n_int * L] = orc.input_gen(pt, np.zeros(L, np.float32), L, 0, float(Fs), 0.0, 1.0,
                                  1.0).ravel()
    gamma = ohc[None].astype(np.float32)
    v, _, _ = orc.bm_run(mv.section_params(), gamma, sc, units, x, rows)
    v = v * np.float32(1.0 + plant)
    nerve = ihc.NerveConfig()
    stage = SimpleNamespace(ac=ihc.design_ac_lowpass().astype(np.float32),
                            dc=nerve.dc_taps(Fs), dmg_host=ihc.ihc_damage(ihc_vec)[None])
    fr = frames[0]
    n_lam = int(fr["lam_rows"])
    _, lam = orc.ihc_lambda(v[:int(fr["rows"])], int(fr["seg"]), int(fr["frdp"]),
                            int(fr["total"]), n_lam, stage.ac.astype(np.float64),
                            stage.dc.astype(np.float64), nerve.scale, nerve.eta_AC,
                            nerve.eta_DC, stage.dmg_host[0].astype(np.float64), nerve.aihc(),
                            np.asarray(nerve.spontRate, np.float32), nerve.Lambda_SAT, mode=2)
    win = JNDWindow()
    head, length = win.nodes(Fs, L)
    ra, ai = orc.jnd(lam, n_int, L, head, length, prof["dA"], ref_of, nerve.nihc(),
                     np.asarray(nerve.W, np.float32), float(Fs),
                     win.delta_alpha_time_factor * Fs, fp64=False)
    tested = ref_of != np.arange(n_int)
    rate_db = np.array([orc.jnd_db(ra[:, i].sum()) if tested[i] else np.nan
                        for i in range(n_int)])
    ai_db = np.array([orc.jnd_db(ai[:, i].sum()) if tested[i] else np.nan
                      for i in range(n_int)])
    return SimpleNamespace(
        groups=[g], frames=frames, units=units, sc=sc, mv=mv, ihc=stage, nerve=nerve,
        jnd_win=win, d_in=torch.from_numpy(x), d_v=torch.from_numpy(v),
        d_lam=torch.from_numpy(np.ascontiguousarray(lam)),
        d_gamma=torch.from_numpy(gamma), jnd_db=lambda: [(rate_db, ai_db, None, None)])


def test_accuracy_record_measures_the_fp32_chain():
    """The 30 dB tone's FP32 velocity is within 1e-3 of the FP64 method (its
    step sequence is the same); every figure is finite, each top-level figure
    is the worst interval's, and the JNDs agree to a small fraction of a dB."""
    sys.path.insert(0, ROOT)
    import bench
    rec = bench.accuracy_record(_stand_in())
    per = rec["per_interval"]
    assert [p["signal"] for p in per] == ["30 dB tone", "60 dB tone", "noise only"]
    assert per[-1]["jnd_db_abs"] is None
    assert 1e-7 < per[0]["velocity"] < 1e-3
    assert per[0]["velocity_vs_exact_solve"] < 1e-3
    for p in per[:2]:
        for k in ("velocity", "velocity_rel_l2", "velocity_vs_exact_solve", "lambda",
                  "lambda_rel_l2"):
            assert np.isfinite(p[k]) and 0.0 < p[k] < 0.5, (p["signal"], k, p[k])
        assert 0.0 <= p["jnd_db_abs"] < 0.05
    for k in ("velocity", "velocity_rel_l2", "lambda", "lambda_rel_l2"):
        assert rec[k] == max(p[k] for p in per)
    assert rec["jnd_db_abs"] == max(p["jnd_db_abs"] or 0.0 for p in per)


def test_accuracy_record_sees_a_planted_velocity_error():
    sys.path.insert(0, ROOT)
    import bench
    rec = bench.accuracy_record(_stand_in(plant=1e-2))
    assert 0.9e-2 < rec["per_interval"][0]["velocity"] < 1.1e-2
