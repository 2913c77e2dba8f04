"""Full-length parity on the benchmark configurations.

- Configuration 1: the whole 50 ms, one block.
- Configuration 2: one 80 ms tone (Time_Block_Length 10 ms x Decouple_Filter
  8) at each of the five power levels, velocity and all three lambda planes.
- Configuration 3: two whole JND-sweep groups (a 200 ms one with noise at
  40 dB SPL and a 20 ms one without), velocity, lambda and the JNDs.

GPU against the FP32 oracle bit for bit (velocity, lambda in the kernel's own
FP32 order); lambda within the 1e-4 bar of the reference's mixed precision;
JND within 0.1 dB of the reference float arithmetic.  The FP64 method's
error is printed for each output (max |a - b| / max |b| per signal).
"""
import numpy as np
import pytest

from cochlearmodel_gb300 import batch, model
from cochlearmodel_gb300.pipeline import ProfileRun, ProfileSweep
from oracle import oracle as orc
from tests import cases

pytestmark = pytest.mark.gpu

LAMBDA_REL = 1e-4
JND_DB_TOL = 0.1


def _max_rel(a, b):
    return float(np.abs(np.asarray(a, np.float64) - b).max() / max(np.abs(b).max(), 1e-300))


def _lambda_checks(stage, v, frames, lam):
    """Every frame's lambda: bit-exact against oracle mode 2, within the bar of
    mode 0 (the reference's mixed precision); returns the FP64 (mode 1) error."""
    worst64 = 0.0
    for fr in frames:
        r0, n = int(fr["lam_row0"]), int(fr["lam_rows"])
        vin = v[fr["v_row0"]:fr["v_row0"] + fr["rows"]]
        args = (vin, int(fr["seg"]), int(fr["frdp"]), int(fr["total"]), n,
                stage.ac.astype(np.float64), stage.dc.astype(np.float64), stage.nerve.scale,
                stage.nerve.eta_AC, stage.nerve.eta_DC,
                stage.dmg_host[fr["ihc_profile"]].astype(np.float64), stage.nerve.aihc(),
                np.asarray(stage.nerve.spontRate, np.float32), stage.nerve.Lambda_SAT)
        _, o2 = orc.ihc_lambda(*args, mode=2)
        assert np.array_equal(lam[:, r0:r0 + n].view(np.uint32), o2.view(np.uint32))
        _, o0 = orc.ihc_lambda(*args, mode=0)
        _, o1 = orc.ihc_lambda(*args, mode=1)
        for j in range(3):
            assert _max_rel(lam[j, r0:r0 + n], o0[j]) <= LAMBDA_REL
            worst64 = max(worst64, _max_rel(lam[j, r0:r0 + n], o1[j]))
    return worst64


def test_configuration1_full_length(mv, bm_solver):
    cfg, sc, gamma, units, x, rows = cases.cfg1_slice(mv, ms=50.0, db=60.0, freq=1000.0)
    v, f, st = bm_solver.run(sc, gamma, units, x, rows)
    o, of, ost = orc.bm_run(mv.section_params(), gamma, sc, units, x, rows)
    assert np.array_equal(v.view(np.uint32), o.view(np.uint32))
    assert np.array_equal(f, of)
    assert int(st["written_samples"][0]) == 5500
    v64, _, _ = orc.bm_run(mv.section_params(), gamma, sc, units, x, rows, fp64=True)
    e = _max_rel(v, v64)
    print(f"configuration 1, 50 ms: velocity max-rel vs FP64 {e:.2e}")
    assert e <= 2e-4


def test_configuration2_tones_full_length(mv):
    """One log-spaced tone per power level, 80 ms each in 8 decoupled blocks."""
    import torch
    cfg = model.RunConfig(Time_Block_Length=0.01, Decouple_Filter=8, Overlap_Time=0.005)
    freqs = [125.0 * 64 ** (k / 63) for k in (5, 20, 35, 50, 63)]
    runs = []
    for f, db in zip(freqs, (20.0, 40.0, 60.0, 80.0, 100.0)):
        c = model.RunConfig(Time_Block_Length=0.01, Decouple_Filter=8, Overlap_Time=0.005)
        r = ProfileRun("cuda:0", c, ProfileSweep(frequencies=[f], powers=[db]), mv=mv)
        r.step()
        runs.append((r, f, db))
    torch.cuda.synchronize()
    for r, f0, p0 in runs:
        x = r.d_in.cpu().numpy()
        gamma = r.cfg.gamma()[None]
        v = r.d_v.cpu().numpy()
        o, of, _ = orc.bm_run(mv.section_params(), gamma, r.sc, r.units, x, r.rows)
        assert np.array_equal(v.view(np.uint32), o.view(np.uint32))
        assert int(r.cfg.total_time_nodes()) - int(cfg.calc_overlap_nodes()) == 8000
        e_lam = _lambda_checks(r.ihc, v, r.frames, r.d_lam.cpu().numpy())
        v64, _, _ = orc.bm_run(mv.section_params(), gamma, r.sc, r.units, x, r.rows, fp64=True)
        print(f"configuration 2, {f0:.0f} Hz {p0:.0f} dB: velocity vs FP64 "
              f"{_max_rel(v, v64):.2e}, lambda vs FP64 {e_lam:.2e}")


def test_configuration3_groups_full_length(mv):
    import torch
    rng = np.random.default_rng(11)
    noise = rng.standard_normal(20001).astype(np.float32)
    powers = [float(p) for p in range(10, 101, 10)]
    spec = [dict(length=20000, noise=noise,
                 sweep=ProfileSweep(frequencies=[1000.0], powers=powers, noises=[40.0],
                                    calculate_jnd=True)),
            dict(length=2000, noise=noise,
                 sweep=ProfileSweep(frequencies=[1000.0], powers=powers, noises=[1111.0],
                                    calculate_jnd=True))]
    b = batch.BatchSweep("cuda:0", spec, mv=mv)
    b.step()
    torch.cuda.synchronize()
    x = b.d_in.cpu().numpy()
    gamma = b.d_gamma.cpu().numpy()
    v = b.d_v.cpu().numpy()
    o, of, _ = orc.bm_run(mv.section_params(), gamma, b.sc, b.units, x, b.v_rows)
    assert np.array_equal(v.view(np.uint32), o.view(np.uint32))
    lam = b.d_lam.cpu().numpy()
    e_lam = _lambda_checks(b.ihc, v, b.frames, lam)
    res = b.jnd_db()
    worst_db = 0.0
    for gi, g in enumerate(b.groups):
        rate_db, ai_db, _, _ = res[gi]
        n_int, L = len(g.prof), g.L
        glam = lam[:, g.lam_row0:g.lam_row0 + n_int * L]
        head, length = b.jnd_win.nodes(g.cfg.Fs, L)
        ra, ai = orc.jnd(glam, n_int, L, head, length, g.prof["dA"], g.ref_of,
                         b.nerve.nihc(), b.W, float(g.cfg.Fs), 0.2 * g.cfg.Fs, fp64=False)
        tested = g.ref_of != np.arange(n_int)
        for got, ref in ((rate_db, ra), (ai_db, ai)):
            want = np.array([orc.jnd_db(ref[:, i].sum()) for i in range(n_int)])
            worst_db = max(worst_db, float(np.abs(got[tested] - want[tested]).max()))
    assert worst_db <= JND_DB_TOL
    # FP64 method on the 20 ms group (the 200 ms group's FP64 solve is the
    # slow part of the oracle and adds nothing the short one does not show)
    short = b.units[b.units["out_base"] >= b.groups[1].v_row0]
    v64, _, _ = orc.bm_run(mv.section_params(), gamma, b.sc, short, x, b.v_rows, fp64=True)
    g1 = b.groups[1]
    rows = slice(g1.v_row0, b.v_rows)
    print(f"configuration 3 groups (200 ms + 20 ms): JND vs reference float arithmetic "
          f"{worst_db:.2e} dB, lambda vs FP64 {e_lam:.2e}, 20 ms group velocity vs FP64 "
          f"{_max_rel(v[rows], v64[rows]):.2e}")
