"""Parity against the REFERENCE's own compiled kernels.

oracle/_ref/cochlea_ref.cubin is the reference's src/cochlea.cu +
include/cochlea.cuh compiled for sm_103a (oracle/build_ref_gpu.sh);
oracle/ref_gpu.cpp launches its BMOHC_NEW_kernel (Run_Fast_BM_Calculation 0,
the reference default) and kernel 17 with the constants its BMOHCNewKernel
packs.

- The product's reference-arithmetic mode (controller 1, arith 1) must equal
  BMOHC_NEW_kernel bit for bit on every row it owns.  BMOHC_NEW_kernel also
  writes row out_first - 1 of every block after the first, a row the previous
  block owns (both blocks store it; which store lands is a race), and stores
  row n's failure flag at index n + 1 (include/cochlea.cuh:4153-4157); the
  comparison accounts for both.
- Kernel 17 leaves its step controller's full sums only in lane 0 of warp 0
  and lets all 32 lanes write the decision (include/cochlea.cuh:169-186,
  14037-14087).  The product takes lane 0's values (controller 0).  Its
  velocity is compared with the FP64 method and must be at least as close as
  the reference's kernel 17 run here.
"""
import numpy as np
import pytest

from cochlearmodel_gb300 import native
from oracle import oracle as orc
from oracle import ref_gpu
from tests import cases

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_gpu.available(),
                                 reason="reference cubin not built (oracle/build_ref_gpu.sh)")]


def _ref_run(variant, cfg, sc, gamma, x, rows):
    p = ref_gpu.params_from(cfg, sc)
    secs = ref_gpu.sections_from(orc.model_setup(), gamma[0])
    mtt = np.full(cfg.Time_Blocks, cfg.Max_Tolerance, np.float32)
    mmspt = np.full(cfg.Time_Blocks, cfg.Max_M1_SP_Error, np.float32)
    return ref_gpu.bm_run(variant, p, secs, mtt, mmspt, x, rows)


def _owned(units, rows):
    """Rows each block alone writes: [out_first, end), minus row out_first - 1
    of every later block (the reference's shared boundary row)."""
    mask = np.zeros(rows, bool)
    for u in units:
        mask[u["out_first"]:u["end"]] = True
    mask[[int(u["out_first"]) - 1 for u in units[1:]]] = False
    return mask


def _max_rel(a, b):
    return float(np.abs(a.astype(np.float64) - b).max() / np.abs(b).max())


REF_CASES = {
    "cfg1_60dB_1kHz_50ms": lambda mv: cases.cfg1_slice(mv, ms=50.0, db=60.0, freq=1000.0),
    "cfg1_100dB_4kHz_10ms": lambda mv: cases.cfg1_slice(mv, ms=10.0, db=100.0, freq=4000.0),
    "cfg1_20dB_250Hz_10ms": lambda mv: cases.cfg1_slice(mv, ms=10.0, db=20.0, freq=250.0),
    "decoupled_3x4_blocks": lambda mv: cases.decoupled_sweep(mv, n_signals=3, decouple=4,
                                                             block_ms=2.5, overlap_ms=1.0,
                                                             seed=1),
}


@pytest.mark.parametrize("name", sorted(REF_CASES))
def test_reference_arithmetic_bit_exact(mv, bm_solver, name):
    cfg, sc, gamma, units, x, rows = REF_CASES[name](mv)
    r_v, r_f, _ = _ref_run(0, cfg, sc, gamma, x, rows)
    s1 = native.BMScalars.from_buffer_copy(sc)
    s1.controller, s1.arith = 1, 1
    v, f, st = bm_solver.run(s1, gamma, units, x, rows)
    mask = _owned(units, rows)
    assert np.abs(r_v[mask]).max() > 0
    assert np.array_equal(v[mask], r_v[mask]), (
        "differs from BMOHC_NEW_kernel: max-rel %.3e" % _max_rel(v[mask], r_v[mask]))
    r_f_row = np.zeros_like(r_f)
    r_f_row[:-1] = r_f[1:]
    assert np.array_equal(f[mask], r_f_row[mask])


def test_hearing_loss_profile_bit_exact(mv, bm_solver):
    """A non-uniform OHC profile (0.5 ramping to 0.05 over sections 128-255)."""
    cfg, sc, _, units, x, rows = cases.cfg1_slice(mv, ms=10.0, db=70.0, freq=1500.0)
    gamma = cases.hearing_loss_gamma()[None]
    r_v, _, _ = _ref_run(0, cfg, sc, gamma, x, rows)
    s1 = native.BMScalars.from_buffer_copy(sc)
    s1.controller, s1.arith = 1, 1
    v, _, _ = bm_solver.run(s1, gamma, units, x, rows)
    mask = _owned(units, rows)
    assert np.array_equal(v[mask], r_v[mask])


def test_kernel17_against_fp64(mv, bm_solver):
    """Kernel 17 semantics: the product (lane-0 controller values, own
    operation order) is closer to the FP64 method than the reference's
    kernel 17 as it runs on this GPU, on full-length configuration 1."""
    cfg, sc, gamma, units, x, rows = cases.cfg1_slice(mv, ms=50.0, db=60.0, freq=1000.0)
    r17, _, _ = _ref_run(17, cfg, sc, gamma, x, rows)
    v, _, _ = bm_solver.run(sc, gamma, units, x, rows)
    v64, _, _ = orc.bm_run(mv.section_params(), gamma, sc, units, x, rows, fp64=True)
    mask = _owned(units, rows)
    e_prod = _max_rel(v[mask], v64[mask])
    e_ref = _max_rel(r17[mask], v64[mask])
    print(f"max-rel vs FP64: product {e_prod:.3e}, reference kernel 17 {e_ref:.3e}")
    assert e_prod <= 2e-4
    assert e_prod <= e_ref


LAMBDA_REL = 1e-4  # the lambda bar: max |a - b| / max |b| per plane


@pytest.fixture(scope="module")
def ihc_stage():
    from cochlearmodel_gb300 import ihc
    return ihc.IHCStage("cuda:0")


@pytest.mark.parametrize("case", ["decoupled", "cfg1_10ms"])
def test_lambda_against_reference_kernels(mv, ihc_stage, case):
    """The fused IHC/lambda kernel against the reference's CudaUnifiedCalcIHC
    + CudaCalcLambda on the same velocity, one Run_Cuda chunk.  The
    reference accumulates the FIR in double; this kernel in compensated
    FP32 (Dot2).  The oracle's restatement of the reference arithmetic (mode
    0) is checked against the reference kernels too."""
    from cochlearmodel_gb300 import ihc
    if case == "decoupled":
        c = cases.decoupled_sweep(mv, n_signals=2, decouple=2, block_ms=1.5, overlap_ms=0.5)
    else:
        c = cases.cfg1_slice(mv, ms=10.0, db=80.0, freq=2000.0)
    cfg, sc, gamma, units, x, rows = c
    v, _, _ = orc.bm_run(mv.section_params(), gamma, sc, units, x, rows)
    fr = ihc.reference_frame(cfg)
    n, lam_rows = int(fr["rows"][0]), int(fr["lam_rows"][0])
    v = v[:n]
    st = ihc_stage
    lam, ih = st.run(v, fr, lam_rows, want_ihc=True)
    nerve = st.nerve
    r_ihc, r_lam = ref_gpu.ihc_lambda(
        v, int(fr["total"][0]), cfg.calc_time_block_nodes(), cfg.Time_Blocks,
        cfg.Decouple_Filter, st.ac.astype(np.float64), st.dc.astype(np.float64), nerve.scale,
        nerve.eta_AC, nerve.eta_DC, nerve.Lambda_SAT, st.dmg_host[0].astype(np.float64),
        np.asarray(nerve.spontRate, np.float32), np.asarray(nerve.W, np.float32), nerve.aihc())
    _, o_lam = orc.ihc_lambda(v, int(fr["seg"][0]), int(fr["frdp"][0]), int(fr["total"][0]),
                              lam_rows, st.ac.astype(np.float64), st.dc.astype(np.float64),
                              nerve.scale, nerve.eta_AC, nerve.eta_DC,
                              st.dmg_host[0].astype(np.float64), nerve.aihc(),
                              np.asarray(nerve.spontRate, np.float32), nerve.Lambda_SAT, mode=0)
    worst_prod = worst_orc = 0.0
    for j in range(3):
        ref = r_lam[j, :lam_rows]
        worst_prod = max(worst_prod, _max_rel(lam[j, :lam_rows], ref))
        worst_orc = max(worst_orc, _max_rel(o_lam[j, :lam_rows], ref))
    print(f"lambda max-rel vs the reference kernels: product {worst_prod:.2e}, "
          f"oracle mode 0 {worst_orc:.2e}")
    assert worst_prod <= LAMBDA_REL
    assert worst_orc <= 1e-6
    assert np.abs(ih[:lam_rows] - r_ihc[:lam_rows]).max() <= 1e-4 * np.abs(r_ihc).max()


JND_DB_TOL = 0.1  # dB


def test_jnd_against_reference_kernels(mv):
    """The profile-mode path's JND against the reference's
    GlobalCalculateMeanRate + GlobalCalculateJND run on the same lambda.  The
    reference sums in FP32 with rsqrt-squared reciprocals; this library sums
    in FP64.  The final JNDs (calcJNDFinal's dB) agree within 0.1 dB, and the
    Fisher sums within the FP32 summation error."""
    import torch
    from cochlearmodel_gb300 import model
    from cochlearmodel_gb300.pipeline import JNDWindow, ProfileRun, ProfileSweep
    cfg = model.RunConfig(Time_Block_Length=0.002, Decouple_Filter=2, Overlap_Time=0.001,
                          OHC_Vector=np.linspace(0.5, 0.05, 256, dtype=np.float32),
                          IHC_Vector=np.linspace(8, 5, 256, dtype=np.float32))
    sweep = ProfileSweep(frequencies=[1000.0, 3000.0], powers=[40.0, 80.0],
                         noises=[1111.0, 30.0], calculate_jnd=True)
    noise = np.random.default_rng(7).standard_normal(400).astype(np.float32)
    run = ProfileRun("cuda:0", cfg, sweep, noise=noise, mv=mv,
                     jnd=JNDWindow(head=0.001, tail=0.0005))
    run.step()
    torch.cuda.synchronize()
    lam = run.d_lam.cpu().numpy()
    r_ra, r_ai = ref_gpu.jnd(lam, run.n_int, run.L, run.head, run.len, run.prof["dA"],
                             run.ref_of, run.nerve.nihc(), np.asarray(run.nerve.W, np.float32),
                             float(cfg.Fs), 0.2 * cfg.Fs)
    rate_db, ai_db, F_RA, F_AI = run.jnd_db()
    tested = run.ref_of != np.arange(run.n_int)
    assert tested.sum() == 8
    worst_db = 0.0
    for got_db, ref in ((rate_db, r_ra), (ai_db, r_ai)):
        want_db = np.array([orc.jnd_db(ref[:, i].astype(np.float64).sum())
                            for i in range(run.n_int)])
        worst_db = max(worst_db, float(np.abs(got_db[tested] - want_db[tested]).max()))
    rel = max(float((np.abs(F_RA[:, tested] - r_ra[:, tested]) / np.abs(r_ra[:, tested])).max()),
              float((np.abs(F_AI[:, tested] - r_ai[:, tested]) / np.abs(r_ai[:, tested])).max()))
    print(f"JND vs the reference kernels: {worst_db:.2e} dB, Fisher sums max-rel {rel:.2e}")
    assert worst_db <= JND_DB_TOL
    assert rel <= 1e-3


def test_whole_profile_path_on_the_reference_default(mv):
    """Run_Fast_BM_Calculation = 0 end to end: the profile-mode path
    (generated input -> BM -> IHC/lambda -> JND) against the reference's own
    kernels chained on the same input.  Velocity is bit-exact; lambda and the
    JNDs carry only the IHC and JND stages' own differences."""
    import torch
    from cochlearmodel_gb300 import ihc, model
    from cochlearmodel_gb300.pipeline import JNDWindow, ProfileRun, ProfileSweep
    cfg = model.RunConfig(Time_Block_Length=0.003, Decouple_Filter=2, Overlap_Time=0.001,
                          OHC_Vector=cases.hearing_loss_gamma(),
                          IHC_Vector=np.linspace(8, 5, 256, dtype=np.float32),
                          Run_Fast_BM_Calculation=0)
    sweep = ProfileSweep(frequencies=[1000.0], powers=[30.0, 60.0, 90.0],
                         noises=[1111.0, 20.0], calculate_jnd=True)
    noise = np.random.default_rng(5).standard_normal(600).astype(np.float32)
    run = ProfileRun("cuda:0", cfg, sweep, noise=noise, mv=mv,
                     jnd=JNDWindow(head=0.001, tail=0.0005))
    run.step()
    torch.cuda.synchronize()
    x = run.d_in.cpu().numpy()
    r_v, _, _ = _ref_run(0, run.cfg, run.sc, run.cfg.gamma()[None], x, run.rows)
    v = run.d_v.cpu().numpy()
    mask = _owned(run.units, run.rows)
    assert np.array_equal(v[mask], r_v[mask])

    fr = run.frames[0]
    st, nerve = run.ihc, run.nerve
    n, lam_rows = int(fr["rows"]), int(fr["lam_rows"])
    r_vin = v[:n].copy()  # the owned rows agree; the product's copy has no boundary races
    _, r_lam = ref_gpu.ihc_lambda(
        r_vin, int(fr["total"]), cfg.calc_time_block_nodes(), cfg.Time_Blocks,
        cfg.Decouple_Filter, st.ac.astype(np.float64), st.dc.astype(np.float64), nerve.scale,
        nerve.eta_AC, nerve.eta_DC, nerve.Lambda_SAT, st.dmg_host[0].astype(np.float64),
        np.asarray(nerve.spontRate, np.float32), np.asarray(nerve.W, np.float32), nerve.aihc())
    lam = run.d_lam.cpu().numpy()
    for j in range(3):
        assert _max_rel(lam[j], r_lam[j, :lam_rows]) <= LAMBDA_REL
    r_ra, r_ai = ref_gpu.jnd(r_lam[:, :lam_rows], run.n_int, run.L, run.head, run.len,
                             run.prof["dA"], run.ref_of, nerve.nihc(),
                             np.asarray(nerve.W, np.float32), float(cfg.Fs), 0.2 * cfg.Fs)
    rate_db, ai_db, _, _ = run.jnd_db()
    tested = run.ref_of != np.arange(run.n_int)
    for got_db, ref in ((rate_db, r_ra), (ai_db, r_ai)):
        want_db = np.array([orc.jnd_db(ref[:, i].astype(np.float64).sum())
                            for i in range(run.n_int)])
        assert np.abs(got_db[tested] - want_db[tested]).max() <= JND_DB_TOL


def test_jnd_sweep_groups_bit_exact_against_the_reference_default(mv):
    """Whole groups of the JND sweep (hearing-loss profile, seeded noise,
    10-100 dB tones and the noise-only reference) through the reference's
    compiled BMOHC_NEW_kernel as Run_Cuda launches it, and through the
    product's reference-arithmetic mode: bit-exact on every owned row.  The
    shortest group (44 blocks) and the longest (220 blocks, 196 ms signals)."""
    from cochlearmodel_gb300 import batch
    from oracle import ref_gpu_sweep
    specs = batch.jnd_sweep_spec(n_seeds=4)
    md = orc.model_setup()
    order = np.argsort([sp["length"] for sp in specs])
    for gi in (order[0], order[-1]):
        g = ref_gpu_sweep.compare_group(specs[gi], mv, md)
        print(f"JND-sweep group {gi}: {g['blocks']} blocks, {g['owned_rows']} owned rows, "
              f"bit-exact {g['bit_exact']}")
        assert "reference_ms" in g, g.get("reference")
        assert g["owned_rows"] > 0 and g["bit_exact"]
