"""GPU parity of the fused IHC/lambda kernel: bit-exact against the oracle's
kernel-FP32 mode; within 1e-4 max-rel of the reference's mixed-precision
arithmetic (double taps and accumulators), the lambda bar."""
import numpy as np
import pytest

from cochlearmodel_gb300 import ihc, native
from oracle import oracle as orc
from tests import cases

pytestmark = pytest.mark.gpu

REL = 1e-4  # max |a-b| / max |b| per lambda plane


@pytest.fixture(scope="module")
def stage():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return ihc.IHCStage("cuda:0", ihc_profiles=np.stack([np.full(256, 8.0, np.float32),
                                                         np.linspace(8, 5, 256, dtype=np.float32)]))


def _oracle(stage, v, fr, mode):
    return orc.ihc_lambda(v[fr["v_row0"]:fr["v_row0"] + fr["rows"]], int(fr["seg"]),
                          int(fr["frdp"]), int(fr["total"]), int(fr["lam_rows"]),
                          stage.ac.astype(np.float64), stage.dc.astype(np.float64),
                          stage.nerve.scale, stage.nerve.eta_AC, stage.nerve.eta_DC,
                          stage.dmg_host[fr["ihc_profile"]].astype(np.float64),
                          stage.nerve.aihc(), np.asarray(stage.nerve.spontRate, np.float32),
                          stage.nerve.Lambda_SAT, mode=mode)


def _check(stage, v, frames, lam_rows):
    lam, ih = stage.run(v, frames, lam_rows, want_ihc=True)
    for fr in frames:
        r0, n = int(fr["lam_row0"]), int(fr["lam_rows"])
        o_ihc, o_lam = _oracle(stage, v, fr, 2)
        assert np.array_equal(ih[r0:r0 + n].view(np.uint32), o_ihc[:n].view(np.uint32))
        assert np.array_equal(lam[:, r0:r0 + n].view(np.uint32), o_lam.view(np.uint32))
        _, ref_lam = _oracle(stage, v, fr, 0)
        for j in range(3):
            d = np.abs(lam[j, r0:r0 + n] - ref_lam[j]).max() / np.abs(ref_lam[j]).max()
            assert d <= REL, (j, d)
    return lam


def test_reference_run_frame(mv, stage):
    case = cases.decoupled_sweep(mv, n_signals=2, decouple=2, block_ms=1.5, overlap_ms=0.5)
    cfg, sc, gamma, units, x, rows = case
    v, _, _ = orc.bm_run(mv.section_params(), gamma, sc, units, x, rows)
    fr = ihc.reference_frame(cfg)
    v = v[:int(fr["rows"][0])]
    lam = _check(stage, v, fr, int(fr["lam_rows"][0]))
    assert (lam[:, :, 0] == np.asarray(stage.nerve.spontRate, np.float32)[:, None]).all()


def test_many_tiles_and_frames(stage):
    rng = np.random.default_rng(3)
    t = np.arange(3600)[:, None] / 1e5
    f = 300 + 40 * np.arange(256)[None, :]
    v = (1e-3 * np.sin(2 * np.pi * f * t) * (1 + rng.random((1, 256)))).astype(np.float32)
    frames = np.zeros(3, ihc.FRAME_DTYPE)
    # three frames back to back: 1000 + 1500 + 1100 rows, different rules
    starts, lens = [0, 1000, 2500], [1000, 1500, 1100]
    lam0 = 0
    for i, (s, n) in enumerate(zip(starts, lens)):
        frames[i] = (s, lam0, n, n - 100 if i == 2 else n, [500, 1500, 400][i], n if i < 2 else n - 100,
                     ihc.round64(n), i % 2)
        lam0 += frames[i]["lam_rows"]
    _check(stage, v, frames, lam0)
    # a debug stage over the same frames: each frame's rows land at its
    # lambda rows, bit-exact against the oracle's kernel arithmetic
    for st_n in (9, 10, 11):
        _, _, plane = stage.run(v, frames, lam0, stage=st_n)
        for fr in frames:
            r0, n = int(fr["lam_row0"]), int(fr["lam_rows"])
            want = orc.ihc_lambda_stage(
                v[fr["v_row0"]:fr["v_row0"] + fr["rows"]], int(fr["seg"]), int(fr["frdp"]),
                int(fr["total"]), n, stage.ac.astype(np.float64), stage.dc.astype(np.float64),
                stage.nerve.scale, stage.nerve.eta_AC, stage.nerve.eta_DC,
                stage.dmg_host[fr["ihc_profile"]].astype(np.float64), stage.nerve.aihc(),
                np.asarray(stage.nerve.spontRate, np.float32), stage.nerve.Lambda_SAT, st_n,
                mode=2)
            assert np.array_equal(plane[r0:r0 + n].view(np.uint32), want.view(np.uint32)), st_n


@pytest.mark.parametrize("kind", ["asymmetric", "even_symmetric"])
def test_other_ac_filters(kind):
    """The FIR paths besides the default odd symmetric filter (tap pairs plus a
    centre tap): an asymmetric filter takes the plain Dot2 over taps, an even
    symmetric one the tap pairs alone.  Bit-exact against the oracle and
    within the lambda bar, on frames with look-back restarts."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    base = ihc.design_ac_lowpass().astype(np.float64)
    if kind == "asymmetric":
        taps = base * (1.0 + 0.3 * np.arange(len(base)) / (len(base) - 1))
    else:
        taps = 0.5 * (base[:-1] + base[1:])
    taps = (taps / taps.sum()).astype(np.float32)
    st = ihc.IHCStage("cuda:0", ac_taps=taps)
    rng = np.random.default_rng(11)
    t = np.arange(2600)[:, None] / 1e5
    f = 250 + 45 * np.arange(256)[None, :]
    v = (1e-3 * np.sin(2 * np.pi * f * t) * (1 + rng.random((1, 256)))).astype(np.float32)
    frames = np.zeros(2, ihc.FRAME_DTYPE)
    frames[0] = (0, 0, 1300, 1300, 650, 1300, ihc.round64(1300), 0)
    frames[1] = (1300, 1300, 1300, 1200, 1300, 1200, ihc.round64(1300), 0)
    _check(st, v, frames, 2500)


def test_empty_frame_table(stage):
    lam, _ = stage.run(np.zeros((10, 256), np.float32), np.zeros(0, ihc.FRAME_DTYPE), 4)
    assert not lam.any()


def _oracle_iir(stage, v, fr, b, a, mode):
    return orc.ihc_lambda_iir(v[fr["v_row0"]:fr["v_row0"] + fr["rows"]], int(fr["seg"]),
                              int(fr["frdp"]), int(fr["total"]), int(fr["lam_rows"]),
                              b.astype(np.float64), a.astype(np.float64),
                              stage.dc.astype(np.float64), stage.nerve.scale,
                              stage.nerve.eta_AC, stage.nerve.eta_DC,
                              stage.dmg_host[fr["ihc_profile"]].astype(np.float64),
                              stage.nerve.aihc(), np.asarray(stage.nerve.spontRate, np.float32),
                              stage.nerve.Lambda_SAT, mode=mode)


def _check_iir(stage, v, frames, lam_rows, b, a):
    lam, ih, ac = stage.run_iir(v, frames, lam_rows, b, a, want_ihc=True)
    for fr in frames:
        r0, n, v0 = int(fr["lam_row0"]), int(fr["lam_rows"]), int(fr["v_row0"])
        o_ihc, o_lam, o_ac = _oracle_iir(stage, v, fr, b, a, 2)
        assert np.array_equal(ac[v0:v0 + n].view(np.uint32), o_ac[:n].view(np.uint32))
        assert np.array_equal(ih[r0:r0 + n].view(np.uint32), o_ihc[:n].view(np.uint32))
        assert np.array_equal(lam[:, r0:r0 + n].view(np.uint32), o_lam.view(np.uint32))
        _, ref_lam, _ = _oracle_iir(stage, v, fr, b, a, 0)
        for j in range(3):
            d = np.abs(lam[j, r0:r0 + n] - ref_lam[j]).max() / np.abs(ref_lam[j]).max()
            assert d <= REL, (j, d)


@pytest.mark.parametrize("order", [2, 4])
def test_iir_ac_reference_run_frame(mv, stage, order):
    """The AC stage by IIR (is_ac_iir_filter): AC, IHC and lambda bit-exact
    against the oracle; lambda within the bar of the reference arithmetic."""
    case = cases.decoupled_sweep(mv, n_signals=2, decouple=2, block_ms=1.5, overlap_ms=0.5)
    cfg, sc, gamma, units, x, rows = case
    v, _, _ = orc.bm_run(mv.section_params(), gamma, sc, units, x, rows)
    fr = ihc.reference_frame(cfg)
    v = v[:int(fr["rows"][0])]
    b, a = ihc.design_ac_iir_lowpass(order=order)
    _check_iir(stage, v, fr, int(fr["lam_rows"][0]), b, a)


def test_iir_ac_frames_with_rule_switch(stage):
    """Frames whose look-back rule switches to the frame total part-way (the
    recursion must not be split there)."""
    rng = np.random.default_rng(5)
    t = np.arange(3600)[:, None] / 1e5
    f = 300 + 40 * np.arange(256)[None, :]
    v = (1e-3 * np.sin(2 * np.pi * f * t) * (1 + rng.random((1, 256)))).astype(np.float32)
    frames = np.zeros(3, ihc.FRAME_DTYPE)
    starts, lens = [0, 1000, 2500], [1000, 1500, 1100]
    lam0 = 0
    for i, (s, n) in enumerate(zip(starts, lens)):
        frames[i] = (s, lam0, n, n - 100 if i == 2 else n, [500, 1500, 400][i],
                     n if i < 2 else n - 100, ihc.round64(n), i % 2)
        lam0 += frames[i]["lam_rows"]
    b, a = ihc.design_ac_iir_lowpass(order=2)
    _check_iir(stage, v, frames, lam0, b, a)


def test_staging_wait_runs_out_and_reports(stage):
    """Failure detection without a GPU fault: with the test-only injection on,
    each CTA arms its first staging wait but issues no copy, so the wait runs
    out after about one second (nothing in flight) and the kernel reports
    status bit 1, which the host turns into an error.  The context stays
    usable: the next launch without injection gives the normal result."""
    from cochlearmodel_gb300 import native
    lib = native.load()
    rng = np.random.default_rng(4)
    v = (1e-3 * rng.standard_normal((600, 256))).astype(np.float32)
    frames = np.zeros(1, ihc.FRAME_DTYPE)
    frames[0] = (0, 0, 600, 600, 600, 600, ihc.round64(600), 0)
    want, _ = stage.run(v, frames, 600)
    native.check(lib.cgb_ihc_set_fault_injection(1), "fault injection")
    try:
        with pytest.raises(native.CGBError, match="did not complete"):
            stage.run(v, frames, 600)
    finally:
        native.check(lib.cgb_ihc_set_fault_injection(0), "fault injection")
    again, _ = stage.run(v, frames, 600)
    assert np.array_equal(again.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("stage", [9, 10, 11, 12])
def test_debug_stages(mv, stage):
    """RunIHCKernel's debug stages (9 AC, 10 DC, 11 and 12 dS): the plane the
    kernel stores is bit-exact against the oracle's kernel arithmetic, within
    the lambda bar of the reference arithmetic, and the lambda planes equal a
    run without a stage."""
    st = ihc.IHCStage("cuda:0")
    case = cases.decoupled_sweep(mv, n_signals=2, decouple=2, block_ms=1.5, overlap_ms=0.5)
    cfg, sc, gamma, units, x, rows = case
    v, _, _ = orc.bm_run(mv.section_params(), gamma, sc, units, x, rows)
    fr = ihc.reference_frame(cfg)
    v = v[:int(fr["rows"][0])]
    n = int(fr["lam_rows"][0])
    lam0, _ = st.run(v, fr, n)
    lam, _, plane = st.run(v, fr, n, stage=stage)
    assert np.array_equal(lam.view(np.uint32), lam0.view(np.uint32))
    o_stage = 11 if stage == 12 else stage
    args = (v, int(fr["seg"][0]), int(fr["frdp"][0]), int(fr["total"][0]), n,
            st.ac.astype(np.float64), st.dc.astype(np.float64), st.nerve.scale,
            st.nerve.eta_AC, st.nerve.eta_DC, st.dmg_host[0].astype(np.float64),
            st.nerve.aihc(), np.asarray(st.nerve.spontRate, np.float32), st.nerve.Lambda_SAT,
            o_stage)
    want = orc.ihc_lambda_stage(*args, mode=2)
    assert np.array_equal(plane.view(np.uint32), want.view(np.uint32))
    ref = orc.ihc_lambda_stage(*args, mode=0)
    assert np.abs(plane - ref).max() <= REL * np.abs(ref).max()
    assert np.abs(plane).max() > 0


def test_debug_stage_rejected():
    st = ihc.IHCStage("cuda:0")
    v = np.zeros((600, 256), np.float32)
    fr = np.zeros(1, ihc.FRAME_DTYPE)
    fr[0] = (0, 0, 600, 512, 600, 600, ihc.round64(600), 0)
    for bad in (8, 13):
        with pytest.raises(native.CGBError):
            st.run(v, fr, 512, stage=bad)


@pytest.mark.parametrize("stage_n", [9, 10, 11])
def test_iir_debug_stages(mv, stage, stage_n):
    """The debug stages on the IIR AC path: AC is the IIR's output; DC and dS
    bit-exact against the oracle fed the same AC (kernel arithmetic)."""
    case = cases.decoupled_sweep(mv, n_signals=2, decouple=2, block_ms=1.5, overlap_ms=0.5)
    cfg, sc, gamma, units, x, rows = case
    v, _, _ = orc.bm_run(mv.section_params(), gamma, sc, units, x, rows)
    fr = ihc.reference_frame(cfg)
    v = v[:int(fr["rows"][0])]
    n = int(fr["lam_rows"][0])
    b, a = ihc.design_ac_iir_lowpass(order=2)
    lam0, _, ac0 = stage.run_iir(v, fr, n, b, a)
    lam, _, ac, plane = stage.run_iir(v, fr, n, b, a, stage=stage_n)
    assert np.array_equal(lam.view(np.uint32), lam0.view(np.uint32))
    assert np.array_equal(ac.view(np.uint32), ac0.view(np.uint32))
    f = fr[0]
    _, _, want = orc.ihc_lambda_ac(v, ac, int(f["seg"]), int(f["frdp"]), int(f["total"]), n,
                                   stage.dc.astype(np.float64), stage.nerve.scale,
                                   stage.nerve.eta_AC, stage.nerve.eta_DC,
                                   stage.dmg_host[0].astype(np.float64), stage.nerve.aihc(),
                                   np.asarray(stage.nerve.spontRate, np.float32),
                                   stage.nerve.Lambda_SAT, mode=2, stage=stage_n)
    assert np.array_equal(plane.view(np.uint32), want.view(np.uint32))
    if stage_n == 9:
        assert np.array_equal(plane.view(np.uint32), ac[:n].view(np.uint32))
