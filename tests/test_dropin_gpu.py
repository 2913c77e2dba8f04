"""The reference-named API (include/cochlea_common.h), driven by the
Run_Cuda-order harness from a .par file, against the device pipeline that the
other GPU tests pin to the oracle."""
import subprocess

import numpy as np
import pytest

from cochlearmodel_gb300 import build, ihc, model, native
from cochlearmodel_gb300.pipeline import JNDWindow, ProfileRun, ProfileSweep

pytestmark = pytest.mark.gpu

PAR = """Fs = 100000
Time_Block_Length = 0.002
Decouple_Filter = 2
Overlap_Time = 0.001
testedFrequencies = 1000, 3000
testedPowerLevels = [40 80]
testedNoises = 1111 30
Calculate_JND = 1
OHC_Vector = 0.5 0.3 0.1
IHC_Vector = 8 6
JND_Interval_Head = 0.001
JND_Interval_Tail = 0.0005
AC_Filter_File = "{ac}"
Input_Noise_File = "{noise}"
Output_File = "{out}"
Run_Fast_BM_Calculation = 17
"""
# the same run with the reference's default kernel selection (no
# Run_Fast_BM_Calculation key: BMOHC_NEW_kernel)
PAR_DEFAULT_KERNEL = PAR.replace("Run_Fast_BM_Calculation = 17\n", "")


def read_out(path):
    raw = open(path, "rb").read()
    rows, lam_rows, n, _ = np.frombuffer(raw[:32], np.int64)
    off = 32
    def take(count, dt):
        nonlocal off
        a = np.frombuffer(raw[off:off + count * np.dtype(dt).itemsize], dt)
        off += count * np.dtype(dt).itemsize
        return a
    v = take(rows * 256, np.float32).reshape(rows, 256)
    lam = take(3 * lam_rows * 256, np.float32).reshape(3, lam_rows, 256)
    fra = take(3 * n, np.float32).reshape(3, n)
    fai = take(3 * n, np.float32).reshape(3, n)
    jr = take(n, np.float64)
    ja = take(n, np.float64)
    return v, lam, fra, fai, jr, ja


@pytest.mark.parametrize("kernel", [17, 0])
def test_harness_matches_pipeline(tmp_path, mv, kernel):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    noise = np.random.default_rng(11).standard_normal(402).astype(np.float32)
    ac = ihc.design_ac_lowpass()
    (tmp_path / "ac.f32").write_bytes(ac.tobytes())
    (tmp_path / "noise.f32").write_bytes(noise.tobytes())
    out = tmp_path / "out.bin"
    par = tmp_path / "run.par"
    text = PAR if kernel == 17 else PAR_DEFAULT_KERNEL
    par.write_text(text.format(ac=tmp_path / "ac.f32", noise=tmp_path / "noise.f32", out=out))
    build.build()
    res = subprocess.run([str(build.harness_path()), str(par)], capture_output=True, text=True,
                         timeout=300)
    assert res.returncode == 0, res.stderr
    v, lam, fra, fai, jr, ja = read_out(out)

    cfg = model.RunConfig(Time_Block_Length=0.002, Decouple_Filter=2, Overlap_Time=0.001,
                          OHC_Vector=np.array([0.5, 0.3, 0.1], np.float32),
                          IHC_Vector=np.array([8.0, 6.0], np.float32),
                          Run_Fast_BM_Calculation=kernel)
    sweep = ProfileSweep(frequencies=[1000.0, 3000.0], powers=[40.0, 80.0],
                         noises=[1111.0, 30.0], calculate_jnd=True)
    run = ProfileRun("cuda:0", cfg, sweep, noise=noise, mv=mv, ac_taps=ac,
                     jnd=JNDWindow(head=0.001, tail=0.0005))
    run.step()
    torch.cuda.synchronize()
    pv = run.d_v.cpu().numpy()[:v.shape[0]]
    assert np.array_equal(v.view(np.uint32), pv.view(np.uint32))
    assert np.array_equal(lam.view(np.uint32), run.d_lam.cpu().numpy().view(np.uint32))
    rate_db, ai_db, F_RA, F_AI = run.jnd_db()
    tested = run.ref_of != np.arange(run.n_int)
    assert np.allclose(fra[:, tested], F_RA[:, tested], rtol=1e-6)
    assert np.allclose(fai[:, tested], F_AI[:, tested], rtol=1e-6)
    assert np.abs(jr[tested] - rate_db[tested]).max() < 1e-4
    assert np.abs(ja[tested] - ai_db[tested]).max() < 1e-4


def test_harness_iir_ac_filter(tmp_path, mv):
    """IHCNewKernel with is_ac_iir_filter (AC_Filter_A_File): the drop-in's
    lambda equals the IIR path of the C ABI on the same velocity, bit for bit."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    noise = np.random.default_rng(11).standard_normal(402).astype(np.float32)
    b, a = ihc.design_ac_iir_lowpass(order=2)
    (tmp_path / "b.f32").write_bytes(b.tobytes())
    (tmp_path / "a.f32").write_bytes(a.tobytes())
    (tmp_path / "noise.f32").write_bytes(noise.tobytes())
    out = tmp_path / "out.bin"
    par = tmp_path / "run.par"
    par.write_text(PAR.format(ac=tmp_path / "b.f32", noise=tmp_path / "noise.f32", out=out) +
                   f'AC_Filter_A_File = "{tmp_path / "a.f32"}"\n')
    build.build()
    res = subprocess.run([str(build.harness_path()), str(par)], capture_output=True, text=True,
                         timeout=300)
    assert res.returncode == 0, res.stderr
    v, lam, fra, fai, jr, ja = read_out(out)
    cfg = model.RunConfig(Time_Block_Length=0.002, Decouple_Filter=2, Overlap_Time=0.001,
                          IHC_Vector=np.array([8.0, 6.0], np.float32))
    N = cfg.calc_time_block_nodes()
    # 2 frequencies x 2 powers x 2 noises + one reference per noise = 10
    # intervals of Decouple_Filter 2 blocks
    n_lam = N * 10 * 2
    # the drop-in's frame total is Run_Cuda's calcTime: the written rows
    # rounded up to 64
    rows = v.shape[0]
    calc_time = ihc.round64(rows)
    assert n_lam <= rows
    stage = ihc.IHCStage("cuda:0", ihc_profiles=model.expand_vector(cfg.IHC_Vector)[None])
    fr = np.zeros(1, ihc.FRAME_DTYPE)
    fr["v_row0"], fr["lam_row0"], fr["rows"], fr["lam_rows"] = 0, 0, rows, n_lam
    fr["seg"], fr["frdp"], fr["total"], fr["ihc_profile"] = N * 2, n_lam, calc_time, 0
    lam2, _, _ = stage.run_iir(np.ascontiguousarray(v[:rows]), fr, n_lam, b, a)
    assert np.array_equal(lam[:, :n_lam].view(np.uint32), lam2.view(np.uint32))
    assert np.isfinite(jr[np.isfinite(jr)]).all()


def _transpose(v, column_size):
    """transposeVector(v, column_size) of the reference (include/cvector.cpp:520-530)."""
    out = np.empty_like(v)
    row = len(v) // column_size
    for i in range(len(v)):
        out[(i % row) * column_size + i // row] = v[i]
    return out


def test_harness_writes_the_reference_output_files(tmp_path, mv):
    """With the reference's own keys (Output_Result, JND_File_Name,
    Allowed_Outputs) the harness writes the files Run_Cuda writes: raw
    float32 in write_vector order.  The Output_Result file holds the failed
    nodes, the failed blocks, velocity, the three lambda planes (the transient
    tail removed), then the failed signals and the AI and rate JNDs of the
    tested intervals; the JND file holds the two JND vectors transposed to
    frequency-major order."""
    import torch
    noise = np.random.default_rng(11).standard_normal(402).astype(np.float32)
    ac = ihc.design_ac_lowpass()
    (tmp_path / "ac.f32").write_bytes(ac.tobytes())
    (tmp_path / "noise.f32").write_bytes(noise.tobytes())
    out, res_bin, jnd_bin = tmp_path / "out.bin", tmp_path / "result.bin", tmp_path / "jnd.bin"
    par = tmp_path / "run.par"
    par.write_text(PAR.format(ac=tmp_path / "ac.f32", noise=tmp_path / "noise.f32", out=out) +
                   f'Output_Result = "{res_bin}"\nJND_File_Name = "{jnd_bin}"\n'
                   "Allowed_Outputs = 15\n")
    build.build()
    res = subprocess.run([str(build.harness_path()), str(par)], capture_output=True, text=True,
                         timeout=300)
    assert res.returncode == 0, res.stderr
    v, lam, fra, fai, jr, ja = read_out(out)

    cfg = model.RunConfig(Time_Block_Length=0.002, Decouple_Filter=2, Overlap_Time=0.001,
                          OHC_Vector=np.array([0.5, 0.3, 0.1], np.float32),
                          IHC_Vector=np.array([8.0, 6.0], np.float32))
    sweep = ProfileSweep(frequencies=[1000.0, 3000.0], powers=[40.0, 80.0],
                         noises=[1111.0, 30.0], calculate_jnd=True)
    run = ProfileRun("cuda:0", cfg, sweep, noise=noise, mv=mv, ac_taps=ac,
                     jnd=JNDWindow(head=0.001, tail=0.0005))
    run.step()
    torch.cuda.synchronize()
    nodes = run.N * cfg.Time_Blocks
    tested = run.ref_of != np.arange(run.n_int)
    n_calc = int(tested.sum())
    failed = run.d_failed.cpu().numpy()
    st = run.d_stats.cpu().numpy().view(native.STATS_DTYPE).reshape(-1)

    raw = np.fromfile(res_bin, np.float32)
    sizes = [nodes, cfg.Time_Blocks, nodes * 256, nodes * 256, nodes * 256, nodes * 256,
             n_calc, n_calc, n_calc]
    assert raw.size == sum(sizes)
    parts = np.split(raw, np.cumsum(sizes)[:-1])
    assert np.array_equal(parts[0], failed[:nodes].astype(np.float32))
    assert np.array_equal(parts[1], st["failed_samples"].astype(np.float32))
    assert np.array_equal(parts[2].reshape(nodes, 256).view(np.uint32),
                          run.d_v.cpu().numpy()[:nodes].view(np.uint32))
    for j in range(3):
        assert np.array_equal(parts[3 + j].reshape(nodes, 256).view(np.uint32),
                              lam[j, :nodes].view(np.uint32))
    assert np.array_equal(parts[6], run.failed_per_interval().astype(np.float32))
    ai, rate = ja[tested].astype(np.float32), jr[tested].astype(np.float32)
    assert np.array_equal(parts[7], ai) and np.array_equal(parts[8], rate)
    rate_db, ai_db, _, _ = run.jnd_db()
    assert np.abs(parts[7] - ai_db[tested]).max() < 1e-3

    cols = n_calc // (2 * 2) * 2  # tested intervals / (powers x frequencies) x powers
    jnd = np.fromfile(jnd_bin, np.float32)
    assert np.array_equal(jnd, np.concatenate([_transpose(ai, cols), _transpose(rate, cols)]))


def test_harness_writes_the_ihc_stage_file(tmp_path, mv):
    """TEST_File_Target with Type_TEST_Output AC, DC, dS, Shigh or IHC: the
    harness writes RunIHCKernel's backup of that stage, write_time x 256 raw
    floats, as the reference's AudioGramCreator does.  Each file equals the
    stage plane of the IHC kernel on the same velocity (bit for bit).  The
    default type, MeanRate, writes the JND's mean rates, JND_Lambda the
    lambda planes, and the JND's debug stages (AvgMeanRate, dMeanRate,
    dLambda, preFisherAI, preFisherAITimeReduced, CRLB_RA) their values; an
    unknown type is refused."""
    import torch
    noise = np.random.default_rng(11).standard_normal(402).astype(np.float32)
    ac = ihc.design_ac_lowpass()
    (tmp_path / "ac.f32").write_bytes(ac.tobytes())
    (tmp_path / "noise.f32").write_bytes(noise.tobytes())
    build.build()
    cfg = model.RunConfig(Time_Block_Length=0.002, Decouple_Filter=2, Overlap_Time=0.001,
                          OHC_Vector=np.array([0.5, 0.3, 0.1], np.float32),
                          IHC_Vector=np.array([8.0, 6.0], np.float32))
    sweep = ProfileSweep(frequencies=[1000.0, 3000.0], powers=[40.0, 80.0],
                         noises=[1111.0, 30.0], calculate_jnd=True)
    run = ProfileRun("cuda:0", cfg, sweep, noise=noise, mv=mv, ac_taps=ac,
                     jnd=JNDWindow(head=0.001, tail=0.0005))
    run.step()
    torch.cuda.synchronize()
    nodes = run.N * cfg.Time_Blocks
    v = run.d_v.cpu().numpy()
    lam_rows = int(run.d_lam.shape[1])
    for name, stage in (("AC", 9), ("DC", 10), ("dS", 11), ("Shigh", 12), ("IHC", 13)):
        target = tmp_path / f"stage_{name}.bin"
        par = tmp_path / f"run_{name}.par"
        par.write_text(PAR.format(ac=tmp_path / "ac.f32", noise=tmp_path / "noise.f32",
                                  out=tmp_path / f"out_{name}.bin") +
                       f'TEST_File_Target = "{target}"\nType_TEST_Output = "{name}"\n')
        res = subprocess.run([str(build.harness_path()), str(par)], capture_output=True,
                             text=True, timeout=300)
        assert res.returncode == 0, res.stderr
        got = np.fromfile(target, np.float32)
        assert got.size % 256 == 0 and got.size // 256 >= nodes
        got = got.reshape(-1, 256)
        if stage == 13:
            _, want = run.ihc.run(v, run.frames, lam_rows, want_ihc=True)
        else:
            _, _, want = run.ihc.run(v, run.frames, lam_rows, stage=stage)
        assert np.array_equal(got[:nodes].view(np.uint32), want[:nodes].view(np.uint32)), name
    # MeanRate, the default type: the JND's mean rates, [3][intervals][256]
    par = tmp_path / "run_mr.par"
    par.write_text(PAR.format(ac=tmp_path / "ac.f32", noise=tmp_path / "noise.f32",
                              out=tmp_path / "out_mr.bin") +
                   f'TEST_File_Target = "{tmp_path / "mr.bin"}"\n')
    res = subprocess.run([str(build.harness_path()), str(par)], capture_output=True, text=True,
                         timeout=300)
    assert res.returncode == 0, res.stderr
    mr = np.fromfile(tmp_path / "mr.bin", np.float32).reshape(3, run.n_int, 256)
    lam = run.d_lam.cpu().numpy()
    for i in range(run.n_int):
        w = lam[:, i * run.L + run.head:i * run.L + run.head + run.len].astype(np.float64)
        want = w.mean(axis=1)
        assert np.abs(mr[:, i] - want).max() <= 1e-6 * np.abs(want).max()
    # JND_Lambda: the three lambda planes; JND_Lambda(k): plane k
    for name, planes in (("JND_Lambda", [0, 1, 2]), ("JND_Lambda(1)", [1])):
        target = tmp_path / "jl.bin"
        par.write_text(PAR.format(ac=tmp_path / "ac.f32", noise=tmp_path / "noise.f32",
                                  out=tmp_path / "out_mr.bin") +
                       f'TEST_File_Target = "{target}"\nType_TEST_Output = "{name}"\n')
        res = subprocess.run([str(build.harness_path()), str(par)], capture_output=True,
                             text=True, timeout=300)
        assert res.returncode == 0, res.stderr
        got = np.fromfile(target, np.float32).reshape(len(planes), -1, 256)
        for k, j in enumerate(planes):
            assert np.array_equal(got[k, :nodes].view(np.uint32), lam[j, :nodes].view(np.uint32))
    # the JND's debug stages, against the same quantities formed here from lambda
    L, head, ln, n = run.L, run.head, run.len, run.n_int
    dA = run.prof["dA"].astype(np.float64)
    win = np.stack([lam[:, i * L + head:i * L + head + ln].astype(np.float64) for i in range(n)],
                   axis=1)                                  # [3][n][len][256]
    MR = win.mean(axis=2)                                   # [3][n][256]
    ref = run.ref_of
    with np.errstate(divide="ignore", invalid="ignore"):
        dmr = (MR - MR[:, ref]) / dA[None, :, None]   # NaN where dA = 0, as the reference
    T, Fs = 0.2, 100000.0
    with np.errstate(divide="ignore", invalid="ignore"):
        dl = np.where(dA[None, :, None, None] > 0,
                      (win - win[:, ref]) / dA[None, :, None, None], 0.0)
    pre = dl * dl / (Fs * win[:, ref])
    nihc = np.full(256, float(np.float32(30000.0 / 256.0)))
    with np.errstate(divide="ignore", invalid="ignore"):
        want = {"AvgMeanRate": MR.mean(axis=2), "dMeanRate": dmr,
                "CRLB_RA": 1.0 / np.sqrt(T * dmr * dmr / MR[:, ref]),
                "preFisherAITimeReduced": (T / (ln / Fs)) * nihc * pre.sum(axis=2),
                "dLambda": dl, "dLambda(2)": dl[2:], "preFisherAI": pre}
    for name, w in want.items():
        target = tmp_path / "js.bin"
        par.write_text(PAR.format(ac=tmp_path / "ac.f32", noise=tmp_path / "noise.f32",
                                  out=tmp_path / "out_mr.bin") +
                       f'TEST_File_Target = "{target}"\nType_TEST_Output = "{name}"\n')
        res = subprocess.run([str(build.harness_path()), str(par)], capture_output=True,
                             text=True, timeout=300)
        assert res.returncode == 0, (name, res.stderr)
        got = np.fromfile(target, np.float32).astype(np.float64)
        if name.startswith(("dLambda", "preFisherAI")) and name != "preFisherAITimeReduced":
            planes = got.reshape(w.shape[0], -1, 256)
            got = np.stack([planes[:, i * L + head:i * L + head + ln] for i in range(n)], axis=1)
        got = got.reshape(w.shape)
        fin = np.isfinite(w)
        assert np.array_equal(np.isfinite(got), fin), name
        scale = np.abs(w[fin]).max()
        assert np.abs(got[fin] - w[fin]).max() <= 1e-5 * scale, name
    par.write_text(PAR.format(ac=tmp_path / "ac.f32", noise=tmp_path / "noise.f32",
                              out=tmp_path / "out_mr.bin") +
                   f'TEST_File_Target = "{tmp_path / "x.bin"}"\nType_TEST_Output = "Nonsense"\n')
    res = subprocess.run([str(build.harness_path()), str(par)], capture_output=True, text=True,
                         timeout=300)
    assert res.returncode != 0 and "not served" in res.stderr


def test_unbuilt_kernel_selectors_raise(tmp_path, mv):
    """BMOHCNewKernel raises for Run_Fast_BM_Calculation values, cache hints
    and enable flags it does not build, instead of running another solver."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    noise = np.random.default_rng(11).standard_normal(402).astype(np.float32)
    (tmp_path / "ac.f32").write_bytes(ihc.design_ac_lowpass().tobytes())
    (tmp_path / "noise.f32").write_bytes(noise.tobytes())
    build.build()
    for extra in ("Run_Fast_BM_Calculation = 5\n", "BMOHC_Kernel_Configuration = 7\n"):
        par = tmp_path / "bad.par"
        par.write_text(PAR_DEFAULT_KERNEL.format(ac=tmp_path / "ac.f32",
                                                 noise=tmp_path / "noise.f32",
                                                 out=tmp_path / "o.bin") + extra)
        res = subprocess.run([str(build.harness_path()), str(par)], capture_output=True,
                             text=True, timeout=300)
        assert res.returncode != 0
        assert "Run_Fast_BM_Calculation" in res.stderr or "BMOHC_Kernel_Configuration" in res.stderr


def test_relative_error_tolerances(tmp_path, mv):
    """RELATIVE_ERRORS = 1: setupToleranceProfile scales each block's throw and
    m1-sp tolerances by 10^(factor x the interval's dB SPL)
    (src/cochlea.cu:4256-4287).  The harness's velocity equals the solver run
    on the same input with those per-block tolerances, and differs from the
    run with the plain constants."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cochlearmodel_gb300.solver import BMSolver
    noise = np.random.default_rng(11).standard_normal(402).astype(np.float32)
    (tmp_path / "ac.f32").write_bytes(ihc.design_ac_lowpass().tobytes())
    (tmp_path / "noise.f32").write_bytes(noise.tobytes())
    out = tmp_path / "out.bin"
    par = tmp_path / "rel.par"
    par.write_text(PAR.format(ac=tmp_path / "ac.f32", noise=tmp_path / "noise.f32", out=out) +
                   "RELATIVE_ERRORS = 1\nM1_SP_Fix_Factor = 0.1\nTolerance_Fix_Factor = 0.1\n")
    build.build()
    res = subprocess.run([str(build.harness_path()), str(par)], capture_output=True, text=True,
                         timeout=300)
    assert res.returncode == 0, res.stderr
    v = read_out(out)[0]

    cfg = model.RunConfig(Time_Block_Length=0.002, Decouple_Filter=2, Overlap_Time=0.001,
                          OHC_Vector=np.array([0.5, 0.3, 0.1], np.float32),
                          IHC_Vector=np.array([8.0, 6.0], np.float32))
    sweep = ProfileSweep(frequencies=[1000.0, 3000.0], powers=[40.0, 80.0],
                         noises=[1111.0, 30.0], calculate_jnd=True)
    run = ProfileRun("cuda:0", cfg, sweep, noise=noise, mv=mv, ac_taps=ihc.design_ac_lowpass(),
                     jnd=JNDWindow(head=0.001, tail=0.0005))
    run.step()
    torch.cuda.synchronize()
    plain = run.d_v.cpu().numpy()[:v.shape[0]]
    units = run.units.copy()
    D = cfg.Decouple_Filter
    f32 = np.float32
    for i in range(run.n_int):
        db = 0.0 if run.is_ref[i] else [40.0, 80.0][(i % 5) // 2]
        units["mtt"][i * D:(i + 1) * D] = f32(f32(1e-10) * np.power(f32(10), f32(0.1) * f32(db)))
        units["mmspt"][i * D:(i + 1) * D] = f32(f32(1e-15) * np.power(f32(10), f32(0.1) * f32(db)))
    x = run.d_in.cpu().numpy()
    want, _, _ = BMSolver("cuda:0", mv).run(run.sc, cfg.gamma()[None], units, x, run.rows)
    assert np.array_equal(v.view(np.uint32), want[:v.shape[0]].view(np.uint32))
    assert not np.array_equal(v, plain)


def test_ihc_staging_timeout_raises_in_the_drop_in(tmp_path, mv):
    """The drop-in's RunIHCKernel turns the IHC kernel's timed-out staging
    wait (made to run out by the harness's test key) into std::runtime_error."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    noise = np.random.default_rng(11).standard_normal(402).astype(np.float32)
    (tmp_path / "ac.f32").write_bytes(ihc.design_ac_lowpass().tobytes())
    (tmp_path / "noise.f32").write_bytes(noise.tobytes())
    par = tmp_path / "fault.par"
    par.write_text(PAR.format(ac=tmp_path / "ac.f32", noise=tmp_path / "noise.f32",
                              out=tmp_path / "o.bin") + "Test_Fault_IHC_Staging = 1\n")
    build.build()
    res = subprocess.run([str(build.harness_path()), str(par)], capture_output=True, text=True,
                         timeout=300)
    assert res.returncode != 0
    assert "IHC staging copy timed out" in res.stderr
