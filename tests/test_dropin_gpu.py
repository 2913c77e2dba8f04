"""The reference-named API (include/cochlea_common.h), driven by the
Run_Cuda-order harness from a .par file, against the device pipeline that the
other GPU tests pin to the oracle."""
import subprocess

import numpy as np
import pytest

from cochlearmodel_gb300 import build, ihc, model
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
"""


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


def test_harness_matches_pipeline(tmp_path, mv):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    noise = np.random.default_rng(11).standard_normal(402).astype(np.float32)
    ac = ihc.design_ac_lowpass()
    (tmp_path / "ac.f32").write_bytes(ac.tobytes())
    (tmp_path / "noise.f32").write_bytes(noise.tobytes())
    out = tmp_path / "out.bin"
    par = tmp_path / "run.par"
    par.write_text(PAR.format(ac=tmp_path / "ac.f32", noise=tmp_path / "noise.f32", out=out))
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
