"""Hearing-aid shaping of the generated input (src/cochlea.cu:4105-4150,
4454-4503): the device kernels against the oracle bit for bit, the profile
pipeline with a hearing aid, and the drop-in driven by the .par keys
Hearing_AID_FIR_Transfer_Function / Hearing_AID_IIR_Transfer_Function."""
import subprocess

import numpy as np
import pytest

from cochlearmodel_gb300 import build, ihc, model, native
from cochlearmodel_gb300.pipeline import JNDWindow, ProfileRun, ProfileSweep
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _ha_dev(x, fir, iir):
    import torch
    d = torch.from_numpy(np.ascontiguousarray(x, np.float32)).cuda()
    aux = torch.zeros_like(d)
    f = torch.from_numpy(np.ascontiguousarray(fir, np.float32)).cuda()
    g = torch.from_numpy(np.ascontiguousarray(iir, np.float32)).cuda() if len(iir) else None
    native.check(native.load().cgb_hearing_aid_dev(
        native.ptr(d), x.shape[0], x.shape[1], native.ptr(f), len(fir), native.ptr(g), len(iir),
        native.ptr(aux), None), "hearing aid")
    torch.cuda.synchronize()
    return d.cpu().numpy()


@pytest.mark.parametrize("fir_len,iir_len", [(9, 4), (1, 0), (31, 0), (1, 6)])
def test_kernels_match_oracle(fir_len, iir_len):
    rng = np.random.default_rng(fir_len * 10 + iir_len)
    x = rng.normal(size=(5, 1000)).astype(np.float32)
    fir = rng.normal(size=fir_len).astype(np.float32) if fir_len > 1 else np.ones(1, np.float32)
    iir = (-0.3 * rng.random(iir_len)).astype(np.float32) if iir_len else np.zeros(0, np.float32)
    if iir_len:
        iir[0] = 1.0
    g = _ha_dev(x, fir, iir)
    o = orc.hearing_aid(x, fir, iir)
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))
    assert np.all(g[:, 0] == 0.0)  # the first sample of an interval gets no FIR term


def test_profile_run_with_hearing_aid(mv):
    import torch
    cfg = model.RunConfig(Time_Block_Length=0.002, Decouple_Filter=2, Overlap_Time=0.001)
    sweep = ProfileSweep(frequencies=[1000.0, 3000.0], powers=[60.0], noises=[1111.0])
    fir = np.array([0.5, 0.3, 0.2, -0.1], np.float32)
    iir = np.array([1.0, 0.4, -0.1], np.float32)
    plain = ProfileRun("cuda:0", cfg, sweep, mv=mv, want_lambda=False)
    aided = ProfileRun("cuda:0", cfg, sweep, mv=mv, want_lambda=False, hearing_aid=(fir, iir))
    plain.generate_input()
    aided.generate_input()
    torch.cuda.synchronize()
    n = plain.n_int * plain.L
    x = plain.d_in.cpu().numpy()[:n].reshape(plain.n_int, plain.L)
    o = orc.hearing_aid(x, fir, iir)
    g = aided.d_in.cpu().numpy()[:n].reshape(plain.n_int, plain.L)
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))
    # identity functions leave the input untouched
    ident = ProfileRun("cuda:0", cfg, sweep, mv=mv, want_lambda=False,
                       hearing_aid=(np.ones(1, np.float32), np.ones(1, np.float32)))
    assert ident.ha is None


def test_harness_hearing_aid(tmp_path, mv):
    import torch
    from tests.test_dropin_gpu import PAR, read_out
    noise = np.random.default_rng(11).standard_normal(402).astype(np.float32)
    ac = ihc.design_ac_lowpass()
    (tmp_path / "ac.f32").write_bytes(ac.tobytes())
    (tmp_path / "noise.f32").write_bytes(noise.tobytes())
    out = tmp_path / "out.bin"
    par = tmp_path / "run.par"
    par.write_text(PAR.format(ac=tmp_path / "ac.f32", noise=tmp_path / "noise.f32", out=out) +
                   "Hearing_AID_FIR_Transfer_Function = [0.6 0.3 0.1]\n"
                   "Hearing_AID_IIR_Transfer_Function = [1 -0.2]\n")
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
    # stored form of the IIR vector: negated, element 0 = 1
    run = ProfileRun("cuda:0", cfg, sweep, noise=noise, mv=mv, ac_taps=ac,
                     jnd=JNDWindow(head=0.001, tail=0.0005),
                     hearing_aid=(np.array([0.6, 0.3, 0.1], np.float32),
                                  np.array([1.0, 0.2], np.float32)))
    run.step()
    torch.cuda.synchronize()
    pv = run.d_v.cpu().numpy()[:v.shape[0]]
    assert np.array_equal(v.view(np.uint32), pv.view(np.uint32))
    assert np.array_equal(lam.view(np.uint32), run.d_lam.cpu().numpy().view(np.uint32))
