"""GPU parity of input generation, JND and the whole profile-mode path
(input -> BM -> IHC/lambda -> JND) against the oracle chain."""
import numpy as np
import pytest

from cochlearmodel_gb300 import model
from cochlearmodel_gb300.pipeline import JNDWindow, ProfileRun, ProfileSweep
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

JND_DB_TOL = 0.1    # dB, final JND against the reference float arithmetic
F_REL_FP64 = 1e-6   # Fisher sums against the FP64 oracle (FP32 terms, compensated sums)


@pytest.fixture(scope="module")
def run(mv):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    cfg = model.RunConfig(Time_Block_Length=0.002, Decouple_Filter=2, Overlap_Time=0.001,
                          OHC_Vector=np.linspace(0.5, 0.05, 256, dtype=np.float32),
                          IHC_Vector=np.linspace(8, 5, 256, dtype=np.float32))
    sweep = ProfileSweep(frequencies=[1000.0, 3000.0], powers=[40.0, 80.0],
                         noises=[1111.0, 30.0], calculate_jnd=True)
    noise = np.random.default_rng(7).standard_normal(400).astype(np.float32)
    r = ProfileRun("cuda:0", cfg, sweep, noise=noise, mv=mv,
                   jnd=JNDWindow(head=0.001, tail=0.0005))
    r.step()
    torch.cuda.synchronize()
    return r


def test_input_generation(run):
    got = run.d_in.cpu().numpy()[:run.n_int * run.L].reshape(run.n_int, run.L)
    prof = np.stack([run.prof["dA"], run.prof["Wn"], run.prof["frequency"]], 1)
    want = orc.input_gen(prof, run.noise, run.L, 0, float(run.cfg.Fs), 0.0, 1.0, 1.0)
    ulp = np.spacing(np.abs(want)).astype(np.float64)
    err = np.abs(got.astype(np.float64) - want) / np.maximum(ulp, 1e-45)
    assert err.max() <= 1.0 and (err > 0).mean() < 1e-3


def test_bm_and_lambda_stages(run, mv):
    x = run.d_in.cpu().numpy()
    v_o, f_o, st_o = orc.bm_run(mv.section_params(), run.cfg.gamma()[None], run.sc, run.units,
                                x, run.rows)
    v = run.d_v.cpu().numpy()
    assert np.array_equal(v.view(np.uint32), v_o.view(np.uint32))
    fr = run.frames[0]
    st = run.ihc
    _, lam_o = orc.ihc_lambda(v[:fr["rows"]], int(fr["seg"]), int(fr["frdp"]), int(fr["total"]),
                              int(fr["lam_rows"]), st.ac.astype(np.float64),
                              st.dc.astype(np.float64), 1.0, 1.0, 100.0,
                              st.dmg_host[0].astype(np.float64), st.nerve.aihc(),
                              np.asarray(st.nerve.spontRate, np.float32), 500.0, mode=2)
    assert np.array_equal(run.d_lam.cpu().numpy().view(np.uint32), lam_o.view(np.uint32))


def test_jnd_sums_and_db(run):
    lam = run.d_lam.cpu().numpy()
    args = (lam, run.n_int, run.L, run.head, run.len, run.prof["dA"], run.ref_of,
            run.nerve.nihc(), np.asarray(run.nerve.W, np.float32), float(run.cfg.Fs),
            0.2 * run.cfg.Fs)
    ra64, ai64 = orc.jnd(*args, fp64=True)
    ra32, ai32 = orc.jnd(*args, fp64=False)
    rate_db, ai_db, F_RA, F_AI = run.jnd_db()
    tested = run.ref_of != np.arange(run.n_int)
    assert tested.sum() == 8
    for got, want in ((F_RA, ra64), (F_AI, ai64)):
        rel = np.abs(got[:, tested] - want[:, tested]) / np.abs(want[:, tested])
        assert rel.max() <= F_REL_FP64
    for got_db, ref in ((rate_db, ra32), (ai_db, ai32)):
        want_db = np.array([orc.jnd_db(ref[:, i].sum()) for i in range(run.n_int)])
        assert np.abs(got_db[tested] - want_db[tested]).max() <= JND_DB_TOL
    assert np.isnan(rate_db[~tested]).all()


def test_profile_step_host_equals_step_and_copies(mv):
    """The host-buffer step of a profile run, whose kernels store their
    results into the pinned host buffers as they write them, returns exactly
    what step() followed by plain copies returns (buffers starting as NaN)."""
    import torch
    cfg = model.RunConfig(Time_Block_Length=0.00128, Decouple_Filter=2, Overlap_Time=0.0005,
                          OHC_Vector=np.linspace(0.5, 0.05, 256, dtype=np.float32))
    sweep = ProfileSweep(frequencies=[500.0, 1000.0, 2000.0, 3000.0, 4000.0],
                         powers=[40.0, 80.0], noises=[1111.0, 30.0], calculate_jnd=True)
    noise = np.random.default_rng(3).standard_normal(300).astype(np.float32)
    r = ProfileRun("cuda:0", cfg, sweep, noise=noise, mv=mv,
                   jnd=JNDWindow(head=0.0003, tail=0.0002))
    h_tables = [r.d_prof.cpu().pin_memory()]
    r.step()
    torch.cuda.synchronize()
    v0, lam0, f0 = r.d_v.cpu(), r.d_lam.cpu(), r.d_FRA.clone()
    h_v = torch.empty(r.d_v.shape, dtype=torch.float32).pin_memory()
    h_lam = torch.empty(r.d_lam.shape, dtype=torch.float32).pin_memory()
    h_v.fill_(float("nan"))
    h_lam.fill_(float("nan"))
    r.step_host(h_tables, h_v, h_lam)
    torch.cuda.synchronize()
    assert torch.equal(h_v, v0) and torch.equal(h_lam, lam0)
    assert torch.equal(r.d_FRA, f0)
