"""The oracle and the host setup against the committed fixtures."""
import os

import numpy as np

from cochlearmodel_gb300 import ihc, model
from oracle import oracle as orc
from tests import cases

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_ac_filter_fixture():
    want = np.load(os.path.join(G, "ac_lowpass_800hz_100khz_255.npy"))
    got = ihc.design_ac_lowpass()
    assert np.array_equal(got, want)
    # low-pass: unit DC gain, attenuated well above the cut-off
    w = np.fft.rfft(got.astype(np.float64), 1 << 16)
    f = np.fft.rfftfreq(1 << 16, 1 / 100000.0)
    assert abs(abs(w[0]) - 1) < 1e-6
    assert np.abs(w[f > 2500]).max() < 0.01


def test_bm_oracle_fixture(mv):
    z = np.load(os.path.join(G, "bm_cfg1_2ms.npz"))
    cfg, sc, gamma, units, x, rows = cases.cfg1_slice(mv, ms=2.0)
    v, failed, st = orc.bm_run(mv.section_params(), gamma, sc, units, x, rows, threads=1)
    e = int(units["end"][0])
    assert np.array_equal(v[:e], z["v"])
    assert np.array_equal(failed[:e], z["failed"])
    assert np.array_equal(st["substeps"], z["substeps"])
    assert np.array_equal(st["sweeps"], z["sweeps"])


def test_own_log10_accuracy():
    xs = np.concatenate([10.0 ** np.linspace(-20, 10, 30001), np.linspace(0.5, 2, 3001)])
    xs = xs.astype(np.float32)
    got = np.array([orc.load().orc_log10f(float(x)) for x in xs], np.float64)
    exact = np.log10(xs.astype(np.float64))
    ulp = np.spacing(np.abs(exact).astype(np.float32)).astype(np.float64)
    ulp[exact == 0] = np.spacing(np.float32(1))
    assert (np.abs(got - exact) / ulp).max() <= 4.0


def test_reference_frame_layout():
    cfg = model.RunConfig(Time_Block_Length=0.01, Time_Blocks=16, Decouple_Filter=8)
    f = ihc.reference_frame(cfg)[0]
    assert f["rows"] == 16 * 1000 + 500 and f["lam_rows"] == 16000
    assert f["seg"] == 8000 and f["frdp"] == 16000 and f["total"] == 16512
    nc = ihc.NerveConfig()
    # long Fs times float Tdelta is formed in float: 200.00002f (src/AudioGramCreator.cpp:810)
    tap = np.float32(1) / (np.float32(100000) * np.float32(0.002))
    assert len(nc.dc_taps(100000)) == 200 and nc.dc_taps(100000)[0] == tap
    a = nc.aihc()
    assert a.shape == (3, 256) and a[0, 0] == 70 and a[2, 255] == 30
