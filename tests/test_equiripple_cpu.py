"""The equiripple (Parks-McClellan) AC filter designer: agreement with an
independent Remez implementation (scipy), linear phase, unit DC gain, the
equiripple property of the weighted error, and the reference's parameter
front-end (minimum order, weights)."""
import math

import numpy as np
import pytest

from cochlearmodel_gb300 import ihc

sg = pytest.importorskip("scipy.signal")


@pytest.mark.parametrize("nt,fp,fsb,wp,ws", [(255, 800, 1600, 1, 10), (101, 2000, 4000, 1, 1),
                                             (64, 1000, 3000, 2, 5), (31, 5000, 15000, 1, 1)])
def test_matches_remez(nt, fp, fsb, wp, ws):
    taps, delta = ihc.design_ac_equiripple(fp, fsb, 1e5, nt, wp, ws)
    ref = sg.remez(nt, [0, fp, fsb, 5e4], [1, 0], weight=[wp, ws], fs=1e5, maxiter=100)
    ref = ref / ref.sum()
    assert np.abs(taps.astype(np.float64) - ref).max() <= 1e-3 * np.abs(ref).max()
    assert np.allclose(taps, taps[::-1], atol=1e-9)          # linear phase
    assert abs(float(taps.astype(np.float64).sum()) - 1.0) < 1e-6  # unit DC gain


def test_equiripple_error():
    taps, delta = ihc.design_ac_equiripple(2000, 4000, 1e5, 101, 1.0, 4.0)
    w, h = sg.freqz(taps.astype(np.float64), worN=20000, fs=1e5)
    H = np.abs(h)
    # DC gain normalisation moves the pass band by the ripple; the weighted
    # errors in the two bands are within a few percent of each other
    ep = np.abs(H[w <= 2000] - np.mean(H[w <= 2000])).max()
    es = 4.0 * H[w >= 4000].max()
    assert ep > 0 and es > 0 and abs(ep - es) / es < 0.1


def test_spec_front_end():
    taps, delta = ihc.design_ac_from_spec(800.0, 2000.0, 1e5, apass_db=1.0, astop_db=40.0)
    dp, ds = 10 ** (-1 / 20), 10 ** (-40 / 20)
    n = math.ceil((-10 * math.log10(dp * ds) - 13) / (2.324 * (1200 / 5e4) * math.pi))
    assert len(taps) == n
    # the reference's ripple conversion (toDelta = 10^(-A/20)) makes the pass
    # "ripple" 0.89 for 1 dB, so this order alone gives a shallow filter (its
    # later searches are not reproduced); it is still a low-pass
    w, h = sg.freqz(taps.astype(np.float64), worN=8192, fs=1e5)
    assert np.abs(h[w >= 2000]).max() < 0.5 * np.abs(h[w <= 800]).min()
