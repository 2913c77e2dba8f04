"""ihc.split_frame: a Run_Cuda frame cut at interval boundaries keeps every
row's filter look-back (the reference's (k + 1) % seg rule and the full
filter on the last row) and its DC anchor phase (k % 32), so the IHC kernel
computes the same rows whether it gets the frame whole or cut."""
import numpy as np
import pytest

from cochlearmodel_gb300 import ihc, model


def _taps_used(k, f, n):
    sg = int(f["seg"]) if k < int(f["frdp"]) - 1 else int(f["total"])
    return min((k + 1) % sg, n)


@pytest.mark.parametrize("tbl,D,blocks", [(0.01, 8, 8 * 40), (0.002, 2, 2 * 20),
                                          (0.00128, 2, 2 * 24), (0.0037, 3, 3 * 9)])
@pytest.mark.parametrize("parts", [2, 3, 4, 7])
def test_split_keeps_every_row(tbl, D, blocks, parts):
    cfg = model.RunConfig(Time_Block_Length=tbl, Decouple_Filter=D, Time_Blocks=blocks)
    whole = ihc.reference_frame(cfg, v_row0=123, lam_row0=45)
    f = whole[0]
    cut = ihc.split_frame(whole, parts)
    assert 1 <= len(cut) <= parts
    L = int(f["lam_rows"])
    o = 0
    for g in cut:
        assert int(g["lam_row0"]) - int(f["lam_row0"]) == o
        assert int(g["v_row0"]) - int(f["v_row0"]) == o
        assert int(g["rows"]) == int(f["rows"]) - o and int(g["lam_rows"]) > 0
        for k_loc in range(int(g["lam_rows"])):
            k = o + k_loc
            assert k % 32 == k_loc % 32
            for n in (1, 31, 200, 255, 1024):
                assert _taps_used(k_loc, g, n) == _taps_used(k, f, n), (k, n)
        o += int(g["lam_rows"])
    assert o == L
    if int(f["seg"]) % 32 == 0 and L >= parts * (1024 + int(f["seg"])):
        assert len(cut) == parts  # frames long enough are split as asked


def test_split_one_part_is_the_frame():
    cfg = model.RunConfig(Time_Block_Length=0.002, Decouple_Filter=2, Time_Blocks=40)
    whole = ihc.reference_frame(cfg)
    assert np.array_equal(ihc.split_frame(whole, 1), whole)
