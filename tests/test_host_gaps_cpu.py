"""Host logic of the host mirrors: the row ranges no kernel writes, which the
host-buffer step zeroes itself (the kernels store only the rows they write)."""
import numpy as np
import torch

from cochlearmodel_gb300 import model, native
from cochlearmodel_gb300.ihc import reference_frame
from cochlearmodel_gb300.solver import host_gaps, unit_rows, unwritten_ranges, zero_host_gaps


def _brute(starts, ends, rows):
    w = np.zeros(rows, bool)
    for a, b in zip(starts, ends):
        w[a:b] = True
    out, r = [], 0
    while r < rows:
        if w[r]:
            r += 1
            continue
        a = r
        while r < rows and not w[r]:
            r += 1
        out.append((a, r))
    return out


def test_unwritten_ranges_match_brute_force():
    rng = np.random.default_rng(5)
    for _ in range(200):
        rows = int(rng.integers(1, 60))
        n = int(rng.integers(0, 6))
        starts = rng.integers(0, rows, n)
        ends = np.minimum(rows, starts + rng.integers(0, 20, n))
        assert unwritten_ranges(starts, ends, rows) == _brute(starts, ends, rows)
    assert unwritten_ranges([], [], 7) == [(0, 7)]
    assert unwritten_ranges([0], [7], 7) == []
    assert unwritten_ranges([0, 3], [3, 7], 7) == []  # adjacent spans leave no gap


def test_reference_run_gaps():
    """A Run_Cuda run writes every velocity row up to its last output sample;
    the rows after it (the overlap tail and the padding) are its only gap.
    Its lambda frame covers every lambda row."""
    cfg = model.RunConfig(Time_Block_Length=0.00128, Decouple_Filter=2, Overlap_Time=0.0005,
                          Time_Blocks=8)
    units = model.reference_units(cfg)
    rows = cfg.total_time_nodes_p1() + 4
    first, end = unit_rows(units)
    u = units.view(native.UNIT_DTYPE)
    assert (first >= u["out_base"] + u["start"]).all() and (end <= rows).all()
    frames = reference_frame(cfg)
    gv, gl = host_gaps(units, rows, frames, int(frames["lam_rows"][0]))
    assert gl == []
    assert gv[-1] == (int(end.max()), rows)
    assert sum(b - a for a, b in gv) == rows - int((end - first).sum())


def test_zero_host_gaps_touches_only_the_gaps():
    h_v = torch.full((10, 4), 7.0)
    h_lam = torch.full((3, 6, 4), 7.0)
    zero_host_gaps(h_v, h_lam, ([(0, 2), (8, 10)], [(5, 6)]))
    assert (h_v[:2] == 0).all() and (h_v[8:] == 0).all() and (h_v[2:8] == 7).all()
    assert (h_lam[:, 5] == 0).all() and (h_lam[:, :5] == 7).all()


def test_host_mirror_check_rejects_mismatched_buffers():
    """The kernels store straight into a host mirror, so the Python layer
    accepts only a pinned, contiguous tensor of the device buffer's exact
    shape and dtype; everything else raises before any launch."""
    import pytest
    like = torch.zeros((8, 256), dtype=torch.float32)
    bad = [None,
           torch.zeros((7, 256), dtype=torch.float32),            # short
           torch.zeros((8, 256), dtype=torch.float64),            # dtype
           torch.zeros((256, 8), dtype=torch.float32).t(),        # not contiguous
           torch.zeros((8, 256), dtype=torch.float32)]            # pageable
    for t in bad:
        with pytest.raises(ValueError):
            native.check_host_mirror(t, like, "h_v")
