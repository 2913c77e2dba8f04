"""The mixed batch (signals of different lengths, types and hearing profiles
in one step): every group's velocity equals the group solved alone, lambda
of the silent reference is the spontaneous rate, a noise reference differs
from its test, the JND is finite where the window fits, and graph replay
reproduces the eager step."""
import numpy as np
import pytest

from cochlearmodel_gb300 import mixed, model

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    spec = mixed.mixed_batch_spec(n_signals=12, seed=5, min_ms=10.0, max_ms=60.0)
    b = mixed.MixedBatch("cuda:0", spec)
    b.step()
    torch.cuda.synchronize()
    return b, spec


def test_groups_equal_solo_runs(batch, bm_solver):
    b, spec = batch
    v = b.d_v.cpu().numpy()
    row = 0
    for i, (N, D, s) in enumerate(spec[:4]):
        ints = [s.test] + ([s.reference] if s.reference is not None else [])
        cfg = model.RunConfig(Time_Block_Length=N / 1e5, Decouple_Filter=D,
                              Time_Blocks=len(ints) * D, Overlap_Time=0.005)
        rows = cfg.total_time_nodes_p1() + 4
        x = np.zeros(rows, np.float32)
        for k, iv in enumerate(ints):
            x[k * N * D:(k + 1) * N * D] = iv
        units = model.reference_units(cfg)
        sv, _, st = bm_solver.run(model.bm_scalars(cfg, bm_solver.mv), s.ohc[None], units, x,
                                  rows)
        assert st["status"].max() == 0
        assert np.array_equal(sv.view(np.uint32), v[row:row + rows].view(np.uint32)), i
        row += rows


def test_silence_and_references(batch):
    b, spec = batch
    lam = b.d_lam.cpu().numpy()
    r0, L, _ = b.group_rows[-1]
    spont = np.asarray(b.nerve.spontRate, np.float32)
    for j in range(3):
        assert np.all(lam[j, r0:r0 + L] == spont[j])
    for i, s in enumerate(b.signals):
        r0, L, k = b.group_rows[i]
        if k == 2:
            assert not np.array_equal(lam[0, r0:r0 + L], lam[0, r0 + L:r0 + 2 * L])


def test_jnd_finite_where_window_fits(batch):
    b, spec = batch
    rate, ai = b.jnd_db()
    fits = b.jnd_of >= 0
    assert fits.any()
    assert np.all(np.isfinite(rate[fits])) and np.all(np.isfinite(ai[fits]))
    assert np.all(np.isnan(rate[~fits]))


def test_graph_replay(batch):
    import torch
    b, _ = batch
    v0, lam0, f0 = b.d_v.clone(), b.d_lam.clone(), b.d_FRA.clone()
    b.capture()
    b.d_lam.zero_()
    b.replay()
    torch.cuda.synchronize()
    assert torch.equal(b.d_v, v0) and torch.equal(b.d_lam, lam0) and torch.equal(b.d_FRA, f0)
