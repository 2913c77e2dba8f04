"""Batched sweeps: groups of different lengths solved in one BM launch and one
IHC launch (and replayed from a CUDA graph) give exactly what each group gives
when run on its own."""
import numpy as np
import pytest

from cochlearmodel_gb300 import batch
from cochlearmodel_gb300.pipeline import JNDWindow, ProfileRun

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sweep(mv):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    spec = batch.jnd_sweep_spec(n_seeds=2, seed=3, min_ms=3.0, max_ms=6.0,
                                noises=(1111.0, 30.0), powers=(40.0, 80.0))
    b = batch.BatchSweep("cuda:0", spec, mv=mv, overlap_time=0.001, block_target=150,
                         jnd=JNDWindow(head=0.0005, tail=0.0002))
    b.step()
    torch.cuda.synchronize()
    return b, spec


def test_groups_match_single_runs(sweep, mv):
    import torch
    b, spec = sweep
    res = b.jnd_db()
    v_all = b.d_v.cpu().numpy()
    lam_all = b.d_lam.cpu().numpy()
    for gi, (g, s) in enumerate(zip(b.groups, spec)):
        cfg = batch.RunConfig(Fs=g.cfg.Fs, Time_Block_Length=g.cfg.Time_Block_Length,
                              Decouple_Filter=g.cfg.Decouple_Filter,
                              Overlap_Time=g.cfg.Overlap_Time, OHC_Vector=g.cfg.OHC_Vector,
                              IHC_Vector=g.cfg.IHC_Vector)
        run = ProfileRun("cuda:0", cfg, s["sweep"], noise=g.noise, mv=mv, jnd=b.jnd_win)
        run.step()
        torch.cuda.synchronize()
        rows = run.rows - 4
        v1 = run.d_v.cpu().numpy()[:rows]
        assert np.array_equal(v1.view(np.uint32), v_all[g.v_row0:g.v_row0 + rows].view(np.uint32))
        lam1 = run.d_lam.cpu().numpy()
        n = lam1.shape[1]
        assert np.array_equal(lam1.view(np.uint32),
                              lam_all[:, g.lam_row0:g.lam_row0 + n].view(np.uint32))
        r1, a1, _, _ = run.jnd_db()
        rb, ab, _, _ = res[gi]
        tested = ~np.isnan(r1)
        assert np.array_equal(r1[tested], rb[tested]) and np.array_equal(a1[tested], ab[tested])


def test_graph_replay_matches_eager(sweep):
    import torch
    b, _ = sweep
    v0 = b.d_v.clone()
    lam0 = b.d_lam.clone()
    F0 = b.d_FRA.clone()
    b.d_v.zero_()
    b.d_lam.zero_()
    b.capture()
    b.d_v.zero_()
    b.d_lam.zero_()
    b.replay()
    torch.cuda.synchronize()
    assert torch.equal(b.d_v, v0) and torch.equal(b.d_lam, lam0)
    assert torch.equal(b.d_FRA, F0)


def test_units_longest_first(sweep):
    b, _ = sweep
    span = b.units["end"] - b.units["start"]
    assert (np.diff(span) <= 0).all()


def test_step_host_equals_step_and_copies(sweep):
    """The host-buffer step, whose kernels store their results into the
    pinned host buffers as they write them, returns exactly what step()
    followed by plain copies returns.  The buffers start as NaN, so the rows
    no kernel writes must be zeroed; a second step into the same buffers
    gives the same values."""
    import torch
    b, _ = sweep
    h_tables = [pg["d_prof"].cpu().pin_memory() for pg in b.per_group]
    b.step()
    torch.cuda.synchronize()
    v0, lam0, f0 = b.d_v.cpu(), b.d_lam.cpu(), b.d_FRA.clone()
    h_v = torch.empty(b.d_v.shape, dtype=torch.float32).pin_memory()
    h_lam = torch.empty(b.d_lam.shape, dtype=torch.float32).pin_memory()
    h_v.fill_(float("nan"))
    h_lam.fill_(float("nan"))
    for _ in range(2):
        b.step_host(h_tables, h_v, h_lam)
        torch.cuda.synchronize()
        assert torch.equal(h_v, v0) and torch.equal(h_lam, lam0)
        assert torch.equal(b.d_FRA, f0)
    assert len(b._gaps[0]) > 0  # the groups' padding rows were zeroed


def test_host_mirror_rejects_bad_buffers(sweep):
    """A host mirror must match its device buffer and be pinned: the Python
    layer rejects a short or pageable tensor, and the library rejects a
    pageable host pointer and a device pointer, before anything launches."""
    import ctypes as C
    import torch
    from cochlearmodel_gb300 import native
    b, _ = sweep
    short = torch.empty((b.d_v.shape[0] - 1, 256), dtype=torch.float32).pin_memory()
    with pytest.raises(ValueError):
        b.solve_bm(h_v=short)
    with pytest.raises(ValueError):
        b.ihc_lambda(h_lam=torch.empty(b.d_lam.shape, dtype=torch.float32))
    lib = native.load()
    pageable = np.zeros((b.d_v.shape[0], 256), np.float32)
    full = b.d_v.numel() * 4
    pinned = torch.empty(b.d_v.shape, dtype=torch.float32).pin_memory()
    for bad, nbytes, msg in ((pageable.ctypes.data, full, b"host mirror"),
                             (b.d_v.data_ptr(), full, b"host mirror"),
                             (pinned.data_ptr(), full - 4, b"shorter")):
        ex = native.BMExtras()
        ex.h_out, ex.h_out_bytes = bad, nbytes
        rc = lib.cgb_bm_run_ex_dev(
            native.ptr(b.bm.secp), native.ptr(b.d_gamma), 1, C.byref(b.sc), native.ptr(b.d_units),
            len(b.units), native.ptr(b.d_in), int(b.d_in.numel()), native.ptr(b.d_v),
            int(b.d_v.shape[0]), None, None, None, native.ptr(b.bm.work),
            C.cast(C.byref(ex), C.c_void_p), None)
        assert rc != 0 and msg in lib.cgb_last_error()
    torch.cuda.synchronize()


def test_jnd_table_order_does_not_change_the_sums(sweep):
    """cgb_jnd_batch_dev writes each descriptor's sums to its own output slot,
    so the table's order (longest windows first, as BatchSweep builds it, or
    any other) changes nothing; an empty table enqueues nothing."""
    import torch
    from cochlearmodel_gb300 import native
    b, _ = sweep
    lens = b.jnd_iv["len"]
    assert (np.diff(lens) <= 0).all()           # longest first
    b.jnd_sums()
    torch.cuda.synchronize()
    F0, A0 = b.d_FRA.clone(), b.d_FAI.clone()
    perm = np.random.default_rng(5).permutation(len(b.jnd_iv))
    shuffled = torch.from_numpy(b.jnd_iv[perm].view(np.uint8).copy()).to(b.d_jnd_iv.device)
    lib = native.load()
    b.d_FRA.zero_()
    b.d_FAI.zero_()
    native.check(lib.cgb_jnd_batch_dev(
        native.ptr(b.d_lam), b.lam_rows, native.ptr(shuffled), len(b.jnd_iv), len(b.jnd_iv),
        native.ptr(b.d_nihc), native.ptr(b.W), float(b.Fs), b.jnd_win.delta_alpha_time_factor * b.Fs,
        native.ptr(b.d_FRA), native.ptr(b.d_FAI), None, None), "cgb_jnd_batch_dev")
    torch.cuda.synchronize()
    assert torch.equal(b.d_FRA, F0) and torch.equal(b.d_FAI, A0)
    native.check(lib.cgb_jnd_batch_dev(
        native.ptr(b.d_lam), b.lam_rows, native.ptr(shuffled), 0, 1,
        native.ptr(b.d_nihc), native.ptr(b.W), float(b.Fs), b.jnd_win.delta_alpha_time_factor * b.Fs,
        native.ptr(b.d_FRA), native.ptr(b.d_FAI), None, None), "cgb_jnd_batch_dev")
