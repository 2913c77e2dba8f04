"""The autotuner on the GPU: every candidate gives the same results bit for
bit (IHC run lengths here; BM launch shapes in test_bm_gpu.py), a search on a
small sweep picks a candidate and caches it, and the next call takes the cache."""
import numpy as np
import pytest

from cochlearmodel_gb300 import autotune, batch, ihc, native
from cochlearmodel_gb300.pipeline import JNDWindow

pytestmark = pytest.mark.gpu


def test_every_ihc_run_length_bit_exact():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    st = ihc.IHCStage("cuda:0")
    rng = np.random.default_rng(8)
    t = np.arange(9000)[:, None] / 1e5
    v = (1e-3 * np.sin(2 * np.pi * (300 + 30 * np.arange(256))[None, :] * t) *
         (1 + rng.random((1, 256)))).astype(np.float32)
    fr = np.zeros(2, ihc.FRAME_DTYPE)
    fr[0] = (0, 0, 5000, 5000, 1000, 5000, ihc.round64(5000), 0)
    fr[1] = (5000, 5000, 4000, 3900, 4000, 3900, ihc.round64(4000), 0)
    lib = native.load()
    try:
        ref = None
        for run in autotune.IHC_RUNS + (1, 3):
            native.check(lib.cgb_ihc_set_run_length(run), "run length")
            lam, _ = st.run(v, fr, 8900)
            if ref is None:
                ref = lam
            assert np.array_equal(lam.view(np.uint32), ref.view(np.uint32)), run
    finally:
        native.check(lib.cgb_ihc_set_run_length(0), "run length")
    with pytest.raises(native.CGBError):
        native.check(lib.cgb_ihc_set_run_length(65), "run length")


def test_tune_searches_then_uses_the_cache(tmp_path, monkeypatch, mv):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    monkeypatch.setenv("CGB_TUNE_CACHE", str(tmp_path / "tuning.json"))
    spec = batch.jnd_sweep_spec(n_seeds=1, seed=5, min_ms=4.0, max_ms=8.0,
                                noises=(1111.0, 30.0), powers=(40.0, 80.0))
    b = batch.BatchSweep("cuda:0", spec, mv=mv, overlap_time=0.001, block_target=200,
                         jnd=JNDWindow(head=0.0005, tail=0.0002))
    try:
        choice, source = b.tune()
        assert source == "search"
        assert 0 <= choice.bm_shape < native.load().cgb_bm_launch_shape_count()
        assert choice.ihc_run in autotune.IHC_RUNS
        again, source2 = b.tune()
        assert source2 == "cache" and again == choice
    finally:
        autotune.apply(autotune.Choice())


def test_launch_keeps_the_run_length_of_its_upload(mv):
    """Tables uploaded under one run length and launched after the setting
    changed still give the full, unchanged lambda (the launch keeps the run
    length of its upload); after a re-upload the new length does too."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    spec = batch.jnd_sweep_spec(n_seeds=1, seed=6, min_ms=20.0, max_ms=40.0,
                                noises=(1111.0, 30.0), powers=(40.0, 80.0))
    b = batch.BatchSweep("cuda:0", spec, mv=mv)
    lib = native.load()
    try:
        b.step()
        torch.cuda.synchronize()
        want = b.d_lam.cpu().numpy()
        for run in (8, 1):
            native.check(lib.cgb_ihc_set_run_length(run), "run length")
            for reupload in (False, True):
                if reupload:
                    b.upload_ihc_tables()
                b.d_lam.fill_(float("nan"))
                b.ihc_lambda()
                torch.cuda.synchronize()
                got = b.d_lam.cpu().numpy()
                assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (run, reupload)
    finally:
        native.check(lib.cgb_ihc_set_run_length(0), "run length")
        b.upload_ihc_tables()


def test_occupancy_profile_times_prefixes(mv):
    """The occupancy profile times each launch shape on prefixes of the unit
    table and returns the statistics of the whole table."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    spec = batch.jnd_sweep_spec(n_seeds=1, seed=5, min_ms=4.0, max_ms=8.0,
                                noises=(1111.0, 30.0), powers=(40.0, 80.0))
    b = batch.BatchSweep("cuda:0", spec, mv=mv, overlap_time=0.001, block_target=200,
                         jnd=JNDWindow(head=0.0005, tail=0.0002))
    n = len(b.units)
    prof, stats = autotune.occupancy_profile(b, [0, 3], [1, n], reps=1)
    assert set(prof) == {0, 3} and all(set(r) == {1, n} for r in prof.values())
    assert all(t > 0 for r in prof.values() for t in r.values())
    assert len(stats) == n and (stats["written_samples"] > 0).all()
