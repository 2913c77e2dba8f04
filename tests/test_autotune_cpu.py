"""Autotuner logic on the CPU: the search picks the fastest candidate of each
stage, rejects a candidate whose outputs differ, and the cache round-trips
under a key that carries the device, the library hash and the workload."""
import numpy as np
import pytest

from cochlearmodel_gb300 import autotune, native


class FakeLib:
    def __init__(self):
        self.shape, self.run = 0, 0

    def cgb_bm_launch_shape_count(self):
        return 4

    def cgb_bm_set_launch_shape(self, s):
        self.shape = s
        return 0

    def cgb_ihc_set_run_length(self, r):
        self.run = r
        return 0


@pytest.fixture
def fake(monkeypatch):
    lib = FakeLib()
    monkeypatch.setattr(native, "load", lambda *a, **k: lib)
    return lib


def test_search_picks_fastest_and_checks_outputs(fake):
    bm_ms = {0: 5.0, 1: 4.0, 2: 6.0, 3: 4.5}
    ihc_ms = {0: 3.0, 8: 3.5, 16: 2.5, 32: 2.8}
    calls = {"stage": None}

    def stage_bm():
        calls["stage"] = "bm"

    def stage_ihc():
        calls["stage"] = "ihc"

    def timer(fn):
        fn()
        return bm_ms[fake.shape] if calls["stage"] == "bm" else ihc_ms[fake.run]

    choice, t = autotune.search(stage_bm, stage_ihc, timer, lambda: (b"v", b"l"))
    assert (choice.bm_shape, choice.ihc_run) == (1, 16)
    assert fake.shape == 1 and fake.run == 16
    assert t["bm_shape"]["2"] == 6.0 and t["ihc_run"]["32"] == 2.8

    outs = iter([(b"v", b""), (b"x", b"")])
    with pytest.raises(native.CGBError, match="shape 1"):
        autotune.search(stage_bm, stage_ihc, timer, lambda: next(outs))


def test_pick_keeps_the_default_within_the_margin():
    assert autotune.pick({0: 10.0, 1: 9.9, 2: 9.85}) == 0
    assert autotune.pick({0: 10.0, 1: 9.7}) == 1
    assert autotune.pick({0: 10.0, 1: 9.7, 3: 9.5}) == 3
    assert autotune.pick({0: 10.0, 1: 9.9}, margin=0.0) == 1


def test_search_warms_up_and_times_round_robin(fake):
    """Untimed warm-up calls come first; then the candidates are timed in
    turn, round after round, and each keeps its best time."""
    order, t = [], iter(range(100))

    def stage_bm():
        order.append(("bm", fake.shape))

    def stage_ihc():
        order.append(("ihc", fake.run))

    def timer(fn):
        fn()
        order.append("timed")
        return 10.0 - 0.001 * next(t)  # later calls a little faster

    autotune.search(stage_bm, stage_ihc, timer, lambda: (b"v", b"l"), shapes=[0, 1],
                    runs=[0, 8], rounds=2, warmup=3)
    bm = [o for o in order if o != "timed" and o[0] == "bm"]
    assert bm[:3] == [("bm", 0)] * 3            # warm-up on the default
    assert bm[3:7] == [("bm", 0), ("bm", 1), ("bm", 0), ("bm", 1)]


def test_cache_round_trip(tmp_path, monkeypatch):
    monkeypatch.setenv("CGB_TUNE_CACHE", str(tmp_path / "t.json"))
    key = autotune.cache_key("NVIDIA GB300", "BatchSweep:units=3025", lib_hash="abc")
    assert key == "NVIDIA GB300|abc|BatchSweep:units=3025"
    assert autotune.lookup(key) is None
    autotune.store(key, autotune.Choice(bm_shape=2, ihc_run=16), {"bm_shape": {"2": 1.0}})
    got = autotune.lookup(key)
    assert got == autotune.Choice(bm_shape=2, ihc_run=16)
    assert autotune.lookup(key.replace("abc", "abd")) is None
    (tmp_path / "t.json").write_text("not json")
    assert autotune.lookup(key) is None


def test_library_hash_is_stable():
    h = autotune.library_hash()
    assert len(h) == 16 and h == autotune.library_hash()
    assert np.all([c in "0123456789abcdef" for c in h])
