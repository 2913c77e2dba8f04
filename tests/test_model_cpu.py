"""Host logic of the product against the oracle, no GPU needed:
model vectors (row a4), the block partition (row a2), section packing."""
import numpy as np
import pytest

from cochlearmodel_gb300 import model
from oracle import oracle as orc


def test_model_vectors_match_oracle(mv):
    o = orc.model_setup()
    for k in ("M", "R", "S", "Q", "S_ohc", "S_tm", "R_tm", "diag_m", "diag_l", "diag_u"):
        assert np.array_equal(getattr(mv, k), o[k]), k
    assert np.array_equal(mv.scal, o["scal"])


def test_model_vectors_closed_form(mv):
    """KAT: M0 e^{M1 x}, R0 e^{R1 x}, S0 e^{S1 x} at s = 0, 128, 255."""
    dx = 3.5 / 256
    for s in (0, 128, 255):
        x = dx * s
        assert mv.M[s] == pytest.approx(1.286e-6 * np.exp(1.5 * x), rel=1e-6)
        assert mv.R[s] == pytest.approx(0.25 * np.exp(-0.06 * x), rel=1e-6)
        assert mv.S[s] == pytest.approx(1.282e4 * np.exp(-1.5 * x), rel=1e-6)
        assert mv.Q[s] == pytest.approx(2 * 1.0 * 0.003 / (0.5 * mv.M[s]), rel=1e-6)
    assert mv.diag_m[255] == 1.0 and mv.diag_l[254] == 0.0 and mv.diag_l[255] == 0.0
    assert mv.diag_m[0] == pytest.approx(-(1 + dx * 0.024), rel=1e-6)


@pytest.mark.parametrize("tb,dec,blk,ov", [(1, 1, 0.05, 0.005), (8, 8, 0.01, 0.005),
                                          (16, 8, 0.01, 0.005), (6, 2, 0.002, 0.001),
                                          (5, 0, 0.004, 0.002), (4, 1, 0.003, 0.001)])
def test_block_partition_matches_oracle(tb, dec, blk, ov):
    cfg = model.RunConfig(Time_Blocks=tb, Decouple_Filter=dec, Time_Block_Length=blk,
                          Overlap_Time=ov)
    args = (tb, cfg.total_time_nodes_p1(), cfg.calc_overlap_nodes(), dec)
    got = model.block_partition(*args)
    want = orc.block_partition(*args)
    for g, w in zip(got, want):
        assert np.array_equal(g, w)


def test_block_partition_decoupled_semantics():
    """Decouple_Filter=8, 10 ms blocks at 100 kHz: a group opens with a block
    that writes from its start, mid-group blocks warm up for the overlap, and
    the group's last block stops at the group boundary."""
    cfg = model.RunConfig(Time_Blocks=16, Decouple_Filter=8, Time_Block_Length=0.01)
    st, of, en = model.block_partition(16, cfg.total_time_nodes_p1(), 500, 8)
    N = 1000
    assert list(st) == [b * N for b in range(16)]
    assert of[0] == 0 and of[8] == 8 * N
    assert of[1] == N + 500 and en[1] == 2 * N + 500
    assert en[7] == 8 * N and en[15] == 16 * N + 500


def test_derived_node_counts():
    cfg = model.RunConfig(Time_Block_Length=0.01, Time_Blocks=8, Overlap_Time=0.005)
    assert cfg.calc_time_block_nodes() == 1000
    assert cfg.calc_overlap_nodes() == 500
    assert cfg.total_time_nodes_p1() == 500 + 9000
    assert cfg.cuda_iterations_per_kernel() == 10
    assert cfg.time_step_out() == np.float32(1e-6) * np.float32(10)


def test_expand_vector():
    v = model.expand_vector([1.0, 2.0, 3.0])
    assert v.shape == (256,)
    assert (v[:86] == 1).all() and (v[86:171] == 2).all() and (v[171:] == 3).all()
    assert (model.expand_vector(0.5) == 0.5).all()


def test_section_packing(mv):
    sp = mv.section_params()
    assert sp.dtype == np.float32 and sp.shape == (8, 256)
    assert sp[0, 10] == np.float32(1.0) / np.float32(mv.M[10])
    assert sp[1, 0] == np.float32(1.0) / np.float32(mv.diag_m[0])
    assert sp[1, 255] == 1.0


def test_noise_normalization_matches_formula():
    """calculateDCANDNornalizationFactor (src/cochlea.cu:4219-4254): the energy
    starts from the first sample's raw square, later samples have the dc removed."""
    from cochlearmodel_gb300 import native
    lib = native.load()
    rng = np.random.default_rng(1)
    x = (rng.standard_normal(1000) + 0.3).astype(np.float32)
    dc, fac = np.zeros(1), np.zeros(1)
    for ntype, remove in ((0, 1.0), (1, 1.0), (2, 0.0), (3, 1.0)):
        native.check(lib.cgb_noise_normalization(native.ptr(x), ntype, 0.16, remove, 100, 900,
                                                 50, 950, 100000.0, native.ptr(dc),
                                                 native.ptr(fac)))
        d = remove * x[100:900].astype(np.float64).sum() / 800
        e = float(x[50]) ** 2 + ((x[51:950].astype(np.float64) - d) ** 2).sum()
        e = np.sqrt(e)
        e = {0: e, 1: e / np.sqrt(900), 2: e / np.sqrt(100000.0 * 0.16), 3: 1.0}[ntype]
        assert dc[0] == pytest.approx(d, rel=1e-12, abs=1e-15)
        assert fac[0] == pytest.approx(e, rel=1e-12)
    native.check(lib.cgb_noise_normalization(None, 0, 0.0, 0.0, 0, 10, 0, 800, 100000.0,
                                             native.ptr(dc), native.ptr(fac)))
    assert fac[0] == pytest.approx(np.sqrt(400.0)) and dc[0] == 0.0


def test_profile_sweep_grid():
    from cochlearmodel_gb300.pipeline import ProfileSweep
    sw = ProfileSweep(frequencies=[1000.0], powers=[10.0 * k for k in range(1, 11)],
                      noises=[1111.0, 0.0, 10.0, 20.0, 30.0, 40.0], calculate_jnd=True)
    p, is_ref, ref_of = sw.build()
    assert len(p) == 66 and is_ref.sum() == 6
    assert list(np.flatnonzero(is_ref)) == [10, 21, 32, 43, 54, 65]
    assert ref_of[0] == 10 and ref_of[11] == 21 and ref_of[65] == 65
    assert p["Wn"][0] == 0.0 and p["dA"][10] == 0.0
    assert p["dA"][5] == pytest.approx(10 * 10 ** (60 / 20) * 2e-5)


def test_jnd_sweep_configuration():
    from cochlearmodel_gb300 import batch
    spec = batch.jnd_sweep_spec(n_seeds=4)
    assert len(spec) == 24
    n = sum(len(s["sweep"].build()[0]) for s in spec)
    assert n == 264
    lens = [s["length"] for s in spec]
    assert min(lens) >= 2000 and max(lens) <= 20000
    for s in spec:
        N, D = batch.block_nodes_for(s["length"], 1000, 100000)
        assert abs(N * D - s["length"]) <= 3 * D and N <= 1000 + 3
    o, i = batch.hearing_loss_ohc(), batch.hearing_loss_ihc()
    assert o[0] == 0.5 and o[127] == 0.5 and o[255] == np.float32(0.05)
    assert i[0] == 8 and i[255] == 5 and (np.diff(i[127:]) < 0).all()
