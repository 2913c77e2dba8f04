"""GPU parity of the BM/OHC solver against the FP32 oracle: bit-exact velocity,
failure flags and per-unit counters (the kernel and the oracle evaluate the
same floating-point sequence)."""
import numpy as np
import pytest

from oracle import oracle as orc
from tests import cases

pytestmark = pytest.mark.gpu


def _compare(mv, bm_solver, case, threads=None):
    cfg, sc, gamma, units, x, rows = case
    secp = mv.section_params()
    o_v, o_f, o_st = orc.bm_run(secp, gamma, sc, units, x, rows, threads=threads)
    g_v, g_f, g_st = bm_solver.run(sc, gamma, units, x, rows)
    assert np.array_equal(g_v.view(np.uint32), o_v.view(np.uint32)), (
        "velocity differs: max abs %g" % np.abs(g_v - o_v).max())
    assert np.array_equal(g_f, o_f)
    for k in ("substeps", "iterations", "sweeps", "failed_samples", "written_samples",
              "status"):
        assert np.array_equal(g_st[k], o_st[k]), k
    return g_v, o_st


def test_cfg1_slice_bit_exact(mv, bm_solver):
    case = cases.cfg1_slice(mv, ms=3.0)
    v, st = _compare(mv, bm_solver, case)
    units = case[3]
    assert np.abs(v).max() > 0
    assert st["written_samples"][0] == units["end"][0] - units["out_first"][0]


@pytest.mark.parametrize("sigma_ow", [0.25, 0.3])
def test_oval_window_scale_bit_exact(mv, bm_solver, sigma_ow):
    """The oval-window acceleration divides by sigma_ow; where sigma_ow is a
    power of two the kernel multiplies by its exact reciprocal instead.  Both
    forms are bit-exact against the oracle's division."""
    from cochlearmodel_gb300 import native
    cfg, sc, gamma, units, x, rows = cases.cfg1_slice(mv, ms=1.5, db=80.0)
    s2 = native.BMScalars.from_buffer_copy(sc)
    s2.sigma_ow = sigma_ow
    _compare(mv, bm_solver, (cfg, s2, gamma, units, x, rows))


@pytest.mark.parametrize("db", [20.0, 100.0])
def test_levels_bit_exact(mv, bm_solver, db):
    _compare(mv, bm_solver, cases.cfg1_slice(mv, ms=1.5, db=db, freq=4000.0))


def test_decoupled_blocks_bit_exact(mv, bm_solver):
    _compare(mv, bm_solver, cases.decoupled_sweep(mv, n_signals=3, decouple=2, block_ms=1.5,
                                                 overlap_ms=0.5, seed=1))


def test_framed_batch_profiles_bit_exact(mv, bm_solver):
    _compare(mv, bm_solver, cases.framed_batch(mv, [1.0, 2.5, 0.6, 1.7], seed=2, block_ms=0.8,
                                              overlap_ms=0.3))


def test_deterministic_replay(mv, bm_solver):
    cfg, sc, gamma, units, x, rows = cases.cfg1_slice(mv, ms=1.0)
    a = bm_solver.run(sc, gamma, units, x, rows)[0]
    b = bm_solver.run(sc, gamma, units, x, rows)[0]
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_nonconvergence_flags(mv, bm_solver):
    """An impossible tolerance makes every step hit Cuda_Outern_Loops; the
    failure flags and counts match the oracle."""
    cfg, sc, gamma, units, x, rows = cases.cfg1_slice(mv, ms=0.5)
    units = units.copy()
    units["mtt"] = np.float32(-1.0)
    v, st = _compare(mv, bm_solver, (cfg, sc, gamma, units, x, rows))
    assert st["failed_samples"][0] > 0


def test_empty_and_rejected_tables(mv, bm_solver):
    from cochlearmodel_gb300 import native
    cfg, sc, gamma, units, x, rows = cases.cfg1_slice(mv, ms=0.5)
    out = bm_solver.run(sc, gamma, units[:0], x, rows)
    assert not out[0].any()
    bad = units.copy()
    bad["end"] = rows + 10
    with pytest.raises(native.CGBError):
        bm_solver.run(sc, gamma, bad, x, rows)


def test_substep_guard_stops_unit(mv, bm_solver):
    """A unit whose sample needs more steps than max_substeps_per_sample
    stops with status 1 (no hang), identically to the oracle."""
    cfg, sc, gamma, units, x, rows = cases.cfg1_slice(mv, ms=0.5)
    sc.max_substeps_per_sample = 5
    v, st = _compare(mv, bm_solver, (cfg, sc, gamma, units, x, rows))
    assert st["status"][0] == 1 and st["written_samples"][0] == 0


def test_per_sample_convergence_stats(mv, bm_solver):
    cfg, sc, gamma, units, x, rows = cases.cfg1_slice(mv, ms=1.0)
    conv_o = np.zeros((rows, 3), np.float32)
    orc.bm_run(mv.section_params(), gamma, sc, units, x, rows, conv=conv_o)
    _, _, _, conv_g = bm_solver.run(sc, gamma, units, x, rows, want_conv=True)
    assert np.array_equal(conv_g.view(np.uint32), conv_o.view(np.uint32))
    e = int(units["end"][0])
    assert (conv_g[:e, 1] >= 10).all() and (conv_g[:e, 2] >= 2).all()


def test_every_launch_shape_bit_exact(mv, bm_solver):
    """Each built launch shape (register-only state, previous-step state and
    G/P_tm in shared memory, bounded register counts) runs the same
    floating-point sequence: bit-exact against the oracle on units of uneven
    length from six signals."""
    from cochlearmodel_gb300 import native
    lib = native.load()
    case = cases.framed_batch(mv, [1.0, 2.5, 0.6, 1.7, 0.9, 1.3], seed=7, block_ms=0.4,
                              overlap_ms=0.2)
    try:
        for shape in range(lib.cgb_bm_launch_shape_count()):
            native.check(lib.cgb_bm_set_launch_shape(shape), "set launch shape")
            _compare(mv, bm_solver, case)
    finally:
        native.check(lib.cgb_bm_set_launch_shape(0), "set launch shape")


@pytest.mark.parametrize("case", ["cfg1", "decoupled"])
def test_fault_count_controller_bit_exact(mv, bm_solver, case):
    """BMOHC_NEW_kernel's controller (another outer iteration while any
    section fails the speed test) in the own operation order: bit-exact
    against the oracle's controller 1."""
    from cochlearmodel_gb300 import native
    c = (cases.cfg1_slice(mv, ms=5.0) if case == "cfg1" else
         cases.decoupled_sweep(mv, n_signals=2, decouple=2, block_ms=1.5, overlap_ms=0.5, seed=3))
    cfg, sc, gamma, units, x, rows = c
    s1 = native.BMScalars.from_buffer_copy(sc)
    s1.controller = 1
    _compare(mv, bm_solver, (cfg, s1, gamma, units, x, rows))


def test_controller_arguments_rejected(mv, bm_solver):
    from cochlearmodel_gb300 import native
    cfg, sc, gamma, units, x, rows = cases.cfg1_slice(mv, ms=0.5)
    for ctl, ar, jm in [(2, 0, 0), (0, 1, 0), (1, 2, 0), (1, 0, 2)]:
        s = native.BMScalars.from_buffer_copy(sc)
        s.controller, s.arith, s.jacobi_mode = ctl, ar, jm
        if jm == 2:
            s.jacobi_cap, s.jacobi_tol = 8, 1e-6
        with pytest.raises(native.CGBError):
            bm_solver.run(s, gamma, units, x, rows)
