"""Known-answer and property tests of the CPU oracle itself."""
import numpy as np

from cochlearmodel_gb300 import model
from oracle import oracle as orc
from tests import cases


def test_own_tanh_accuracy():
    """The project's float tanh (rational, one path) stays within 6.5 ulp of the
    exact value (6.03 at most over every float in [0, 9.5]), is odd, and
    saturates to +-1 from |x| = 9.5."""
    xs = np.concatenate([np.linspace(-12, 12, 20001), np.linspace(-0.6, 0.6, 20001),
                         np.geomspace(1e-8, 1e-1, 2001), np.linspace(8.5, 9.0, 2001),
                         [0.55, 0.5499999, 8.999999, 9.0, 20.0, 25.0]])
    xs = xs.astype(np.float32)
    got = np.array([orc.tanhf(float(x)) for x in xs], np.float32)
    exact = np.tanh(xs.astype(np.float64))
    ulp = np.spacing(np.abs(exact).astype(np.float32)).astype(np.float64)
    err = np.abs(got.astype(np.float64) - exact) / ulp
    assert err.max() <= 6.5, (xs[err.argmax()], err.max())
    assert np.all(np.abs(got) <= 1.0)
    neg = np.array([orc.tanhf(float(-x)) for x in xs], np.float32)
    assert np.array_equal(neg, -got)
    assert orc.tanhf(0.0) == 0.0 and orc.tanhf(30.0) == 1.0 and orc.tanhf(-30.0) == -1.0
    for big in (9.5, 9.500001, 1e30, float("inf")):
        assert orc.tanhf(big) == 1.0 and orc.tanhf(-big) == -1.0, big


def test_thomas_matches_dense_solve():
    o = orc.model_setup()
    m, l, u = o["diag_m"], o["diag_l"], o["diag_u"]
    rng = np.random.default_rng(0)
    v = rng.standard_normal(256)
    A = np.diag(m) + np.diag(u[:-1], 1) + np.diag(l[:-1], -1)
    assert np.allclose(orc.thomas(m, l, u, v), np.linalg.solve(A, v), rtol=1e-9, atol=1e-12)


def test_fixed_sweeps_approach_exact_solution(mv):
    """More Jacobi sweeps move the FP64 solution toward the exact tridiagonal
    solve; the default 20/2 sweeps stay within 1e-3 of it."""
    cfg, sc, gamma, units, x, rows = cases.cfg1_slice(mv, ms=1.0)
    secp = mv.section_params()
    ex, _, _ = orc.bm_run(secp, gamma, sc, units, x, rows, fp64=True, jacobi_mode=1)
    e = units["end"][0]
    scale = np.abs(ex[:e]).max()
    errs = []
    for slow, fast in ((20, 2), (200, 50)):
        sc.jacobi_slow, sc.jacobi_fast = slow, fast
        v, _, _ = orc.bm_run(secp, gamma, sc, units, x, rows, fp64=True)
        errs.append(np.abs(v[:e] - ex[:e]).max() / scale)
    assert errs[1] < errs[0] < 1e-3


def test_fp32_vs_fp64_small(mv):
    cfg, sc, gamma, units, x, rows = cases.cfg1_slice(mv, ms=2.0)
    secp = mv.section_params()
    v32, f32, st32 = orc.bm_run(secp, gamma, sc, units, x, rows)
    v64, f64, st64 = orc.bm_run(secp, gamma, sc, units, x, rows, fp64=True)
    e = units["end"][0]
    rel = np.abs(v32[:e] - v64[:e]).max() / np.abs(v64[:e]).max()
    assert rel < 1e-3
    assert st32["written_samples"][0] == units["end"][0] - units["out_first"][0]


def test_reduction_width_changes_only_rounding(mv):
    cfg, sc, gamma, units, x, rows = cases.cfg1_slice(mv, ms=1.0)
    secp = mv.section_params()
    a, _, _ = orc.bm_run(secp, gamma, sc, units, x, rows)
    sc.red_lanes = 64
    b, _, _ = orc.bm_run(secp, gamma, sc, units, x, rows)
    e = units["end"][0]
    assert np.abs(a[:e] - b[:e]).max() <= 1e-4 * np.abs(a[:e]).max()


def test_threads_do_not_change_results(mv):
    case = cases.decoupled_sweep(mv, n_signals=2, decouple=2, block_ms=1.0, overlap_ms=0.5)
    cfg, sc, gamma, units, x, rows = case
    secp = mv.section_params()
    a = orc.bm_run(secp, gamma, sc, units, x, rows, threads=1)[0]
    b = orc.bm_run(secp, gamma, sc, units, x, rows, threads=4)[0]
    assert np.array_equal(a, b)


def test_ihc_kernel_arithmetic_within_lambda_bar():
    """The GPU kernel's IHC/lambda arithmetic (oracle mode 2: Dot2 AC FIR,
    running compensated DC window sum) against the reference's mixed
    precision (mode 0): every lambda plane within 1e-4 max-rel, on a frame
    whose look-back rule restarts the windows (seg 700, frdp 2)."""
    from cochlearmodel_gb300 import ihc
    rng = np.random.default_rng(7)
    rows = 1600
    t = np.arange(rows)[:, None] / 1e5
    f = 200.0 * 40.0 ** (np.arange(256)[None, :] / 255.0)
    env = np.exp(-np.arange(256) / 90.0)[None, :]
    v = (1e-3 * env * np.sin(2 * np.pi * f * t) + 1e-6 * rng.normal(size=(rows, 256)))
    v = v.astype(np.float32)
    nerve = ihc.NerveConfig()
    ac = ihc.design_ac_lowpass().astype(np.float64)
    dc = np.full(200, np.float32(1.0 / (np.float32(100000) * np.float32(0.002))), np.float64)
    dmg = np.full(256, 10.0 ** 8, np.float64)
    args = (v, 700, 2, 1400, rows, ac, dc, nerve.scale, nerve.eta_AC, nerve.eta_DC, dmg,
            nerve.aihc(), np.asarray(nerve.spontRate, np.float32), nerve.Lambda_SAT)
    _, lam2 = orc.ihc_lambda(*args, mode=2)
    _, lam0 = orc.ihc_lambda(*args, mode=0)
    for j in range(3):
        d = np.abs(lam2[j] - lam0[j]).max() / np.abs(lam0[j]).max()
        assert d <= 1e-4, (j, d)
