"""CPU checks of the warm-start pieces: the FP64 network restatement against
finite differences, and the tolerance-mode oracle's basic properties."""
import numpy as np

from cochlearmodel_gb300 import model
from oracle import oracle as orc
from tests import cases


def _params(seed):
    rng = np.random.default_rng(seed)
    parts = []
    for cout, cin in ((64, 8), (64, 64), (64, 64), (1, 64)):
        b = np.sqrt(6.0 / (cin * 5))
        parts += [rng.uniform(-b, b, 5 * cout * cin), rng.uniform(-0.1, 0.1, cout)]
    return np.concatenate(parts).astype(np.float32)


def test_network_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = _params(1)
    feat = rng.uniform(-1, 1, (2, 256, 8)).astype(np.float32)
    target = rng.normal(0, 1, (2, 256)).astype(np.float32)
    _, loss, g = orc.ws_forward_backward(p, feat, target, 0.7, round_bf16=False)
    assert loss > 0
    bounds = np.cumsum([0, 2560, 64, 20480, 64, 20480, 64, 320, 1])
    idx = [int(rng.integers(bounds[k], bounds[k + 1])) for k in range(8) for _ in range(3)]
    # parameters are float32: perturb in float32 and difference in float64
    for i in idx:
        eps = np.float32(1e-4) * max(np.float32(1e-2), abs(p[i]))
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        step = float(pp[i]) - float(pm[i])
        _, lp, _ = orc.ws_forward_backward(pp, feat, target, 0.7, round_bf16=False,
                                           want_grad=False)
        _, lm, _ = orc.ws_forward_backward(pm, feat, target, 0.7, round_bf16=False,
                                           want_grad=False)
        fd = (lp - lm) / step
        assert abs(fd - g[i]) <= 1e-4 * max(abs(g[i]), 1e-3 * np.abs(g).max()), (i, fd, g[i])


def test_tolerance_mode_tighter_tolerance_converges_closer(mv):
    """Tolerance mode against the exact tridiagonal solve (FP64): a tighter
    tolerance brings the velocity closer, and the extrapolated guess reaches
    the same tolerance with fewer sweeps than the previous-step guess."""
    cfg, sc, gamma, units, x, rows = cases.cfg1_slice(mv, ms=1.0, db=60.0, freq=1000.0)
    secp = mv.section_params()
    ex, _, _ = orc.bm_run(secp, gamma, sc, units, x, rows, fp64=True, jacobi_mode=1)
    errs, sweeps = [], {}
    for tol in (1e-4, 1e-6):
        v, _, st = orc.bm_run(secp, gamma, model.tolerance_mode(sc, guess=0, tol=tol), units, x,
                              rows, fp64=True)
        errs.append(np.abs(v - ex).max() / np.abs(ex).max())
    assert errs[1] < errs[0]
    for guess in (0, 1):
        _, _, st = orc.bm_run(secp, gamma, model.tolerance_mode(sc, guess=guess), units, x, rows)
        sweeps[guess] = st["sweeps"].sum() / st["substeps"].sum()
    assert sweeps[1] < sweeps[0]
