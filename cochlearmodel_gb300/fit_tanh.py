"""Derives the coefficients of the solver's float tanh (csrc/cgb_device.cuh
own_tanhf / own_tanhf2 and the oracle's copy).

    python -m cochlearmodel_gb300.fit_tanh

tanh(x) = x P(z) / Q(z), z = x^2, P and Q of degree 4 in z with Q(0) = 1;
the evaluation clamps z to 9.5^2 (from there on |x| P / Q exceeds 1) and
the result to [-1, 1], so it saturates to +-1 exactly.  The fit minimises the maximum relative error of P/Q
against tanh(x)/x on [0, 9] by linearised least squares (Sanathanan-Koerner
iteration: P - f Q weighted by 1/Q_prev) with Lawson's multiplicative
reweighting towards the minimax solution; the best iterate is kept.  The
printed float32 values are the ones the kernel and the oracle use; the float
evaluation (Horner in z, x P times own_rcpf(Q)) stays within 6.1 ulp of tanh
(every float in [0, 9.5] checked against double tanh: at most 6.03 ulp).
"""
from __future__ import annotations

import numpy as np

X_MAX = 9.0
DEG = 5  # coefficients of P and of Q


def fit(npc: int = DEG, nqc: int = DEG, x_max: float = X_MAX, iters: int = 200):
    x = np.unique(np.maximum(np.linspace(0.0, 1.0, 8000) ** 1.5 * x_max, 1e-6))
    z = x * x
    f = np.tanh(x) / x
    q_prev = np.ones_like(z)
    w = np.full_like(z, 1.0 / len(z))
    best = (np.inf, None, None)
    for _ in range(iters):
        a = np.concatenate([np.stack([z ** k for k in range(npc)], 1),
                            -np.stack([f * z ** k for k in range(1, nqc)], 1)], 1)
        sw = np.sqrt(w) / (q_prev * f)
        coef, *_ = np.linalg.lstsq(a * sw[:, None], f * sw, rcond=None)
        p = coef[:npc]
        q = np.concatenate([[1.0], coef[npc:]])
        qv = sum(q[k] * z ** k for k in range(nqc))
        err = (sum(p[k] * z ** k for k in range(npc)) / qv - f) / f
        e = float(np.abs(err).max())
        if e < best[0]:
            best = (e, p.copy(), q.copy())
        q_prev = qv
        w = w * (np.abs(err) + 1e-30)
        w /= w.sum()
    return best


if __name__ == "__main__":
    e, p, q = fit()
    print("max relative fit error %.3e" % e)
    print("P:", ", ".join(repr(float(np.float32(c))) + "f" for c in p))
    print("Q:", ", ".join(repr(float(np.float32(c))) + "f" for c in q))
