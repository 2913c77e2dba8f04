"""The own-order BM solve takes pairs of Jacobi sweeps as one update over the
second neighbours,

    p''_s = C_s + a_s p_{s-2} + b_s p_s + c_s p_{s+2},

with C one sweep applied to Y/m and a, b, c products of 1/m values (the
oracle's two_step_coefficients, the kernel's coefficient rows 8-10).  In exact
arithmetic that update is the reference's two sweeps
(include/cochlea.cuh:13736, l_s = 0 on rows 254 and 255, p_{-1} = p_256 = 0).
Checked here in FP64 on the model's 1/m vector, boundary rows included; and
the FP32 oracle that uses it stays within the FP32 method's error of the FP64
solve."""
import numpy as np

from cochlearmodel_gb300 import model
from oracle import oracle as orc
from tests import cases

NS = 256


def _sweep(src, Yrm, rm):
    ext = np.concatenate([[0.0], src, [0.0]])
    t = ext[:-2] + ext[2:]
    t[NS - 2:] = ext[NS:NS + 2]  # l_254 = l_255 = 0
    return Yrm - rm * t


def _coefficients(rm):
    s = np.arange(NS)
    rl = np.concatenate([[0.0], rm[:-1]])
    ru = np.concatenate([rm[1:], [0.0]])
    a = np.where((s >= 2) & (s <= NS - 3), rm * rl, 0.0)
    c = np.where(s <= NS - 3, rm * ru, 0.0)
    lo = np.where((s >= 1) & (s <= NS - 3), rl, 0.0)
    up = np.where(s + 1 <= NS - 3, ru, 0.0)
    return a, rm * (lo + up), c


def test_two_step_update_equals_two_sweeps():
    rm = model.ModelVectors.build().section_params()[1].astype(np.float64)
    a, b, c = _coefficients(rm)
    rng = np.random.default_rng(3)
    for _ in range(4):
        p = rng.standard_normal(NS)
        Yrm = rng.standard_normal(NS) * rm
        two = _sweep(_sweep(p, Yrm, rm), Yrm, rm)
        C = _sweep(Yrm, Yrm, rm)
        pe = np.concatenate([[0.0, 0.0], p, [0.0, 0.0]])
        one = C + a * pe[:-4] + b * p + c * pe[4:]
        assert np.abs(one - two).max() <= 1e-13 * np.abs(two).max()


def test_fp32_oracle_with_two_step_stays_near_fp64():
    mv = model.ModelVectors.build()
    cfg, sc, gamma, units, x, rows = cases.cfg1_slice(mv, ms=3.0)
    v, _, _ = orc.bm_run(mv.section_params(), gamma, sc, units, x, rows, threads=1)
    v64, _, _ = orc.bm_run(mv.section_params(), gamma, sc, units, x, rows, fp64=True,
                           threads=1)
    rel = np.abs(v.astype(np.float64) - v64).max() / np.abs(v64).max()
    print(f"configuration 1, 3 ms: FP32 oracle vs FP64 {rel:.2e}")
    assert 0 < rel <= 3e-4
