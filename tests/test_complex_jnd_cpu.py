"""Complex-JND aggregation (src/ComplexJNDProfile.cpp:19-100) through the C
ABI, against a direct restatement of the two reference methods, and the
complex-profile level adjustments of updateInputProfile."""
import math

import numpy as np
import pytest

from cochlearmodel_gb300.pipeline import ProfileSweep, complex_jnd


def ref_min(vals, failed):
    """calculateMinValue: the last strict interior minimum, else a lower
    boundary (warning); None where the reference keeps a stale value."""
    caps = [i for i in range(1, len(vals) - 1) if vals[i] < vals[i - 1] and vals[i] < vals[i + 1]]
    if caps:
        return vals[caps[-1]], 0, failed[caps[-1]]
    if len(vals) == 1:
        return vals[0], 1, failed[0]
    if vals[0] < vals[1]:
        return vals[0], 1, failed[0]
    if vals[-1] < vals[-2]:
        return vals[-1], 1, failed[-1]
    return None, 1, 0


def ref_grad(vals, failed, eps):
    """calculateGradientMinMaxValue: std::adjacent_find with rhs - lhs > eps."""
    for i in range(len(vals) - 1):
        if vals[i + 1] - vals[i] > eps:
            return vals[i], 0, failed[i]
    return vals[0], 1, failed[0]


@pytest.mark.parametrize("seed", range(6))
def test_methods_match_restatement(seed):
    rng = np.random.default_rng(seed)
    n_prof, n_lev = 7, 6
    values = np.round(rng.uniform(0, 30, n_prof * n_lev), 1)
    failed = rng.integers(0, 3, n_prof * n_lev).astype(np.int32)
    intervals = rng.permutation(n_prof * n_lev).reshape(n_prof, n_lev).astype(np.int32)
    for method in (0, 1):
        eps = 2.0
        val, warn, fo = complex_jnd(values, intervals, method, eps, failed)
        for p in range(n_prof):
            v = [float(values[i]) for i in intervals[p]]
            f = [int(failed[i]) for i in intervals[p]]
            r = ref_min(v, f) if method == 0 else ref_grad(v, f, eps)
            if r[0] is None:
                assert math.isnan(val[p]) and warn[p] == 1
            else:
                assert val[p] == np.float32(r[0]) and warn[p] == r[1] and fo[p] == r[2]


def test_edge_cases():
    # monotone decreasing: no interior minimum, the last is the lowest boundary
    val, warn, _ = complex_jnd([5.0, 4.0, 3.0], [[0, 1, 2]], 0)
    assert val[0] == 3.0 and warn[0] == 1
    # a plateau has no strict minimum and neither boundary is lower: NaN
    val, warn, _ = complex_jnd([2.0, 2.0, 2.0], [[0, 1, 2]], 0)
    assert math.isnan(val[0]) and warn[0] == 1
    # one level
    val, warn, _ = complex_jnd([7.5], [[0]], 0)
    assert val[0] == 7.5 and warn[0] == 1
    # gradient: first rise above eps
    val, warn, _ = complex_jnd([10.0, 9.0, 9.5, 14.0], [[0, 1, 2, 3]], 1, eps=1.0)
    assert val[0] == 9.5 and warn[0] == 0


def test_complex_profile_levels():
    sw = ProfileSweep(frequencies=[1000.0, 2000.0], powers=[10.0, 20.0, 30.0],
                      noises=[1111.0, 20.0], calculate_jnd=True,
                      power_divisor=[0.0, 0.0, 10.0, 0.0], noise_fix_factor=[0.0, 0.0, 0.5, 0.25],
                      noise_fix_addition=[0.0, 0.0, 1.0, -2.0])
    # noise 1111: no adjustment
    assert sw.signal_db(0, 2, 1) == 30.0
    # profile 2 (noise 20, freq 0): 10 + (30 - 10) * 10 / 20 + 0.5 * 20 + 1
    assert sw.signal_db(1, 2, 0) == pytest.approx(10 + 20 * 10 / 20 + 10 + 1)
    # profile 3 (noise 20, freq 1): no divisor; 30 + 0.25 * 20 - 2
    assert sw.signal_db(1, 2, 1) == pytest.approx(33.0)
    iv = sw.complex_intervals()
    assert iv.shape == (4, 3)
    # calculated intervals run noise-major, then power, then frequency
    assert iv[0].tolist() == [0, 2, 4] and iv[3].tolist() == [7, 9, 11]
