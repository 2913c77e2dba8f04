"""A complex-JND run (Sim_Type 4) end to end: a sweep with complex-profile
level adjustments through the device pipeline, then the per-profile
aggregation of its rate JNDs (src/AudioGramCreator.cpp:548-571)."""
import math

import numpy as np
import pytest

from cochlearmodel_gb300 import model
from cochlearmodel_gb300.pipeline import JNDWindow, ProfileRun, ProfileSweep, complex_jnd
from tests.test_complex_jnd_cpu import ref_grad, ref_min

pytestmark = pytest.mark.gpu


def test_complex_sweep_end_to_end(mv):
    import torch
    cfg = model.RunConfig(Time_Block_Length=0.004, Decouple_Filter=1, Overlap_Time=0.001)
    sweep = ProfileSweep(frequencies=[1000.0, 2000.0], powers=[20.0, 40.0, 60.0, 80.0],
                         noises=[1111.0, 30.0], calculate_jnd=True,
                         noise_fix_factor=[0.0, 0.0, 0.5, 0.5])
    noise = np.random.default_rng(2).standard_normal(401).astype(np.float32)
    run = ProfileRun("cuda:0", cfg, sweep, noise=noise, mv=mv,
                     jnd=JNDWindow(head=0.001, tail=0.0005))
    run.step()
    torch.cuda.synchronize()
    rate, ai, _, _ = run.jnd_db()
    values = rate[~run.is_ref]
    assert np.all(np.isfinite(values)) and len(values) == 16
    failed = run.failed_per_interval()
    assert failed.shape == (16,)
    iv = sweep.complex_intervals()
    for method in (0, 1):
        val, warn, fo = complex_jnd(values, iv, method, 0.5, failed)
        for p in range(iv.shape[0]):
            v = [float(values[i]) for i in iv[p]]
            f = [int(failed[i]) for i in iv[p]]
            r = ref_min(v, f) if method == 0 else ref_grad(v, f, 0.5)
            if r[0] is None:
                assert math.isnan(val[p])
            else:
                assert val[p] == np.float32(r[0]) and warn[p] == r[1] and fo[p] == r[2]
