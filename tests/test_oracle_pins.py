"""Pins the oracle (and the product's host setup) to the reference's own code,
compiled from its sources by oracle/build_ref.sh: the constants of
include/const.h and the Thomas solve of src/tridiag.cpp.  Skipped where the
reference tree was not available to build oracle/_ref/."""
import ctypes as C
import math
import os

import numpy as np
import pytest

from cochlearmodel_gb300 import ihc, model
from oracle import oracle as orc

LIB = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref",
                   "libref_pins.so")
pytestmark = pytest.mark.skipif(not os.path.exists(LIB), reason="oracle/_ref not built")


@pytest.fixture(scope="module")
def ref():
    lib = C.CDLL(LIB)
    out = np.zeros(64, np.float64)
    lib.ref_consts.argtypes = [C.c_void_p]
    lib.ref_consts(out.ctypes.data)
    lib.ref_thomas.argtypes = [C.c_void_p] * 5 + [C.c_int]
    return lib, out


def test_model_constants_match_const_h(ref, mv):
    _, k = ref
    o = orc.model_setup()["scal"]
    # w_ohc, dx, alpha_r, alpha_L, alpha_s, Gme, a0, a1, a2, sigma_ow, eta_1, eta_2, w_ow, Cme,
    # ratio_K, psi0
    want = k[:16]
    assert np.array_equal(o, want)
    assert np.array_equal(mv.scal, want)


def test_model_vectors_match_const_h_formulas(ref, mv):
    _, k = ref
    dx, M0, M1, R0, R1, S0, S1 = k[1], k[16], k[17], k[18], k[19], k[20], k[21]
    area, rho, beta, w_ohc, ratio = k[22], k[23], k[24], k[0], k[14]
    o = orc.model_setup()
    for i in range(256):
        M = M0 * math.exp(M1 * dx * i)
        R = R0 * math.exp(R1 * dx * i)
        S = S0 * math.exp(S1 * dx * i)
        assert o["M"][i] == M and mv.M[i] == M
        assert o["R"][i] == R and o["S"][i] == S
        assert o["S_tm"][i] == R * (S / M) / w_ohc
        assert o["S_ohc"][i] == ratio * (R * (S / M) / w_ohc)
        assert o["Q"][i] == 2 * rho * beta / (area * M)


def test_thomas_matches_reference_tridiag(ref):
    lib, _ = ref
    o = orc.model_setup()
    rng = np.random.default_rng(5)
    for _ in range(3):
        v = rng.standard_normal(256)
        got = orc.thomas(o["diag_m"], o["diag_l"], o["diag_u"], v)
        want = np.zeros(256)
        lib.ref_thomas(*[np.ascontiguousarray(a).ctypes.data for a in
                         (o["diag_m"], o["diag_l"], o["diag_u"], v)], want.ctypes.data, 256)
        assert np.array_equal(got, want)


def test_solver_and_nerve_defaults_match_const_h(ref):
    _, k = ref
    cfg = model.RunConfig()
    nerve = ihc.NerveConfig()
    assert np.float32(cfg.cuda_max_time_step) == np.float32(k[25])
    assert np.float32(cfg.cuda_min_time_step) == np.float32(k[26])
    assert np.float32(cfg.Max_M1_SP_Error) == np.float32(k[27])
    assert np.float32(cfg.Max_Tolerance) == np.float32(k[28])
    assert (cfg.JACOBBY_Loops_Slow, cfg.JACOBBY_Loops_Fast, cfg.Cuda_Outern_Loops) == \
        (k[29], k[30], k[31])
    assert k[32] == 2  # TM/OHC update on outer iterations 0-1 (CUDA_AUX_TM_LOOPS)
    assert np.float32(cfg.SPLRef) == np.float32(k[33])
    assert (nerve.Lambda_SAT, nerve.eta_AC, nerve.eta_DC) == (k[34], k[35], k[36])
    assert np.float32(nerve.Tdelta) == np.float32(k[37])
    assert nerve.spontRate == (k[38], k[39], k[40])
    assert nerve.Aihc == (k[41], k[42], k[43])
    assert nerve.W == (k[44], k[45], k[46])
    assert np.float32(nerve.M_tot) == np.float32(np.float32(k[47]) / np.float32(k[48]))
