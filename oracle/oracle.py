"""Test infrastructure: ctypes binding of the CPU oracle (oracle/cochlea_oracle.cpp).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
arm may import this module.  It builds the oracle library on first use.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libcochlea_oracle.so"

UNIT_DTYPE = np.dtype([
    ("in_base", "<i8"), ("out_base", "<i8"), ("start", "<i4"), ("out_first", "<i4"),
    ("end", "<i4"), ("profile", "<i4"), ("mtt", "<f4"), ("mmspt", "<f4"),
])
STATS_DTYPE = np.dtype([
    ("substeps", "<i8"), ("iterations", "<i8"), ("sweeps", "<i8"),
    ("failed_samples", "<i4"), ("written_samples", "<i4"), ("status", "<i4"), ("pad_", "<i4"),
])


class OrcScalars(C.Structure):
    _fields_ = [(n, C.c_float) for n in (
        "w_ohc", "time_step", "time_step_out", "delta_x", "alpha_r", "Ts",
        "alpha_l", "alpha_s", "Gme", "a0", "a1", "a2", "sigma_ow", "eta_1", "eta_2",
        "dt_min", "dt_max")] + [(n, C.c_int32) for n in (
            "jacobi_fast", "jacobi_slow", "max_outer", "red_lanes", "jacobi_mode",
            "max_substeps_per_sample")] + [("jacobi_tol", C.c_float), ("jacobi_cap", C.c_int32),
                                           ("guess_mode", C.c_int32),
                                           ("learned_every", C.c_int32),
                                           ("controller", C.c_int32), ("arith", C.c_int32)]


_lib = None
_p = C.c_void_p


def build(force: bool = False) -> Path:
    srcs = [HERE / "cochlea_oracle.cpp", HERE / "warmstart_oracle.cpp", HERE / "build.sh"]
    if force or not LIB.exists() or any(LIB.stat().st_mtime < f.stat().st_mtime for f in srcs):
        subprocess.run(["sh", str(HERE / "build.sh")], check=True)
    return LIB


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB))
        lib.orc_tanhf.restype = C.c_float
        lib.orc_tanhf.argtypes = [C.c_float]
        lib.orc_log10f.restype = C.c_float
        lib.orc_log10f.argtypes = [C.c_float]
        lib.orc_model_setup.argtypes = [_p] * 11
        lib.orc_thomas.argtypes = [_p, _p, _p, _p, _p, C.c_int]
        lib.orc_block_partition.argtypes = [C.c_int, C.c_int64, C.c_int, C.c_int, _p, _p, _p]
        for nm in ("orc_bm_run_f32", "orc_bm_run_f64"):
            getattr(lib, nm).argtypes = [_p, _p, C.POINTER(OrcScalars), _p, C.c_int, _p, _p,
                                         _p, _p, _p, C.c_int]
        lib.orc_ihc_lambda.argtypes = [_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                       _p, C.c_int, _p, C.c_int, C.c_double, C.c_double,
                                       C.c_double, _p, _p, _p, C.c_double, _p, _p, C.c_int64,
                                       C.c_int]
        lib.orc_jnd.argtypes = [_p, C.c_int64, C.c_int, C.c_int, C.c_int, C.c_int, _p, _p, _p,
                                _p, C.c_double, C.c_double, _p, _p, C.c_int]
        lib.orc_jnd_db.restype = C.c_double
        lib.orc_jnd_db.argtypes = [C.c_double, C.c_double, C.c_double]
        lib.orc_iir_ac.argtypes = [_p, C.c_int, C.c_int, C.c_int, C.c_int, _p, _p, C.c_int,
                                   C.c_double, _p]
        lib.orc_ihc_lambda_iir.argtypes = [_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _p,
                                           _p, C.c_int, _p, C.c_int, C.c_double, C.c_double,
                                           C.c_double, _p, _p, _p, C.c_double, _p, _p, C.c_int64,
                                           C.c_int, _p]
        lib.orc_ihc_lambda_stage.argtypes = [_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                             _p, C.c_int, _p, C.c_int, C.c_double, C.c_double,
                                             C.c_double, _p, _p, _p, C.c_double, _p, _p,
                                             C.c_int64, C.c_int, C.c_int, _p]
        lib.orc_ihc_lambda_ac.argtypes = [_p, _p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                          _p, C.c_int, C.c_double, C.c_double, C.c_double, _p,
                                          _p, _p, C.c_double, _p, _p, C.c_int64, C.c_int,
                                          C.c_int, _p]
        lib.orc_hearing_aid.argtypes = [_p, C.c_int, C.c_int, _p, C.c_int, _p, C.c_int, _p]
        lib.orc_ws_param_count.restype = C.c_int
        lib.orc_ws_forward_backward.argtypes = [_p, _p, _p, C.c_int, C.c_float, C.c_int, _p, _p,
                                                _p]
        lib.orc_input_gen.argtypes = [_p, C.c_int, _p, C.c_int, C.c_int, C.c_float,
                                      C.c_double, C.c_double, C.c_double, _p]
        _lib = lib
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


def scalars_from(sc) -> OrcScalars:
    """Copies a product BMScalars (same field list) into the oracle's struct."""
    o = OrcScalars()
    for name, _ in OrcScalars._fields_:
        setattr(o, name, getattr(sc, name))
    return o


def tanhf(x: float) -> float:
    return load().orc_tanhf(x)


def model_setup():
    arrs = [np.zeros(256, np.float64) for _ in range(10)]
    scal = np.zeros(16, np.float64)
    load().orc_model_setup(*[_ptr(a) for a in arrs], _ptr(scal))
    names = ["M", "R", "S", "Q", "S_ohc", "S_tm", "R_tm", "diag_m", "diag_l", "diag_u"]
    d = dict(zip(names, arrs))
    d["scal"] = scal
    return d


def thomas(m, l, u, v):
    n = len(v)
    res = np.zeros(n, np.float64)
    load().orc_thomas(*[_ptr(np.ascontiguousarray(a, np.float64)) for a in (m, l, u, v)],
                      _ptr(res), n)
    return res


def block_partition(time_blocks, samples_p1, overlap, decouple):
    st = np.zeros(time_blocks, np.int32)
    of = np.zeros(time_blocks, np.int32)
    en = np.zeros(time_blocks, np.int32)
    load().orc_block_partition(time_blocks, samples_p1, overlap, decouple, _ptr(st), _ptr(of),
                               _ptr(en))
    return st, of, en


def bm_run(secp, gamma, sc, units, inp, out_rows, fp64=False, threads=None, jacobi_mode=None,
           conv=None):
    """Runs the BM step over `units`; returns (velocity[out_rows,256], failed, stats).
    conv: optional float32[out_rows, 3] filled with the per-sample statistics."""
    osc = scalars_from(sc)
    if jacobi_mode is not None:
        osc.jacobi_mode = jacobi_mode
    if osc.arith and not fp64:
        raise ValueError("the FP32 oracle evaluates the own operation order (arith 0); the "
                         "reference order (arith 1) is checked against the reference's kernel")
    units = np.ascontiguousarray(units).view(UNIT_DTYPE)
    secp = np.ascontiguousarray(secp, np.float32)
    gamma = np.ascontiguousarray(gamma, np.float32)
    inp = np.ascontiguousarray(inp, np.float32)
    out = np.zeros((out_rows, 256), np.float64 if fp64 else np.float32)
    failed = np.zeros(out_rows, np.int32)
    stats = np.zeros(len(units), STATS_DTYPE)
    fn = load().orc_bm_run_f64 if fp64 else load().orc_bm_run_f32
    fn(_ptr(secp), _ptr(gamma), C.byref(osc), _ptr(units), len(units), _ptr(inp), _ptr(out),
       _ptr(failed), _ptr(conv), _ptr(stats), threads or (os.cpu_count() or 1))
    return out, failed, stats


def ihc_lambda(v, seg, frdp, total, lam_rows, ac_taps, dc_taps, scale, eta_ac, eta_dc,
               ihc_damage, aihc, spont, lambda_sat, mode=0):
    """mode 0: the reference's mixed precision; 1: FP64; 2: the GPU kernel's FP32."""
    v = np.ascontiguousarray(v, np.float32)
    rows = v.shape[0]
    ihc = np.zeros((rows, 256), np.float32)
    lam = np.zeros((3, lam_rows, 256), np.float32)
    ac = np.ascontiguousarray(ac_taps, np.float64)
    dc = np.ascontiguousarray(dc_taps, np.float64)
    load().orc_ihc_lambda(_ptr(v), rows, seg, frdp, total, lam_rows, _ptr(ac), len(ac),
                          _ptr(dc), len(dc), scale, eta_ac, eta_dc,
                          _ptr(np.ascontiguousarray(ihc_damage, np.float64)),
                          _ptr(np.ascontiguousarray(aihc, np.float32)),
                          _ptr(np.ascontiguousarray(spont, np.float32)), lambda_sat,
                          _ptr(ihc), _ptr(lam), lam_rows, mode)
    return ihc, lam


def jnd(lam, n_int, interval_nodes, head, length, dA, ref_of, nIHC, W, Fs, factor, fp64=True):
    lam = np.ascontiguousarray(lam, np.float32)
    stride = lam.shape[1]
    F_RA = np.zeros((3, n_int), np.float64)
    F_AI = np.zeros((3, n_int), np.float64)
    load().orc_jnd(_ptr(lam), stride, n_int, interval_nodes, head, length,
                   _ptr(np.ascontiguousarray(dA, np.float64)),
                   _ptr(np.ascontiguousarray(ref_of, np.int32)),
                   _ptr(np.ascontiguousarray(nIHC, np.float64)),
                   _ptr(np.ascontiguousarray(W, np.float32)), Fs, factor, _ptr(F_RA), _ptr(F_AI),
                   1 if fp64 else 0)
    return F_RA, F_AI


def jnd_db(fisher_sum, spl_ref=2e-5, max_db=150.0):
    return load().orc_jnd_db(float(fisher_sum), spl_ref, max_db)


def input_gen(prof, wn, interval_len, head, Fs, wn_dc, wn_norm, sig_norm):
    prof = np.ascontiguousarray(prof, np.float64)
    wn = np.ascontiguousarray(wn, np.float32)
    out = np.zeros((prof.shape[0], interval_len), np.float32)
    load().orc_input_gen(_ptr(prof), prof.shape[0], _ptr(wn), interval_len, head, Fs, wn_dc,
                         wn_norm, sig_norm, _ptr(out))
    return out


def ws_forward_backward(params, feat, target, s_out, round_bf16=True, want_grad=True):
    """The warm-start network in FP64 (cochlearmodel_gb300/csrc/warmstart.cu):
    returns (output[n,256], mean loss, grad[param_count] or None).
    feat: float[n,256,8]; target: float[n,256]."""
    params = np.ascontiguousarray(params, np.float32)
    feat = np.ascontiguousarray(feat, np.float32)
    target = np.ascontiguousarray(target, np.float32)
    n = feat.shape[0]
    out = np.zeros((n, 256), np.float64)
    loss = np.zeros(1, np.float64)
    grad = np.zeros(load().orc_ws_param_count(), np.float64) if want_grad else None
    load().orc_ws_forward_backward(_ptr(params), _ptr(feat), _ptr(target), n, s_out,
                                   1 if round_bf16 else 0, _ptr(out), _ptr(loss), _ptr(grad))
    return out, float(loss[0]), grad


def ihc_lambda_stage(v, seg, frdp, total, lam_rows, ac_taps, dc_taps, scale, eta_ac, eta_dc,
                     ihc_damage, aihc, spont, lambda_sat, stage, mode=0):
    """One intermediate plane of the IHC stage for every lambda row: stage 9
    AC, 10 DC, 11 dS, in `mode`'s arithmetic (as ihc_lambda).  Returns
    float32 [lam_rows][256]."""
    v = np.ascontiguousarray(v, np.float32)
    rows = v.shape[0]
    lam = np.zeros((3, lam_rows, 256), np.float32)
    out = np.zeros((lam_rows, 256), np.float32)
    ac = np.ascontiguousarray(ac_taps, np.float64)
    dc = np.ascontiguousarray(dc_taps, np.float64)
    load().orc_ihc_lambda_stage(_ptr(v), rows, seg, frdp, total, lam_rows, _ptr(ac), len(ac),
                                _ptr(dc), len(dc), scale, eta_ac, eta_dc,
                                _ptr(np.ascontiguousarray(ihc_damage, np.float64)),
                                _ptr(np.ascontiguousarray(aihc, np.float32)),
                                _ptr(np.ascontiguousarray(spont, np.float32)), lambda_sat,
                                None, _ptr(lam), lam_rows, mode, stage, _ptr(out))
    return out


def ihc_lambda_ac(v, ac, seg, frdp, total, lam_rows, dc_taps, scale, eta_ac, eta_dc,
                  ihc_damage, aihc, spont, lambda_sat, mode=0, stage=0):
    """IHC/lambda with the AC stage given (rows x 256 floats) in place of the
    FIR; the rest in `mode` as ihc_lambda.  Returns (ihc, lambda), and with
    stage 9-11 (as ihc_lambda_stage) also that plane [lam_rows][256]."""
    v = np.ascontiguousarray(v, np.float32)
    ac = np.ascontiguousarray(ac, np.float32)
    assert ac.shape == v.shape
    rows = v.shape[0]
    ihc = np.zeros((rows, 256), np.float32)
    lam = np.zeros((3, lam_rows, 256), np.float32)
    out = np.zeros((lam_rows, 256), np.float32) if stage else None
    dc = np.ascontiguousarray(dc_taps, np.float64)
    load().orc_ihc_lambda_ac(_ptr(v), _ptr(ac), rows, seg, frdp, total, lam_rows, _ptr(dc),
                             len(dc), scale, eta_ac, eta_dc,
                             _ptr(np.ascontiguousarray(ihc_damage, np.float64)),
                             _ptr(np.ascontiguousarray(aihc, np.float32)),
                             _ptr(np.ascontiguousarray(spont, np.float32)), lambda_sat,
                             _ptr(ihc), _ptr(lam), lam_rows, mode, stage,
                             _ptr(out) if stage else None)
    return (ihc, lam, out) if stage else (ihc, lam)


def ihc_lambda_iir(v, seg, frdp, total, lam_rows, b, a, dc_taps, scale, eta_ac, eta_dc,
                   ihc_damage, aihc, spont, lambda_sat, mode=0):
    """IHC/lambda with the AC stage by the reference's IIR recursion; returns
    (ihc, lambda[3][lam_rows][256], ac[rows][256])."""
    v = np.ascontiguousarray(v, np.float32)
    rows = v.shape[0]
    ihc = np.zeros((rows, 256), np.float32)
    lam = np.zeros((3, lam_rows, 256), np.float32)
    ac = np.zeros((rows, 256), np.float32)
    b = np.ascontiguousarray(b, np.float64)
    a = np.ascontiguousarray(a, np.float64)
    dc = np.ascontiguousarray(dc_taps, np.float64)
    load().orc_ihc_lambda_iir(_ptr(v), rows, seg, frdp, total, lam_rows, _ptr(b), _ptr(a), len(b),
                              _ptr(dc), len(dc), scale, eta_ac, eta_dc,
                              _ptr(np.ascontiguousarray(ihc_damage, np.float64)),
                              _ptr(np.ascontiguousarray(aihc, np.float32)),
                              _ptr(np.ascontiguousarray(spont, np.float32)), lambda_sat,
                              _ptr(ihc), _ptr(lam), lam_rows, mode, _ptr(ac))
    return ihc, lam, ac


def hearing_aid(x, fir, iir):
    """Hearing-aid shaping of float[n_prof][L] input (reference semantics)."""
    x = np.ascontiguousarray(x, np.float32)
    fir = np.ascontiguousarray(fir, np.float32)
    iir = np.ascontiguousarray(iir, np.float32)
    out = np.zeros_like(x)
    load().orc_hearing_aid(_ptr(x), x.shape[0], x.shape[1], _ptr(fir), len(fir), _ptr(iir),
                           len(iir), _ptr(out))
    return out
