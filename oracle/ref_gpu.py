"""Test infrastructure: ctypes binding of the launcher of the REFERENCE's own
CUDA kernels (oracle/ref_gpu.cpp, oracle/_ref/cochlea_ref.cubin).

The cubin is the reference's src/cochlea.cu + include/cochlea.cuh compiled for
sm_103a by oracle/build_ref_gpu.sh where the reference tree is present; it is
device code only, so a copy built on one machine runs on any host with an
sm_103a GPU.  Only tests/ and bench.py's reporting legs may import this module.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libref_gpu.so"
CUBIN = HERE / "_ref" / "cochlea_ref.cubin"

_p = C.c_void_p
_lib = None


class RefBMParams(C.Structure):
    """The BMOHCNewKernel arguments that reach the kernels
    (src/cochlea.cu:990-1042)."""
    _fields_ = (
        [(n, C.c_float) for n in ("w_ohc", "time_step", "time_step_out", "delta_x", "alpha_r")]
        + [("enable_psi", C.c_int), ("enable_OW", C.c_int)]
        + [(n, C.c_float) for n in ("Ts", "alpha_l", "alpha_s", "Gme", "a0", "a1", "a2",
                                    "sigma_ow", "eta_1", "eta_2")]
        + [(n, C.c_int) for n in ("Time_Blocks", "samplesBufferLengthP1",
                                  "overlap_nodes_for_block")]
        + [("overlapTimeMicroSec", C.c_longlong), ("show_transient", C.c_int)]
        + [(n, C.c_float) for n in ("cuda_max_time_step", "cuda_min_time_step")]
        + [("Decouple_Filter", C.c_int)]
        + [(n, C.c_float) for n in ("Max_M1_SP_Error_Parameter", "Max_Tolerance_Parameter")]
        + [("Relative_Error_Parameters", C.c_int)]
        + [(n, C.c_float) for n in ("M1_SP_Fix_Factor", "Tolerance_Fix_Factor", "SPLREfVal")]
        + [(n, C.c_int) for n in ("JACOBBY_Loops_Fast", "JACOBBY_Loops_Slow",
                                  "Cuda_Outern_Loops")])


def available() -> bool:
    """True when the reference cubin is present (it is built only where the
    reference tree exists, and travels with the repository copy)."""
    return CUBIN.exists()


def load():
    global _lib
    if _lib is None:
        if not LIB.exists():
            subprocess.run(["sh", str(HERE / "build.sh")], check=True)
        lib = C.CDLL(str(LIB))
        lib.refgpu_last_error.restype = C.c_char_p
        lib.refgpu_last_bm_ms.restype = C.c_float
        lib.refgpu_load.argtypes = [C.c_char_p]
        lib.refgpu_bm_run.argtypes = [C.c_int, C.POINTER(RefBMParams), _p, _p, _p, _p,
                                      C.c_longlong, _p, C.c_longlong, _p, _p]
        lib.refgpu_ihc_lambda.argtypes = [_p, C.c_int, C.c_int, C.c_int, C.c_int, _p, C.c_int,
                                          _p, C.c_int, C.c_double, C.c_double, C.c_double,
                                          C.c_double, _p, _p, _p, _p, _p]
        lib.refgpu_jnd.argtypes = [_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _p, _p, _p,
                                   _p, C.c_double, C.c_double, _p, _p]
        if not CUBIN.exists():
            raise FileNotFoundError(f"{CUBIN} is missing (built by oracle/build_ref_gpu.sh)")
        if lib.refgpu_load(str(CUBIN).encode()):
            raise RuntimeError(lib.refgpu_last_error().decode())
        _lib = lib
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


def params_from(cfg, sc) -> RefBMParams:
    """RefBMParams of one Run_Cuda parameter set: `cfg` a RunConfig-like object
    (Time_Blocks, Decouple_Filter, node counts, loop counts, tolerances) and
    `sc` the float scalars as Run_Cuda forms them."""
    p = RefBMParams()
    for n in ("w_ohc", "time_step", "time_step_out", "delta_x", "alpha_r", "Ts", "eta_1",
              "eta_2", "a0", "a1", "a2", "sigma_ow", "alpha_l", "alpha_s", "Gme"):
        setattr(p, n, getattr(sc, n))
    p.enable_psi, p.enable_OW = 1, 1
    p.Time_Blocks = cfg.Time_Blocks
    p.samplesBufferLengthP1 = cfg.total_time_nodes_p1()
    p.overlap_nodes_for_block = cfg.calc_overlap_nodes()
    p.overlapTimeMicroSec = cfg.overlap_time_microsec
    p.show_transient = 1
    p.cuda_max_time_step, p.cuda_min_time_step = sc.dt_max, sc.dt_min
    p.Decouple_Filter = cfg.Decouple_Filter
    p.Max_M1_SP_Error_Parameter = cfg.Max_M1_SP_Error
    p.Max_Tolerance_Parameter = cfg.Max_Tolerance
    p.Relative_Error_Parameters = 0
    p.M1_SP_Fix_Factor = p.Tolerance_Fix_Factor = 0.0
    p.SPLREfVal = cfg.SPLRef
    p.JACOBBY_Loops_Fast, p.JACOBBY_Loops_Slow = sc.jacobi_fast, sc.jacobi_slow
    p.Cuda_Outern_Loops = sc.max_outer
    return p


def sections_from(model: dict, gamma) -> list[np.ndarray]:
    """The eleven float[256] vectors of BMOHCKernel_Init in its order (gamma,
    mass, rsM = 1/m, U, L, R, S, Q, S_ohc, S_tm, R_tm), cast as Run_Cuda casts
    them (src/solver.cpp:357-376), from the oracle's model (oracle.model_setup)."""
    f = np.float32
    m = model
    return [np.ascontiguousarray(gamma, f), m["M"].astype(f),
            (f(1.0) / m["diag_m"].astype(f)).astype(f), m["diag_u"].astype(f),
            m["diag_l"].astype(f), m["R"].astype(f), m["S"].astype(f), m["Q"].astype(f),
            m["S_ohc"].astype(f), m["S_tm"].astype(f), m["R_tm"].astype(f)]


def bm_run(variant: int, params: RefBMParams, sections, mtt, mmspt, inp, out_rows: int):
    """Runs the reference's BM kernel (0: BMOHC_NEW_kernel, 17: kernel 17);
    returns (saved_speeds float32[out_rows,256], failed_nodes int32[out_rows],
    failed_blocks int32[Time_Blocks])."""
    lib = load()
    secs = [np.ascontiguousarray(s, np.float32) for s in sections]
    arr = (C.c_void_p * 11)(*[s.ctypes.data for s in secs])
    mtt = np.ascontiguousarray(mtt, np.float32)
    mmspt = np.ascontiguousarray(mmspt, np.float32)
    inp = np.ascontiguousarray(inp, np.float32)
    out = np.zeros((out_rows, 256), np.float32)
    fn = np.zeros(out_rows, np.int32)
    fb = np.zeros(params.Time_Blocks, np.int32)
    rc = lib.refgpu_bm_run(variant, C.byref(params), C.cast(arr, C.c_void_p), _ptr(mtt),
                           _ptr(mmspt), _ptr(inp), inp.size, _ptr(out), out_rows, _ptr(fn),
                           _ptr(fb))
    if rc:
        raise RuntimeError(lib.refgpu_last_error().decode())
    return out, fn, fb


def last_bm_ms() -> float:
    """Device time (ms, CUDA events around the launch) of the last bm_run."""
    return float(load().refgpu_last_bm_ms())


def ihc_lambda(v, calc_time, interval, time_blocks, decouple, ac, dc, scale, eta_ac, eta_dc,
               lambda_sat, ihc_damage, spont, W, aihc):
    """The reference's CudaUnifiedCalcIHC + CudaCalcLambda over one chunk of
    calc_time velocity rows (see refgpu_ihc_lambda); returns
    (ihc float32[calc_time,256], lambda float32[3, calc_time, 256])."""
    lib = load()
    vin = np.zeros((calc_time, 256), np.float32)
    vin[:len(v)] = v
    ihc = np.zeros((calc_time, 256), np.float32)
    lam = np.zeros((3, calc_time, 256), np.float32)
    ac = np.ascontiguousarray(ac, np.float64)
    dc = np.ascontiguousarray(dc, np.float64)
    nerves = np.zeros(9, np.float32)
    nerves[:3] = spont
    nerves[6:] = W
    rc = lib.refgpu_ihc_lambda(_ptr(vin), calc_time, interval, time_blocks, decouple, _ptr(ac),
                               len(ac), _ptr(dc), len(dc), scale, eta_ac, eta_dc, lambda_sat,
                               _ptr(np.ascontiguousarray(ihc_damage, np.float64)),
                               _ptr(nerves), _ptr(np.ascontiguousarray(aihc, np.float32)),
                               _ptr(ihc), _ptr(lam))
    if rc:
        raise RuntimeError(lib.refgpu_last_error().decode())
    return ihc, lam


def jnd(lam, n_int, interval_nodes, head, length, dA, ref_of, nihc, W, Fs, factor):
    """The reference's GlobalCalculateMeanRate + GlobalCalculateJND over every
    interval (see refgpu_jnd); returns (F_RA, F_AI) float32[3, n_int]."""
    lib = load()
    lam = np.ascontiguousarray(lam, np.float32)
    F_RA = np.zeros((3, n_int), np.float32)
    F_AI = np.zeros((3, n_int), np.float32)
    rc = lib.refgpu_jnd(_ptr(lam), lam.shape[1], n_int, interval_nodes, head, length,
                        _ptr(np.ascontiguousarray(dA, np.float64)),
                        _ptr(np.ascontiguousarray(ref_of, np.int32)),
                        _ptr(np.ascontiguousarray(nihc, np.float64)),
                        _ptr(np.ascontiguousarray(W, np.float32)), Fs, factor, _ptr(F_RA),
                        _ptr(F_AI))
    if rc:
        raise RuntimeError(lib.refgpu_last_error().decode())
    return F_RA, F_AI
