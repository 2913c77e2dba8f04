"""Host-side mirror of the reference's configuration surface for the solver path.

Names follow the reference's parameter keys (src/params.cpp:784-1682):
Fs, Time_Blocks, Time_Block_Length, Overlap_Time, Decouple_Filter,
OHC_Vector, IHC_Vector, JACOBBY_Loops_Fast/Slow, Cuda_Outern_Loops,
MAX_TOLERANCE, MAX_M1_SP_ERROR, ... and the derived node counts of
include/params.h:288-395.  Float quantities are formed in float32 exactly as
the reference's C++ forms them, because they feed the float solver.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import native

F32 = np.float32
SECTIONS = native.SECTIONS


@dataclass
class ModelVectors:
    """Per-section model vectors (CModel, src/model.cpp:72-86) and the
    pressure-system diagonals (src/solver.cpp:155-176), in float64."""
    M: np.ndarray
    R: np.ndarray
    S: np.ndarray
    Q: np.ndarray
    S_ohc: np.ndarray
    S_tm: np.ndarray
    R_tm: np.ndarray
    diag_m: np.ndarray
    diag_l: np.ndarray
    diag_u: np.ndarray
    scal: np.ndarray  # w_ohc, dx, alpha_r, alpha_L, alpha_s, Gme, a0, a1, a2,
                      # sigma_ow, eta_1, eta_2, w_ow, Cme, ratio_K, psi0

    @classmethod
    def build(cls) -> "ModelVectors":
        lib = native.load()
        arrs = [np.zeros(SECTIONS, np.float64) for _ in range(10)]
        scal = np.zeros(16, np.float64)
        native.check(lib.cgb_model_setup(*[native.ptr(a) for a in arrs], native.ptr(scal)),
                     "cgb_model_setup")
        return cls(*arrs, scal)

    def section_params(self) -> np.ndarray:
        """float32[8][256]: 1/M, 1/m, R, S, Q, S_ohc, S_tm, R_tm."""
        out = np.zeros((8, SECTIONS), np.float32)
        lib = native.load()
        native.check(lib.cgb_pack_sections(*[native.ptr(a) for a in (
            self.M, self.diag_m, self.R, self.S, self.Q, self.S_ohc, self.S_tm, self.R_tm)],
            native.ptr(out)), "cgb_pack_sections")
        return out

    @property
    def w_ohc(self): return self.scal[0]
    @property
    def dx(self): return self.scal[1]


def expand_vector(v, size: int = SECTIONS) -> np.ndarray:
    """expandVectorToSize (include/cvector.cpp:609-623): each entry repeated
    size//len times, the first size%len entries once more."""
    v = list(np.atleast_1d(np.asarray(v, np.float32)))
    times, rem = divmod(size, len(v))
    out = []
    for i, x in enumerate(v):
        out += [x] * times
        if i < rem:
            out.append(x)
    return np.asarray(out, np.float32)


@dataclass
class RunConfig:
    """The subset of CParams the solver path reads (Appendix-C keys)."""
    Fs: int = 100000
    Time_Blocks: int = 1
    Time_Block_Length: float = 0.05
    Overlap_Time: float = 0.005
    Decouple_Filter: int = 1
    OHC_Vector: np.ndarray = field(default_factory=lambda: np.full(SECTIONS, 0.5, np.float32))
    IHC_Vector: np.ndarray = field(default_factory=lambda: np.full(SECTIONS, 8.0, np.float32))
    JACOBBY_Loops_Fast: int = 2
    JACOBBY_Loops_Slow: int = 20
    Cuda_Outern_Loops: int = 10
    Max_Tolerance: float = 1e-10      # MAX_TOLERANCE default (include/const.h:208)
    Max_M1_SP_Error: float = 1e-15    # MAX_M1_SP_ERROR default (include/const.h:207)
    cuda_max_time_step: float = 1e-6  # CUDA_MAX_TIME_STEP
    cuda_min_time_step: float = 1e-18  # CUDA_MIN_TIME_STEP
    SPLRef: float = 2e-5
    # BM kernel (src/cochlea.cu:1258-2331): 17 = kernel 17 with the full-sum
    # value of its step controller, in this library's own operation order
    # (the CPU oracle mirrors it bit for bit); 0 = BMOHC_NEW_kernel, the
    # reference's default, with its fault-count controller and its own
    # operation order (checked against the reference's compiled kernel).
    # The reference's CParams defaults to 0; this host mirror defaults to 17,
    # the kernel the reference recommends for speed (README.md:44,57).
    Run_Fast_BM_Calculation: int = 17

    # --- derived node counts (include/params.h:288-395) ---
    @property
    def overlap_time_microsec(self) -> int:
        return int(round(self.Overlap_Time * 1000) * 1000)

    def calc_overlap_nodes(self) -> int:
        return (self.overlap_time_microsec * int(self.Fs)) // 1000000

    def calc_time_block_nodes(self) -> int:
        return int(math.ceil(float(F32(self.Time_Block_Length) * F32(self.Fs))))

    def total_time_nodes(self) -> int:
        return self.calc_overlap_nodes() + self.calc_time_block_nodes() * self.Time_Blocks

    def total_time_nodes_p1(self) -> int:
        return self.calc_overlap_nodes() + self.calc_time_block_nodes() * (self.Time_Blocks + 1)

    def cuda_iterations_per_kernel(self) -> int:
        return int(F32(1.0) / (F32(self.Fs) * F32(self.cuda_max_time_step)))

    def time_step(self) -> np.float32:
        return F32(1e-6)  # INIT_TIME_STEP (src/solver.cpp:21)

    def time_step_out(self) -> np.float32:
        return F32(self.time_step() * F32(self.cuda_iterations_per_kernel()))

    def Ts(self) -> np.float32:
        return F32(1.0 / float(self.Fs))

    def gamma(self) -> np.ndarray:
        return expand_vector(self.OHC_Vector)

    def ihc(self) -> np.ndarray:
        return expand_vector(self.IHC_Vector)


def bm_scalars(cfg: RunConfig, mv: ModelVectors) -> native.BMScalars:
    """The float arguments of BMOHCNewKernel as Run_Cuda forms them
    (src/solver.cpp:437-438, 629-659)."""
    s = mv.scal
    sc = native.BMScalars()
    sc.w_ohc = float(F32(s[0]))
    sc.time_step = float(cfg.time_step())
    sc.time_step_out = float(cfg.time_step_out())
    sc.delta_x = float(F32(s[1]))
    sc.alpha_r = float(F32(s[2]))
    sc.Ts = float(cfg.Ts())
    sc.alpha_l = float(F32(s[3]))
    sc.alpha_s = float(F32(s[4]))
    sc.Gme = float(F32(s[5]))
    sc.a0 = float(F32(s[6]))
    sc.a1 = float(F32(s[7]))
    sc.a2 = float(F32(s[8]))
    sc.sigma_ow = float(F32(s[9]))
    sc.eta_1 = float(F32(s[10]))
    sc.eta_2 = float(F32(s[11]))
    sc.dt_min = float(F32(cfg.cuda_min_time_step))
    sc.dt_max = float(F32(cfg.cuda_max_time_step))
    sc.jacobi_fast = cfg.JACOBBY_Loops_Fast
    sc.jacobi_slow = cfg.JACOBBY_Loops_Slow
    sc.max_outer = cfg.Cuda_Outern_Loops
    sc.red_lanes = 32
    sc.jacobi_mode = 0
    sc.max_substeps_per_sample = 1 << 20
    sc.jacobi_tol = 0.0
    sc.jacobi_cap = 0
    sc.guess_mode = 0
    sc.learned_every = 1
    if cfg.Run_Fast_BM_Calculation not in (0, 17):
        raise native.CGBError(f"Run_Fast_BM_Calculation {cfg.Run_Fast_BM_Calculation} is not "
                              "built (0: BMOHC_NEW_kernel, 17: kernel 17)")
    sc.controller = sc.arith = 1 if cfg.Run_Fast_BM_Calculation == 0 else 0
    return sc


# Tolerance of the tolerance-mode Jacobi solve: the corrector's acceptance
# test compares successive velocities to |v| dt, so the pressure must settle
# to about 1e-6 of its maximum; at 1e-5 outer iterations grow and steps fail.
JACOBI_TOL = 1e-6
JACOBI_CAP = 400


def tolerance_mode(sc: native.BMScalars, guess: int = 1, tol: float = JACOBI_TOL,
                   cap: int = JACOBI_CAP, learned_every: int = 1) -> native.BMScalars:
    """A copy of `sc` in jacobi_mode 2: every pressure solve sweeps (in pairs)
    until max|p2 - p1| <= tol * max|p2|, at most `cap` sweeps; the first solve
    of a step starts from the previous pressure (guess 0), its linear
    extrapolation (1) or the extrapolation plus the network's correction (2,
    every learned_every-th step).  The reference runs fixed sweep counts
    (JACOBBY_Loops_Slow/Fast) instead."""
    o = native.BMScalars.from_buffer_copy(sc)
    o.jacobi_mode = 2
    o.jacobi_tol = tol
    o.jacobi_cap = cap
    o.guess_mode = guess
    o.learned_every = learned_every
    return o


def block_partition(time_blocks: int, samples_p1: int, overlap: int, decouple: int):
    lib = native.load()
    st = np.zeros(time_blocks, np.int32)
    of = np.zeros(time_blocks, np.int32)
    en = np.zeros(time_blocks, np.int32)
    native.check(lib.cgb_block_partition(time_blocks, samples_p1, overlap, decouple,
                                         native.ptr(st), native.ptr(of), native.ptr(en)),
                 "cgb_block_partition")
    return st, of, en


def reference_units(cfg: RunConfig, in_base: int = 0, out_base: int = 0, profile: int = 0,
                    mtt: float | None = None, mmspt: float | None = None) -> np.ndarray:
    """The unit table of one reference run (one CUDA block per unit)."""
    st, of, en = block_partition(cfg.Time_Blocks, cfg.total_time_nodes_p1(),
                                 cfg.calc_overlap_nodes(), cfg.Decouple_Filter)
    u = np.zeros(cfg.Time_Blocks, native.UNIT_DTYPE)
    u["in_base"] = in_base
    u["out_base"] = out_base
    u["start"], u["out_first"], u["end"] = st, of, en
    u["profile"] = profile
    u["mtt"] = F32(cfg.Max_Tolerance if mtt is None else mtt)
    u["mmspt"] = F32(cfg.Max_M1_SP_Error if mmspt is None else mmspt)
    return u


def spl_to_amplitude(db_spl: float, spl_ref: float = 2e-5) -> float:
    """SPL2PA (include/params.h:325): 10*10^(dB/20)*SPLRef, in dyn/cm^2."""
    return 0.0 if db_spl == 1111.0 else 10.0 * 10.0 ** (db_spl / 20.0) * spl_ref


def sine_input(n: int, freq: float, amp: float, Fs: int, start_time: float = 0.0) -> np.ndarray:
    """CState::gen_input_data (src/state.cpp:411-436): amp*sin(2*PI*f*t) with
    t advanced by Ts each sample and PI the float constant of const.h."""
    two_pi = 2.0 * float(F32(3.141592653589793))
    out = np.empty(n, np.float32)
    t = float(start_time)
    ts = 1.0 / float(Fs)
    for i in range(n):
        out[i] = F32(amp * math.sin(two_pi * float(freq) * t))
        t += ts
    return out
