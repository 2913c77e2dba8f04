"""The solver path as Run_Cuda drives it in profile mode (src/solver.cpp:234-962):
input generation -> BM/OHC solver -> IHC/lambda -> JND, on device buffers.

ProfileSweep mirrors CParams::updateInputProfile (src/params.cpp:661-782):
per noise level, per power level, per frequency one tested interval, plus one
noise-only reference interval per noise level when JND is computed.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import native
from .ihc import IHCStage, NerveConfig, reference_frame
from .model import ModelVectors, RunConfig, bm_scalars, reference_units, spl_to_amplitude

F32 = np.float32


@dataclass
class ProfileSweep:
    frequencies: list
    powers: list                       # dB SPL
    noises: list = field(default_factory=lambda: [1111.0])  # 1111 = no noise
    calculate_jnd: bool = False
    spl_ref: float = 2e-5
    # complex-JND profile adjustments, indexed by profile n_freq * noise + freq
    # (Complex_Profile_Power_Level_Divisor / _Noise_Level_Fix_Factor /
    # _Noise_Level_Fix_Addition); missing entries count as 0
    power_divisor: list = field(default_factory=list)
    noise_fix_factor: list = field(default_factory=list)
    noise_fix_addition: list = field(default_factory=list)

    def signal_db(self, nlevel: int, plevel: int, flevel: int) -> float:
        """The tested signal level (src/params.cpp:700-711), in float."""
        cid = len(self.frequencies) * nlevel + flevel
        get = lambda v: F32(v[cid]) if cid < len(v) else F32(0.0)
        noise = F32(self.noises[nlevel])
        base = F32(self.powers[plevel])
        div = get(self.power_divisor)
        if div != 0 and noise != F32(1111.0) and noise > 0:
            p0 = F32(self.powers[0])
            base = F32(p0 + F32(F32(F32(base - p0) * div) / noise))
        if noise != F32(1111.0):
            base = F32(base + F32(F32(get(self.noise_fix_factor) * noise) +
                                  get(self.noise_fix_addition)))
        return float(base)

    def complex_intervals(self) -> np.ndarray:
        """int32[n_noise * n_freq][n_power]: per complex profile (noise, freq),
        the calculated-interval index of each tested power level
        (ComplexJNDProfile::setInterval, src/params.cpp:723-729)."""
        nf, npw = len(self.frequencies), len(self.powers)
        out = np.zeros((len(self.noises) * nf, npw), np.int32)
        idx = 0
        for nl in range(len(self.noises)):
            for pl in range(npw):
                for fl in range(nf):
                    out[nl * nf + fl, pl] = idx
                    idx += 1
        return out

    def build(self):
        """Returns (profiles PROFILE_DTYPE[n], is_reference bool[n], ref_of int32[n])."""
        prof, is_ref, ref_of = [], [], []
        for nli, nl in enumerate(self.noises):
            wn = spl_to_amplitude(float(nl), self.spl_ref)
            first = len(prof)
            for pli in range(len(self.powers)):
                for fli, f in enumerate(self.frequencies):
                    db = self.signal_db(nli, pli, fli)
                    prof.append((spl_to_amplitude(db, self.spl_ref), wn, float(f)))
                    is_ref.append(False)
            if self.calculate_jnd:
                prof.append((0.0, wn, 0.0))
                is_ref.append(True)
                r = len(prof) - 1
                ref_of += [r] * (r - first) + [r]
            else:
                ref_of += list(range(first, len(prof)))
        p = np.array(prof, dtype=native.PROFILE_DTYPE)
        return p, np.array(is_ref), np.array(ref_of, np.int32)


def complex_jnd(values, intervals, method: int = 0, eps: float = 0.0, failed=None):
    """Complex-JND aggregation (cgb_complex_jnd): per complex profile, one
    value from its JND values across the tested power levels.  values: per
    calculated interval (dB); intervals: ProfileSweep.complex_intervals().
    Returns (value float32[n], warning int32[n], failed int32[n])."""
    lib = native.load()
    values = np.ascontiguousarray(values, np.float64)
    intervals = np.ascontiguousarray(intervals, np.int32)
    n, m = intervals.shape
    fl = None if failed is None else np.ascontiguousarray(failed, np.int32)
    val = np.zeros(n, np.float32)
    warn = np.zeros(n, np.int32)
    fo = np.zeros(n, np.int32)
    native.check(lib.cgb_complex_jnd(native.ptr(values), len(values), native.ptr(fl),
                                     native.ptr(intervals), n, m, method, eps, native.ptr(val),
                                     native.ptr(warn), native.ptr(fo)), "cgb_complex_jnd")
    return val, warn, fo


@dataclass
class JNDWindow:
    """JND_Interval_Head / JND_Interval_Tail / JND_Delta_Alpha_Time_Factor."""
    head: float = 0.014
    tail: float = 0.002
    delta_alpha_time_factor: float = 0.2
    max_db: float = 150.0

    def nodes(self, Fs: int, interval_len: int):
        head = int(round(F32(Fs) * F32(self.head)))
        length = interval_len - head - int(round(F32(Fs) * F32(self.tail)))
        return head, length


class ProfileRun:
    """One Run_Cuda chunk in profile mode: a sweep of intervals of equal length
    laid end to end, partitioned into Decouple_Filter blocks per interval."""

    def __init__(self, device, cfg: RunConfig, sweep: ProfileSweep, noise: np.ndarray | None = None,
                 nerve: NerveConfig | None = None, jnd: JNDWindow | None = None,
                 mv: ModelVectors | None = None, ac_taps=None, want_lambda=True,
                 hearing_aid=None):
        import torch
        from .solver import BMSolver, units_to_device
        self.torch = torch
        self.device = torch.device(device)
        self.cfg = cfg
        self.lib = native.load()
        self.mv = mv or ModelVectors.build()
        self.prof, self.is_ref, self.ref_of = sweep.build()
        self.n_int = len(self.prof)
        if cfg.Decouple_Filter < 1:
            raise ValueError("profile runs need Decouple_Filter >= 1")
        cfg.Time_Blocks = self.n_int * cfg.Decouple_Filter
        self.N = cfg.calc_time_block_nodes()
        self.L = self.N * cfg.Decouple_Filter
        self.sc = bm_scalars(cfg, self.mv)
        self.units = reference_units(cfg)
        self.rows = cfg.total_time_nodes_p1() + 4
        self.bm = BMSolver(self.device, self.mv)
        self.bm.check_units(self.units, 1, self.rows, self.rows)
        self.d_units = units_to_device(self.units, self.device)
        self.d_gamma = torch.from_numpy(cfg.gamma()[None].copy()).to(self.device)
        self.d_prof = torch.from_numpy(self.prof.view(np.uint8).copy()).to(self.device)
        self.d_in = torch.zeros(self.rows, dtype=torch.float32, device=self.device)
        self.d_v = torch.zeros((self.rows, 256), dtype=torch.float32, device=self.device)
        self.d_failed = torch.zeros(self.rows, dtype=torch.int32, device=self.device)
        self.d_stats = torch.zeros((len(self.units), native.STATS_DTYPE.itemsize),
                                   dtype=torch.uint8, device=self.device)
        # noise (Input_Noise) and its normalisation (type 3: no energy scaling)
        # the noise draft is cut or zero-padded to one interval (WN resize,
        # src/solver.cpp:497-500); the input kernel reads noise[0, L)
        self.noise = None
        if noise is not None:
            self.noise = np.zeros(self.L, np.float32)
            n = min(self.L, len(noise))
            self.noise[:n] = np.asarray(noise, np.float32)[:n]
        self.d_wn = None if self.noise is None else torch.from_numpy(self.noise).to(self.device)
        self.wn_dc, self.wn_norm, self.sig_norm = 0.0, 1.0, 1.0
        self.want_lambda = want_lambda
        self.nerve = nerve or NerveConfig()
        self.jnd_win = jnd or JNDWindow()
        if want_lambda:
            self.ihc = IHCStage(self.device, self.nerve, cfg.IHC_Vector[None], ac_taps, cfg.Fs)
            self.frames = reference_frame(cfg)
            self.lam_rows = int(self.frames["lam_rows"][0])
            self.d_lam = torch.zeros((3, self.lam_rows, 256), dtype=torch.float32,
                                     device=self.device)
        if sweep.calculate_jnd:
            self.head, self.len = self.jnd_win.nodes(cfg.Fs, self.L)
            self.d_dA = torch.from_numpy(np.ascontiguousarray(self.prof["dA"])).to(self.device)
            self.d_ref = torch.from_numpy(self.ref_of).to(self.device)
            self.d_nihc = torch.from_numpy(self.nerve.nihc()).to(self.device)
            self.d_FRA = torch.zeros((3, self.n_int), dtype=torch.float64, device=self.device)
            self.d_FAI = torch.zeros((3, self.n_int), dtype=torch.float64, device=self.device)
        self.calc_jnd = sweep.calculate_jnd
        # hearing-aid transfer functions (fir, iir), applied to the generated
        # input when either is not the identity (src/cochlea.cu:4454-4503);
        # iir holds the reference's stored form (-a with element 0 = 1)
        self.ha = None
        if hearing_aid is not None:
            fir, iir = (np.atleast_1d(np.asarray(t, np.float32)) for t in hearing_aid)
            active = len(fir) > 1 or (len(fir) > 0 and fir[0] != 1) or \
                len(iir) > 1 or (len(iir) > 0 and iir[0] != 1)
            if active:
                iir_on = len(iir) > 1 or (len(iir) > 0 and iir[0] != 1)
                self.ha = (torch.from_numpy(fir.copy()).to(self.device), len(fir),
                           torch.from_numpy(iir.copy()).to(self.device) if iir_on else None,
                           len(iir) if iir_on else 0,
                           torch.zeros(self.n_int * self.L, dtype=torch.float32,
                                       device=self.device))

    @property
    def audio_seconds(self) -> float:
        return self.n_int * self.L / self.cfg.Fs

    def _stream(self, stream):
        s = stream if stream is not None else self.torch.cuda.current_stream(self.device)
        return C.c_void_p(s.cuda_stream)

    def tune(self, use_cache: bool = True):
        """Applies the autotuner's launch choices for this run on this GPU
        (cached, or searched and cached); returns (Choice, 'cache'|'search')."""
        from . import autotune
        return autotune.tune_sweep(self, self.device, use_cache=use_cache)

    def generate_input(self, stream=None):
        native.check(self.lib.cgb_input_gen_dev(
            native.ptr(self.d_prof), self.n_int, native.ptr(self.d_wn), None, 0, self.L, 0,
            float(self.cfg.Fs), self.wn_dc, self.wn_norm, 0.0, self.sig_norm,
            native.ptr(self.d_in), self._stream(stream)), "cgb_input_gen_dev")
        if self.ha is not None:
            fir, nf, iir, ni, aux = self.ha
            native.check(self.lib.cgb_hearing_aid_dev(
                native.ptr(self.d_in), self.n_int, self.L, native.ptr(fir), nf, native.ptr(iir),
                ni, native.ptr(aux), self._stream(stream)), "cgb_hearing_aid_dev")

    def solve_bm(self, stream=None, h_v=None):
        """The BM stage; with h_v (pinned, shaped like d_v) every velocity row
        is stored there too as the kernel writes it."""
        self.bm.run_dev(self.sc, self.d_gamma, self.d_units, len(self.units), self.d_in,
                        self.d_v, self.d_failed, self.d_stats, stream, h_out=h_v)

    def ihc_lambda(self, stream=None):
        self.ihc.run_dev(self.d_v, self.frames, self.d_lam, None, stream)

    def jnd_sums(self, stream=None):
        W = np.asarray(self.nerve.W, np.float32)
        native.check(self.lib.cgb_jnd_dev(
            native.ptr(self.d_lam), self.lam_rows, self.n_int, self.L, self.head, self.len,
            native.ptr(self.d_dA), native.ptr(self.d_ref), native.ptr(self.d_nihc),
            native.ptr(W), float(self.cfg.Fs),
            self.jnd_win.delta_alpha_time_factor * self.cfg.Fs,
            native.ptr(self.d_FRA), native.ptr(self.d_FAI), None, self._stream(stream)),
            "cgb_jnd_dev")

    def step_host(self, h_tables, h_v, h_lam):
        """One step through host buffers (pinned): the profile table in, the
        whole path, velocity and the three lambda planes out.  The kernels
        store their results into h_v and h_lam as they write them, over the
        CPU-GPU link while they run: BM each velocity row, the IHC stage each
        lambda value.  Rows that no kernel writes are zeroed here, as they
        are on the device, so the results equal step() followed by copies of
        d_v and d_lam."""
        from .solver import host_gaps, zero_host_gaps
        torch = self.torch
        if not self.want_lambda:
            raise ValueError("step_host needs the lambda stage")
        if getattr(self, "_whole", None) is None:
            self._whole = self.ihc.upload_chunks([self.frames], self.rows, self.lam_rows)[0]
            self._gaps = host_gaps(self.units, self.rows, self.frames, self.lam_rows)
        self.d_prof.copy_(h_tables[0], non_blocking=True)
        self.generate_input()
        self.solve_bm(h_v=h_v)
        self.ihc.launch_chunk(self.d_v, self._whole, self.d_lam,
                              torch.cuda.current_stream(self.device), h_lam=h_lam)
        if self.calc_jnd:
            self.jnd_sums()
        # no kernel writes these rows, so the host zeroes them while the
        # kernels run
        zero_host_gaps(h_v, h_lam, self._gaps)

    def step(self, stream=None):
        """One pass of the path over the whole sweep (device buffers only)."""
        self.generate_input(stream)
        self.solve_bm(stream)
        if self.want_lambda:
            self.ihc_lambda(stream)
        if self.calc_jnd:
            self.jnd_sums(stream)

    def failed_per_interval(self) -> np.ndarray:
        """Failed-convergence count of each tested interval: the failed
        samples of its Decouple_Filter blocks (calcJNDFinal,
        src/AudioGramCreator.cpp:489-493), in calculated-interval order."""
        st = self.d_stats.cpu().numpy().view(native.STATS_DTYPE).reshape(-1)
        D = self.cfg.Decouple_Filter
        per = st["failed_samples"].reshape(self.n_int, D).sum(axis=1).astype(np.int32)
        return per[~self.is_ref]

    def jnd_db(self):
        F_RA = self.d_FRA.cpu().numpy()
        F_AI = self.d_FAI.cpu().numpy()
        rate = np.zeros(self.n_int)
        ai = np.zeros(self.n_int)
        native.check(self.lib.cgb_jnd_final(native.ptr(F_RA), native.ptr(F_AI), self.n_int,
                                            native.ptr(self.ref_of), self.cfg.SPLRef,
                                            self.jnd_win.max_db, native.ptr(rate),
                                            native.ptr(ai)), "cgb_jnd_final")
        return rate, ai, F_RA, F_AI
