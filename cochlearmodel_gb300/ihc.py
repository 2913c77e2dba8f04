"""IHC + lambda stage (reference RunIHCKernel, src/cochlea.cu:3573-3644) over
the C ABI, and the host-side setup the reference does in IHCNewKernel and
AudioGramCreator::setupIHCOHC (src/cochlea.cu:2417-2598,
src/AudioGramCreator.cpp:604-828)."""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import native
from .model import RunConfig, expand_vector

F32 = np.float32

FRAME_DTYPE = np.dtype([
    ("v_row0", "<i8"), ("lam_row0", "<i8"), ("rows", "<i4"), ("lam_rows", "<i4"),
    ("seg", "<i4"), ("frdp", "<i4"), ("total", "<i4"), ("ihc_profile", "<i4"),
])
assert FRAME_DTYPE.itemsize == 40


class IHCParams(C.Structure):
    _fields_ = [("scale", C.c_float), ("eta_ac", C.c_float), ("eta_dc", C.c_float),
                ("lambda_sat", C.c_float), ("spont", C.c_float * 3), ("pad_", C.c_int32)]


@dataclass
class NerveConfig:
    """Hair-cell / nerve constants (include/const.h:254-290, src/params.cpp:111-140)."""
    eta_AC: float = 1.0          # AMP_AC
    eta_DC: float = 100.0        # AMP_DC
    Lambda_SAT: float = 500.0    # RSAT
    Tdelta: float = 2e-3         # Tdc
    spontRate: tuple = (60.0, 3.0, 0.1)
    Aihc: tuple = (70.0, 50.0, 30.0)
    W: tuple = (0.61, 0.23, 0.16)
    M_tot: float = 30000.0 / 256.0  # AN_FIBERS / SECTIONS
    scale: float = 1.0            # Scale_BM_Velocity_For_Lambda_Calculation

    def params(self) -> IHCParams:
        p = IHCParams()
        p.scale, p.eta_ac, p.eta_dc = self.scale, self.eta_AC, self.eta_DC
        p.lambda_sat = self.Lambda_SAT
        for j in range(3):
            p.spont[j] = F32(self.spontRate[j])
        return p

    def aihc(self) -> np.ndarray:
        """model_Aihc[3][256]: each A repeated over the sections (src/params.cpp:1384-1386)."""
        return expand_vector(np.asarray(self.Aihc, np.float32), 768).reshape(3, 256)

    def dc_taps(self, Fs: int) -> np.ndarray:
        """round(Fs*Tdelta) taps of 1/(Fs*Tdelta) in float (AudioGramCreator.cpp:622, 810-812)."""
        n = int(round(Fs * self.Tdelta))
        v = F32(1.0) / F32(F32(Fs) * F32(self.Tdelta))
        return np.full(n, v, np.float32)

    def nihc(self) -> np.ndarray:
        return np.full(256, float(F32(self.M_tot)), np.float64)


def ihc_damage(ihc_vector) -> np.ndarray:
    """10^IHC_s per section (AudioGramCreator::setupIHCOHC), as float."""
    v = expand_vector(ihc_vector).astype(np.float64)
    return (10.0 ** v).astype(np.float32)


def design_ac_lowpass(fc: float = 800.0, fs: float = 100000.0, ntaps: int = 255) -> np.ndarray:
    """AC low-pass FIR: a Hamming-windowed ideal low-pass (sinc) of odd length,
    normalised to unit DC gain.  Stands in for the reference's equiripple
    design (src/SubModel.cpp:153-512), which is not reproduced."""
    if ntaps % 2 == 0:
        raise ValueError("ntaps must be odd")
    n = np.arange(ntaps, dtype=np.float64) - (ntaps - 1) / 2.0
    h = 2.0 * fc / fs * np.sinc(2.0 * fc / fs * n)
    h *= 0.54 - 0.46 * np.cos(2.0 * math.pi * np.arange(ntaps) / (ntaps - 1))
    h /= h.sum()
    return h.astype(np.float32)


def design_ac_equiripple(fpass: float = 800.0, fstop: float = 1600.0, fs: float = 100000.0,
                         num_taps: int = 255, weight_pass: float = 1.0,
                         weight_stop: float = 10.0):
    """Equiripple (Parks-McClellan) AC low-pass: the design the reference
    makes with firpm for an "equiripple" AC filter (src/SubModel.cpp:147-149,
    pass band to fpass, stop band from fstop, weights {pass, stop}), unit DC
    gain.  Returns (taps float32, weighted ripple)."""
    lib = native.load()
    nyq = fs / 2.0
    taps = np.zeros(num_taps, np.float64)
    delta = np.zeros(1, np.float64)
    native.check(lib.cgb_design_equiripple_lowpass(num_taps, fpass / nyq, (fstop - fpass) / nyq,
                                                   weight_pass, weight_stop, native.ptr(taps),
                                                   native.ptr(delta), None),
                 "cgb_design_equiripple_lowpass")
    return taps.astype(np.float32), float(delta[0])


def design_ac_from_spec(fpass: float, fstop: float, fs: float = 100000.0,
                        apass_db: float = 1.0, astop_db: float = 60.0, num_taps=None):
    """The reference's equiripple AC design from a pass/stop specification
    (SubModel::analyzeACFilter, src/SubModel.cpp:150-240): ripples
    10^(-A/20), the minimum order of Oppenheim & Schafer eq. 7.104
    (calcMinimumOrder, :143-146) when num_taps is not given, stop weight 10
    and pass weight max(0.01, 10 deltaStop / deltaPass) (with the stop weight
    raised when the floor applies), then the equiripple design with unit DC
    gain.  The reference's further searches (frequency-error correction and
    band-edge search) are not reproduced.  Returns (taps float32, ripple)."""
    nyq = fs / 2.0
    dp = 10.0 ** (-apass_db / 20.0)
    ds = 10.0 ** (-astop_db / 20.0)
    pw = (fstop - fpass) / nyq
    if num_taps is None:
        num_taps = int(math.ceil((-10.0 * math.log10(dp * ds) - 13.0) / (2.324 * pw * math.pi)))
    ws = 10.0
    wp = max(0.01, 10.0 * ds / dp)
    if wp > 10.0 * ds / dp:
        ws = ws * (wp / (10.0 * ds / dp))
    return design_ac_equiripple(fpass, fstop, fs, int(num_taps), wp, ws)


def design_ac_iir_lowpass(fc: float = 800.0, fs: float = 100000.0, order: int = 2):
    """AC low-pass IIR for the reference's is_ac_iir_filter path: a Butterworth
    low-pass of even `order`, by the bilinear transform with the cutoff
    prewarped, as cascaded second-order sections multiplied out into one
    direct-form (b, a) of order + 1 coefficients each (a[0] = 1)."""
    if order < 2 or order % 2:
        raise ValueError("order must be even and >= 2")
    K = math.tan(math.pi * fc / fs)
    b = np.array([1.0])
    a = np.array([1.0])
    for m in range(order // 2):
        # pole pair of the analog prototype: q = 1 / (2 sin((2m+1) pi / (2 order)))
        two_zeta = 2.0 * math.sin((2 * m + 1) * math.pi / (2 * order))
        norm = 1.0 / (1.0 + two_zeta * K + K * K)
        bs = np.array([K * K, 2 * K * K, K * K]) * norm
        as_ = np.array([1.0, 2.0 * (K * K - 1.0) * norm, (1.0 - two_zeta * K + K * K) * norm])
        b = np.convolve(b, bs)
        a = np.convolve(a, as_)
    return b.astype(np.float32), a.astype(np.float32)


def round64(n: int) -> int:
    return (n + 63) // 64 * 64


def reference_frame(cfg: RunConfig, v_row0: int = 0, lam_row0: int = 0,
                    ihc_profile: int = 0) -> np.ndarray:
    """The frame of one Run_Cuda chunk: rows = write time, lambda for
    Time_Blocks x block nodes rows (src/solver.cpp:691-699, cochlea.cu:3431-3506)."""
    N = cfg.calc_time_block_nodes()
    rows = cfg.total_time_nodes()
    f = np.zeros(1, FRAME_DTYPE)
    f["v_row0"], f["lam_row0"], f["rows"] = v_row0, lam_row0, rows
    f["lam_rows"] = N * cfg.Time_Blocks
    total = round64(rows)
    f["seg"] = N * cfg.Decouple_Filter if cfg.Decouple_Filter > 0 else total
    f["frdp"] = N * cfg.Time_Blocks
    f["total"] = total
    f["ihc_profile"] = ihc_profile
    return f


class IHCStage:
    """Device-side IHC/lambda stage: damage/A tables, scratch and status."""

    def __init__(self, device, nerve: NerveConfig | None = None, ihc_profiles=None,
                 ac_taps=None, Fs: int = 100000):
        import torch
        self.torch = torch
        self.device = torch.device(device)
        self.lib = native.load()
        self.nerve = nerve or NerveConfig()
        prof = np.atleast_2d(np.asarray(ihc_profiles if ihc_profiles is not None
                                        else np.full(256, 8.0, np.float32), np.float32))
        self.dmg_host = np.stack([ihc_damage(p) for p in prof])
        self.dmg = torch.from_numpy(self.dmg_host).to(self.device)
        self.aihc = torch.from_numpy(self.nerve.aihc()).to(self.device)
        self.ac = np.ascontiguousarray(ac_taps if ac_taps is not None else design_ac_lowpass(),
                                       np.float32)
        self.dc = self.nerve.dc_taps(Fs)
        self.prm = self.nerve.params()
        self.status = torch.zeros(4, dtype=torch.int32, device=self.device)
        self._scratch = None

    def scratch(self, n_frames: int):
        need = self.lib.cgb_ihc_lambda_scratch_bytes(n_frames, len(self.ac), len(self.dc))
        if self._scratch is None or self._scratch.numel() < need:
            self._scratch = self.torch.empty(int(need), dtype=self.torch.uint8,
                                             device=self.device)
        return self._scratch

    def run_dev(self, v, frames: np.ndarray, lam, ihc=None, stream=None, stage: int = 0,
                stage_out=None) -> None:
        """stage 9-12 (with stage_out shaped like ihc): RunIHCKernel's debug
        stage of every lambda row, 9 AC, 10 DC, 11 and 12 dS."""
        frames = np.ascontiguousarray(frames).view(FRAME_DTYPE)
        st = stream if stream is not None else self.torch.cuda.current_stream(self.device)
        sc = self.scratch(len(frames))
        head = (native.ptr(v), int(v.shape[0]), native.ptr(frames), len(frames),
                native.ptr(self.ac), len(self.ac), native.ptr(self.dc), len(self.dc),
                C.byref(self.prm), native.ptr(self.dmg), int(self.dmg.shape[0]),
                native.ptr(self.aihc), native.ptr(lam), int(lam.shape[1]), native.ptr(ihc))
        tail = (native.ptr(sc), int(sc.numel()), native.ptr(self.status),
                C.c_void_p(st.cuda_stream))
        if stage:
            native.check(self.lib.cgb_ihc_lambda_stage_dev(*head, int(stage),
                                                           native.ptr(stage_out), *tail),
                         "cgb_ihc_lambda_stage_dev")
        else:
            native.check(self.lib.cgb_ihc_lambda_dev(*head, *tail), "cgb_ihc_lambda_dev")

    def upload_chunks(self, frame_groups, v_rows: int, lam_rows: int, stream=None):
        """Per-call tables (frames, tile prefix, taps) of each group of frames
        uploaded to its own scratch buffer, for launches that run one group at
        a time.  Returns [(frames, scratch, first lambda row, end lambda row)]."""
        torch = self.torch
        st = stream if stream is not None else torch.cuda.current_stream(self.device)
        out = []
        for fr in frame_groups:
            fr = np.ascontiguousarray(fr).view(FRAME_DTYPE)
            need = self.lib.cgb_ihc_lambda_scratch_bytes(len(fr), len(self.ac), len(self.dc))
            sc = torch.empty(int(need), dtype=torch.uint8, device=self.device)
            native.check(self.lib.cgb_ihc_lambda_upload_dev(
                native.ptr(fr), len(fr), native.ptr(self.ac), len(self.ac), native.ptr(self.dc),
                len(self.dc), C.byref(self.prm), v_rows, lam_rows, int(self.dmg.shape[0]),
                native.ptr(sc), int(sc.numel()), C.c_void_p(st.cuda_stream)),
                "cgb_ihc_lambda_upload_dev")
            r0 = int(fr["lam_row0"][0])
            r1 = int(fr["lam_row0"][-1] + fr["lam_rows"][-1])
            out.append((fr, sc, r0, r1))
        return out

    def launch_chunk(self, v, chunk, lam, stream, h_lam=None) -> None:
        """The IHC/lambda launch of one uploaded group (upload_chunks).  With
        h_lam (a pinned host tensor shaped like lam) the kernel also stores
        every lambda value there."""
        fr, sc, _, _ = chunk
        args = [native.ptr(v), int(v.shape[0]), native.ptr(fr), len(fr), native.ptr(self.ac),
                len(self.ac), native.ptr(self.dc), len(self.dc), C.byref(self.prm),
                native.ptr(self.dmg), int(self.dmg.shape[0]), native.ptr(self.aihc),
                native.ptr(lam), int(lam.shape[1]), None, native.ptr(sc), int(sc.numel()),
                native.ptr(self.status)]
        if h_lam is None:
            native.check(self.lib.cgb_ihc_lambda_launch_dev(
                *args, C.c_void_p(stream.cuda_stream)), "cgb_ihc_lambda_launch_dev")
        else:
            native.check_host_mirror(h_lam, lam, "h_lam")
            native.check(self.lib.cgb_ihc_lambda_launch_mirror_dev(
                *args, native.ptr(h_lam), h_lam.numel() * h_lam.element_size(),
                C.c_void_p(stream.cuda_stream)),
                "cgb_ihc_lambda_launch_mirror_dev")

    def run_iir(self, v: np.ndarray, frames: np.ndarray, lam_rows: int, b, a,
                want_ihc: bool = False, stage: int = 0):
        """Host-buffer call of the IIR AC path; returns (lambda, ihc or None,
        ac), and with stage 9-12 also that debug stage's [lam_rows][256]
        plane as a fourth element."""
        torch = self.torch
        frames = np.ascontiguousarray(frames).view(FRAME_DTYPE)
        b = np.ascontiguousarray(b, np.float32)
        a = np.ascontiguousarray(a, np.float32)
        d_v = torch.from_numpy(np.require(v, np.float32, ["C", "W"])).to(self.device)
        lam = torch.zeros((3, lam_rows, 256), dtype=torch.float32, device=self.device)
        ihc = torch.zeros((lam_rows, 256), dtype=torch.float32, device=self.device) \
            if want_ihc else None
        ac = torch.zeros_like(d_v)
        out = torch.zeros((lam_rows, 256), dtype=torch.float32, device=self.device) \
            if stage else None
        need = self.lib.cgb_ihc_lambda_iir_scratch_bytes(native.ptr(frames), len(frames), len(b),
                                                         len(self.dc))
        if need < 0:
            raise native.CGBError("bad IIR filter or frame table")
        sc = torch.empty(int(need), dtype=torch.uint8, device=self.device)
        self.status.zero_()
        st = torch.cuda.current_stream(self.device)
        head = (native.ptr(d_v), int(d_v.shape[0]), native.ptr(frames), len(frames),
                native.ptr(b), native.ptr(a), len(b), native.ptr(self.dc), len(self.dc),
                C.byref(self.prm), native.ptr(self.dmg), int(self.dmg.shape[0]),
                native.ptr(self.aihc), native.ptr(lam), lam_rows, native.ptr(ihc),
                native.ptr(ac))
        tail = (native.ptr(sc), int(sc.numel()), native.ptr(self.status),
                C.c_void_p(st.cuda_stream))
        if stage:
            native.check(self.lib.cgb_ihc_lambda_iir_stage_dev(*head, int(stage),
                                                               native.ptr(out), *tail),
                         "cgb_ihc_lambda_iir_stage_dev")
        else:
            native.check(self.lib.cgb_ihc_lambda_iir_dev(*head, *tail), "cgb_ihc_lambda_iir_dev")
        torch.cuda.synchronize(self.device)
        if int(self.status[0].item()) != 0:
            raise native.CGBError("IHC stage: a staged copy did not complete")
        res = (lam.cpu().numpy(), (ihc.cpu().numpy() if want_ihc else None), ac.cpu().numpy())
        return res + (out.cpu().numpy(),) if stage else res

    def run(self, v: np.ndarray, frames: np.ndarray, lam_rows: int, want_ihc: bool = False,
            stage: int = 0):
        """Host-buffer call; returns (lambda float32[3][lam_rows][256], ihc or
        None), and with stage 9-12 also that debug stage's [lam_rows][256]
        plane as a third element."""
        torch = self.torch
        d_v = torch.from_numpy(np.require(v, np.float32, ["C", "W"])).to(self.device)
        lam = torch.zeros((3, lam_rows, 256), dtype=torch.float32, device=self.device)
        ihc = torch.zeros((lam_rows, 256), dtype=torch.float32, device=self.device) \
            if want_ihc else None
        out = torch.zeros((lam_rows, 256), dtype=torch.float32, device=self.device) \
            if stage else None
        self.status.zero_()
        self.run_dev(d_v, frames, lam, ihc, stage=stage, stage_out=out)
        torch.cuda.synchronize(self.device)
        if int(self.status[0].item()) != 0:
            raise native.CGBError("IHC stage: a staged copy did not complete")
        res = (lam.cpu().numpy(), (ihc.cpu().numpy() if want_ihc else None))
        return res + (out.cpu().numpy(),) if stage else res
