"""Batched sweeps: many Run_Cuda profile runs of different lengths solved together.

Each group is one reference run (src/solver.cpp:234-962): intervals of one length
laid end to end, Decouple_Filter blocks per interval, one noise level and one
noise-only reference interval when JND is computed.  The BM units of all groups
go into one unit table (longest first) drained by one persistent kernel; the IHC
frames of all groups go into one launch; each group's JND is one launch.  The
whole step can be captured in a CUDA graph and replayed.

jnd_sweep() builds the configuration-3 sweep: a 1 kHz tone at 10..100 dB SPL x
noise levels {none, 0, 10, 20, 30, 40} dB SPL, seeded white Gaussian noise,
hearing-loss OHC/IHC profiles and interval lengths drawn per group.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import native
from .ihc import IHCStage, NerveConfig, reference_frame
from .model import ModelVectors, RunConfig, bm_scalars, reference_units
from .pipeline import JNDWindow, ProfileSweep

F32 = np.float32


def hearing_loss_ohc() -> np.ndarray:
    """OHC_Vector of configuration 3: 0.5 on sections 0-127, then linear to 0.05 at 255."""
    g = np.full(256, 0.5, np.float64)
    g[128:] = 0.5 + (0.05 - 0.5) * np.arange(1, 129) / 128.0
    return g.astype(np.float32)


def hearing_loss_ihc() -> np.ndarray:
    """IHC_Vector of configuration 3: 8 on sections 0-127, then linear to 5 at 255."""
    g = np.full(256, 8.0, np.float64)
    g[128:] = 8.0 + (5.0 - 8.0) * np.arange(1, 129) / 128.0
    return g.astype(np.float32)


def block_nodes_for(length: int, block_target: int, Fs: int) -> tuple[int, int]:
    """(N, D) with N*D == length-ish: D blocks of N nodes, N as close to
    block_target as possible and Time_Block_Length = N/Fs reproducing N
    through the reference's float ceil (include/params.h:291)."""
    D = max(1, int(math.ceil(length / block_target)))
    N = max(1, int(round(length / D)))
    for dn in (0, -1, 1, -2, 2, -3, 3):
        n = N + dn
        if n > 0 and int(math.ceil(float(F32(n / Fs) * F32(Fs)))) == n:
            return n, D
    raise ValueError(f"no block length reproduces {N} nodes")


@dataclass
class Group:
    cfg: RunConfig
    prof: np.ndarray
    ref_of: np.ndarray
    noise: np.ndarray | None
    N: int
    L: int
    in_base: int
    v_row0: int
    lam_row0: int


class BatchSweep:
    """Device buffers and launches for a list of groups."""

    def __init__(self, device, groups_spec, ohc=None, ihc_vec=None, mv=None, nerve=None,
                 jnd=None, ac_taps=None, overlap_time=0.005, Fs=100000, block_target=1000):
        import torch
        from .solver import BMSolver, units_to_device
        self.torch = torch
        self.device = torch.device(device)
        self.lib = native.load()
        self.mv = mv or ModelVectors.build()
        self.nerve = nerve or NerveConfig()
        self.jnd_win = jnd or JNDWindow()
        self.Fs = Fs
        ohc = hearing_loss_ohc() if ohc is None else np.asarray(ohc, np.float32)
        ihc_vec = hearing_loss_ihc() if ihc_vec is None else np.asarray(ihc_vec, np.float32)
        self.groups: list[Group] = []
        units, frames = [], []
        in_base = v_row0 = lam_row0 = 0
        for spec in groups_spec:
            N, D = block_nodes_for(spec["length"], block_target, Fs)
            sweep: ProfileSweep = spec["sweep"]
            prof, _, ref_of = sweep.build()
            n_int = len(prof)
            cfg = RunConfig(Fs=Fs, Time_Block_Length=N / Fs, Decouple_Filter=D,
                            Time_Blocks=n_int * D, Overlap_Time=overlap_time,
                            OHC_Vector=ohc, IHC_Vector=ihc_vec)
            assert cfg.calc_time_block_nodes() == N
            L = N * D
            noise = None
            if spec.get("noise") is not None:
                noise = np.zeros(L, np.float32)
                nz = np.asarray(spec["noise"], np.float32)[:L]
                noise[:len(nz)] = nz
            rows = cfg.total_time_nodes_p1() + 4
            g = Group(cfg, prof, ref_of, noise, N, L, in_base, v_row0, lam_row0)
            u = reference_units(cfg, in_base=in_base, out_base=v_row0)
            units.append(u)
            frames.append(reference_frame(cfg, v_row0=v_row0, lam_row0=lam_row0))
            self.groups.append(g)
            in_base += rows
            v_row0 += rows
            lam_row0 += int(frames[-1]["lam_rows"][0])
        self.sc = bm_scalars(self.groups[0].cfg, self.mv)
        units = np.concatenate(units)
        order = np.argsort(-(units["end"] - units["start"]), kind="stable")
        self.units = units[order]
        self.frames = np.concatenate(frames)
        self.in_len, self.v_rows, self.lam_rows = in_base, v_row0, lam_row0
        self.bm = BMSolver(self.device, self.mv)
        self.bm.check_units(self.units, 1, self.in_len, self.v_rows)
        d = self.device
        self.d_units = units_to_device(self.units, d)
        self.d_gamma = torch.from_numpy(ohc[None].copy()).to(d)
        self.d_in = torch.zeros(self.in_len, dtype=torch.float32, device=d)
        self.d_v = torch.zeros((self.v_rows, 256), dtype=torch.float32, device=d)
        self.d_failed = torch.zeros(self.v_rows, dtype=torch.int32, device=d)
        self.d_stats = torch.zeros((len(self.units), native.STATS_DTYPE.itemsize),
                                   dtype=torch.uint8, device=d)
        self.d_lam = torch.zeros((3, self.lam_rows, 256), dtype=torch.float32, device=d)
        self.ihc = IHCStage(d, self.nerve, ihc_vec[None], ac_taps, Fs)
        self.upload_ihc_tables()
        self.W = np.asarray(self.nerve.W, np.float32)
        self.d_nihc = torch.from_numpy(self.nerve.nihc()).to(d)
        self.per_group = []
        ivs = []
        for gi, g in enumerate(self.groups):
            head, length = self.jnd_win.nodes(Fs, g.L)
            n = len(g.prof)
            self.per_group.append(dict(
                d_prof=torch.from_numpy(g.prof.view(np.uint8).copy()).to(d),
                d_wn=None if g.noise is None else torch.from_numpy(g.noise).to(d),
                head=head, len=length, n=n, out0=len(ivs)))
            # the group's lambda rows start at its frame's first row; interval
            # i's window at + i * L + head
            r0 = int(self.frames["lam_row0"][gi])
            for i in range(n):
                ivs.append((r0 + i * g.L + head, r0 + int(g.ref_of[i]) * g.L + head,
                            float(g.prof["dA"][i]), length, len(ivs)))
        # longest windows first (each keeps its output slot): the kernel issues
        # the table in order, so the long intervals do not trail the launch
        iv = np.array(ivs, dtype=native.JND_INTERVAL_DTYPE)
        self.jnd_iv = iv[np.argsort(-iv["len"], kind="stable")]
        self.d_jnd_iv = torch.from_numpy(self.jnd_iv.view(np.uint8).copy()).to(d)
        self.d_FRA = torch.zeros((3, len(ivs)), dtype=torch.float64, device=d)
        self.d_FAI = torch.zeros((3, len(ivs)), dtype=torch.float64, device=d)
        self.graph = None
        self.extras = None  # tolerance-mode extras (network weights), see solver.run_dev

    @property
    def n_signals(self) -> int:
        return sum(len(g.prof) for g in self.groups)

    @property
    def audio_seconds(self) -> float:
        return sum(len(g.prof) * g.L for g in self.groups) / self.Fs

    def _stream(self, stream):
        s = stream if stream is not None else self.torch.cuda.current_stream(self.device)
        return C.c_void_p(s.cuda_stream)

    def upload_ihc_tables(self, stream=None):
        """Uploads the IHC/lambda per-call tables (frames, tile prefix, taps) for
        ihc_lambda(); again after a change of the IHC run length."""
        sc = self.ihc.scratch(len(self.frames))
        native.check(self.lib.cgb_ihc_lambda_upload_dev(
            native.ptr(self.frames), len(self.frames), native.ptr(self.ihc.ac), len(self.ihc.ac),
            native.ptr(self.ihc.dc), len(self.ihc.dc), C.byref(self.ihc.prm), self.v_rows,
            self.lam_rows, 1, native.ptr(sc), int(sc.numel()), self._stream(stream)),
            "cgb_ihc_lambda_upload_dev")

    def tune(self, use_cache: bool = True):
        """Applies the autotuner's launch choices for this sweep on this GPU
        (cached, or searched and cached); returns (Choice, 'cache'|'search')."""
        from . import autotune
        return autotune.tune_sweep(self, self.device, use_cache=use_cache)

    def generate_input(self, stream=None):
        for g, pg in zip(self.groups, self.per_group):
            native.check(self.lib.cgb_input_gen_dev(
                native.ptr(pg["d_prof"]), pg["n"], native.ptr(pg["d_wn"]), None, 0, g.L, 0,
                float(self.Fs), 0.0, 1.0, 0.0, 1.0,
                native.ptr(self.d_in) + 4 * g.in_base, self._stream(stream)),
                "cgb_input_gen_dev")

    def solve_bm(self, stream=None, h_v=None):
        """The BM stage; with h_v (pinned, shaped like d_v) every velocity row
        is stored there too as the kernel writes it."""
        self.bm.run_dev(self.sc, self.d_gamma, self.d_units, len(self.units), self.d_in,
                        self.d_v, self.d_failed, self.d_stats, stream, extras=self.extras,
                        h_out=h_v)

    def ihc_lambda(self, stream=None, h_lam=None):
        """The IHC/lambda stage; with h_lam (pinned, shaped like d_lam) every
        lambda value is stored there too."""
        sc = self.ihc.scratch(len(self.frames))
        args = [native.ptr(self.d_v), self.v_rows, native.ptr(self.frames), len(self.frames),
                native.ptr(self.ihc.ac), len(self.ihc.ac), native.ptr(self.ihc.dc),
                len(self.ihc.dc), C.byref(self.ihc.prm), native.ptr(self.ihc.dmg), 1,
                native.ptr(self.ihc.aihc), native.ptr(self.d_lam), self.lam_rows, None,
                native.ptr(sc), int(sc.numel()), native.ptr(self.ihc.status)]
        if h_lam is None:
            native.check(self.lib.cgb_ihc_lambda_launch_dev(*args, self._stream(stream)),
                         "cgb_ihc_lambda_launch_dev")
        else:
            native.check_host_mirror(h_lam, self.d_lam, "h_lam")
            native.check(self.lib.cgb_ihc_lambda_launch_mirror_dev(
                *args, native.ptr(h_lam), h_lam.numel() * h_lam.element_size(),
                self._stream(stream)),
                "cgb_ihc_lambda_launch_mirror_dev")

    def jnd_sums(self, stream=None):
        """Fisher sums of every interval of every group in one launch."""
        native.check(self.lib.cgb_jnd_batch_dev(
            native.ptr(self.d_lam), self.lam_rows, native.ptr(self.d_jnd_iv), len(self.jnd_iv),
            len(self.jnd_iv), native.ptr(self.d_nihc), native.ptr(self.W), float(self.Fs),
            self.jnd_win.delta_alpha_time_factor * self.Fs, native.ptr(self.d_FRA),
            native.ptr(self.d_FAI), None, self._stream(stream)), "cgb_jnd_batch_dev")

    def step_host(self, h_tables, h_v, h_lam):
        """One step through host buffers (pinned): the profile tables in, the
        whole path, velocity and the three lambda planes out.  The kernels
        store their results into h_v and h_lam as they write them, over the
        CPU-GPU link while they run: BM each velocity row, the IHC stage each
        lambda value.  No copy follows the compute.  Rows that no kernel
        writes are zeroed here, as they are on the device, so the results
        equal step() followed by copies of d_v and d_lam."""
        from .solver import host_gaps, zero_host_gaps
        if getattr(self, "_gaps", None) is None:
            self._gaps = host_gaps(self.units, self.v_rows, self.frames, self.lam_rows)
        for pg, h in zip(self.per_group, h_tables):
            pg["d_prof"].copy_(h, non_blocking=True)
        self.generate_input()
        self.solve_bm(h_v=h_v)
        self.ihc_lambda(h_lam=h_lam)
        self.jnd_sums()
        # no kernel writes these rows, so the host zeroes them while the
        # kernels run
        zero_host_gaps(h_v, h_lam, self._gaps)

    def step(self, stream=None):
        self.generate_input(stream)
        self.solve_bm(stream)
        self.ihc_lambda(stream)
        self.jnd_sums(stream)

    def capture(self):
        """Captures step() into a CUDA graph (after one eager step to warm up)."""
        torch = self.torch
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            self.step(s)
        torch.cuda.current_stream(self.device).wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            self.step(s)
        self.graph = g
        return g

    def replay(self):
        self.graph.replay()

    def jnd_db(self):
        """Per group: (rate dB, AI dB) of every interval (NaN on references)."""
        out = []
        FRA_all = self.d_FRA.cpu().numpy()
        FAI_all = self.d_FAI.cpu().numpy()
        for g, pg in zip(self.groups, self.per_group):
            n = pg["n"]
            F_RA = np.ascontiguousarray(FRA_all[:, pg["out0"]:pg["out0"] + n])
            F_AI = np.ascontiguousarray(FAI_all[:, pg["out0"]:pg["out0"] + n])
            rate, ai = np.zeros(n), np.zeros(n)
            ref = np.ascontiguousarray(g.ref_of, np.int32)
            native.check(self.lib.cgb_jnd_final(native.ptr(F_RA), native.ptr(F_AI), n,
                                                native.ptr(ref), g.cfg.SPLRef,
                                                self.jnd_win.max_db, native.ptr(rate),
                                                native.ptr(ai)), "cgb_jnd_final")
            out.append((rate, ai, F_RA, F_AI))
        return out


def jnd_sweep_spec(n_seeds=4, seed=0, min_ms=20.0, max_ms=200.0, Fs=100000,
                   noises=(1111.0, 0.0, 10.0, 20.0, 30.0, 40.0),
                   powers=tuple(float(p) for p in range(10, 101, 10)), freq=1000.0):
    """Configuration 3: per (seed, noise level) one group of 10 tone intervals
    and one reference interval of a common length drawn uniformly in
    [min_ms, max_ms]; seeded unit-variance white Gaussian noise per seed."""
    rng = np.random.default_rng(seed)
    specs = []
    for s in range(n_seeds):
        noise = rng.standard_normal(int(max_ms * Fs / 1000) + 1).astype(np.float32)
        for nl in noises:
            length = int(round(rng.uniform(min_ms, max_ms) * Fs / 1000))
            specs.append(dict(length=length, noise=noise,
                              sweep=ProfileSweep(frequencies=[freq], powers=list(powers),
                                                 noises=[nl], calculate_jnd=True)))
    return specs
