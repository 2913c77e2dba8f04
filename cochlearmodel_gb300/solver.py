"""Device-side runner of the BM/OHC solver over the C ABI.

torch supplies device memory and streams; the compute is the native kernel
(cgb_bm_run_dev).  There is no CPU path: on a machine without CUDA the
constructor raises.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import native
from .model import ModelVectors


def _require_cuda(device: torch.device) -> None:
    if device.type != "cuda" or not torch.cuda.is_available():
        raise native.CGBError("the cochlear solver runs on a CUDA device only")


def units_to_device(units: np.ndarray, device) -> torch.Tensor:
    u = np.ascontiguousarray(units).view(native.UNIT_DTYPE)
    return torch.from_numpy(u.view(np.uint8).copy()).to(device)


def unwritten_ranges(starts, ends, rows: int) -> list[tuple[int, int]]:
    """Row ranges of [0, rows) outside every written span [starts[i], ends[i])."""
    cover = np.zeros(rows + 1, np.int64)
    np.add.at(cover, np.asarray(starts, np.int64), 1)
    np.add.at(cover, np.asarray(ends, np.int64), -1)
    written = (np.cumsum(cover[:-1]) > 0).astype(np.int8)
    edges = np.flatnonzero(np.diff(np.concatenate([[1], written, [1]])))
    return [(int(a), int(b)) for a, b in zip(edges[0::2], edges[1::2])]


def unit_rows(units: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """First and one-past-last output row each unit writes (when it completes)."""
    u = np.ascontiguousarray(units).view(native.UNIT_DTYPE)
    first = u["out_base"] + np.maximum(u["start"], u["out_first"])
    return first, u["out_base"] + u["end"]


def host_gaps(units: np.ndarray, v_rows: int, frames: np.ndarray, lam_rows: int):
    """Velocity and lambda row ranges that no kernel writes (they stay zero
    on the device): the padding rows between runs, and rows before a unit's
    first output."""
    return (unwritten_ranges(*unit_rows(units), v_rows),
            unwritten_ranges(frames["lam_row0"], frames["lam_row0"] + frames["lam_rows"],
                             lam_rows))


def zero_host_gaps(h_v, h_lam, gaps) -> None:
    """Zeroes the host mirrors' rows that no kernel writes."""
    hv, hl = h_v.numpy(), h_lam.numpy()
    for a, b in gaps[0]:
        hv[a:b] = 0
    for a, b in gaps[1]:
        hl[:, a:b] = 0


class BMSolver:
    """Holds the section parameters and the work-queue scratch on one device."""

    def __init__(self, device: str | torch.device = "cuda:0", mv: ModelVectors | None = None):
        self.device = torch.device(device)
        _require_cuda(self.device)
        self.lib = native.load()
        self.mv = mv or ModelVectors.build()
        self.secp = torch.from_numpy(self.mv.section_params()).to(self.device)
        self.work = torch.zeros(4, dtype=torch.int32, device=self.device)

    def check_units(self, units: np.ndarray, n_profiles: int, in_len: int, out_rows: int):
        u = np.ascontiguousarray(units).view(native.UNIT_DTYPE)
        native.check(self.lib.cgb_check_units(native.ptr(u), len(u), n_profiles, in_len,
                                              out_rows), "cgb_check_units")

    def run_dev(self, sc: native.BMScalars, gamma: torch.Tensor, units: torch.Tensor,
                n_units: int, inp: torch.Tensor, out: torch.Tensor,
                failed: torch.Tensor | None = None, stats: torch.Tensor | None = None,
                stream: torch.cuda.Stream | None = None, conv: torch.Tensor | None = None,
                extras: native.BMExtras | None = None,
                h_out: torch.Tensor | None = None) -> None:
        """Enqueues the solver on `stream` (default: torch's current stream).
        All tensors live on this solver's device; `units` holds cgb_unit
        records (see units_to_device) already validated by check_units.
        extras: network weights / training-record logging of the tolerance
        mode (jacobi_mode 2).  h_out: a pinned host tensor shaped like `out`
        that receives every velocity row as the kernel writes it."""
        st = stream if stream is not None else torch.cuda.current_stream(self.device)
        if h_out is not None:
            native.check_host_mirror(h_out, out, "h_out")
            ex = native.BMExtras()
            if extras is not None:
                C.memmove(C.addressof(ex), C.addressof(extras), C.sizeof(ex))
            ex.h_out = h_out.data_ptr()
            ex.h_out_bytes = h_out.numel() * h_out.element_size()
            extras = ex
        native.check(self.lib.cgb_bm_run_ex_dev(
            native.ptr(self.secp), native.ptr(gamma), int(gamma.shape[0]), C.byref(sc),
            native.ptr(units), int(n_units), native.ptr(inp), int(inp.numel()),
            native.ptr(out), int(out.shape[0]), native.ptr(failed), native.ptr(conv),
            native.ptr(stats), native.ptr(self.work),
            C.cast(C.byref(extras), C.c_void_p) if extras is not None else None,
            C.c_void_p(st.cuda_stream)), "cgb_bm_run_dev")

    def run(self, sc: native.BMScalars, gamma: np.ndarray, units: np.ndarray,
            inp: np.ndarray, out_rows: int, want_conv: bool = False,
            extras: native.BMExtras | None = None):
        """Host-buffer call: validates, uploads, solves, downloads.
        Returns (velocity float32[out_rows,256], failed int32[out_rows], stats)
        and, with want_conv, the per-sample statistics float32[out_rows,3]."""
        gamma = np.ascontiguousarray(np.atleast_2d(gamma), np.float32)
        inp = np.ascontiguousarray(inp, np.float32)
        self.check_units(units, gamma.shape[0], inp.size, out_rows)
        d = self.device
        g = torch.from_numpy(gamma).to(d)
        u = units_to_device(units, d)
        x = torch.from_numpy(inp).to(d)
        out = torch.zeros((out_rows, native.SECTIONS), dtype=torch.float32, device=d)
        failed = torch.zeros(out_rows, dtype=torch.int32, device=d)
        stats = torch.zeros((len(units), native.STATS_DTYPE.itemsize), dtype=torch.uint8,
                            device=d)
        conv = torch.zeros((out_rows, 3), dtype=torch.float32, device=d) if want_conv else None
        self.run_dev(sc, g, u, len(units), x, out, failed, stats, conv=conv, extras=extras)
        torch.cuda.synchronize(d)
        st = stats.cpu().numpy().view(native.STATS_DTYPE).reshape(-1)
        if want_conv:
            return out.cpu().numpy(), failed.cpu().numpy(), st, conv.cpu().numpy()
        return out.cpu().numpy(), failed.cpu().numpy(), st
