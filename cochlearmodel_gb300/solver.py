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
                extras: native.BMExtras | None = None) -> None:
        """Enqueues the solver on `stream` (default: torch's current stream).
        All tensors live on this solver's device; `units` holds cgb_unit
        records (see units_to_device) already validated by check_units.
        extras: network weights / training-record logging of the tolerance
        mode (jacobi_mode 2)."""
        st = stream if stream is not None else torch.cuda.current_stream(self.device)
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
