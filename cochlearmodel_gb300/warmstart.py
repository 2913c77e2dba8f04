"""Learned Jacobi warm start: data, training and evaluation on the GPU.

The BM solver's tolerance mode (jacobi_mode 2) sweeps every pressure solve
until max|p2 - p1| <= tol * max|p2|.  The first solve of a step needs the
most sweeps; its starting guess is the previous step's pressure (guess 0),
the linear extrapolation of the last two steps (guess 1), or the
extrapolation corrected by a small network (guess 2):

    pe = p1 + rho (p1 - p2),   guess = pe + max|rt| * s_out * net(features)

with rt the Jacobi update from pe.  The network (four width-5 1-D
convolutions over the 256 sections, 8 -> 64 -> 64 -> 64 -> 1 channels, BF16
weights and activations, FP32 accumulation) is trained on (state, exact
pressure) pairs that the solver logs while it runs, by the library's own
forward / backward / Adam kernels (csrc/warmstart.cu).  The Jacobi loop still
runs to the same tolerance, so the guess changes the sweep count, not the
stopping criterion.

torch supplies device memory and streams only; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass
from pathlib import Path

import numpy as np
import torch

from . import model, native
from .solver import BMSolver, units_to_device

FEAT_ROWS = 280          # feature rows per record (section s at row s + 8)
RECORD_FLOATS = 6 * 256  # logged record: Y/m, p1, p2, v, x, {rho, ...}


# ---------------------------------------------------------------------------
# Training and held-out signals
# ---------------------------------------------------------------------------
def warmstart_signal(rng: np.random.Generator, n: int, fs: float) -> tuple[np.ndarray, dict]:
    """One seeded signal of the warm-start data set: a pure tone (125 Hz -
    8 kHz, log-uniform) or a 3-10-harmonic complex (f0 80-400 Hz, random
    phases) with 4-16 Hz sinusoidal amplitude modulation, at 20-100 dB SPL
    (RMS of a tone of that level)."""
    t = np.arange(n) / fs
    db = float(rng.uniform(20.0, 100.0))
    amp = model.spl_to_amplitude(db)
    if rng.uniform() < 0.5:
        f = float(125.0 * 64.0 ** rng.uniform())
        x = amp * np.sin(2 * np.pi * f * t + rng.uniform(0, 2 * np.pi))
        meta = {"kind": "tone", "f": f, "db": db}
    else:
        h = int(rng.integers(3, 11))
        f0 = float(80.0 * 5.0 ** rng.uniform())
        ph = rng.uniform(0, 2 * np.pi, h)
        x = sum(np.sin(2 * np.pi * f0 * (k + 1) * t + ph[k]) for k in range(h))
        fm = float(rng.uniform(4.0, 16.0))
        depth = float(rng.uniform(0.5, 1.0))
        x = x * (1.0 - depth * 0.5 * (1.0 - np.cos(2 * np.pi * fm * t + rng.uniform(0, 2 * np.pi))))
        x = x * (amp / np.sqrt(2.0)) / max(np.sqrt(np.mean(x * x)), 1e-30)
        meta = {"kind": "complex", "f0": f0, "harmonics": h, "am_hz": fm, "db": db}
    return x.astype(np.float32), meta


@dataclass
class SignalBatch:
    """Signals of one length, one unit each (a single time block)."""
    cfg: model.RunConfig
    units: np.ndarray
    inp: np.ndarray
    rows_per_signal: int
    n_signals: int
    meta: list

    @property
    def out_rows(self) -> int:
        return self.rows_per_signal * self.n_signals

    @property
    def audio_seconds(self) -> float:
        return self.n_signals * self.cfg.Time_Block_Length


def signal_batch(n_signals: int, ms: float, seed: int) -> SignalBatch:
    cfg = model.RunConfig(Time_Block_Length=ms / 1000.0, Time_Blocks=1, Decouple_Filter=1)
    rows = cfg.total_time_nodes_p1() + 4
    rng = np.random.default_rng(seed)
    inp = np.zeros(n_signals * rows, np.float32)
    units, meta = [], []
    for i in range(n_signals):
        x, m = warmstart_signal(rng, rows, cfg.Fs)
        inp[i * rows:(i + 1) * rows] = x
        units.append(model.reference_units(cfg, in_base=i * rows, out_base=i * rows))
        meta.append(m)
    return SignalBatch(cfg, np.concatenate(units), inp, rows, n_signals, meta)


# ---------------------------------------------------------------------------
# The network on the device
# ---------------------------------------------------------------------------
class WarmStartNet:
    """Canonical FP32 parameters, Adam moments and the packed BF16 blobs."""

    def __init__(self, device="cuda:0", seed: int = 0, params: np.ndarray | None = None,
                 s_out: float = 1.0, rm_scale: float | None = None):
        self.device = torch.device(device)
        if self.device.type != "cuda" or not torch.cuda.is_available():
            raise native.CGBError("the warm-start network runs on a CUDA device only")
        self.lib = native.load()
        self.n_params = self.lib.cgb_ws_param_count()
        if params is None:
            params = init_params(seed)
        assert params.size == self.n_params
        self.params = torch.from_numpy(np.ascontiguousarray(params, np.float32)).to(self.device)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.step = 0
        self.s_out = float(s_out)
        if rm_scale is None:
            rm = model.ModelVectors.build().section_params()[1]
            rm_scale = float(1.0 / np.abs(rm).max())
        self.rm_scale = float(rm_scale)
        self.blob = torch.zeros(self.lib.cgb_ws_blob_bytes(), dtype=torch.uint8, device=self.device)
        self.blobT = torch.zeros(self.lib.cgb_ws_blobT_bytes(), dtype=torch.uint8,
                                 device=self.device)
        self.pack()

    def pack(self, stream=None) -> None:
        st = _stream(self.device, stream)
        native.check(self.lib.cgb_ws_pack_dev(native.ptr(self.params), self.s_out, self.rm_scale,
                                              native.ptr(self.blob), native.ptr(self.blobT), st),
                     "cgb_ws_pack_dev")

    # -- data ---------------------------------------------------------------
    def prepare(self, records: torch.Tensor):
        """Features, raw targets (p* - pe) / max|rt| and max|rt| of logged records."""
        n = int(records.shape[0])
        d = self.device
        rm = torch.from_numpy(model.ModelVectors.build().section_params()[1].copy()).to(d)
        feat = torch.zeros((n, FEAT_ROWS, 8), dtype=torch.bfloat16, device=d)
        target = torch.zeros((n, 256), dtype=torch.float32, device=d)
        nr = torch.zeros(n, dtype=torch.float32, device=d)
        work = torch.zeros((n, 512), dtype=torch.float64, device=d)
        native.check(self.lib.cgb_ws_prepare_dev(native.ptr(records), n, native.ptr(rm),
                                                 self.rm_scale, native.ptr(feat),
                                                 native.ptr(target), native.ptr(nr),
                                                 native.ptr(work), _stream(d)),
                     "cgb_ws_prepare_dev")
        return feat, target, nr

    # -- forward / backward ---------------------------------------------------
    def buffers(self, n: int) -> dict:
        d = self.device
        return {
            "hid": torch.zeros((3, n, 256, 64), dtype=torch.bfloat16, device=d),
            "out": torch.zeros((n, 256), dtype=torch.float32, device=d),
            "dout": torch.zeros((n, 256, 8), dtype=torch.bfloat16, device=d),
            "dpre": torch.zeros((3, n, 256, 64), dtype=torch.bfloat16, device=d),
            "loss": torch.zeros(n, dtype=torch.float64, device=d),
            "grad": torch.zeros(self.n_params, dtype=torch.float32, device=d),
        }

    def forward(self, feat: torch.Tensor, buf: dict | None = None) -> torch.Tensor:
        n = int(feat.shape[0])
        buf = buf or self.buffers(n)
        native.check(self.lib.cgb_ws_forward_dev(native.ptr(self.blob), native.ptr(feat), n,
                                                 native.ptr(buf["hid"]), native.ptr(buf["out"]),
                                                 _stream(self.device)), "cgb_ws_forward_dev")
        return buf["out"]

    def infer(self, feat: torch.Tensor) -> torch.Tensor:
        """The BM kernel's fused per-warp inference routine, standalone."""
        n = int(feat.shape[0])
        out = torch.zeros((n, 256), dtype=torch.float32, device=self.device)
        native.check(self.lib.cgb_ws_infer_dev(native.ptr(self.blob), native.ptr(feat), n,
                                               native.ptr(out), _stream(self.device)),
                     "cgb_ws_infer_dev")
        return out

    def gradients(self, feat: torch.Tensor, target: torch.Tensor, buf: dict | None = None,
                  n_parts: int | None = None):
        """Forward, loss and backward; returns (mean loss tensor, grad tensor)."""
        n = int(feat.shape[0])
        buf = buf or self.buffers(n)
        st = _stream(self.device)
        lib = self.lib
        self.forward(feat, buf)
        native.check(lib.cgb_ws_loss_dev(native.ptr(buf["out"]), native.ptr(target), n,
                                         self.s_out, native.ptr(buf["dout"]),
                                         native.ptr(buf["loss"]), st), "cgb_ws_loss_dev")
        native.check(lib.cgb_ws_backward_dev(native.ptr(self.blobT), native.ptr(buf["dout"]),
                                             native.ptr(buf["hid"]), n, native.ptr(buf["dpre"]),
                                             st), "cgb_ws_backward_dev")
        parts = n_parts or max(1, min(n, 2 * _sm_count(self.device)))
        if "partial" not in buf or buf["partial"].shape[0] < parts:
            buf["partial"] = torch.zeros((parts, self.n_params), dtype=torch.float32,
                                         device=self.device)
        native.check(lib.cgb_ws_wgrad_dev(native.ptr(feat), native.ptr(buf["hid"]),
                                          native.ptr(buf["dpre"]), native.ptr(buf["dout"]), n,
                                          native.ptr(buf["partial"]), parts,
                                          native.ptr(buf["grad"]), st), "cgb_ws_wgrad_dev")
        return buf["loss"].sum() / (n * 256), buf["grad"]

    def adam(self, grad: torch.Tensor, lr: float) -> None:
        self.step += 1
        native.check(self.lib.cgb_ws_adam_dev(native.ptr(self.params), native.ptr(grad),
                                              native.ptr(self.m), native.ptr(self.v), self.step,
                                              lr, 0.9, 0.999, 1e-8, _stream(self.device)),
                     "cgb_ws_adam_dev")
        self.pack()

    # -- persistence ------------------------------------------------------------
    def save(self, path: str | Path) -> None:
        np.savez(path, params=self.params.cpu().numpy(), s_out=np.float32(self.s_out),
                 rm_scale=np.float32(self.rm_scale))

    @classmethod
    def load(cls, path: str | Path, device="cuda:0") -> "WarmStartNet":
        z = np.load(path)
        return cls(device, params=z["params"], s_out=float(z["s_out"]),
                   rm_scale=float(z["rm_scale"]))

    def extras(self) -> native.BMExtras:
        ex = native.BMExtras()
        ex.d_ws_blob = native.ptr(self.blob)
        return ex


def init_params(seed: int) -> np.ndarray:
    """He-uniform weights, zero biases; the output layer starts small so the
    untrained guess stays near the extrapolation."""
    rng = np.random.default_rng(seed)
    parts = []
    for cout, cin, scale in ((64, 8, 1.0), (64, 64, 1.0), (64, 64, 1.0), (1, 64, 0.1)):
        bound = scale * math.sqrt(6.0 / (cin * 5))
        parts.append(rng.uniform(-bound, bound, 5 * cout * cin))
        parts.append(np.zeros(cout))
    return np.concatenate(parts).astype(np.float32)


def _stream(device, stream=None) -> C.c_void_p:
    st = stream if stream is not None else torch.cuda.current_stream(device)
    return C.c_void_p(st.cuda_stream)


def _sm_count(device) -> int:
    return torch.cuda.get_device_properties(device).multi_processor_count


# ---------------------------------------------------------------------------
# Logging, training, evaluation
# ---------------------------------------------------------------------------
def log_records(solver: BMSolver, batch: SignalBatch, cap: int, every: int,
                tol: float = model.JACOBI_TOL) -> torch.Tensor:
    """Runs the batch in tolerance mode with the extrapolated guess and logs
    every `every`-th step start of each signal (at most `cap` records)."""
    d = solver.device
    sc = model.tolerance_mode(model.bm_scalars(batch.cfg, solver.mv), guess=1, tol=tol)
    log = torch.zeros((cap, RECORD_FLOATS), dtype=torch.float32, device=d)
    count = torch.zeros(1, dtype=torch.int32, device=d)
    ex = native.BMExtras()
    ex.d_log = native.ptr(log)
    ex.log_cap = cap
    ex.log_every = every
    ex.d_log_count = native.ptr(count)
    gamma = torch.from_numpy(np.ascontiguousarray(batch.cfg.gamma()[None], np.float32)).to(d)
    u = units_to_device(batch.units, d)
    x = torch.from_numpy(batch.inp).to(d)
    out = torch.zeros((batch.out_rows, 256), dtype=torch.float32, device=d)
    solver.run_dev(sc, gamma, u, len(batch.units), x, out, extras=ex)
    n = min(int(count.item()), cap)
    return log[:n]


def train(net: WarmStartNet, feat: torch.Tensor, target: torch.Tensor, steps: int,
          batch: int = 256, lr: float = 1e-3, seed: int = 0, log_every: int = 0):
    """Adam on random minibatches; returns the list of (step, mean loss)."""
    n = int(feat.shape[0])
    g = torch.Generator(device="cpu").manual_seed(seed)
    buf = net.buffers(min(batch, n))
    hist = []
    for it in range(steps):
        idx = torch.randint(0, n, (min(batch, n),), generator=g).to(net.device)
        f = feat.index_select(0, idx).contiguous()
        t = target.index_select(0, idx).contiguous()
        # cosine decay to 10 %
        cur = lr * (0.55 + 0.45 * math.cos(math.pi * it / max(1, steps)))
        loss, grad = net.gradients(f, t, buf)
        net.adam(grad, cur)
        if log_every and (it % log_every == 0 or it == steps - 1):
            hist.append((it, float(loss.item())))
    return hist


def fit_output_scale(target: torch.Tensor) -> float:
    return float(target.float().std().item()) or 1.0


def evaluate(solver: BMSolver, batch: SignalBatch, guess: int, net: WarmStartNet | None = None,
             learned_every: int = 1, tol: float = model.JACOBI_TOL, repeats: int = 1) -> dict:
    """Runs the batch in tolerance mode with the given guess; returns the
    velocity, per-unit statistics and the device time of the solve."""
    d = solver.device
    sc = model.tolerance_mode(model.bm_scalars(batch.cfg, solver.mv), guess=guess, tol=tol,
                              learned_every=learned_every)
    gamma = torch.from_numpy(np.ascontiguousarray(batch.cfg.gamma()[None], np.float32)).to(d)
    u = units_to_device(batch.units, d)
    x = torch.from_numpy(batch.inp).to(d)
    out = torch.zeros((batch.out_rows, 256), dtype=torch.float32, device=d)
    failed = torch.zeros(batch.out_rows, dtype=torch.int32, device=d)
    stats = torch.zeros((len(batch.units), native.STATS_DTYPE.itemsize), dtype=torch.uint8,
                        device=d)
    ex = net.extras() if (guess == 2 and net is not None) else None
    solver.run_dev(sc, gamma, u, len(batch.units), x, out, failed, stats, extras=ex)
    torch.cuda.synchronize(d)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(repeats):
        solver.run_dev(sc, gamma, u, len(batch.units), x, out, failed, stats, extras=ex)
    e1.record()
    torch.cuda.synchronize(d)
    ms = e0.elapsed_time(e1) / repeats
    st = stats.cpu().numpy().view(native.STATS_DTYPE).reshape(-1)
    sub = int(st["substeps"].sum())
    return {
        "velocity": out.cpu().numpy(), "failed": failed.cpu().numpy(), "stats": st,
        "ms": ms, "substeps": sub,
        "sweeps_per_step": float(st["sweeps"].sum()) / max(sub, 1),
        "iterations_per_step": float(st["iterations"].sum()) / max(sub, 1),
        "audio_s_per_s": batch.audio_seconds / (ms / 1000.0),
        "status": int(st["status"].max()) if len(st) else 0,
    }


def max_rel(a: np.ndarray, b: np.ndarray) -> float:
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


WEIGHTS = Path(__file__).resolve().parent / "warmstart_weights.npz"
