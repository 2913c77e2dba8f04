"""Tolerance-mode Jacobi and the learned warm start on the GPU.

* tolerance mode (jacobi_mode 2) with the previous-step and the extrapolated
  guess: bit-exact against the FP32 oracle (same sweeps, same stopping points);
* the network: the BM kernel's fused per-warp inference equals the training
  forward bit for bit, and forward, loss and gradients of the training
  kernels match the FP64 oracle restatement (oracle/warmstart_oracle.cpp);
* the learned guess runs inside the BM kernel to the same tolerance.
"""
import numpy as np
import pytest

from cochlearmodel_gb300 import model
from oracle import oracle as orc
from tests import cases

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("guess", [0, 1])
@pytest.mark.parametrize("db,freq", [(60.0, 1000.0), (100.0, 4000.0)])
def test_tolerance_mode_bit_exact(mv, bm_solver, guess, db, freq):
    cfg, sc, gamma, units, x, rows = cases.cfg1_slice(mv, ms=2.0, db=db, freq=freq)
    tsc = model.tolerance_mode(sc, guess=guess)
    o_v, o_f, o_st = orc.bm_run(mv.section_params(), gamma, tsc, units, x, rows)
    g_v, g_f, g_st = bm_solver.run(tsc, gamma, units, x, rows)
    assert np.array_equal(g_v.view(np.uint32), o_v.view(np.uint32)), np.abs(g_v - o_v).max()
    assert np.array_equal(g_f, o_f)
    for k in ("substeps", "iterations", "sweeps", "status"):
        assert np.array_equal(g_st[k], o_st[k]), k
    assert g_st["sweeps"].sum() > 0


@pytest.fixture(scope="module")
def ws_data(bm_solver):
    """Records logged by the solver on a few warm-start signals, prepared."""
    from cochlearmodel_gb300 import warmstart as W
    batch = W.signal_batch(6, ms=4.0, seed=11)
    rec = W.log_records(bm_solver, batch, cap=96, every=37)
    assert rec.shape[0] >= 48
    net = W.WarmStartNet(seed=3)
    feat, target, nr = net.prepare(rec)
    net.s_out = W.fit_output_scale(target)
    net.pack()
    return W, net, rec, feat, target, nr


def test_features_and_targets(ws_data):
    W, net, rec, feat, target, nr = ws_data
    f = feat.float().cpu().numpy()
    assert np.all(f[:, :8] == 0) and np.all(f[:, 264:] == 0)
    body = f[:, 8:264]
    # normalised channels lie in [-1, 1] and reach 1 in magnitude
    for c in (0, 1, 3, 5, 6):
        m = np.abs(body[:, :, c]).max(axis=1)
        assert np.all(m <= 1.0 + 1e-6)
        assert np.all((m > 0.99) | (m == 0))
    assert np.all(np.isfinite(target.cpu().numpy()))
    assert float(nr.min().item()) > 0.0
    # the exact pressure solves the scaled tridiagonal system
    r = rec.cpu().numpy().astype(np.float64)
    rm = mv_rm()
    t = target.cpu().numpy().astype(np.float64)
    i = 0
    Yrm, p1, p2 = r[i, 0:256], r[i, 256:512], r[i, 512:768]
    rho = r[i, 1280]
    pe = (np.float32(rho) * (p1 - p2).astype(np.float32) + p1.astype(np.float32)).astype(
        np.float64)
    pstar = pe + t[i] * float(nr[i].item())
    lo = np.where(np.arange(256) < 254, 1.0, 0.0)
    res = pstar + rm * (np.concatenate([[0.0], pstar[:-1]]) * lo +
                        np.concatenate([pstar[1:], [0.0]])) - Yrm
    assert np.abs(res).max() <= 1e-4 * np.abs(Yrm).max()


def mv_rm():
    return model.ModelVectors.build().section_params()[1].astype(np.float64)


def test_fused_inference_equals_training_forward(ws_data):
    W, net, rec, feat, target, nr = ws_data
    a = net.forward(feat).cpu().numpy()
    b = net.infer(feat).cpu().numpy()
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), np.abs(a - b).max()


def test_forward_and_gradients_match_oracle(ws_data):
    W, net, rec, feat, target, nr = ws_data
    n = min(32, feat.shape[0])
    f = feat[:n].contiguous()
    t = target[:n].contiguous()
    loss, grad = net.gradients(f, t)
    g_out = net.forward(f).cpu().numpy()
    g_grad = grad.cpu().numpy().astype(np.float64)
    fnp = f[:, 8:264].float().cpu().numpy()
    o_out, o_loss, o_grad = orc.ws_forward_backward(net.params.cpu().numpy(), fnp,
                                                    t.cpu().numpy(), net.s_out, round_bf16=True)
    assert np.abs(g_out - o_out).max() <= 1e-3 * np.abs(o_out).max()
    assert abs(float(loss.item()) - o_loss) <= 1e-3 * o_loss
    # per tensor: W1, b1, W2, b2, W3, b3, W4, b4
    bounds = np.cumsum([0, 2560, 64, 20480, 64, 20480, 64, 320, 1])
    for k in range(8):
        a, b = g_grad[bounds[k]:bounds[k + 1]], o_grad[bounds[k]:bounds[k + 1]]
        rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        assert rel <= 5e-3, (k, rel)


@pytest.mark.parametrize("which", ["fixture", "trained"])
def test_learned_guess_in_the_solver(mv, bm_solver, ws_data, which):
    """The network's guess inside the BM kernel (the fixture's barely trained
    network and the shipped weights): the solve still runs to the tolerance,
    every step converges, and the velocity is as close to the FP64 exact solve
    (exact tridiagonal pressure, FP64 state) as with the other guesses.

    Two tolerance-mode runs are not held to 1e-4 of each other: the 1e-6
    pressure tolerance leaves each FP32 run 1e-4 to 3e-3 from the FP64 exact
    solve.  Measured on four seeds of this batch: previous-pressure guess
    1.2e-4 to 3.3e-3, extrapolated 1.3e-4 to 3.3e-3, trained network 1.5e-4 to
    1.2e-3, reference schedule 1.2e-4 to 8.2e-4.  So each run is checked
    against FP64: with the shipped weights the learned run within 1.5x the
    worse of the two plain guesses, and every run within 5e-3.

    The stopping rule compares successive sweeps (|p2 - p1| <= tol |p2|), not
    the residual, so a poor start can stop further from the exact pressure:
    the fixture's network leaves 6.3e-3 on seed 5 against 3.3e-3 for the plain
    guesses.  It is held to 1e-2."""
    W, net, rec, feat, target, nr = ws_data
    if which == "trained":
        net = W.WarmStartNet.load(W.WEIGHTS)
    batch = W.signal_batch(4, ms=3.0, seed=5)
    r0 = W.evaluate(bm_solver, batch, guess=0)
    r1 = W.evaluate(bm_solver, batch, guess=1)
    r2 = W.evaluate(bm_solver, batch, guess=2, net=net)
    assert r0["status"] == 0 and r1["status"] == 0 and r2["status"] == 0
    assert r2["failed"].sum() <= r1["failed"].sum() + 2
    sc = model.bm_scalars(batch.cfg, mv)
    v64, _, _ = orc.bm_run(mv.section_params(), batch.cfg.gamma()[None], sc, batch.units,
                           batch.inp, batch.out_rows, fp64=True, jacobi_mode=1)
    e0, e1, e2 = (W.max_rel(r["velocity"], v64) for r in (r0, r1, r2))
    print(f"{which} network: velocity max-rel vs the FP64 exact solve: previous {e0:.2e}, "
          f"extrapolated {e1:.2e}, learned {e2:.2e}")
    assert max(e0, e1) <= 5e-3
    if which == "trained":
        assert e2 <= 1.5 * max(e0, e1)
    else:
        assert e2 <= 1e-2


def test_trained_network_gain(mv, bm_solver):
    """What the trained network (weights trained on the GPU by the library's
    own kernels, cochlearmodel_gb300/warmstart_weights.npz) gains on held-out
    seeds at the unchanged tolerance:
      * its prediction of the exact-pressure correction on held-out records
        leaves < 5 % of the error of no correction;
      * the first solve of every step started from its guess needs fewer
        Jacobi sweeps per step than from the plain previous-step guess.
    The extrapolation alone (guess 1) is measured beside it."""
    import torch
    from cochlearmodel_gb300 import warmstart as W
    net = W.WarmStartNet.load(W.WEIGHTS)
    held = W.signal_batch(16, ms=10.0, seed=4321)
    rec = W.log_records(bm_solver, held, cap=2000, every=53)
    feat, target, nr = net.prepare(rec)
    with torch.no_grad():
        o = net.forward(feat)
        mse = float(((net.s_out * o - target) ** 2).mean().item())
        zero = float((target ** 2).mean().item())
    assert mse < 0.05 * zero, (mse, zero)
    r0 = W.evaluate(bm_solver, held, guess=0)
    r1 = W.evaluate(bm_solver, held, guess=1)
    r2 = W.evaluate(bm_solver, held, guess=2, net=net)
    print("sweeps per step: previous %.2f extrapolated %.2f learned %.2f" %
          (r0["sweeps_per_step"], r1["sweeps_per_step"], r2["sweeps_per_step"]))
    assert r0["status"] == r1["status"] == r2["status"] == 0
    assert r2["sweeps_per_step"] < 0.85 * r0["sweeps_per_step"]


def test_host_mirror_keeps_the_extras(bm_solver, ws_data):
    """A host mirror merged into extras that carry the network weights (the
    learned guess): the kernel still finds the weights, the device velocity
    equals the run without the mirror, and the pinned host buffer holds
    exactly the rows the kernel wrote."""
    import torch
    from cochlearmodel_gb300.solver import unit_rows, units_to_device
    W, net = ws_data[0], ws_data[1]
    batch = W.signal_batch(2, ms=2.0, seed=9)
    d = bm_solver.device
    sc = model.tolerance_mode(model.bm_scalars(batch.cfg, bm_solver.mv), guess=2,
                              learned_every=4)
    gamma = torch.from_numpy(np.ascontiguousarray(batch.cfg.gamma()[None], np.float32)).to(d)
    u = units_to_device(batch.units, d)
    x = torch.from_numpy(batch.inp).to(d)
    runs = []
    for mirror in (False, True):
        out = torch.zeros((batch.out_rows, 256), dtype=torch.float32, device=d)
        h = torch.full((batch.out_rows, 256), float("nan")).pin_memory() if mirror else None
        bm_solver.run_dev(sc, gamma, u, len(batch.units), x, out, extras=net.extras(), h_out=h)
        torch.cuda.synchronize(d)
        runs.append((out.cpu(), h))
    (v0, _), (v1, h) = runs
    assert torch.equal(v0, v1)
    first, end = unit_rows(batch.units)
    assert (end > first).all()
    for a, b in zip(first, end):
        assert torch.equal(h[a:b], v1[a:b])
