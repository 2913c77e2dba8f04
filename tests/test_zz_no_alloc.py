"""The no-allocation IHC/lambda entry point (cgb_ihc_lambda_noalloc_dev).

It serves callers that cannot allocate device memory -- a host that hands the
library only buffers it already owns, or a real-time audio thread that must not
enter the device allocator -- by keeping its per-call tables in a fixed array
inside the library.  Its results must equal those of cgb_ihc_lambda_dev (the
entry point with caller scratch) bit for bit, the tolerance the other IHC tests
use, call after call: the array keeps the previous call's contents."""
import ctypes as C

import numpy as np
import pytest

from cochlearmodel_gb300 import ihc, native

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def stage():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return ihc.IHCStage("cuda:0", ihc_profiles=np.stack([np.full(256, 8.0, np.float32),
                                                         np.linspace(8, 5, 256, dtype=np.float32)]))


def _signal(seed, rows):
    rng = np.random.default_rng(seed)
    t = np.arange(rows)[:, None] / 1e5
    f = 200 + 37 * np.arange(256)[None, :]
    return (1e-3 * np.sin(2 * np.pi * f * t + rng.random((1, 256)) * 6) *
            (1 + rng.random((1, 256)))).astype(np.float32)


def _frames(lens, segs):
    fr = np.zeros(len(lens), ihc.FRAME_DTYPE)
    v0 = lam0 = 0
    for i, (n, seg) in enumerate(zip(lens, segs)):
        fr[i] = (v0, lam0, n, n, seg, n, ihc.round64(n), i % 2)
        v0 += n
        lam0 += n
    return fr, lam0


def _noalloc(stage, v, frames, lam_rows):
    import torch
    d = stage.device
    d_v = torch.from_numpy(v).to(d)
    lam = torch.zeros((3, lam_rows, 256), dtype=torch.float32, device=d)
    ih = torch.zeros((lam_rows, 256), dtype=torch.float32, device=d)
    status = torch.zeros(4, dtype=torch.int32, device=d)
    fr = np.ascontiguousarray(frames)
    rc = native.load().cgb_ihc_lambda_noalloc_dev(
        native.ptr(d_v), int(v.shape[0]), native.ptr(fr), len(fr), native.ptr(stage.ac),
        len(stage.ac), native.ptr(stage.dc), len(stage.dc), C.byref(stage.prm),
        native.ptr(stage.dmg), int(stage.dmg.shape[0]), native.ptr(stage.aihc), native.ptr(lam),
        lam_rows, native.ptr(ih), native.ptr(status),
        C.c_void_p(torch.cuda.current_stream(d).cuda_stream))
    native.check(rc, "cgb_ihc_lambda_noalloc_dev")
    torch.cuda.synchronize(d)
    assert int(status[0].item()) == 0
    return lam.cpu().numpy(), ih.cpu().numpy()


def test_matches_scratch_entry_point_on_consecutive_calls(stage):
    cases = [(_signal(1, 2500), *_frames([1000, 1500], [500, 1500])),
             (_signal(2, 1800), *_frames([700, 400, 700], [700, 200, 350]))]
    for v, frames, lam_rows in cases:
        want_lam, want_ihc = stage.run(v, frames, lam_rows, want_ihc=True)
        got_lam, got_ihc = _noalloc(stage, v, frames, lam_rows)
        assert np.array_equal(got_lam.view(np.uint32), want_lam.view(np.uint32))
        assert np.array_equal(got_ihc.view(np.uint32), want_ihc.view(np.uint32))


def test_rejects_sizes_beyond_the_fixed_array(stage):
    v = np.zeros((8, 256), np.float32)
    frames = np.zeros(4097, ihc.FRAME_DTYPE)
    with pytest.raises(native.CGBError, match="4096 frames"):
        _noalloc(stage, v, frames, 8)
