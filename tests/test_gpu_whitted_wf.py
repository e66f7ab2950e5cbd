"""The Whitted tracer's wavefront stages (QR_FP_WAVEFRONT) against the
per-pixel kernels (the default), bit for bit.

The wavefront (camera rays, nearest-hit and shading, shadow rays light by
light, light sums, secondary rays, a bottom-up fold) must give the frame of
the per-pixel kernels: every AA mode, ragged sizes, depths 0 to 10,
clippers and booleans, textures, the other quadric kinds, several chunks a
frame, and chunks whose queues overflow (the frame is then rendered by the
per-pixel code).  The other GPU parity tests render through the default
path against the oracle and the reference's frames.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ctx(qr, samples=None):
    old = os.environ.get("QR_WH_SAMPLES")
    if samples:
        os.environ["QR_WH_SAMPLES"] = str(samples)
    else:
        os.environ.pop("QR_WH_SAMPLES", None)
    try:
        return qr.Context(0)
    finally:
        if old is None:
            os.environ.pop("QR_WH_SAMPLES", None)
        else:
            os.environ["QR_WH_SAMPLES"] = old


def _both(qr, ctx, kind, seed, nq, w, h, fsaa, depth, flags=0, t=0):
    g = qr.GenScene(kind, seed, nq, flags)
    f = qr.Flat(g, w, h, fsaa)
    desc, params = f.update(t, depth)
    sid = ctx.upload(desc)
    b = ctx.render_host(sid, params).copy()
    p = qr.QrFrameParams.from_buffer_copy(params)
    p.flags = p.flags | qr.FP_WAVEFRONT
    a = ctx.render_host(sid, p).copy()
    ctx.release(sid)
    return a, b


CASES = [  # kind, seed, nq, w, h, fsaa, depth, flags, t
    (2, 1, 64, 320, 180, 2, 4, 0, 0),
    (2, 2, 64, 203, 117, 1, 4, 0, 16),
    (2, 3, 64, 160, 90, 0, 10, 0, 32),
    (2, 4, 128, 96, 54, 2, 0, 0, 0),
    (2, 6, 64, 128, 72, 0, 4, 512, 48),
    (1, 1, 16, 320, 192, 0, 10, 0, 0),
    (1, 7, 16, 161, 93, 2, 10, 32 | 64, 0),
    (1, 12, 8, 160, 96, 0, 10, 128, 0),
    (1, 17, 16, 160, 96, 1, 10, 256, 0),
    (1, 4, 16, 7, 3, 0, 10, 0, 0),
    (3, 2, 32, 128, 72, 2, 8, 0, 0),
]


@pytest.mark.parametrize("kind,seed,nq,w,h,fsaa,depth,flags,t", CASES)
def test_whitted_wavefront_equals_megakernel(qr, kind, seed, nq, w, h, fsaa, depth, flags, t):
    ctx = _ctx(qr)
    a, b = _both(qr, ctx, kind, seed, nq, w, h, fsaa, depth, flags, t)
    assert (a != b).sum() == 0
    assert ctx.fault() == (0, 0, 0, 0)
    ctx.close()


@pytest.mark.parametrize("samples", [128, 4096, 50000])
def test_whitted_wavefront_chunks_and_overflow(qr, samples):
    """many chunks a frame, and chunks small enough for a deep reflective
    tree to overflow their queues (the per-pixel code renders the frame):
    the same bits"""
    ctx = _ctx(qr, samples)
    for case in [(2, 7, 64, 160, 90, 2, 10, 0, 16), (1, 3, 16, 97, 61, 0, 10, 0, 0)]:
        a, b = _both(qr, ctx, *case)
        assert (a != b).sum() == 0, case
    ctx.close()


def test_whitted_wavefront_two_streams(qr):
    """frames of one context on two streams take turns on the scratch"""
    import torch
    ctx = _ctx(qr)
    g = qr.GenScene(qr.SCN_ANIM, 9, 64, 0)
    f = qr.Flat(g, 192, 108, 2)
    desc, params = f.update(0, 4)
    sid = ctx.upload(desc)
    ref = ctx.render_host(sid, params).copy()
    p = qr.QrFrameParams.from_buffer_copy(params)
    p.flags = p.flags | qr.FP_WAVEFRONT
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    outs = []
    for s in (s1, s2, s1, s2):
        fr = torch.zeros((params.y_res, params.x_row), dtype=torch.int32, device="cuda")
        ctx.render_device(sid, p, fr.data_ptr(), s.cuda_stream)
        outs.append(fr)
    torch.cuda.synchronize()
    for fr in outs:
        assert (fr.cpu().numpy().view(np.uint32)[:, :params.x_res] != ref).sum() == 0
    ctx.close()
