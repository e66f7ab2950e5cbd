"""qr_render_pt_noalloc: the path tracer with its running sums in the
library's fixed device array, against qr_render_pt with caller-owned sums.

The entry point is for callers that may not allocate device memory inside
their render loop.  Collected last (file name), and independent of the other
tests: it passes alone and after them.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scene(qr, w, h, seed=4):
    g = qr.GenScene(qr.SCN_PT, seed, 32, 0)
    f = qr.Flat(g, w, h, 0)
    desc, params = f.update(0, 8)
    return g, f, desc, params


def _noalloc(qr, ctx, sid, p, frame_ptr, stream=None):
    return qr.lib().qr_render_pt_noalloc(ctx.h, sid, ctypes.byref(p),
                                         ctypes.c_void_p(frame_ptr),
                                         ctypes.c_void_p(stream) if stream else None)


def test_noalloc_matches_render_pt_two_calls(qr):
    import torch
    ctx = qr.Context(0)
    g, f, desc, params = _scene(qr, 128, 72)
    sid = ctx.upload(desc)
    acc = torch.zeros((params.y_res, params.x_row, 3), dtype=torch.float32, device="cuda")
    fa = torch.zeros((params.y_res, params.x_row), dtype=torch.int32, device="cuda")
    fb = torch.zeros_like(fa)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        p = qr.QrFrameParams.from_buffer_copy(params)
        p.pt_on, p.pts_c, p.seed, p.frame_idx = 8, 8.0 * call, 31, call
        ctx.render_pt(sid, p, acc.data_ptr(), fa.data_ptr(), stream)
        rc = _noalloc(qr, ctx, sid, p, fb.data_ptr(), stream)
        assert rc == qr.QR_OK, ctx.error()
        torch.cuda.synchronize()
        assert torch.equal(fa, fb), call
        assert int((fb != 0).sum()) > 0
    assert torch.cuda.current_device() == 0
    ctx.close()


def test_noalloc_rejects_oversize_frame(qr):
    """a frame beyond the fixed sums is refused before any launch; the frame
    handed over is a real device buffer of that size, so a regression of the
    size check would render into it instead of faulting"""
    import torch
    ctx = qr.Context(0)
    g, f, desc, params = _scene(qr, 1920, 1080)
    sid = ctx.upload(desc)
    params.pt_on, params.pts_c = 1, 0.0
    frame = torch.zeros((params.y_res, params.x_row), dtype=torch.int32, device="cuda")
    rc = _noalloc(qr, ctx, sid, params, frame.data_ptr())
    torch.cuda.synchronize()
    assert rc == qr.QR_ERR_LIMIT
    assert "exceeds" in ctx.error()
    assert int((frame != 0).sum()) == 0
    ctx.close()


def test_noalloc_needs_started_sums(qr):
    """adding to sums needs a start of the same context, scene and frame
    shape: the same pixel count in another shape, another scene, or no start
    at all are refused with QR_ERR_STATE"""
    import torch
    ctx = qr.Context(0)
    g, f, desc, params = _scene(qr, 100, 64)
    sid = ctx.upload(desc)
    g2, f2, desc2, params2 = _scene(qr, 64, 100, seed=5)
    sid2 = ctx.upload(desc2)
    frame = torch.zeros((128, 128), dtype=torch.int32, device="cuda")
    p = qr.QrFrameParams.from_buffer_copy(params)
    p.pt_on, p.pts_c, p.seed = 2, 2.0, 3
    # nothing started for this scene yet (other tests may have started sums
    # for other scenes or contexts)
    assert _noalloc(qr, ctx, sid, p, frame.data_ptr()) == qr.QR_ERR_STATE
    assert "pts_c == 0" in ctx.error()
    p.pts_c = 0.0
    assert _noalloc(qr, ctx, sid, p, frame.data_ptr()) == qr.QR_OK
    torch.cuda.synchronize()
    # same pixel count, other shape and scene: refused
    p2 = qr.QrFrameParams.from_buffer_copy(params2)
    p2.pt_on, p2.pts_c, p2.seed = 2, 2.0, 3
    assert p2.x_row * p2.y_res == p.x_row * p.y_res
    assert _noalloc(qr, ctx, sid2, p2, frame.data_ptr()) == qr.QR_ERR_STATE
    # the started scene and shape: accepted
    p.pts_c = 2.0
    assert _noalloc(qr, ctx, sid, p, frame.data_ptr()) == qr.QR_OK
    torch.cuda.synchronize()
    ctx.close()
