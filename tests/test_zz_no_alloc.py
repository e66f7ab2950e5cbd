"""qr_render_pt_noalloc: the path tracer with its running sums in the
library's fixed device array, against qr_render_pt with caller-owned sums.

Collected last (file name), and independent of the other tests: it passes
alone and after them.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scene(qr, w, h):
    g = qr.GenScene(qr.SCN_PT, 4, 32, 0)
    f = qr.Flat(g, w, h, 0)
    desc, params = f.update(0, 8)
    return g, f, desc, params


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
        rc = qr.lib().qr_render_pt_noalloc(ctx.h, sid, ctypes.byref(p),
                                           ctypes.c_void_p(fb.data_ptr()),
                                           ctypes.c_void_p(stream))
        assert rc == qr.QR_OK, ctx.error()
        torch.cuda.synchronize()
        assert torch.equal(fa, fb), call
        assert int((fb != 0).sum()) > 0
    ctx.close()


def test_noalloc_rejects_oversize_frame(qr):
    ctx = qr.Context(0)
    g, f, desc, params = _scene(qr, 1920, 1080)
    sid = ctx.upload(desc)
    params.pt_on, params.pts_c = 1, 0.0
    rc = qr.lib().qr_render_pt_noalloc(ctx.h, sid, ctypes.byref(params),
                                       ctypes.c_void_p(16), None)
    assert rc == 7                      # QR_ERR_LIMIT
    assert "exceeds" in ctx.error()
    ctx.close()


def test_noalloc_needs_started_sums(qr):
    import torch
    ctx = qr.Context(0)
    g, f, desc, params = _scene(qr, 100, 61)
    sid = ctx.upload(desc)
    frame = torch.zeros((params.y_res, params.x_row), dtype=torch.int32, device="cuda")
    params.pt_on, params.pts_c = 2, 2.0
    rc = qr.lib().qr_render_pt_noalloc(ctx.h, sid, ctypes.byref(params),
                                       ctypes.c_void_p(frame.data_ptr()), None)
    assert rc == 5                      # QR_ERR_STATE
    assert "pts_c == 0" in ctx.error()
    ctx.close()
