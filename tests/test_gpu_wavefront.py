"""The wavefront path tracer (queues per tree level, warp-vote compaction)
against the per-pixel kernel and the oracle, bit for bit.

Both CUDA forms and the oracle draw counter-based random numbers keyed by
(seed, frame, pixel, sample, tree node, purpose), so the wavefront's
breadth-first evaluation gives the depth-first frame exactly: frame and
running sums are compared as bits.  Chunked frames (more paths than a chunk
holds) and frames whose queues overflow (and are rendered by the per-pixel
kernel instead) must give the same bits too.
"""
import os

import numpy as np
import pytest

from conftest import oracle_pt_par

pytestmark = pytest.mark.gpu


def _ctx(qr, caps=None):
    old = os.environ.get("QR_WF_CAPS")
    if caps:
        os.environ["QR_WF_CAPS"] = caps
    else:
        os.environ.pop("QR_WF_CAPS", None)
    try:
        return qr.Context(0)
    finally:
        if old is None:
            os.environ.pop("QR_WF_CAPS", None)
        else:
            os.environ["QR_WF_CAPS"] = old


def _render(qr, ctx, sid, params, launches, pixel):
    """launches of params.pt_on samples each (accumulating); returns the
    frame and sums after each"""
    import torch
    fr = torch.zeros((params.y_res, params.x_row), dtype=torch.int32, device="cuda")
    acc = torch.zeros((params.y_res, params.x_row, 3), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    out = []
    for k in range(launches):
        p = qr.QrFrameParams.from_buffer_copy(params)
        p.pts_c = float(k * params.pt_on)
        p.frame_idx = 3
        if pixel:
            p.flags = p.flags | qr.FP_PIXEL_PT
        ctx.render_pt(sid, p, acc.data_ptr(), fr.data_ptr(), stream)
        torch.cuda.synchronize()
        out.append((fr.cpu().numpy().view(np.uint32)[:, :params.x_res].copy(),
                    acc.cpu().numpy()[:, :params.x_res].copy()))
    return out


CASES = [  # kind, seed, nq, w, h, depth, spp, launches
    (3, 1, 32, 160, 90, 8, 8, 2),
    (3, 2, 32, 97, 61, 8, 33, 1),       # ragged, the single-loop form's range
    (3, 3, 64, 128, 72, 10, 4, 3),      # depth 10: three children a node
    (1, 4, 16, 120, 80, 6, 6, 1),       # plain scene (no emitter: black frame)
    (2, 5, 64, 96, 54, 4, 5, 1),        # animated scene: clippers, booleans (no
                                        # emitter: black frame)
]


@pytest.mark.parametrize("kind,seed,nq,w,h,depth,spp,launches", CASES)
def test_wavefront_equals_pixel_kernel(qr, kind, seed, nq, w, h, depth, spp, launches):
    ctx = _ctx(qr)
    g = qr.GenScene(kind, seed, nq, 0)
    f = qr.Flat(g, w, h, 0)
    desc, params = f.update(0, depth)
    params.pt_on, params.seed = spp, 77
    sid = ctx.upload(desc)
    a = _render(qr, ctx, sid, params, launches, pixel=False)
    b = _render(qr, ctx, sid, params, launches, pixel=True)
    for k, ((fa, sa), (fb, sb)) in enumerate(zip(a, b)):
        assert (fa != fb).sum() == 0, k
        assert np.array_equal(sa.view(np.uint32), sb.view(np.uint32)), k
    if kind == 3:
        assert (a[-1][0] != 0).mean() > 0.2
    assert ctx.fault() == (0, 0, 0, 0)
    ctx.close()


def test_wavefront_equals_oracle(qr, oracle):
    ctx = _ctx(qr)
    g = qr.GenScene(qr.SCN_PT, 6, 32, 0)
    f = qr.Flat(g, 200, 120, 0)
    desc, params = f.update(0, 8)
    params.pt_on, params.seed, params.frame_idx, params.pts_c = 12, 9, 0, 0.0
    sid = ctx.upload(desc)
    (fa, sa), = _render(qr, ctx, sid, params, 1, pixel=False)
    p = qr.QrFrameParams.from_buffer_copy(params)
    p.frame_idx = 3
    cf, ca = oracle_pt_par(oracle, desc, p, 0, p.y_res)
    assert (fa != cf).sum() == 0
    assert np.array_equal(sa.view(np.uint32), ca.view(np.uint32))
    ctx.close()


@pytest.mark.parametrize("caps", ["1000,2,8", "64,2,8", "4096,1,2", "512,1,1"])
def test_wavefront_chunks_and_overflow(qr, caps):
    """small chunks (many chunks a frame, chunk boundaries inside a pixel's
    samples) and capacities too small for the trees (the queues overflow and
    the frame falls back to the per-pixel kernel): the same bits"""
    ctx = _ctx(qr, caps)
    g = qr.GenScene(qr.SCN_PT, 7, 32, 0)
    f = qr.Flat(g, 72, 40, 0)
    desc, params = f.update(0, 8)
    params.pt_on, params.seed = 7, 5
    sid = ctx.upload(desc)
    a = _render(qr, ctx, sid, params, 2, pixel=False)
    b = _render(qr, ctx, sid, params, 2, pixel=True)
    for (fa, sa), (fb, sb) in zip(a, b):
        assert (fa != fb).sum() == 0
        assert np.array_equal(sa.view(np.uint32), sb.view(np.uint32))
    ctx.close()


def test_wavefront_two_streams(qr):
    """frames of one context on two streams take turns on the scratch: both
    equal their frames rendered alone"""
    import torch
    ctx = _ctx(qr)
    g = qr.GenScene(qr.SCN_PT, 8, 32, 0)
    f = qr.Flat(g, 160, 96, 0)
    desc, params = f.update(0, 8)
    params.pt_on, params.seed, params.pts_c = 6, 2, 0.0
    sid = ctx.upload(desc)
    ref = _render(qr, ctx, sid, params, 1, pixel=True)[0]
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    outs = []
    for s in (s1, s2, s1, s2):
        fr = torch.zeros((params.y_res, params.x_row), dtype=torch.int32, device="cuda")
        acc = torch.zeros((params.y_res, params.x_row, 3), dtype=torch.float32, device="cuda")
        p = qr.QrFrameParams.from_buffer_copy(params)
        p.frame_idx = 3
        ctx.render_pt(sid, p, acc.data_ptr(), fr.data_ptr(), s.cuda_stream)
        outs.append((fr, acc))
    torch.cuda.synchronize()
    for fr, acc in outs:
        assert (fr.cpu().numpy().view(np.uint32)[:, :params.x_res] != ref[0]).sum() == 0
        assert np.array_equal(acc.cpu().numpy()[:, :params.x_res].view(np.uint32),
                              ref[1].view(np.uint32))
    ctx.close()
