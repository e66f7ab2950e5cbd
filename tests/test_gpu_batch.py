"""Batched persistent rendering (qr_batch_*): every frame of a batch of
mixed requests (Whitted and path-traced, several scenes and sizes) is the
frame of the same request rendered alone, bit for bit, whatever the tile
configuration."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [  # kind, seed, nq, w, h, fsaa, depth, spp
    (1, 11, 8, 64, 48, 0, 3, 0), (1, 12, 40, 100, 75, 2, 6, 0),
    (2, 13, 64, 96, 54, 0, 4, 0), (3, 14, 16, 80, 45, 0, 8, 4),
    (3, 15, 32, 48, 36, 0, 8, 12), (1, 16, 120, 33, 17, 0, 1, 0),
    (2, 17, 64, 50, 30, 1, 4, 0),
]


def _setup(qr, ctx):
    import torch
    reqs, keep, bufs = [], [], []
    for i, (kind, seed, nq, w, h, fsaa, depth, spp) in enumerate(CASES):
        g = qr.GenScene(kind, seed, nq, 0)
        f = qr.Flat(g, w, h, fsaa)
        desc, params = f.update(16 * i, depth)
        sid = ctx.upload(desc)
        keep.append((g, f))
        r = qr.QrRequest()
        r.scene_id = sid
        r.fp = params
        r.fp.pt_on, r.fp.pts_c, r.fp.seed, r.fp.frame_idx = spp, 0.0, 100 + i, 0
        fr = torch.zeros((h, params.x_row), dtype=torch.int32, device="cuda")
        acc = torch.zeros((h, params.x_row, 3), dtype=torch.float32, device="cuda")
        r.dev_frame = fr.data_ptr()
        r.dev_acc = acc.data_ptr() if spp else None
        bufs.append((fr, acc))
        reqs.append(r)
    return reqs, keep, bufs


def _alone(qr, ctx, r):
    return ctx.render_host(r.scene_id, r.fp)


def test_batch_frames_equal_single_frames(qr):
    import torch
    ctx = qr.Context(0)
    reqs, keep, bufs = _setup(qr, ctx)
    alone = [_alone(qr, ctx, r).copy() for r in reqs]
    b = qr.Batch(ctx, 16)
    b.set(reqs)
    for tw, grab, persistent in [(8, 1, 1), (16, 4, 1), (32, 1, 1), (4, 2, 1), (8, 1, 0),
                                 (16, 4, 0)]:
        for fr, _ in bufs:
            fr.zero_()
        b.config(tw, grab)
        b.persistent(persistent)
        b.launch(torch.cuda.current_stream().cuda_stream)
        b.wait()
        for i, (fr, _) in enumerate(bufs):
            got = fr.cpu().numpy().view(np.uint32)[:, :reqs[i].fp.x_res]
            assert (got != alone[i]).sum() == 0, (tw, grab, persistent, i)
    b.persistent(1)
    tw, grab, ms = b.tune()
    assert tw in (4, 8, 16, 32) and grab >= 1 and ms > 0
    b.launch(0)
    while not b.poll():
        pass
    for i, (fr, _) in enumerate(bufs):
        got = fr.cpu().numpy().view(np.uint32)[:, :reqs[i].fp.x_res]
        assert (got != alone[i]).sum() == 0, ("tuned", i)
    b.close()
    ctx.close()


def test_batch_rejects_bad_requests(qr):
    ctx = qr.Context(0)
    g = qr.GenScene(qr.SCN_PT, 1, 8, 0)
    f = qr.Flat(g, 32, 24, 0)
    desc, params = f.update(0, 8)
    sid = ctx.upload(desc)
    b = qr.Batch(ctx, 2)
    r = qr.QrRequest()
    r.scene_id = sid
    r.fp = params
    r.fp.pt_on = 4
    r.dev_frame = 256
    r.dev_acc = None                      # path tracer without sums
    with pytest.raises(RuntimeError):
        b.set([r])
    r.scene_id = 99                       # unknown scene
    with pytest.raises(RuntimeError):
        b.set([r])
    with pytest.raises(RuntimeError):     # more requests than the batch holds
        b.set([r, r, r])
    b.close()
    ctx.close()


def test_request_completion_flags(qr):
    """A request's completion word turns 1 once its frame is complete, while
    the rest of the batch may still run: the first request (a small Whitted
    frame) is read back as soon as its word is set, on another stream than
    the batch's, and must equal the frame rendered alone; after the batch
    every word is 1 and every frame equals its frame alone."""
    import time
    import torch
    ctx = qr.Context(0)
    cases = [(1, 21, 16, 64, 48, 0, 4, 0)] + [(3, 22 + i, 32, 320, 240, 0, 8, 64)
                                             for i in range(3)]
    reqs, keep, bufs = [], [], []
    for i, (kind, seed, nq, w, h, fsaa, depth, spp) in enumerate(cases):
        g = qr.GenScene(kind, seed, nq, 0)
        f = qr.Flat(g, w, h, fsaa)
        desc, params = f.update(0, depth)
        sid = ctx.upload(desc)
        keep.append((g, f))
        r = qr.QrRequest()
        r.scene_id = sid
        r.fp = params
        r.fp.pt_on, r.fp.pts_c, r.fp.seed, r.fp.frame_idx = spp, 0.0, 300 + i, 0
        fr = torch.zeros((h, params.x_row), dtype=torch.int32, device="cuda")
        acc = torch.zeros((h, params.x_row, 3), dtype=torch.float32, device="cuda")
        r.dev_frame = fr.data_ptr()
        r.dev_acc = acc.data_ptr() if spp else None
        bufs.append((fr, acc))
        reqs.append(r)
    alone = [ctx.render_host(r.scene_id, r.fp).copy() for r in reqs]
    torch.cuda.synchronize()
    b = qr.Batch(ctx, len(reqs))
    b.set(reqs)
    side = torch.cuda.Stream()
    b.launch(side.cuda_stream)
    flags = b.done_flags(len(reqs))
    t_end = time.monotonic() + 120.0
    while flags[0] != 1 and time.monotonic() < t_end:
        time.sleep(0.0002)
    assert flags[0] == 1
    other = torch.cuda.Stream()
    with torch.cuda.stream(other):
        early = bufs[0][0].to("cpu", non_blocking=False)
    got = early.numpy().view(np.uint32)[:, :reqs[0].fp.x_res]
    assert (got != alone[0]).sum() == 0
    b.wait()
    assert list(flags) == [1] * len(reqs)
    for i, (fr, _) in enumerate(bufs):
        got = fr.cpu().numpy().view(np.uint32)[:, :reqs[i].fp.x_res]
        assert (got != alone[i]).sum() == 0, i
    b.close()
    ctx.close()
