"""Frame server (quadray-engine_gb300/serve.py): continuous batching of mixed
requests gives, for every request, the frame it gets when rendered alone;
admission by the HBM budget delays requests without changing them."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SCENES = [  # kind, seed, nq, flags, depth
    (1, 31, 16, 1 << 4, 10), (1, 32, 40, 1 << 4, 10), (1, 33, 100, 1 << 4, 10),
    (3, 34, 16, 0, 8),
]
SIZES = [(64, 48), (96, 54), (128, 72)]


def _server(qr, ctx, budget, max_batch, device_anim=False, urgent=None):
    serve = importlib.import_module("quadray-engine_gb300.serve")
    scenes = [dict(gen=qr.GenScene(k, s, n, f), pt=(k == 3), depth=d,
                   anim=bool(f & qr.GEN_SPIN))
              for (k, s, n, f, d) in SCENES]
    return serve, serve.Server(qr, ctx, scenes, budget_bytes=budget, max_batch=max_batch,
                               prep_threads=3, device_anim=device_anim, urgent=urgent)


def _alone(qr, ctx, req):
    kind, seed, nq, flags, depth = SCENES[req.scene]
    pt = kind == 3
    fsaa = 0 if (pt or req.spp <= 1) else 2
    g = qr.GenScene(kind, seed, nq, flags)
    f = qr.Flat(g, req.w, req.h, fsaa)
    desc, params = f.update(req.time, depth)
    sid = ctx.upload(desc)
    p = qr.QrFrameParams.from_buffer_copy(params)
    p.x_row = req.w
    if pt:
        p.pt_on, p.pts_c, p.seed, p.frame_idx = req.spp, 0.0, 0x5E, req.rid
    return ctx.render_host(sid, p).copy()


def _requests(serve, n, seed):
    rng = np.random.default_rng(seed)
    out, nxt = [], [0] * len(SCENES)
    for i in range(n):
        s = int(rng.integers(0, len(SCENES)))
        w, h = SIZES[int(rng.integers(0, len(SIZES)))]
        spp = int(rng.integers(1, 6))
        out.append(serve.Request(i, s, 16 * nxt[s], w, h, spp, 0.002 * i))
        nxt[s] += 1
    return out


@pytest.mark.parametrize("budget,max_batch,device_anim,urgent", [
    (120 << 30, 6, False, False), (3 << 20, 4, False, False), (120 << 30, 6, True, False),
    (3 << 20, 4, True, False), (120 << 30, 6, True, True)])
def test_served_frames_equal_frames_alone(qr, budget, max_batch, device_anim, urgent):
    """device_anim: spinning scenes whose copies were prepared for it are
    updated on the device (qr_scene_anim_update on the serving stream);
    urgent: the largest frames go into batches of their own on a stream of
    high priority, overlapping the others on the device"""
    ctx = qr.Context(0)
    serve, srv = _server(qr, ctx, budget, max_batch, device_anim,
                         (lambda r: r.w == 128) if urgent else None)
    reqs = _requests(serve, 28, 7)
    done, wall = srv.run(reqs, keep_frames=True)
    if device_anim:
        assert srv.device_updates > 0
    assert len(done) == len(reqs)
    assert all(r.done >= r.arrival for r in done)
    for r in sorted(done, key=lambda r: r.rid):
        got = r.frame.cpu().numpy().view(np.uint32)
        ref = _alone(qr, ctx, r)
        assert (got != ref).sum() == 0, (r.rid, r.scene, r.w, r.h, r.spp)
    srv.close()
    ctx.close()


def test_budget_bounds_memory_in_flight(qr):
    """with a budget that holds one request at a time, requests still all
    complete, in arrival order"""
    ctx = qr.Context(0)
    serve, srv = _server(qr, ctx, 1 << 20, 8)
    reqs = [serve.Request(i, 0, 16 * i, 64, 48, 1, 0.0) for i in range(6)]
    srv.budget = 64 * 48 * 4 + (1 << 20)
    done, wall = srv.run(reqs, keep_frames=False)
    assert [r.rid for r in done] == list(range(6))
    srv.close()
    ctx.close()
