"""Device-side update phases (qr_scene_anim_*): a scene whose animators run
on the host and whose transforms, inverse matrices, surface boxes and
hierarchy are updated by the device gives, frame after frame, the same
frame bit for bit as the same scene updated by the host phases and
uploaded, as the in-order list walk over the device-updated records, and as
the reference's own frames of the golden fixtures."""
import ctypes

import pytest

from conftest import oracle_render

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(qr):
    c = qr.Context(0)
    yield c
    c.close()


def _copy(qr, params):
    return qr.QrFrameParams.from_buffer_copy(params)


def _device_scene(qr, ctx, kind, seed, nq, flags, w, h, fsaa, depth, bound=None,
                  fresh=False):
    """fresh: a new scene prepared in one call (qr_scene_anim_upload), else a
    resident scene prepared in place (qr_scene_anim_init)"""
    g = qr.GenScene(kind, seed, nq, flags)
    f = qr.Flat(g, w, h, fsaa)
    desc, params = f.update(0, depth)
    fp = _copy(qr, params)
    if fresh:
        sid = ctx.anim_upload(desc, f.anim_table(), bound)
    else:
        sid = ctx.upload(desc)
        ctx.anim_init(sid, desc, f.anim_table(), bound)
    return g, f, sid, fp


@pytest.mark.parametrize("kind,seed,nq,flags,fsaa", [
    (2, 1, 64, 0, 0),           # spinning 3-level hierarchy, every surface a node
    (2, 2, 64, 8, 2),           # array-level transform nodes (TARRAY), 4x AA
    (2, 6, 64, 512, 0),         # the reference's default of no Fresnel terms
    (2, 4, 256, 0, 0),          # 256 quadrics: outer hierarchy levels in use
    (1, 3, 32, 16, 0),          # spinning quadrics of the plain scene
])
def test_device_update_equals_host_update(qr, oracle, ctx, kind, seed, nq, flags, fsaa):
    w, h, depth = 192, 108, 4
    g, f, sid, fp = _device_scene(qr, ctx, kind, seed, nq, flags, w, h, fsaa, depth)
    g2 = qr.GenScene(kind, seed, nq, flags)
    f2 = qr.Flat(g2, w, h, fsaa)
    hid = None
    times = [16, 32, 48, 16 * 40, 16 * 97]
    for k, t in enumerate(times):
        rc, p = f.anim_params(t)
        assert rc == 0
        ctx.anim_update(sid, p)
        dev = ctx.render_host(sid, fp).copy()
        desc2, params2 = f2.update(t, depth)
        if hid is None:
            hid = ctx.upload(desc2)
        else:
            ctx.update(hid, desc2)
        host = ctx.render_host(hid, params2)
        assert (dev != host).sum() == 0, (t, int((dev != host).sum()))
        lin = _copy(qr, fp)
        lin.flags |= qr.FP_LINEAR_WALK
        walk = ctx.render_host(sid, lin)
        assert (dev != walk).sum() == 0, t
        if k == 1:
            cpu, _ = oracle_render(oracle, desc2, params2)
            assert (dev != cpu).sum() == 0, t
    assert ctx.anim_status(sid) == (len(times), 0)
    ctx.release(sid)
    ctx.release(hid)


def test_device_update_outside_bound_stays_exact(qr, ctx):
    """a motion bound no larger than the first frame's extent: spinning
    surfaces leave it, the update opens the hierarchy's boxes for those
    frames (counted), and the frames still equal the host's"""
    kind, seed, nq, flags, w, h, depth = 2, 3, 64, 0, 160, 90, 4
    g, f, sid, fp = _device_scene(qr, ctx, kind, seed, nq, flags, w, h, 0, depth,
                                  bound=[0.0] * 6)
    g2 = qr.GenScene(kind, seed, nq, flags)
    f2 = qr.Flat(g2, w, h, 0)
    hid = None
    times = [16 * 25 * k for k in range(1, 7)]
    for t in times:
        rc, p = f.anim_params(t)
        assert rc == 0
        ctx.anim_update(sid, p)
        dev = ctx.render_host(sid, fp).copy()
        desc2, params2 = f2.update(t, depth)
        if hid is None:
            hid = ctx.upload(desc2)
        else:
            ctx.update(hid, desc2)
        host = ctx.render_host(hid, params2)
        assert (dev != host).sum() == 0, t
    frames, missed = ctx.anim_status(sid)
    assert frames == len(times) and missed >= 1
    ctx.release(sid)
    ctx.release(hid)


def test_moving_transforms_leave_the_bound_and_stay_exact(qr, ctx):
    """quadrics that rise (their animators move the transforms): positions
    come from the animators' parameters, and once the risen surfaces leave
    the default bound (rotations about fixed origins) the updates open the
    hierarchy, count the misses, and the frames still equal the host's"""
    w, h, depth = 160, 96, 4
    g, f, sid, fp = _device_scene(qr, ctx, qr.SCN_PLAIN, 11, 24, qr.GEN_RISE, w, h, 0, depth)
    g2 = qr.GenScene(qr.SCN_PLAIN, 11, 24, qr.GEN_RISE)
    f2 = qr.Flat(g2, w, h, 0)
    f2.update(0, depth)
    hid = None
    times = [16, 160, 1600, 4000, 8000]
    for t in times:
        rc, p = f.anim_params(t)
        assert rc == 0
        ctx.anim_update(sid, p)
        dev = ctx.render_host(sid, fp).copy()
        desc2, params2 = f2.update(t, depth)
        if hid is None:
            hid = ctx.upload(desc2)
        else:
            ctx.update(hid, desc2)
        host = ctx.render_host(hid, params2)
        assert (dev != host).sum() == 0, t
    frames, missed = ctx.anim_status(sid)
    assert frames == len(times) and 1 <= missed < len(times)
    ctx.release(sid)
    ctx.release(hid)


def test_device_update_matches_reference_frames(qr, ctx):
    """the reference's own frames of the golden fixtures with animated
    objects (the animated hierarchy, spinning plain quadrics; no camera
    actions), every frame after the first updated on the device"""
    from test_oracle_golden import EXACT, load_golden, check_against_golden, flatten_case
    import os
    done = 0
    for path in EXACT:
        frames, meta = load_golden(path)
        if meta["frames"] < 2 or meta.get("actions") or meta.get("nextcam"):
            continue
        g, f, desc, params = flatten_case(qr, meta, 0)
        table = f.anim_table()
        if len(table) == 0:
            continue
        fp = _copy(qr, params)
        sid = ctx.upload(desc)
        ctx.anim_init(sid, desc, table)
        for k in range(meta["frames"]):
            if k > 0:
                rc, p = f.anim_params(16 * k)
                assert rc == 0
                ctx.anim_update(sid, p)
            img = ctx.render_host(sid, fp)
            mask = None
            if meta["flags"] & 1:
                from conftest import boundary_mask
                _, _, dk, pk = flatten_case(qr, meta, 16 * k)
                mask = boundary_mask(dk, pk)
            check_against_golden(img, frames[k], meta, mask)
        ctx.release(sid)
        done += 1
    assert done >= 4, os.listdir(os.path.dirname(path))


def test_device_update_on_a_stream_and_in_a_batch(qr, ctx):
    """the updates of several scenes in one launch on a caller's stream,
    ahead of a batched render of them: each frame equals its host-updated
    one"""
    import numpy as np
    import torch
    w, h, depth = 128, 72, 4
    s = torch.cuda.Stream()
    scenes = []
    for seed in (1, 2, 3):
        g, f, sid, fp = _device_scene(qr, ctx, qr.SCN_ANIM, seed, 64, 0, w, h, 0, depth,
                                      fresh=True)
        scenes.append((g, f, sid, fp))
    b = qr.Batch(ctx, len(scenes))
    with pytest.raises(RuntimeError):       # one scene twice in one launch
        ctx.anim_update_many([(scenes[0][2], scenes[0][1].anim_params(16)[1])] * 2)
    for t in (48, 160):
        outs, reqs, ups = [], [], []
        for g, f, sid, fp in scenes:
            rc, p = f.anim_params(t)
            assert rc == 0
            ups.append((sid, p))
            out = torch.empty((h, w), dtype=torch.int32, device="cuda")
            q = qr.QrRequest()
            q.scene_id = sid
            q.fp = fp
            q.dev_frame = out.data_ptr()
            q.dev_acc = None
            reqs.append(q)
            outs.append(out)
        ctx.anim_update_many(ups, s.cuda_stream)     # one launch, a block a scene
        b.set(reqs)
        b.launch(s.cuda_stream)
        s.synchronize()
        for (g, f, sid, fp), out in zip(scenes, outs):
            g2 = qr.GenScene(qr.SCN_ANIM, g.seed, 64, 0)
            f2 = qr.Flat(g2, w, h, 0)
            desc2, params2 = f2.update(t, depth)
            hid = ctx.upload(desc2)
            host = ctx.render_host(hid, params2)
            dev = out.cpu().numpy().view(np.uint32)
            assert (dev != host).sum() == 0, (g.seed, t)
            ctx.release(hid)
    b.close()
    for g, f, sid, fp in scenes:
        ctx.release(sid)


@pytest.mark.parametrize("kind,seed,nq,flags,fsaa", [(2, 7, 64, 0, 2), (1, 5, 32, 16, 0),
                                                     (2, 8, 64, 8, 0), (1, 9, 24, 0, 0),
                                                     (1, 13, 24, 1 << 12, 0)])
def test_engine_renders_with_device_updates(qr, kind, seed, nq, flags, fsaa):
    """rt_Scene::render with device updates (the default) against the host
    update phases every frame: 40 frames (past a periodic host rebuild),
    with camera actions and a camera switch between renders; a static scene
    (uploaded once, only its camera refreshed) and one whose transforms move
    too"""
    a = qr.Engine(qr.GenScene(kind, seed, nq, flags), 160, 90, fsaa=fsaa, depth=4)
    b = qr.Engine(qr.GenScene(kind, seed, nq, flags), 160, 90, fsaa=fsaa, depth=4)
    b.set_device_update(False)
    for k in range(40):
        if k % 7 == 3:
            act = (qr.CAMERA_MOVE_FORWARD, qr.CAMERA_ROTATE_LEFT, qr.CAMERA_MOVE_UP)[k % 3]
            a.update(16 * k, act)
            b.update(16 * k, act)
        if k == 20:
            a.next_cam()
            b.next_cam()
        fa = a.render(16 * k).copy()
        fb = b.render(16 * k).copy()
        assert (fa != fb).sum() == 0, k
    a.close()
    b.close()


def test_malformed_tables_and_updates_are_refused(qr, ctx):
    """the table's indices are checked before anything is uploaded: parents
    earlier and carrying a record, records and lights in range and named
    once; an update gives exactly the table's animated transforms"""
    g = qr.GenScene(qr.SCN_ANIM, 2, 64, 0)
    f = qr.Flat(g, 64, 36, 0)
    desc, params = f.update(0, 4)
    table = f.anim_table()
    sid = ctx.upload(desc)
    n = len(table)
    under = next(i for i, e in enumerate(table) if e.parent >= 0)

    def refused(mutate):
        bad = (qr.QrAnimNode * n)()
        ctypes.memmove(bad, table, ctypes.sizeof(bad))
        mutate(bad)
        with pytest.raises(RuntimeError):
            ctx.anim_init(sid, desc, bad)

    refused(lambda t: setattr(t[under], "parent", under))            # not earlier
    refused(lambda t: setattr(t[table[under].parent], "rec", -1))    # parent without record
    refused(lambda t: setattr(t[1], "rec", t[0].rec))                # record named twice
    refused(lambda t: setattr(t[0], "rec", desc.nsrf))               # out of range
    refused(lambda t: setattr(t[0], "kind", 7))                      # unknown recipe
    with pytest.raises(RuntimeError):
        ctx.anim_init(sid, desc, table, bound=[1, 0, 0, 0, 0, 0])     # lo above hi
    ctx.anim_init(sid, desc, table)
    rc, p = f.anim_params(16)
    with pytest.raises(RuntimeError):
        ctx.anim_update(sid, (qr.QrAnimParam * (len(p) - 1))())       # too few transforms
    ctx.anim_update(sid, p)
    assert ctx.anim_status(sid) == (1, 0)
    ctx.release(sid)


@pytest.mark.parametrize("seed,nq", [(1, 32), (4, 96)])
def test_device_update_path_traced_equals_host_update(qr, ctx, seed, nq):
    """the path tracer's tracing stage walks the 4-wide records, which the
    device update refits after the nodes: path-traced frames of the closed
    box with spinning quadrics, updated on the device, equal those of the
    host-updated scene, and those of the per-pixel kernel (which walks the
    binary records)"""
    import torch
    w, h, depth = 96, 54, 6
    g, f, sid, fp = _device_scene(qr, ctx, qr.SCN_PT, seed, nq, qr.GEN_SPIN, w, h, 0, depth)
    g2 = qr.GenScene(qr.SCN_PT, seed, nq, qr.GEN_SPIN)
    f2 = qr.Flat(g2, w, h, 0)
    hid = None
    sp = torch.cuda.current_stream().cuda_stream

    def pt(scene, params, flags=0):
        p = _copy(qr, params)
        p.pt_on, p.pts_c, p.seed, p.frame_idx = 16, 0.0, 9, 0
        p.flags |= flags
        acc = torch.zeros((p.y_res, p.x_row, 3), dtype=torch.float32, device="cuda")
        fr = torch.zeros((p.y_res, p.x_row), dtype=torch.int32, device="cuda")
        ctx.render_pt(scene, p, acc.data_ptr(), fr.data_ptr(), sp)
        torch.cuda.synchronize()
        return fr.cpu().numpy(), acc.cpu().numpy()

    for t in [16, 16 * 40, 16 * 97]:
        rc, p = f.anim_params(t)
        assert rc == 0
        ctx.anim_update(sid, p)
        dev, dacc = pt(sid, fp)
        desc2, params2 = f2.update(t, depth)
        if hid is None:
            hid = ctx.upload(desc2)
        else:
            ctx.update(hid, desc2)
        host, hacc = pt(hid, params2)
        assert (dev != host).sum() == 0 and (dacc != hacc).sum() == 0, t
        pix, pacc = pt(sid, fp, qr.FP_PIXEL_PT)
        assert (dev != pix).sum() == 0 and (dacc != pacc).sum() == 0, t
        assert (dev != 0).mean() > 0.05       # 16 samples: a noisy, not a black frame
    ctx.release(sid)
    ctx.release(hid)
