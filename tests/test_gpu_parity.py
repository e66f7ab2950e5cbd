"""GPU tracer vs the CPU oracle, bit for bit, through the C ABI.

The oracle restates the reference's fp32 tracer and is pinned against the
reference's own frames (test_oracle_golden.py); here the CUDA kernel must
reproduce the oracle exactly (hit IDs and 8-bit colour) on the same
flattened scene.
"""
import numpy as np
import pytest

from conftest import oracle_render

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(qr):
    c = qr.Context(0)
    yield c
    c.close()


def _render_both(qr, oracle, ctx, kind, seed, nq, w, h, fsaa=0, flags=0, depth=10, t=0):
    g = qr.GenScene(kind, seed, nq, flags)
    f = qr.Flat(g, w, h, fsaa)
    desc, params = f.update(t, depth)
    sid = ctx.upload(desc)
    gpu = ctx.render_host(sid, params)
    cpu, _ = oracle_render(oracle, desc, params)
    return gpu, cpu


@pytest.mark.parametrize("seed", [1, 2, 3, 4, 5])
def test_plain_bit_exact(qr, oracle, ctx, seed):
    gpu, cpu = _render_both(qr, oracle, ctx, qr.SCN_PLAIN, seed, 16, 320, 192)
    assert (gpu != cpu).sum() == 0


@pytest.mark.parametrize("seed", [1, 6])
def test_plain_ids_bit_exact(qr, oracle, ctx, seed):
    gpu, cpu = _render_both(qr, oracle, ctx, qr.SCN_PLAIN, seed, 16, 320, 192,
                            flags=qr.GEN_IDS)
    assert (gpu != cpu).sum() == 0


@pytest.mark.parametrize("fsaa,w,h", [(2, 200, 120), (1, 200, 120), (1, 37, 23)])
def test_plain_aa_bit_exact(qr, oracle, ctx, fsaa, w, h):
    """4x rotated grid (fsaa 2) and 2x alternating (fsaa 1), on an odd
    width too (the 2x offsets follow the column's parity)"""
    gpu, cpu = _render_both(qr, oracle, ctx, qr.SCN_PLAIN, 3, 16, w, h, fsaa=fsaa)
    assert (gpu != cpu).sum() == 0


@pytest.mark.parametrize("seed,fsaa,flags", [(7, 0, 32), (11, 2, 32), (9, 0, 64), (10, 2, 96),
                                             (17, 0, 256), (19, 2, 480)])
def test_textured_and_gamma_bit_exact(qr, oracle, ctx, seed, fsaa, flags):
    """bound texel arrays on the ground and on scaled, rotated walls (side
    scales of either sign, rotations, offsets), the reference's gamma mode
    (texels squared, square root before packing), and lights with an
    ambient share and constant, linear and quadratic attenuation"""
    gpu, cpu = _render_both(qr, oracle, ctx, qr.SCN_PLAIN, seed, 16, 320, 192,
                            fsaa=fsaa, flags=flags)
    assert (gpu != cpu).sum() == 0


@pytest.mark.parametrize("seed,fsaa,flags", [(12, 0, 128), (13, 2, 128), (15, 0, 129),
                                             (16, 0, 128 | 32)])
def test_other_quadric_kinds_bit_exact(qr, oracle, ctx, seed, fsaa, flags):
    """paracylinder, hypercylinder, two planes (the two-plane solver), double
    cone (apex adjustment) and hyperbolic paraboloid, at right-angle and other
    rotations; colour and hit IDs"""
    gpu, cpu = _render_both(qr, oracle, ctx, qr.SCN_PLAIN, seed, 8, 320, 192,
                            fsaa=fsaa, flags=flags)
    assert (gpu != cpu).sum() == 0


def test_plain_full_size(qr, oracle, ctx):
    gpu, cpu = _render_both(qr, oracle, ctx, qr.SCN_PLAIN, 1, 16, 800, 480)
    assert (gpu != cpu).sum() == 0


def test_engine_api_matches_c_abi(qr, oracle):
    g = qr.GenScene(qr.SCN_PLAIN, 2, 16, 0)
    eng = qr.Engine(g, 256, 160)
    a = eng.render(0).copy()
    eng.close()
    g2 = qr.GenScene(qr.SCN_PLAIN, 2, 16, 0)
    f = qr.Flat(g2, 256, 160)
    desc, params = f.update(0, 10)
    cpu, _ = oracle_render(oracle, desc, params)
    assert (a != cpu).sum() == 0


@pytest.mark.parametrize("name", ["plain_s24_actions_160x96", "anim_s10_actions_128x72_d4",
                                  "plain_s25_cameras_160x96"])
def test_engine_camera_actions_match_reference(qr, name):
    """rt_Scene::update(time, action) and next_cam, then render(time), frame
    after frame, through the drop-in rt_Scene: the reference's own frames
    under the same camera actions (forward, rotate, up / rotate, back) and
    camera switches"""
    import os
    from test_oracle_golden import check_against_golden, load_golden
    frames, meta = load_golden(os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                            "golden", name + ".npz"))
    g = qr.GenScene(meta["kind"], meta["seed"], meta["nq"], meta["flags"])
    opts = qr.OPTS_NONE if meta["opts"] == "none" else qr.OPTS_DEFAULT
    eng = qr.Engine(g, meta["w"], meta["h"], fsaa=meta["fsaa"], opts=opts, depth=meta["depth"])
    acts = [int(x) for x in meta.get("actions", "").split(",") if x]
    cams = [int(x) for x in meta.get("nextcam", "").split(",") if x]
    for k in range(meta["frames"]):
        for c in cams:
            if c == k:
                eng.next_cam()
        if k > 0 and acts:
            eng.update(16 * k, acts[(k - 1) % len(acts)])
        img = eng.render(16 * k).copy()
        check_against_golden(img, frames[k], meta)
    eng.close()


def test_tiny_and_ragged_frames(qr, oracle, ctx):
    for (w, h) in [(1, 1), (7, 3), (33, 17), (129, 65)]:
        gpu, cpu = _render_both(qr, oracle, ctx, qr.SCN_PLAIN, 4, 16, w, h)
        assert (gpu != cpu).sum() == 0, (w, h)


# ---- animated scene: clippers, booleans, spinning hierarchy, secondary rays

@pytest.mark.parametrize("seed,fsaa,flags", [(1, 0, 0), (2, 2, 0), (3, 0, 0), (6, 2, 512),
                                             (9, 1, 0)])
def test_anim_bit_exact_over_frames(qr, oracle, ctx, seed, fsaa, flags):
    """animated frames; flags 512 keeps the reference's default of no
    Fresnel terms"""
    g = qr.GenScene(qr.SCN_ANIM, seed, 64, flags)
    f = qr.Flat(g, 192, 108, fsaa)
    for k in range(3):
        desc, params = f.update(16 * k, 4)
        sid = ctx.upload(desc)
        gpu = ctx.render_host(sid, params)
        cpu, _ = oracle_render(oracle, desc, params)
        assert (gpu != cpu).sum() == 0, (seed, fsaa, k)


def test_anim_scene_update_in_place(qr, oracle, ctx):
    """qr_scene_update replaces the records of a resident scene per frame."""
    g = qr.GenScene(qr.SCN_ANIM, 5, 64, 0)
    f = qr.Flat(g, 160, 90)
    desc, params = f.update(0, 4)
    sid = ctx.upload(desc)
    for k in range(1, 4):
        desc, params = f.update(16 * k, 4)
        ctx.update(sid, desc)
        gpu = ctx.render_host(sid, params)
        cpu, _ = oracle_render(oracle, desc, params)
        assert (gpu != cpu).sum() == 0, k


def test_anim_ids_bit_exact(qr, oracle, ctx):
    gpu, cpu = _render_both(qr, oracle, ctx, qr.SCN_ANIM, 6, 64, 240, 136,
                            flags=qr.GEN_IDS, depth=4)
    assert (gpu != cpu).sum() == 0


def test_anim_depth_10(qr, oracle, ctx):
    gpu, cpu = _render_both(qr, oracle, ctx, qr.SCN_ANIM, 7, 64, 160, 90, depth=10)
    assert (gpu != cpu).sum() == 0


def test_anim_full_size_frame_properties(qr, ctx):
    """1920x1080 4x AA: the frame is deterministic, animated frames differ,
    and a replayed frame is bit-identical (size-independent checks)."""
    g = qr.GenScene(qr.SCN_ANIM, 1, 64, 0)
    f = qr.Flat(g, 1920, 1080, 2)
    d0, p0 = f.update(0, 4)
    s0 = ctx.upload(d0)
    a = ctx.render_host(s0, p0).copy()
    b = ctx.render_host(s0, p0).copy()
    assert np.array_equal(a, b)
    d1, p1 = f.update(16, 4)
    s1 = ctx.upload(d1)
    c = ctx.render_host(s1, p1)
    assert (a != c).sum() > 0
    assert (a != 0).mean() > 0.5


# ---- the reference's own frames (tests/golden), through the GPU

def test_gpu_matches_reference_goldens(qr, ctx):
    from conftest import boundary_mask
    from test_oracle_golden import EXACT, load_golden, check_against_golden, frames_of
    for path in EXACT:
        frames, meta = load_golden(path)
        for k, (desc, params) in enumerate(frames_of(qr, meta)):
            sid = ctx.upload(desc)
            img = ctx.render_host(sid, params)
            mask = boundary_mask(desc, params) if meta["flags"] & 1 else None
            check_against_golden(img, frames[k], meta, mask)
            ctx.release(sid)


# ---- bounding-volume hierarchy: the same frames as the in-order list walk

@pytest.mark.parametrize("kind,seed,nq,w,h,fsaa,t,depth", [
    (2, 1, 64, 320, 180, 2, 0, 4), (2, 8, 64, 256, 144, 0, 48, 10),
    (2, 9, 128, 192, 108, 2, 32, 4), (1, 3, 16, 320, 192, 0, 0, 10),
    (1, 4, 64, 256, 160, 2, 0, 10)])
def test_bvh_equals_linear_walk(qr, ctx, kind, seed, nq, w, h, fsaa, t, depth):
    g = qr.GenScene(kind, seed, nq, 0)
    f = qr.Flat(g, w, h, fsaa)
    desc, params = f.update(t, depth)
    sid = ctx.upload(desc)
    a = ctx.render_host(sid, params).copy()
    lin = qr.QrFrameParams.from_buffer_copy(params)
    lin.flags = qr.FP_LINEAR_WALK
    b = ctx.render_host(sid, lin)
    assert (a != b).sum() == 0


def test_fault_word_clear_after_renders(qr, ctx):
    """Valid scenes never run past the per-pixel loop bounds: after device
    renders of every kind (Whitted at depth 10 with 4x AA, the animated scene,
    the path tracer at depth 10) the context's fault word holds zeros."""
    import torch
    stream = torch.cuda.current_stream().cuda_stream
    for kind, seed, nq, w, h, fsaa, depth, spp in [
            (1, 2, 40, 160, 96, 2, 10, 0), (2, 3, 64, 192, 108, 2, 10, 0),
            (3, 4, 32, 96, 54, 0, 10, 8)]:
        g = qr.GenScene(kind, seed, nq, 0)
        f = qr.Flat(g, w, h, fsaa)
        desc, params = f.update(0, depth)
        sid = ctx.upload(desc)
        frame = torch.zeros((params.y_res, params.x_row), dtype=torch.int32, device="cuda")
        if spp:
            params.pt_on, params.pts_c, params.seed = spp, 0.0, 5
            acc = torch.zeros((params.y_res, params.x_row, 3), dtype=torch.float32,
                              device="cuda")
            ctx.render_pt(sid, params, acc.data_ptr(), frame.data_ptr(), stream)
        else:
            ctx.render_device(sid, params, frame.data_ptr(), stream)
        torch.cuda.synchronize()
        assert ctx.fault() == (0, 0, 0, 0), (kind, seed)


@pytest.mark.parametrize("kind,seed,nq,w,h,depth", [
    (2, 4, 64, 203, 117, 4), (1, 6, 40, 161, 93, 10), (2, 5, 32, 7, 3, 10)])
def test_aa_subsample_threads_equal_pixel_threads(qr, ctx, kind, seed, nq, w, h, depth):
    """4x AA with a thread per sub-sample (shuffle average) gives the frame
    of a thread per pixel, on ragged sizes too"""
    g = qr.GenScene(kind, seed, nq, 0)
    f = qr.Flat(g, w, h, 2)
    desc, params = f.update(16, depth)
    sid = ctx.upload(desc)
    a = ctx.render_host(sid, params).copy()
    pp = qr.QrFrameParams.from_buffer_copy(params)
    pp.flags = qr.FP_PIXEL_THREADS
    b = ctx.render_host(sid, pp)
    assert (a != b).sum() == 0


def test_upload_rejects_out_of_range_indices(qr, ctx):
    """qr_scene_upload checks every index the kernels follow before any copy:
    descriptors with an element, material, texel or list index out of range
    are refused with QR_ERR_ARG (no kernel ever sees them); the intact
    descriptor is accepted"""
    import ctypes
    g = qr.GenScene(qr.SCN_PLAIN, 7, 16, qr.GEN_TEX)
    f = qr.Flat(g, 64, 48, 0)
    desc, params = f.update(0, 10)
    elems = np.ctypeslib.as_array(ctypes.cast(desc.elems, ctypes.POINTER(ctypes.c_int32)),
                                  shape=(desc.nelem * 4,)).copy()
    mats = np.ctypeslib.as_array(ctypes.cast(desc.mat, ctypes.POINTER(ctypes.c_int32)),
                                 shape=(desc.nmat * 28,)).copy()   # qr_mat: 112 bytes

    def upload(el, mt, **fields):
        d = qr.QrSceneDesc.from_buffer_copy(desc)
        d.elems = el.ctypes.data
        d.mat = mt.ctypes.data
        for k, v in fields.items():
            setattr(d, k, v)
        sid = ctypes.c_int(-1)
        rc = qr.lib().qr_scene_upload(ctx.h, ctypes.byref(d), ctypes.byref(sid))
        if rc == 0:
            ctx.release(sid.value)
        return rc

    assert upload(elems, mats) == 0
    bad = elems.copy()
    bad[1] = desc.nsrf + 5                      # element 0 refers past the records
    assert upload(bad, mats) == 1
    tex = [i for i in range(desc.nmat) if mats[28 * i + 3] & 0x800]   # QR_PROP_TEXTURE
    assert tex
    badm = mats.copy()
    badm[28 * tex[0] + 19] = desc.ntex - 1       # tex_off: the texture runs past the texels
    assert upload(elems, badm) == 1
    assert upload(elems, mats, cam_num=desc.nelem + 1) == 1
    assert upload(elems, mats, nmat=-1) == 1
