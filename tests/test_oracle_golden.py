"""The CPU oracle against the reference engine's own frames (CPU only).

tests/golden/*.npz were rendered by the reference's fp32 CPU renderer
(core/engine/engine.cpp:3014 rt_Scene::render over core/tracer/tracer.cpp)
through oracle/_ref/ref_driver; tests/golden/make_golden.py regenerates them.
The oracle renders the same seeded scene from the host flattening
(csrc/flatten.cpp) and must reproduce them: hit IDs exactly, colour within
1 LSB per channel on at least 99.9% of pixels (the reference's 4-lane SIMD
groups can shift the last bit of a handful of pixels; on x86-64 every fixture
currently matches exactly).

Animated-scene fixtures hold several frames (t = 0, 16, 32 ms), rendered by
the reference with its default options or with RT_OPTS_NONE.  The animated
scene opts out of RT_OPTS_TARRAY: with array-level transform nodes the
reference builds per-surface shadow lists (lsort, bbox_shad,
core/engine/rtgeom.cpp:1004) and per-side secondary-ray lists (ssort,
core/engine/engine.cpp:2184-2376, bbox_side, rtgeom.cpp:1954) that lose
occluders and candidates of this spinning hierarchy, so its frame departs
from its own unculled render (missing shadows).  The fixture rendered with
TARRAY kept on is therefore an expected failure of the oracle, which walks
unculled lists.
"""
import glob
import json
import os

import numpy as np
import pytest

from conftest import boundary_mask, channels, max_channel_diff, oracle_render

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
# generated-scene fixtures (the reference's own test scenes, scn_test*, are
# covered by test_ref_scenes.py)
FIXTURES = sorted(p for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if not os.path.basename(p).startswith("scn_"))

# colour: fraction of pixels allowed to differ, and by at most this many LSBs
COLOR_FRAC = 1e-3
COLOR_LSB = 1
# hit IDs: exact outside the exclusion mask (conftest.boundary_mask: a root
# within 1e-5 relative of a tangent, a clip boundary or another surface's
# distance, where float rounding may pick either surface); the mask itself
# must stay a small share of the frame
ID_MASK_FRAC = 0.03


def load_golden(path):
    z = np.load(path)
    return z["frames"], json.loads(str(z["meta"]))


_TEXDIRS = {}


def texture_dir(qr, seed):
    """a directory holding the BMP textures of GEN_TEXFILE scenes of `seed`"""
    if seed not in _TEXDIRS:
        import tempfile
        d = tempfile.mkdtemp(prefix="qr_tex_")
        qr.write_textures(seed, d)
        _TEXDIRS[seed] = d
    return _TEXDIRS[seed]


def flatten_case(qr, meta, time=0):
    if meta["flags"] & qr.GEN_TEXFILE:
        os.environ["QR_PATH_TEXTURES"] = texture_dir(qr, meta["seed"]) + os.sep
    g = qr.GenScene(meta["kind"], meta["seed"], meta["nq"], meta["flags"])
    opts = qr.OPTS_NONE if meta["opts"] == "none" else qr.OPTS_DEFAULT
    f = qr.Flat(g, meta["w"], meta["h"], meta["fsaa"], opts)
    desc, params = f.update(time, meta.get("depth", 10))
    return g, f, desc, params


def frames_of(qr, meta):
    """Flatten every frame of a fixture (t = 16 ms per frame) in order,
    applying the fixture's camera actions (rt_Scene::update) before frames
    1, 2, ... as the reference's driver did."""
    g, f, desc, params = flatten_case(qr, meta, 0)
    yield desc, params
    acts = [int(a) for a in meta.get("actions", "").split(",") if a]
    cams = [int(a) for a in meta.get("nextcam", "").split(",") if a]
    for k in range(1, meta["frames"]):
        for c in cams:
            if c == k:
                f.next_cam()
        if acts:
            f.action(16 * k, acts[(k - 1) % len(acts)])
        desc, params = f.update(16 * k, meta.get("depth", 10))
        yield desc, params


def check_against_golden(img, ref, meta, mask=None):
    """the golden bar: hit-ID frames exact outside the exclusion mask (exact
    everywhere when no mask is given), colour frames within COLOR_LSB on all
    but COLOR_FRAC of the pixels"""
    assert img.shape == ref.shape
    n = img.size
    if meta["flags"] & 1:
        diff = img != ref
        if mask is not None:
            assert mask.shape == img.shape
            assert mask.mean() <= ID_MASK_FRAC, "exclusion mask %.4f" % mask.mean()
            diff = diff & ~mask
        bad = int(diff.sum())
        assert bad == 0, "hit IDs differ on %d of %d pixels outside the mask" % (bad, n)
        return bad
    d = max_channel_diff(img, ref)
    bad = int((d > COLOR_LSB).sum())
    assert bad <= COLOR_FRAC * n, \
        "colour differs by more than %d LSB on %d of %d pixels (max %d)" % (
            COLOR_LSB, bad, n, int(d.max()))
    return bad


CULLED = {"anim_s1_tarray_160x90_d4"}
PT = set(os.path.basename(p)[:-4] for p in FIXTURES if os.path.basename(p).startswith("pt_"))


def _id(p):
    return os.path.basename(p)[:-4]


def test_fixtures_present():
    assert len(FIXTURES) >= 20


EXACT = [p for p in FIXTURES if _id(p) not in CULLED and _id(p) not in PT]


@pytest.mark.parametrize("path", EXACT, ids=[_id(p) for p in EXACT])
def test_oracle_matches_reference(qr, oracle, path):
    frames, meta = load_golden(path)
    for k, (desc, params) in enumerate(frames_of(qr, meta)):
        img, nrays = oracle_render(oracle, desc, params)
        assert nrays > 0
        mask = boundary_mask(desc, params) if meta["flags"] & 1 else None
        check_against_golden(img, frames[k], meta, mask)


@pytest.mark.xfail(reason="with RT_OPTS_TARRAY the reference's shadow and "
                          "secondary-ray list culling drops occluders of the "
                          "spinning hierarchy; the oracle does not cull", strict=True)
def test_oracle_vs_reference_culled_lists(qr, oracle):
    frames, meta = load_golden(os.path.join(GOLDEN, "anim_s1_tarray_160x90_d4.npz"))
    g, f, desc, params = flatten_case(qr, meta)
    img, _ = oracle_render(oracle, desc, params)
    check_against_golden(img, frames[0], meta)


def test_tarray_culling_loses_shadows_in_the_reference():
    """With RT_OPTS_TARRAY the reference's own frame departs from its
    unculled render of the same scene, mostly brighter (lost occluders);
    without it the two renders are identical."""
    a, _ = load_golden(os.path.join(GOLDEN, "anim_s1_tarray_160x90_d4.npz"))
    b, _ = load_golden(os.path.join(GOLDEN, "anim_s1_tarray_none_160x90_d4.npz"))
    ca, cb = channels(a[0]).sum(-1), channels(b[0]).sum(-1)
    assert int((ca > cb).sum()) > int((ca < cb).sum()) > 0
    c, _ = load_golden(os.path.join(GOLDEN, "anim_s1_full_160x90_d4.npz"))
    d, _ = load_golden(os.path.join(GOLDEN, "anim_s1_none_160x90_d4.npz"))
    assert np.array_equal(c[0], d[0])


def test_planted_error_is_caught(qr, oracle):
    """Errors planted in the oracle's output beyond the bar must fail the check."""
    frames, meta = load_golden(os.path.join(GOLDEN, "plain_s1_160x96.npz"))
    g, f, desc, params = flatten_case(qr, meta)
    img, _ = oracle_render(oracle, desc, params)
    img = img.copy()
    img[40:44, 80:88] ^= 0x000400      # green off by 4 on 32 px (0.2%)
    with pytest.raises(AssertionError):
        check_against_golden(img, frames[0], meta)
    frames, meta = load_golden(os.path.join(GOLDEN, "plain_s1_ids_160x96.npz"))
    g, f, desc, params = flatten_case(qr, meta)
    img, _ = oracle_render(oracle, desc, params)
    img = img.copy()
    mask = boundary_mask(desc, params)
    moved = img.copy()
    moved[::4, :] ^= 2                 # 25% of hit IDs moved to the other side
    with pytest.raises(AssertionError):
        check_against_golden(moved, frames[0], meta, mask)
    one = img.copy()                   # one ID moved where the mask is clear
    yy, xx = np.argwhere(~mask)[len(np.argwhere(~mask)) // 2]
    one[yy, xx] ^= 2
    with pytest.raises(AssertionError):
        check_against_golden(one, frames[0], meta, mask)
    inside = img.copy()                # IDs moved only inside the mask pass
    inside[mask] ^= 2
    check_against_golden(inside, frames[0], meta, mask)


def test_boundary_mask_marks_tangents_and_clips(qr):
    """the exclusion mask is a thin set: a small share of the frame, and in
    the animated scene (clippers, booleans) larger than in the plain one"""
    g, f, desc, params = flatten_case(qr, dict(kind=1, seed=1, nq=16, w=160, h=96, fsaa=0,
                                               flags=1, opts="full", depth=10))
    m1 = boundary_mask(desc, params)
    g, f, desc, params = flatten_case(qr, dict(kind=2, seed=5, nq=64, w=160, h=90, fsaa=0,
                                               flags=1, opts="full", depth=4))
    m2 = boundary_mask(desc, params)
    assert 0 < m1.mean() < 0.01
    assert m1.mean() < m2.mean() < ID_MASK_FRAC


# ---- path tracer: same estimator as the reference, different random streams

def pt_frames(qr, oracle, meta, seeds, spp):
    """oracle path-traced frames (XRGB) of a fixture's scene, one per seed,
    rendered by row bands on all cores"""
    import ctypes
    import threading
    g = qr.GenScene(meta["kind"], meta["seed"], meta["nq"], meta["flags"])
    f = qr.Flat(g, meta["w"], meta["h"], 0)
    desc, params = f.update(0, meta["depth"])
    out = []
    for sd in seeds:
        p = qr.QrFrameParams.from_buffer_copy(params)
        p.pt_on, p.pts_c, p.seed, p.frame_idx = spp, 0.0, sd, 0
        acc = np.zeros((p.y_res, p.x_row, 3), dtype=np.float32)
        fr = np.zeros((p.y_res, p.x_row), dtype=np.uint32)
        nt = min(8, os.cpu_count() or 1)
        bands = np.linspace(0, p.y_res, nt + 1).astype(int)
        th = [threading.Thread(target=oracle.qr_oracle_pt, args=(
            ctypes.addressof(desc), ctypes.addressof(p), acc.ctypes.data, fr.ctypes.data,
            int(bands[i]), int(bands[i + 1]), None)) for i in range(nt)]
        [t.start() for t in th]
        [t.join() for t in th]
        out.append(fr[:, :p.x_res].copy())
    return out


def pt_agreement(a, b, ref):
    """mean squared error of a against ref, over that of a against b (an
    independent frame of the same estimator: the noise); and the difference
    of mean brightness in units of its standard error"""
    A, B, R = (channels(x).astype(np.float64) / 255.0 for x in (a, b, ref))
    noise = np.mean((A - B) ** 2)
    ratio = np.mean((A - R) ** 2) / noise
    se = np.sqrt(noise / A.size)
    return ratio, abs(A.mean() - R.mean()) / se


def test_pt_oracle_agrees_with_reference_path_tracer(qr, oracle):
    """The oracle's path tracer and the reference's (tests/golden, 256
    samples a pixel, its own LCG streams) converge to the same image: their
    distance matches the distance between two independent oracle frames
    (ratio 1 up to sampling error), and mean brightness agrees."""
    frames, meta = load_golden(os.path.join(GOLDEN, "pt_s2_ref256_64x36_d8.npz"))
    a, b = pt_frames(qr, oracle, meta, [11, 12], meta["samples"])
    ratio, z = pt_agreement(a, b, frames[0])
    assert ratio < 1.35, ratio
    assert z < 4.0, z


def test_pt_agreement_catches_a_biased_estimator(qr, oracle):
    """The same check fails for an image 10% too bright (planted on the CPU)."""
    frames, meta = load_golden(os.path.join(GOLDEN, "pt_s2_ref256_64x36_d8.npz"))
    a, b = pt_frames(qr, oracle, meta, [11, 12], meta["samples"])
    c = channels(a).astype(np.float64)
    c = np.minimum(np.rint(c * 1.1), 255).astype(np.uint32)
    biased = (c[..., 0] << 16) | (c[..., 1] << 8) | c[..., 2]
    ratio, z = pt_agreement(biased, b, frames[0])
    assert ratio > 1.35 or z > 4.0
