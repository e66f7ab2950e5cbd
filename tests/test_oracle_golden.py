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

from conftest import channels, max_channel_diff, oracle_render

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))

# colour: fraction of pixels allowed to differ, and by at most this many LSBs
COLOR_FRAC = 1e-3
COLOR_LSB = 1
# hit IDs: host libm differences across machines may move a boundary pixel
ID_FRAC = 1e-3


def load_golden(path):
    z = np.load(path)
    return z["frames"], json.loads(str(z["meta"]))


def flatten_case(qr, meta, time=0):
    g = qr.GenScene(meta["kind"], meta["seed"], meta["nq"], meta["flags"])
    opts = qr.OPTS_NONE if meta["opts"] == "none" else qr.OPTS_DEFAULT
    f = qr.Flat(g, meta["w"], meta["h"], meta["fsaa"], opts)
    desc, params = f.update(time, meta.get("depth", 10))
    return g, f, desc, params


def frames_of(qr, meta):
    """Flatten every frame of a fixture (t = 16 ms per frame) in order."""
    g, f, desc, params = flatten_case(qr, meta, 0)
    yield desc, params
    for k in range(1, meta["frames"]):
        desc, params = f.update(16 * k, meta.get("depth", 10))
        yield desc, params


def check_against_golden(img, ref, meta):
    assert img.shape == ref.shape
    n = img.size
    if meta["flags"] & 1:
        bad = int((img != ref).sum())
        assert bad <= ID_FRAC * n, "hit IDs differ on %d of %d pixels" % (bad, n)
        return bad
    d = max_channel_diff(img, ref)
    bad = int((d > COLOR_LSB).sum())
    assert bad <= COLOR_FRAC * n, \
        "colour differs by more than %d LSB on %d of %d pixels (max %d)" % (
            COLOR_LSB, bad, n, int(d.max()))
    return bad


CULLED = {"anim_s1_tarray_160x90_d4"}


def _id(p):
    return os.path.basename(p)[:-4]


def test_fixtures_present():
    assert len(FIXTURES) >= 18


@pytest.mark.parametrize("path", [p for p in FIXTURES if _id(p) not in CULLED],
                         ids=[_id(p) for p in FIXTURES if _id(p) not in CULLED])
def test_oracle_matches_reference(qr, oracle, path):
    frames, meta = load_golden(path)
    for k, (desc, params) in enumerate(frames_of(qr, meta)):
        img, nrays = oracle_render(oracle, desc, params)
        assert nrays > 0
        check_against_golden(img, frames[k], meta)


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
    img[::4, :] ^= 2                   # 25% of hit IDs moved to the other side
    with pytest.raises(AssertionError):
        check_against_golden(img, frames[0], meta)
