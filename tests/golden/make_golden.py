"""Generate the golden fixtures of tests/golden/ from the reference engine.

TEST INFRASTRUCTURE ONLY.  Runs the reference's own fp32 CPU renderer
(VectorChief/QuadRay-engine rt_Scene::render, core/engine/engine.cpp:3014),
built from the reference sources by ``make -C oracle ref`` into
``oracle/_ref/ref_driver``, on the seeded synthetic scenes of
quadray-engine_gb300/csrc/scenegen.hpp and stores each frame as a compressed
``.npz`` (uint32 XRGB, H x W) plus the case parameters.  The fixtures pin the
CPU restatement in oracle/qr_oracle.c (tests/test_oracle_golden.py) and the
CUDA path (tests/test_gpu_parity.py) without the reference being present.

    python tests/golden/make_golden.py            # (re)write all fixtures
    python tests/golden/make_golden.py NAME ...   # (re)write the named ones

The reference is compiled with its SSE4 128-bit target (4 lanes), so the
frames carry the SIMD-group effects of that target (see the oracle header).
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")

# name: (kind, seed, nq, w, h, fsaa, frames, flags, opts[, depth])
#   kind 1 = plain Whitted scene, 2 = animated scene (clippers, booleans,
#   3-level spinning hierarchy, reflection/refraction with Fresnel; frames
#   at t = 0, 16, 32 ms); flags 1 = hit-ID materials, 8 = animated scene
#   that keeps RT_OPTS_TARRAY on (see test_oracle_golden.py), 32 = textured
#   ground and walls (bound texel arrays, side scales, rotations, offsets),
#   64 = gamma on, 128 = paracylinder, hypercylinder, two-plane, double
#   cone and hyperbolic paraboloid added, 256 = lights with an ambient share
#   and attenuation, 512 = animated scene without Fresnel terms (the
#   reference's default), 1024 = the textures named as BMP files that the
#   reference's load_image reads (the driver writes them to
#   ../data/textures/ of its working directory); fsaa 1 = 2x alternating,
#   2 = 4x rotated grid; 2048 = a second camera (next_cam before the frames
#   listed in NEXTCAM); 16 = plain scene whose quadrics spin;
#   opts "none" renders the reference without its list optimisations
CASES = {
    "plain_s1_160x96":      (1, 1, 16, 160, 96, 0, 1, 0, "full"),
    "plain_s2_160x96":      (1, 2, 16, 160, 96, 0, 1, 0, "full"),
    "plain_s3_160x96":      (1, 3, 16, 160, 96, 0, 1, 0, "full"),
    "plain_s4_160x96":      (1, 4, 16, 160, 96, 0, 1, 0, "full"),
    "plain_s5_none_160x96": (1, 5, 16, 160, 96, 0, 1, 0, "none"),
    "plain_s1_ids_160x96":  (1, 1, 16, 160, 96, 0, 1, 1, "full"),
    "plain_s6_ids_160x96":  (1, 6, 16, 160, 96, 0, 1, 1, "full"),
    "plain_s2_aa4_128x80":  (1, 2, 16, 128, 80, 2, 1, 0, "full"),
    "plain_s8_q32_200x120": (1, 8, 32, 200, 120, 0, 1, 0, "full"),
    "plain_s9_ragged_37x23": (1, 9, 16, 37, 23, 0, 1, 0, "full"),
    "plain_s7_tex_160x96":  (1, 7, 16, 160, 96, 0, 1, 32, "full"),
    "plain_s9_gamma_160x96": (1, 9, 16, 160, 96, 0, 1, 64, "full"),
    "plain_s10_tex_gamma_aa4_128x80": (1, 10, 16, 128, 80, 2, 1, 96, "full"),
    "plain_s12_shapes_160x96": (1, 12, 8, 160, 96, 0, 1, 128, "full"),
    "plain_s15_shapes_ids_160x96": (1, 15, 8, 160, 96, 0, 1, 129, "full"),
    "plain_s13_shapes_aa4_128x80": (1, 13, 8, 128, 80, 2, 1, 128, "full"),
    "plain_s17_attn_160x96": (1, 17, 16, 160, 96, 0, 1, 256, "full"),
    "plain_s19_all_160x96": (1, 19, 8, 160, 96, 0, 1, 480, "full"),
    "plain_s21_aa2_160x96": (1, 21, 16, 160, 96, 1, 1, 0, "full"),
    "anim_s9_none_aa2_128x72_d4": (2, 9, 64, 128, 72, 1, 2, 0, "none", 4),
    "plain_s24_actions_160x96": (1, 24, 16, 160, 96, 0, 4, 0, "full"),
    "anim_s10_actions_128x72_d4": (2, 10, 64, 128, 72, 0, 3, 0, "none", 4),
    "plain_s7_texfile_aa4_128x80": (1, 7, 16, 128, 80, 2, 1, 32 | 1024, "full"),
    "plain_s25_cameras_160x96": (1, 25, 16, 160, 96, 0, 3, 2048, "full"),
    "anim_s1_none_160x90_d4":     (2, 1, 64, 160, 90, 0, 2, 0, "none", 4),
    "anim_s2_none_aa4_128x72_d4": (2, 2, 64, 128, 72, 2, 2, 0, "none", 4),
    "anim_s4_none_96x54_d10":     (2, 4, 64, 96, 54, 0, 1, 0, "none", 10),
    "anim_s5_ids_160x90":         (2, 5, 64, 160, 90, 0, 2, 1, "full", 4),
    "anim_s1_full_160x90_d4":     (2, 1, 64, 160, 90, 0, 2, 0, "full", 4),
    "anim_s3_full_aa4_128x72_d4": (2, 3, 64, 128, 72, 2, 1, 0, "full", 4),
    "anim_s1_tarray_160x90_d4":   (2, 1, 64, 160, 90, 0, 1, 8, "full", 4),
    "anim_s1_tarray_none_160x90_d4": (2, 1, 64, 160, 90, 0, 1, 8, "none", 4),
    "anim_s6_nofresnel_160x90_d4": (2, 6, 64, 160, 90, 0, 2, 512, "full", 4),
    "anim_s8_nofresnel_96x54_d10": (2, 8, 64, 96, 54, 0, 1, 512, "none", 10),
    # six frames in a row (t = 0 .. 80 ms): a longer sequence for animated
    # scenes updated from frame to frame, and spinning plain quadrics (16)
    "anim_s12_full_128x72_d4":    (2, 12, 64, 128, 72, 0, 6, 0, "full", 4),
    "plain_s26_spin_160x96":      (1, 26, 16, 160, 96, 0, 6, 16, "full"),
    "anim_s13_full_aa4_96x54_d4": (2, 13, 64, 96, 54, 2, 4, 0, "full", 4),
    "anim_s14_none_96x54_d10":    (2, 14, 64, 96, 54, 0, 4, 0, "none", 10),
    # the benchmarked configurations at their sizes: the plain frame at
    # 800x480 (seeds 1-3), the animated frame with 4x AA at 480x270 (two
    # frames, the bench's default options)
    "plain_s1_800x480":           (1, 1, 16, 800, 480, 0, 1, 0, "full"),
    "plain_s2_800x480":           (1, 2, 16, 800, 480, 0, 1, 0, "full"),
    "plain_s3_800x480":           (1, 3, 16, 800, 480, 0, 1, 0, "full"),
    "anim_s1_full_aa4_480x270_d4": (2, 1, 64, 480, 270, 2, 2, 0, "full", 4),
    # path tracer (kind 3): the reference's running mean after 256 frames of
    # one sample each (its own random streams); only the last frame is kept
    "pt_s1_ref256_80x45_d8":      (3, 1, 32, 80, 45, 0, 256, 0, "full", 8, "last"),
    "pt_s2_ref256_64x36_d8":      (3, 2, 32, 64, 36, 0, 256, 0, "full", 8, "last"),
}


# camera actions (rt_Scene::update(time, action), codes of
# core/engine/object.h:47-63) applied before frames 1, 2, ... in turn:
# forward, rotate left, up; rotate right, back
ACTIONS = {
    "plain_s24_actions_160x96": "7,12,3",
    "anim_s10_actions_128x72_d4": "13,6",
}
# rt_Scene::next_cam before the listed frames
NEXTCAM = {
    "plain_s25_cameras_160x96": "1,2",
}


def run_case(name, case):
    kind, seed, nq, w, h, fsaa, frames, flags, opts = case[:9]
    depth = case[9] if len(case) > 9 else 10
    last_only = len(case) > 10 and case[10] == "last"
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "frame.bin")
        run = os.path.join(td, "run")
        os.makedirs(run)
        os.makedirs(os.path.join(td, "data", "textures"))
        # the frame does not depend on the worker count (rows are independent)
        cmd = [DRIVER, str(kind), str(seed), str(nq), str(w), str(h),
               str(fsaa), str(frames), str(flags), opts, out,
               str(min(8, os.cpu_count() or 1)), str(depth)]
        env = dict(os.environ)
        env.pop("QR_ACTIONS", None)
        env.pop("QR_NEXTCAM", None)
        if name in ACTIONS:
            env["QR_ACTIONS"] = ACTIONS[name]
        if name in NEXTCAM:
            env["QR_NEXTCAM"] = NEXTCAM[name]
        subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL,
                       stderr=subprocess.DEVNULL, env=env, cwd=run)
        data = np.fromfile(out, dtype="<u4").reshape(frames, h, w)
    meta = dict(kind=kind, seed=seed, nq=nq, w=w, h=h, fsaa=fsaa,
                frames=frames, flags=flags, opts=opts, depth=depth)
    if name in ACTIONS:
        meta["actions"] = ACTIONS[name]
    if name in NEXTCAM:
        meta["nextcam"] = NEXTCAM[name]
    if last_only:
        data = data[-1:]
        meta["samples"] = frames
        meta["frames"] = 1
    np.savez_compressed(os.path.join(HERE, name + ".npz"), frames=data,
                        meta=json.dumps(meta))
    return data


# ---- the reference's own regression scenes (test/scenes/scn_test01-18.h)
#
# Each fixture holds the reference's frame of the scene (rt_Scene::render
# with RT_OPTS_NONE, as test/core_test.cpp:993 renders its first run, and
# with RT_OPTS_FULL, its second run at :1033) and the scene as this
# repository's host engine flattens it from the unchanged scene header
# (oracle/_ref/scene_fixture, built from tests/golden/scene_fixture.cpp):
# the records the tests render.  The library's one image texture (the crate
# of data/objects, named tex_crate01.bmp when images are not compiled in) is
# replaced on both sides by a synthetic image of this script, so no image
# data of the reference enters the fixtures.  Scenes 17 and 18 are the
# reference's path-tracer scenes: their fixtures hold the mean of 256
# one-sample frames of the reference's path tracer.
SCN_W, SCN_H = 400, 240
PT_SCENES = {17: (80, 48, 256), 18: (80, 48, 256)}
FIXTURE = os.path.join(ROOT, "oracle", "_ref", "scene_fixture")


def write_bmp24(path, w, h, rgb):
    """24-bit bottom-up BMP of rgb[h][w] (XRGB integers)"""
    row = (w * 3 + 3) & ~3
    img = row * h
    hd = bytearray(54)
    hd[0:2] = b"BM"
    for at, v in ((2, 54 + img), (10, 54), (14, 40), (18, w), (22, h), (34, img)):
        hd[at:at + 4] = int(v).to_bytes(4, "little")
    hd[26] = 1
    hd[28] = 24
    body = bytearray()
    for y in range(h - 1, -1, -1):
        line = bytearray()
        for x in range(w):
            c = int(rgb[y][x])
            line += bytes((c & 255, (c >> 8) & 255, (c >> 16) & 255))
        body += line + bytes(row - len(line))
    with open(path, "wb") as f:
        f.write(bytes(hd) + bytes(body))


def crate_standin(n=64):
    """a synthetic plank pattern standing in for the crate image"""
    rgb = np.zeros((n, n), dtype=np.int64)
    for y in range(n):
        for x in range(n):
            plank = (y * 4) // n
            edge = x < 3 or x >= n - 3 or y < 3 or y >= n - 3 or (y * 4) % n < 2
            h = (x * 2654435761 + plank * 40503 + y * 97) & 0xFFFFFFFF
            grain = 150 + ((h >> 13) % 40) - 20
            if edge:
                grain = 70
            r, g, b = grain, (grain * 3) // 4, grain // 3
            rgb[y, x] = (r << 16) | (g << 8) | b
    return rgb


def scene_dir(td):
    run = os.path.join(td, "run")
    tex = os.path.join(td, "data", "textures")
    os.makedirs(run, exist_ok=True)
    os.makedirs(tex, exist_ok=True)
    write_bmp24(os.path.join(tex, "tex_crate01.bmp"), 64, 64, crate_standin(64))
    return run, tex


def ref_scene_frames(kind, w, h, frames, opts, run):
    out = os.path.join(run, "frame.bin")
    subprocess.run([DRIVER, str(kind), "0", "0", str(w), str(h), "0", str(frames), "0",
                    opts, out, str(min(8, os.cpu_count() or 1)), "10"],
                   check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL, cwd=run)
    return np.fromfile(out, dtype="<u4").reshape(frames, h, w)


def flat_scene(n, w, h, tex, run):
    out = os.path.join(run, "scene.qrsf")
    env = dict(os.environ, QR_PATH_TEXTURES=tex + os.sep)
    subprocess.run([FIXTURE, str(n), str(w), str(h), "0", "none", "10", out],
                   check=True, env=env)
    with open(out, "rb") as f:
        return np.frombuffer(f.read(), dtype=np.uint8)


def run_ref_scene(n):
    with tempfile.TemporaryDirectory() as td:
        run, tex = scene_dir(td)
        none = ref_scene_frames(100 + n, SCN_W, SCN_H, 1, "none", run)
        full = ref_scene_frames(100 + n, SCN_W, SCN_H, 1, "full", run)
        qrsf = flat_scene(n, SCN_W, SCN_H, tex, run)
        meta = dict(scene=n, w=SCN_W, h=SCN_H, fsaa=0, depth=10, frames=1, opts="none",
                    flags=0)
        np.savez_compressed(os.path.join(HERE, "scn_test%02d_%dx%d.npz" % (n, SCN_W, SCN_H)),
                            frames=none, frames_full=full, qrsf=qrsf, meta=json.dumps(meta))
        if n in PT_SCENES:
            w, h, spp = PT_SCENES[n]
            # the reference's path tracer converges under its full options
            # only (with RT_OPTS_NONE its frames do not accumulate)
            pt = ref_scene_frames(200 + n, w, h, spp, "full", run)[-1:]
            qrsf = flat_scene(n, w, h, tex, run)
            meta = dict(scene=n, w=w, h=h, fsaa=0, depth=10, frames=1, samples=spp,
                        opts="full", flags=0)
            np.savez_compressed(os.path.join(HERE, "scn_test%02d_pt%d_%dx%d.npz" % (n, spp, w, h)),
                                frames=pt, qrsf=qrsf, meta=json.dumps(meta))
        return none


def main():
    if not os.path.exists(DRIVER):
        sys.exit("oracle/_ref/ref_driver is missing: run `make -C oracle ref`")
    names = sys.argv[1:] or list(CASES) + ["scn_test%02d" % n for n in range(1, 19)]
    for name in names:
        if name.startswith("scn_test"):
            data = run_ref_scene(int(name[8:10]))
        else:
            data = run_case(name, CASES[name])
        print("%-24s %s nonzero=%d" % (name, data.shape, int((data != 0).sum())))


if __name__ == "__main__":
    main()
