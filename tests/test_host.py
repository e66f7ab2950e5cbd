"""Host-side logic without a GPU: the C-ABI library, struct layouts, the
seeded scene generator and the host flattening.

Nothing here launches a kernel.  The library must load and export every entry
point include/qr_gpu.h declares; creating a context on a machine without a
GPU must fail with a status code (the product has no CPU fallback).
"""
import ctypes
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "qr_gpu.h")


def header_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|const char \*|void)\s*\*?\s*(qr_\w+)\s*\(",
                                 src, flags=re.M)))


def test_header_declares_entry_points():
    names = header_functions()
    for n in ["qr_ctx_create", "qr_ctx_destroy", "qr_last_error", "qr_scene_upload",
              "qr_scene_update", "qr_scene_release", "qr_render_device",
              "qr_render_host", "qr_sync", "qr_render_stats"]:
        assert n in names


def test_library_exports_every_declared_symbol(qr):
    L = qr.lib()
    missing = [n for n in header_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_context_without_gpu_fails_with_status(qr):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    p = ctypes.c_void_p()
    rc = qr.lib().qr_ctx_create(0, ctypes.byref(p))
    assert rc != qr.QR_OK
    assert not p.value


def test_null_arguments_rejected(qr):
    L = qr.lib()
    assert L.qr_ctx_create(0, None) != qr.QR_OK
    assert L.qr_render_host(None, 0, None, None) != qr.QR_OK
    assert L.qr_scene_upload(None, None, None) != qr.QR_OK
    assert L.qr_scene_anim_init(None, 0, None, None, 0, None) != qr.QR_OK
    assert L.qr_scene_anim_update(None, 0, None, 0, None) != qr.QR_OK
    assert L.qr_scene_anim_status(None, 0, None) != qr.QR_OK


def _c_layout():
    """sizeof/offsetof of the ABI structs as a C compiler lays them out."""
    prog = r"""
#include <stdio.h>
#include <stddef.h>
#include "qr_gpu.h"
#define P(T, F) printf(#T "." #F " %zu\n", offsetof(T, F))
int main(void) {
    printf("qr_srf %zu\nqr_mat %zu\nqr_light %zu\nqr_elem %zu\nqr_lelem %zu\n",
           sizeof(qr_srf), sizeof(qr_mat), sizeof(qr_light), sizeof(qr_elem),
           sizeof(qr_lelem));
    printf("qr_scene_desc %zu\nqr_frame_params %zu\n", sizeof(qr_scene_desc),
           sizeof(qr_frame_params));
    P(qr_frame_params, x_res); P(qr_frame_params, seed); P(qr_frame_params, pts_c);
    P(qr_scene_desc, texels); P(qr_scene_desc, cam_num);
    P(qr_srf, sci); P(qr_srf, amap); P(qr_srf, trnode); P(qr_srf, id);
    printf("qr_anim_node %zu\nqr_anim_param %zu\n", sizeof(qr_anim_node),
           sizeof(qr_anim_param));
    P(qr_anim_node, p); P(qr_anim_node, r); P(qr_anim_param, pos);
    return 0;
}
"""
    with tempfile.TemporaryDirectory() as td:
        c = os.path.join(td, "l.c")
        exe = os.path.join(td, "l")
        open(c, "w").write(prog)
        subprocess.run(["gcc", "-I" + os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    return dict((k, int(v)) for k, v in (ln.split() for ln in out.splitlines()))


def test_struct_layouts_match_ctypes_mirror(qr):
    lay = _c_layout()
    assert lay["qr_srf"] == 256
    assert lay["qr_srf.sci"] % 16 == 0
    assert lay["qr_elem"] == 16 and lay["qr_lelem"] == 16
    assert lay["qr_light"] == 48
    assert lay["qr_mat"] == 112
    assert lay["qr_scene_desc"] == ctypes.sizeof(qr.QrSceneDesc)
    assert lay["qr_frame_params"] == ctypes.sizeof(qr.QrFrameParams)
    assert lay["qr_frame_params.x_res"] == qr.QrFrameParams.x_res.offset
    assert lay["qr_frame_params.seed"] == qr.QrFrameParams.seed.offset
    assert lay["qr_frame_params.pts_c"] == qr.QrFrameParams.pts_c.offset
    assert lay["qr_scene_desc.texels"] == qr.QrSceneDesc.texels.offset
    assert lay["qr_scene_desc.cam_num"] == qr.QrSceneDesc.cam_num.offset
    assert lay["qr_anim_node"] == ctypes.sizeof(qr.QrAnimNode) == 160
    assert lay["qr_anim_param"] == ctypes.sizeof(qr.QrAnimParam) == 48
    assert lay["qr_anim_node.p"] == qr.QrAnimNode.p.offset
    assert lay["qr_anim_node.r"] == qr.QrAnimNode.r.offset
    assert lay["qr_anim_param.pos"] == qr.QrAnimParam.pos.offset


def _desc_arrays(desc, mat_size=112):
    def arr(ptr, n, rec):
        if n == 0:
            return np.zeros((0, rec // 4), dtype=np.int32)
        buf = (ctypes.c_char * (n * rec)).from_address(ptr)
        return np.frombuffer(bytes(buf), dtype=np.int32).reshape(n, rec // 4)
    return dict(srf=arr(desc.srf, desc.nsrf, 256), mat=arr(desc.mat, desc.nmat, mat_size),
                lgt=arr(desc.lgt, desc.nlgt, 48), elems=arr(desc.elems, desc.nelem, 16),
                lelems=arr(desc.lelems, desc.nlelem, 16))


def _flat_arrays(qr, seed):
    f = qr.Flat(qr.GenScene(qr.SCN_PLAIN, seed, 16), 64, 48)
    return _desc_arrays(f.update(0, 10)[0])     # copied while f is alive


def test_generation_is_deterministic(qr):
    a, b, c = _flat_arrays(qr, 11), _flat_arrays(qr, 11), _flat_arrays(qr, 12)
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    assert not np.array_equal(a["srf"], c["srf"])


@pytest.mark.parametrize("nq", [1, 16, 64])
def test_flattened_lists_are_consistent(qr, nq):
    g = qr.GenScene(qr.SCN_PLAIN, 3, nq)
    f = qr.Flat(g, 96, 64)
    desc, params = f.update(0, 10)
    A = _desc_arrays(desc)
    srf, el, le = A["srf"], A["elems"], A["lelems"]
    nsrf, nel = desc.nsrf, desc.nelem
    assert 0 <= desc.cam_off and desc.cam_off + desc.cam_num <= nel
    # qr_elem: kind, ref, last, rel
    for kind, ref, last, rel in el:
        assert kind in (0, 1, 2, 3)
        if kind in (0, 1):
            assert 0 <= ref < nsrf
        if kind == 1:
            assert 0 <= last < nel
    # surface records: list ranges stay inside the element arrays
    # int32 words: clip_off 45, clip_num 46, lgt_off 48-49, lgt_num 50-51,
    # sec_off 52-53, sec_num 54-55, mat 40-41
    for r in srf:
        assert r[45] >= 0 and r[45] + r[46] <= nel
        for s in (0, 1):
            assert r[48 + s] >= 0 and r[48 + s] + r[50 + s] <= desc.nlelem
            assert r[52 + s] >= 0 and r[52 + s] + r[54 + s] <= nel
            assert -1 <= r[40 + s] < desc.nmat
    for light, off, num, _ in le:
        assert 0 <= light < desc.nlgt
        assert 0 <= off and off + num <= nel
    # the camera sees every surface of the plain scene (1 ground plane + nq)
    cam = el[desc.cam_off:desc.cam_off + desc.cam_num]
    seen = set(int(r) for k, r, _, _ in cam if k == 0)
    assert len(seen) == nq + 1
    assert params.x_res == 96 and params.y_res == 64 and params.x_row >= 96


def test_frame_params_camera(qr):
    """The ray basis spans the screen: hor/ver are 1/x_res of the camera axes."""
    g = qr.GenScene(qr.SCN_PLAIN, 1, 16)
    f = qr.Flat(g, 800, 480)
    _, p = f.update(0, 10)
    hor, ver = np.array(p.hor), np.array(p.ver)
    assert abs(np.linalg.norm(hor) * 800 - 1.0) < 1e-5
    assert abs(np.linalg.norm(ver) * 800 - 1.0) < 1e-5
    assert abs(np.dot(hor, ver)) < 1e-6
    assert np.allclose(p.org, [0.0, -25.0, 8.0])
    assert abs(p.t_min - 0.5 / np.tan(np.radians(30.0))) < 1e-5


def test_bmp_textures_load_like_the_reference(qr, tmp_path, monkeypatch):
    """Textures named as files load as the reference's load_image reads
    them: 24-bit uncompressed BMPs, texels in file order; a file of another
    depth, or a missing file, fails the scene's construction"""
    qr.write_textures(7, str(tmp_path))
    monkeypatch.setenv("QR_PATH_TEXTURES", str(tmp_path) + "/")
    ref = qr.Flat(qr.GenScene(qr.SCN_PLAIN, 7, 16, qr.GEN_TEX), 64, 48)
    d_ref, _ = ref.update(0, 10)
    f = qr.Flat(qr.GenScene(qr.SCN_PLAIN, 7, 16, qr.GEN_TEX | qr.GEN_TEXFILE), 64, 48)
    d, _ = f.update(0, 10)
    import ctypes
    a = np.ctypeslib.as_array(ctypes.cast(d.texels, ctypes.POINTER(ctypes.c_uint32)), (d.ntex,))
    b = np.ctypeslib.as_array(ctypes.cast(d_ref.texels, ctypes.POINTER(ctypes.c_uint32)),
                              (d_ref.ntex,))
    assert d.ntex == d_ref.ntex and (a == b).all()
    raw = bytearray((tmp_path / "qr_tex1.bmp").read_bytes())
    raw[28] = 32                                    # bits per pixel
    (tmp_path / "qr_tex1.bmp").write_bytes(bytes(raw))
    with pytest.raises(RuntimeError):
        qr.Flat(qr.GenScene(qr.SCN_PLAIN, 7, 16, qr.GEN_TEX | qr.GEN_TEXFILE), 64, 48)
    (tmp_path / "qr_tex1.bmp").unlink()
    with pytest.raises(RuntimeError):
        qr.Flat(qr.GenScene(qr.SCN_PLAIN, 7, 16, qr.GEN_TEX | qr.GEN_TEXFILE), 64, 48)


@pytest.mark.parametrize("kind,seed,nq,flags,opts", [
    (2, 1, 64, 0, -1),          # every surface under a spinning array a node
    (2, 2, 64, 8, -1),          # array-level transform nodes (TARRAY)
    (2, 5, 64, 0, (1 << 20) | (1 << 21) | (1 << 25)),   # the reference's NONE opts
    (1, 3, 32, 16, -1),         # spinning quadrics, no hierarchy of arrays
    (1, 11, 24, 1 << 12, -1),   # quadrics that turn and rise: moving transforms
])
def test_device_update_table_reproduces_host_update(qr, kind, seed, nq, flags, opts):
    """the device update table taken at one frame, with the animators'
    transforms of later frames, gives the records and lights of the host
    update phases of those frames bit for bit (the device's matrix steps run
    on the host here; the GPU tests compare the device's own output)"""
    f = qr.Flat(qr.GenScene(kind, seed, nq, flags), 160, 96, 0, opts)
    f.update(16, 4)
    table = f.anim_table()
    assert len(table) > 0
    assert all(e.parent < i for i, e in enumerate(table))
    nparam = max(e.param for e in table) + 1
    for t in (32, 48, 16 * 55, 16 * 301):
        rc, p = f.anim_params(t)
        assert rc == 0 and len(p) == nparam
        f.update(t, 4)
        assert f.anim_check(table, p) == 0, t
    # a stale table does not reproduce frames it was not given
    rc, p = f.anim_params(16 * 302)
    assert f.anim_check(table, p) > 0


def test_static_scene_has_an_empty_update_table(qr):
    f = qr.Flat(qr.GenScene(qr.SCN_PLAIN, 4, 16, 0), 64, 48)
    f.update(0, 4)
    assert len(f.anim_table()) == 0
    rc, p = f.anim_params(16)
    assert rc == 0 and len(p) == 0


def _bound(qr, desc, table):
    out = (ctypes.c_float * 6)()
    qr.lib().qrpy_rotation_bound(ctypes.byref(desc), table, len(table), out)
    return list(out)


def _extent(qr, desc):
    out = (ctypes.c_double * 6)()
    qr.lib().qrpy_extent(ctypes.byref(desc), out)
    return list(out)


@pytest.mark.parametrize("kind,seed,nq,flags", [
    (2, 1, 64, 0),          # spinning 3-level hierarchy, every surface a node
    (2, 5, 64, 8),          # array-level transform nodes (TARRAY)
    (2, 3, 256, 0),
    (1, 3, 64, 16),         # spinning quadrics
])
def test_rotation_bound_holds_every_later_frame(qr, kind, seed, nq, flags):
    """the default motion bound of a device update table, taken at the first
    frame: for animators that only rotate, the scene's extent (surface boxes
    without rounding allowance and record positions) at every later frame
    lies inside it"""
    f = qr.Flat(qr.GenScene(kind, seed, nq, flags), 64, 48, 0)
    desc, _ = f.update(0, 4)
    table = f.anim_table()
    b = _bound(qr, desc, table)
    e0 = _extent(qr, desc)
    assert all(b[k] <= e0[k] and b[3 + k] >= e0[3 + k] for k in range(3))
    for t in [16 * k for k in range(1, 400, 7)]:
        desc, _ = f.update(t, 4)
        e = _extent(qr, desc)
        for k in range(3):
            assert b[k] <= e[k] + 1e-4 and e[3 + k] - 1e-4 <= b[3 + k], (t, k, b, e)


def test_moving_transforms_leave_the_rotation_bound(qr):
    """animators that move their transforms (quadrics that rise) are not
    covered by the default bound: later frames leave it, which the device
    update's own check catches"""
    f = qr.Flat(qr.GenScene(qr.SCN_PLAIN, 11, 24, 1 << 12), 64, 48, 0)
    desc, _ = f.update(0, 4)
    b = _bound(qr, desc, f.anim_table())
    desc, _ = f.update(16000, 4)
    e = _extent(qr, desc)
    assert e[5] > b[5]


@pytest.mark.parametrize("kind,seed,nq,flags", [
    (2, 1, 64, 0), (2, 5, 64, 8), (2, 3, 256, 0), (1, 3, 64, 16),
])
def test_float_box_stage_contains_the_exact_boxes(qr, kind, seed, nq, flags):
    """the device update's box stage (the kernel's float steps, run here on
    the host) gives, at later frames, boxes that contain the exact boxes of
    the same terms in double arithmetic: the pad covers float rounding"""
    f0 = qr.Flat(qr.GenScene(kind, seed, nq, flags), 64, 48, 0)
    d0, _ = f0.update(0, 4)
    table = f0.anim_table()
    ft = qr.Flat(qr.GenScene(kind, seed, nq, flags), 64, 48, 0)
    for t in (16, 16 * 37, 16 * 211, 16 * 997):
        dt, _ = ft.update(t, 4)
        assert qr.lib().qrpy_anim_box_check(ctypes.byref(d0), table, len(table),
                                            ctypes.byref(dt)) == 0, t


def test_update_table_refusals(qr):
    """anim_params reports a frame the table no longer fits: an animated
    transform whose scale changes (2), one that comes to rest at right
    angles (1); a table taken where an animated object has no free rotation
    is refused"""
    f = qr.Flat(qr.GenScene(qr.SCN_PLAIN, 5, 8, qr.GEN_SETTLE), 64, 48, 0)
    f.update(0, 4)
    table = f.anim_table()
    assert len(table) == 8
    rc, p = f.anim_params(500)
    assert rc == 0
    f.update(500, 4)
    assert f.anim_check(table, p) == 0
    rc, _ = f.anim_params(1200)
    assert rc == 2
    f.update(1200, 4)
    table = f.anim_table()          # a new table at the new scale fits again
    rc, p = f.anim_params(1500)
    assert rc == 0
    f.update(1500, 4)
    assert f.anim_check(table, p) == 0
    rc, _ = f.anim_params(2500)
    assert rc == 1
    f.update(2500, 4)
    with pytest.raises(ValueError):
        f.anim_table()


@pytest.mark.parametrize("kind,seed,nq,flags", [
    (1, 1, 16, 0), (1, 5, 256, 0), (2, 1, 64, 0), (2, 4, 256, 0), (2, 9, 512, 0),
    (3, 1, 32, 0), (3, 2, 96, 1 << 4)])
def test_walk_views_of_the_hierarchy(qr, kind, seed, nq, flags):
    """the binary child records and the 4-wide records the walks read
    reach exactly the binary tree's items, each once, with its boxes and
    codes; leaves hold at most 15 items; the stack need bounds the 4-wide
    walk (qrpy_accel_check, on the host)"""
    g = qr.GenScene(kind, seed, nq, flags)
    f = qr.Flat(g, 320, 240, 0)
    desc, _ = f.update(0, 4)
    levels = ctypes.c_int(0)
    bad = qr.lib().qrpy_accel_check(ctypes.byref(desc), ctypes.byref(levels))
    assert bad == 0
    assert levels.value >= 1
    if nq >= 256 and kind == 2:
        assert levels.value == 3          # the outer levels are built and checked


@pytest.mark.parametrize("kind,seed,nq,always", [
    (3, 1, 32, 5),      # the closed box: its five walls are tested by every ray
    (2, 1, 64, 1),      # the animated hierarchy: only the unbounded ground plane
    (1, 1, 16, 1),      # the plain scene: only the unbounded ground plane
])
def test_room_walls_leave_the_tree(qr, kind, seed, nq, always):
    """surfaces covering more than a fifth of the bounded extent's area join
    the unbounded ones (every ray tests them) instead of the tree"""
    g = qr.GenScene(kind, seed, nq, 0)
    f = qr.Flat(g, 320, 240, 0)
    desc, _ = f.update(0, 4)
    out = (ctypes.c_int * 3)()
    qr.lib().qrpy_accel_counts(ctypes.byref(desc), out)
    assert out[1] == always, list(out)
    assert out[0] > 0 and out[2] > 0
