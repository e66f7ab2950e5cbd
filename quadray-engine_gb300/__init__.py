"""GB300 QuadRay engine: Python host bindings.

Thin ctypes layer over ``_build/libquadray_gb300.so`` (built by
``build.py``): seeded synthetic scenes, the host flattening (no GPU needed),
the C ABI of ``include/qr_gpu.h`` and the ``rt_Scene`` engine API.  The
render itself always runs in the CUDA library; there is no CPU fallback and
loading fails loudly if the library is missing.

The directory name is not a Python identifier, so import it with
``importlib.import_module("quadray-engine_gb300")`` after putting the repo
root on ``sys.path``.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libquadray_gb300.so")

# scene kinds and generator flags (csrc/scenegen.hpp)
SCN_PLAIN = 1
SCN_ANIM = 2
SCN_PT = 3
GEN_IDS = 1 << 0
GEN_TARRAY = 1 << 3      # animated scene keeps RT_OPTS_TARRAY on
GEN_SPIN = 1 << 4        # plain scene whose quadrics spin
GEN_TEX = 1 << 5         # plain scene with textured ground and quadrics
GEN_GAMMA = 1 << 6       # the reference's gamma mode on
GEN_SHAPES = 1 << 7      # plain scene with the other quadric kinds too
GEN_ATTN = 1 << 8        # plain scene whose lights have ambient and attenuation
GEN_NOFRESNEL = 1 << 9   # animated scene without Fresnel terms (the default)
GEN_TEXFILE = 1 << 10    # with GEN_TEX: textures named as BMP files (write_textures)
GEN_CAMERAS = 1 << 11    # plain scene with a second camera (next_cam)
GEN_RISE = 1 << 12       # plain scene whose quadrics turn and rise (transforms move)
GEN_SETTLE = 1 << 13     # plain scene whose quadrics grow (from 1 s), rest at right angles (2 s)
# camera actions (rt_Scene::update; codes of core/engine/object.h:47-63)
CAMERA_MOVE_DOWN, CAMERA_MOVE_UP, CAMERA_MOVE_LEFT, CAMERA_MOVE_RIGHT = 2, 3, 4, 5
CAMERA_MOVE_BACK, CAMERA_MOVE_FORWARD = 6, 7
CAMERA_ROTATE_DOWN, CAMERA_ROTATE_UP, CAMERA_ROTATE_LEFT, CAMERA_ROTATE_RIGHT = 10, 11, 12, 13

# runtime options (csrc/format.h): -1 selects the default (FULL minus the
# scene's opt-outs)
OPTS_DEFAULT = -1
OPTS_NONE = (1 << 20) | (1 << 21) | (1 << 25)

QR_OK = 0
FP_LINEAR_WALK = 1        # qr_frame_params.flags: no BVH (same frame)
FP_PIXEL_THREADS = 2      # qr_frame_params.flags: 4x AA, a thread per pixel (same frame)
FP_PIXEL_PT = 4           # qr_frame_params.flags: path tracer, a thread per pixel instead
                          # of the wavefront stages (same frame)
FP_WAVEFRONT = 8          # qr_frame_params.flags: Whitted, wavefront stages instead of a
                          # thread per pixel or sub-sample tracing its whole ray tree


class QrSceneDesc(ctypes.Structure):
    """qr_scene_desc of include/qr_gpu.h."""
    _fields_ = [
        ("nsrf", ctypes.c_int32), ("srf", ctypes.c_void_p),
        ("nmat", ctypes.c_int32), ("mat", ctypes.c_void_p),
        ("nlgt", ctypes.c_int32), ("lgt", ctypes.c_void_p),
        ("nelem", ctypes.c_int32), ("elems", ctypes.c_void_p),
        ("nlelem", ctypes.c_int32), ("lelems", ctypes.c_void_p),
        ("ntex", ctypes.c_int32), ("texels", ctypes.c_void_p),
        ("cam_off", ctypes.c_int32), ("cam_num", ctypes.c_int32),
    ]


class QrFrameParams(ctypes.Structure):
    """qr_frame_params of include/qr_gpu.h."""
    _fields_ = [
        ("org", ctypes.c_float * 3), ("t_min", ctypes.c_float),
        ("dir", ctypes.c_float * 3), ("t_max", ctypes.c_float),
        ("hor", ctypes.c_float * 3), ("flags", ctypes.c_int32),
        ("ver", ctypes.c_float * 3), ("pad1", ctypes.c_float),
        ("amb", ctypes.c_float * 3), ("l_amb", ctypes.c_float),
        ("x_res", ctypes.c_int32), ("y_res", ctypes.c_int32),
        ("x_row", ctypes.c_int32), ("fsaa", ctypes.c_int32),
        ("depth", ctypes.c_int32), ("ctx_props", ctypes.c_int32),
        ("pt_on", ctypes.c_int32), ("frame_idx", ctypes.c_int32),
        ("seed", ctypes.c_uint64),
        ("pts_c", ctypes.c_float), ("pad2", ctypes.c_float),
    ]


class QrRequest(ctypes.Structure):
    """qr_request of include/qr_gpu.h (one frame of a batch)."""
    _fields_ = [
        ("scene_id", ctypes.c_int32), ("pad", ctypes.c_int32),
        ("fp", QrFrameParams),
        ("dev_frame", ctypes.c_void_p), ("dev_acc", ctypes.c_void_p),
    ]


class QrAnimNode(ctypes.Structure):
    """qr_anim_node of include/qr_gpu.h (one entry of a device update table)."""
    _fields_ = [
        ("kind", ctypes.c_int32), ("parent", ctypes.c_int32),
        ("param", ctypes.c_int32), ("rec", ctypes.c_int32),
        ("light", ctypes.c_int32), ("pad", ctypes.c_int32 * 3),
        ("p", ctypes.c_float * 16), ("r", ctypes.c_float * 16),
    ]


class QrAnimParam(ctypes.Structure):
    """qr_anim_param of include/qr_gpu.h (one animated transform)."""
    _fields_ = [
        ("sin", ctypes.c_float * 3), ("cos", ctypes.c_float * 3),
        ("pos", ctypes.c_float * 3), ("pad", ctypes.c_float * 3),
    ]


class QrAnimRequest(ctypes.Structure):
    """qr_anim_request of include/qr_gpu.h (one scene of a batched update)."""
    _fields_ = [
        ("scene_id", ctypes.c_int32), ("nparams", ctypes.c_int32),
        ("params", ctypes.POINTER(QrAnimParam)),
    ]


ANIM_OWN, ANIM_UNDER, ANIM_NODE = 0, 1, 2
QR_ERR_STATE = 5
QR_ERR_LIMIT = 7
QR_ERR_BUSY = 8
QR_ERR_TRACE = 9
FAULT_TREE, FAULT_STACK = 1, 2

_lib = None


def lib():
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libquadray_gb300.so is not built: run "
                               "quadray-engine_gb300/build.py (or "
                               "__graft_entry__.build())")
        L = ctypes.CDLL(LIB_PATH)
        vp, i32, i64, u64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_ulonglong
        L.qrpy_gen_new.restype = vp
        L.qrpy_gen_new.argtypes = [i32, u64, i32, i32]
        L.qrpy_gen_free.argtypes = [vp]
        L.qrpy_gen_nsurf.argtypes = [vp]
        L.qrpy_flat_new.restype = vp
        L.qrpy_flat_new.argtypes = [vp, i32, i32, i32, i32]
        L.qrpy_flat_update.argtypes = [vp, i64, i32]
        L.qrpy_flat_action.argtypes = [vp, i64, i32]
        L.qrpy_flat_next_cam.argtypes = [vp]
        L.qrpy_scene_next_cam.argtypes = [vp]
        L.qrpy_gen_write_textures.argtypes = [ctypes.c_ulonglong, ctypes.c_char_p]
        L.qrpy_flat_action.restype = None
        L.qrpy_scene_update.argtypes = [vp, i64, i32]
        L.qrpy_scene_update.restype = None
        L.qrpy_flat_desc.argtypes = [vp, ctypes.POINTER(QrSceneDesc),
                                     ctypes.POINTER(QrFrameParams)]
        L.qrpy_flat_free.argtypes = [vp]
        L.qrpy_flat_anim_table.argtypes = [vp, ctypes.POINTER(QrAnimNode), i32,
                                           ctypes.POINTER(ctypes.c_int), ctypes.c_char_p, i32]
        L.qrpy_flat_anim_params.argtypes = [vp, i64, ctypes.POINTER(QrAnimParam), i32,
                                            ctypes.POINTER(ctypes.c_int)]
        L.qrpy_anim_check.argtypes = [vp, ctypes.POINTER(QrAnimNode), i32,
                                      ctypes.POINTER(QrAnimParam)]
        L.qrpy_rotation_bound.argtypes = [ctypes.POINTER(QrSceneDesc), ctypes.POINTER(QrAnimNode),
                                          i32, ctypes.POINTER(ctypes.c_float)]
        L.qrpy_rotation_bound.restype = None
        L.qrpy_extent.argtypes = [ctypes.POINTER(QrSceneDesc), ctypes.POINTER(ctypes.c_double)]
        L.qrpy_accel_check.argtypes = [ctypes.POINTER(QrSceneDesc), ctypes.POINTER(ctypes.c_int)]
        L.qrpy_accel_counts.argtypes = [ctypes.POINTER(QrSceneDesc), ctypes.POINTER(ctypes.c_int)]
        L.qrpy_accel_counts.restype = None
        L.qrpy_extent.restype = None
        L.qrpy_anim_box_check.argtypes = [ctypes.POINTER(QrSceneDesc), ctypes.POINTER(QrAnimNode),
                                          i32, ctypes.POINTER(QrSceneDesc)]
        L.qr_scene_anim_init.argtypes = [vp, i32, ctypes.POINTER(QrSceneDesc),
                                         ctypes.POINTER(QrAnimNode), i32,
                                         ctypes.POINTER(ctypes.c_float)]
        L.qr_scene_anim_update.argtypes = [vp, i32, ctypes.POINTER(QrAnimParam), i32, vp]
        L.qr_scene_anim_upload.argtypes = [vp, ctypes.POINTER(QrSceneDesc),
                                           ctypes.POINTER(QrAnimNode), i32,
                                           ctypes.POINTER(ctypes.c_float), ctypes.POINTER(i32)]
        L.qr_scene_anim_status.argtypes = [vp, i32, ctypes.POINTER(ctypes.c_int32)]
        L.qr_scene_anim_update_many.argtypes = [vp, ctypes.POINTER(QrAnimRequest), i32, vp]
        L.qrpy_scene_new.restype = vp
        L.qrpy_scene_new.argtypes = [vp, i32, i32, i32, i32, i32, vp]
        L.qrpy_scene_render.argtypes = [vp, i64, vp]
        L.qrpy_scene_render_device.argtypes = [vp, i64, vp, vp]
        L.qrpy_scene_ctx.restype = vp
        L.qrpy_scene_ctx.argtypes = [vp]
        L.qrpy_scene_free.argtypes = [vp]
        L.qrpy_scene_set_pton.argtypes = [vp, i32]
        L.qrpy_scene_set_device_update.argtypes = [vp, i32]
        L.qr_ctx_create.argtypes = [i32, ctypes.POINTER(vp)]
        L.qr_ctx_destroy.argtypes = [vp]
        L.qr_last_error.restype = ctypes.c_char_p
        L.qr_last_error.argtypes = [vp]
        L.qr_scene_upload.argtypes = [vp, ctypes.POINTER(QrSceneDesc),
                                      ctypes.POINTER(ctypes.c_int)]
        L.qr_scene_update.argtypes = [vp, i32, ctypes.POINTER(QrSceneDesc)]
        L.qr_scene_release.argtypes = [vp, i32]
        L.qr_render_device.argtypes = [vp, i32, ctypes.POINTER(QrFrameParams), vp, vp]
        L.qr_render_host.argtypes = [vp, i32, ctypes.POINTER(QrFrameParams), vp]
        L.qr_render_pt.argtypes = [vp, i32, ctypes.POINTER(QrFrameParams), vp, vp, vp]
        L.qr_render_pt_noalloc.argtypes = [vp, i32, ctypes.POINTER(QrFrameParams), vp, vp]
        L.qr_batch_create.argtypes = [vp, i32, ctypes.POINTER(vp)]
        L.qr_batch_destroy.argtypes = [vp]
        L.qr_batch_set.argtypes = [vp, ctypes.POINTER(QrRequest), i32]
        L.qr_batch_config.argtypes = [vp, i32, i32]
        L.qr_batch_persistent.argtypes = [vp, i32]
        L.qr_batch_tune.argtypes = [vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                    ctypes.POINTER(ctypes.c_float)]
        L.qr_batch_launch.argtypes = [vp, vp]
        L.qr_batch_poll.argtypes = [vp]
        L.qr_batch_done.argtypes = [vp, ctypes.POINTER(ctypes.c_void_p)]
        L.qr_batch_wait.argtypes = [vp]
        L.qr_sync.argtypes = [vp, vp]
        L.qr_fp32_peak.argtypes = [i32, i32, ctypes.POINTER(ctypes.c_double)]
        L.qr_kernel_launches.argtypes = []
        L.qr_kernel_launches.restype = ctypes.c_ulonglong
        L.qr_fault.argtypes = [vp, ctypes.POINTER(ctypes.c_int32)]
        L.qr_render_stats.argtypes = [vp, i32, ctypes.POINTER(QrFrameParams), vp,
                                      ctypes.POINTER(ctypes.c_uint64)]
        _lib = L
    return _lib


class GenScene:
    """A seeded synthetic scene in the scene-struct format (scenegen.hpp)."""

    def __init__(self, kind=SCN_PLAIN, seed=1, nq=16, flags=0):
        self.kind, self.seed, self.nq, self.flags = kind, seed, nq, flags
        self.h = lib().qrpy_gen_new(kind, seed, nq, flags)
        if not self.h:
            raise RuntimeError("scene generation failed")

    @property
    def nsurf(self):
        return lib().qrpy_gen_nsurf(self.h)

    def close(self):
        if self.h:
            lib().qrpy_gen_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def kernel_launches():
    """kernels the library has launched in this process (qr_kernel_launches)"""
    return int(lib().qr_kernel_launches())


def write_textures(seed, directory):
    """write the BMP files qr_tex0-2.bmp that GEN_TEXFILE scenes of `seed`
    name into `directory` (the engine reads them from $QR_PATH_TEXTURES,
    default data/textures/)"""
    if lib().qrpy_gen_write_textures(int(seed), os.fsencode(directory)) != 0:
        raise RuntimeError("cannot write textures into %s" % directory)


class Flat:
    """Host flattening of a scene (update phases); CPU only."""

    def __init__(self, gen, x_res, y_res, fsaa=0, opts=OPTS_DEFAULT):
        self.gen = gen
        self.h = lib().qrpy_flat_new(gen.h, opts, x_res, y_res, fsaa)
        if not self.h:
            raise RuntimeError("flattening failed")
        self.desc = QrSceneDesc()
        self.params = QrFrameParams()

    def update(self, time=0, depth=10):
        rc = lib().qrpy_flat_update(self.h, int(time), int(depth))
        if rc != QR_OK:
            raise RuntimeError("update failed: %d" % rc)
        lib().qrpy_flat_desc(self.h, ctypes.byref(self.desc), ctypes.byref(self.params))
        return self.desc, self.params

    def next_cam(self):
        """switch to the next camera (rt_Scene::next_cam); returns its index
        in the reference's camera list"""
        return lib().qrpy_flat_next_cam(self.h)

    def frame_params(self):
        """the frame parameters of the last update (a copy)"""
        d, fp = QrSceneDesc(), QrFrameParams()
        lib().qrpy_flat_desc(self.h, ctypes.byref(d), ctypes.byref(fp))
        return fp

    def action(self, time, action):
        """camera movement before the next update (rt_Scene::update(time,
        action); CAMERA_* codes)"""
        lib().qrpy_flat_action(self.h, int(time), int(action))

    def anim_table(self):
        """the device update table after the last update: a QrAnimNode
        array; raises ValueError (with the reason) when the scene cannot be
        updated on the device"""
        n = ctypes.c_int(0)
        why = ctypes.create_string_buffer(160)
        rc = lib().qrpy_flat_anim_table(self.h, None, 0, ctypes.byref(n), why, 160)
        if rc == QR_ERR_STATE:
            raise ValueError(why.value.decode())
        arr = (QrAnimNode * n.value)()
        rc = lib().qrpy_flat_anim_table(self.h, arr, n.value, ctypes.byref(n), why, 160)
        if rc != QR_OK:
            raise ValueError(why.value.decode() or "anim table: %d" % rc)
        return arr

    def anim_params(self, time):
        """run the animators for `time`; returns (status, QrAnimParam array):
        status 0, or 1 / 2 when an animated transform lost its free rotation
        or changed scale (the frame then needs update() and a new table)"""
        n = ctypes.c_int(0)
        cap = getattr(self, "_anim_n", 0)
        buf = (QrAnimParam * cap)()
        rc = lib().qrpy_flat_anim_params(self.h, int(time), buf, cap, ctypes.byref(n))
        if rc == -1:
            # the animators ran; a second call at the same time only reads
            buf = (QrAnimParam * n.value)()
            rc = lib().qrpy_flat_anim_params(self.h, int(time), buf, n.value, ctypes.byref(n))
        self._anim_n = n.value
        return rc, buf

    def anim_check(self, table, params):
        """entries of `table` whose records or lights, formed from `params`
        by the device update's matrix steps on the host, differ from this
        scene's last update (0: all equal bit for bit)"""
        return lib().qrpy_anim_check(self.h, table, len(table), params)

    def close(self):
        if self.h:
            lib().qrpy_flat_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Context:
    """A device context of the C ABI (qr_ctx)."""

    def __init__(self, device=0):
        p = ctypes.c_void_p()
        rc = lib().qr_ctx_create(device, ctypes.byref(p))
        if rc != QR_OK:
            raise RuntimeError("qr_ctx_create failed: %d" % rc)
        self.h = p

    def error(self):
        return lib().qr_last_error(self.h).decode()

    def upload(self, desc):
        sid = ctypes.c_int(-1)
        rc = lib().qr_scene_upload(self.h, ctypes.byref(desc), ctypes.byref(sid))
        if rc != QR_OK:
            raise RuntimeError("qr_scene_upload: %d %s" % (rc, self.error()))
        return sid.value

    def update(self, sid, desc):
        rc = lib().qr_scene_update(self.h, sid, ctypes.byref(desc))
        if rc != QR_OK:
            raise RuntimeError("qr_scene_update: %d %s" % (rc, self.error()))

    def anim_init(self, sid, desc, table, bound=None):
        """upload desc into scene sid with its device update table (and a
        motion bound lo[3] + hi[3], default: the scene's extent widened)"""
        b = (ctypes.c_float * 6)(*bound) if bound is not None else None
        rc = lib().qr_scene_anim_init(self.h, sid, ctypes.byref(desc), table, len(table), b)
        if rc != QR_OK:
            raise RuntimeError("qr_scene_anim_init: %d %s" % (rc, self.error()))

    def anim_upload(self, desc, table, bound=None):
        """a new resident scene prepared for device updates; returns its id"""
        b = (ctypes.c_float * 6)(*bound) if bound is not None else None
        sid = ctypes.c_int32(-1)
        rc = lib().qr_scene_anim_upload(self.h, ctypes.byref(desc), table, len(table), b,
                                        ctypes.byref(sid))
        if rc != QR_OK:
            raise RuntimeError("qr_scene_anim_upload: %d %s" % (rc, self.error()))
        return sid.value

    def anim_update(self, sid, params, stream=0):
        """one frame's device update of scene sid on `stream`"""
        rc = lib().qr_scene_anim_update(self.h, sid, params, len(params), ctypes.c_void_p(stream))
        if rc != QR_OK:
            raise RuntimeError("qr_scene_anim_update: %d %s" % (rc, self.error()))

    def anim_update_many(self, updates, stream=0):
        """the updates [(sid, params), ...] of distinct scenes in one launch
        on `stream`"""
        arr = (QrAnimRequest * len(updates))()
        for q, (sid, params) in zip(arr, updates):
            q.scene_id = sid
            q.nparams = len(params)
            q.params = ctypes.cast(params, ctypes.POINTER(QrAnimParam))
        rc = lib().qr_scene_anim_update_many(self.h, arr, len(updates), ctypes.c_void_p(stream))
        if rc != QR_OK:
            raise RuntimeError("qr_scene_anim_update_many: %d %s" % (rc, self.error()))

    def anim_status(self, sid):
        """(frames updated on the device, frames whose update left the
        motion bound)"""
        out = (ctypes.c_int32 * 2)()
        rc = lib().qr_scene_anim_status(self.h, sid, out)
        if rc != QR_OK:
            raise RuntimeError("qr_scene_anim_status: %d %s" % (rc, self.error()))
        return tuple(out)

    def release(self, sid):
        rc = lib().qr_scene_release(self.h, sid)
        if rc != QR_OK:
            raise RuntimeError("qr_scene_release: %d %s" % (rc, self.error()))

    def render_host(self, sid, params):
        out = np.zeros((params.y_res, params.x_row), dtype=np.uint32)
        rc = lib().qr_render_host(self.h, sid, ctypes.byref(params),
                                  out.ctypes.data_as(ctypes.c_void_p))
        if rc != QR_OK:
            raise RuntimeError("qr_render_host: %d %s" % (rc, self.error()))
        return out[:, :params.x_res]

    def render_device(self, sid, params, dev_ptr, stream=0):
        rc = lib().qr_render_device(self.h, sid, ctypes.byref(params),
                                    ctypes.c_void_p(dev_ptr), ctypes.c_void_p(stream))
        if rc != QR_OK:
            raise RuntimeError("qr_render_device: %d %s" % (rc, self.error()))

    def render_pt(self, sid, params, dev_acc, dev_frame, stream=0):
        """Path-trace params.pt_on samples per pixel into caller-owned device
        sums (3 floats a pixel) and the device frame."""
        rc = lib().qr_render_pt(self.h, sid, ctypes.byref(params), ctypes.c_void_p(dev_acc),
                                ctypes.c_void_p(dev_frame), ctypes.c_void_p(stream))
        if rc != QR_OK:
            raise RuntimeError("qr_render_pt: %d %s" % (rc, self.error()))

    def sync(self, stream=0):
        rc = lib().qr_sync(self.h, ctypes.c_void_p(stream))
        if rc != QR_OK:
            raise RuntimeError("qr_sync: %d %s" % (rc, self.error()))

    def fault(self):
        """read and clear the fault word: (QR_FAULT_* bits, x, y of the first
        pixel, count of pixels); (0, 0, 0, 0) when no loop ran past its
        bound"""
        out = (ctypes.c_int32 * 4)()
        rc = lib().qr_fault(self.h, out)
        if rc not in (QR_OK, QR_ERR_TRACE):
            raise RuntimeError("qr_fault: %d %s" % (rc, self.error()))
        return tuple(out)

    def close(self):
        if self.h:
            lib().qr_ctx_destroy(self.h)
            self.h = None


class Batch:
    """Batched persistent rendering of many requests (qr_batch_*)."""

    def __init__(self, ctx, max_requests):
        self.ctx = ctx
        p = ctypes.c_void_p()
        rc = lib().qr_batch_create(ctx.h, max_requests, ctypes.byref(p))
        if rc != QR_OK:
            raise RuntimeError("qr_batch_create: %d %s" % (rc, ctx.error()))
        self.h = p

    def _check(self, rc, what):
        if rc != QR_OK:
            raise RuntimeError("%s: %d %s" % (what, rc, self.ctx.error()))

    def set(self, requests):
        arr = (QrRequest * len(requests))(*requests)
        self._check(lib().qr_batch_set(self.h, arr, len(requests)), "qr_batch_set")

    def config(self, tile_w, grab):
        self._check(lib().qr_batch_config(self.h, tile_w, grab), "qr_batch_config")

    def persistent(self, on):
        self._check(lib().qr_batch_persistent(self.h, 1 if on else 0), "qr_batch_persistent")

    def tune(self):
        tw, gr, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_float()
        self._check(lib().qr_batch_tune(self.h, ctypes.byref(tw), ctypes.byref(gr),
                                        ctypes.byref(ms)), "qr_batch_tune")
        return tw.value, gr.value, ms.value

    def launch(self, stream=0):
        self._check(lib().qr_batch_launch(self.h, ctypes.c_void_p(stream)), "qr_batch_launch")

    def poll(self):
        rc = lib().qr_batch_poll(self.h)
        if rc not in (QR_OK, QR_ERR_BUSY):
            self._check(rc, "qr_batch_poll")
        return rc == QR_OK

    def wait(self):
        self._check(lib().qr_batch_wait(self.h), "qr_batch_wait")

    def done_flags(self, n):
        """the per-request completion words of the last launch (n of them,
        1 = that request's frame is complete); a live view of host memory
        the device writes"""
        p = ctypes.c_void_p()
        self._check(lib().qr_batch_done(self.h, ctypes.byref(p)), "qr_batch_done")
        return (ctypes.c_uint32 * n).from_address(p.value)

    def close(self):
        if self.h:
            lib().qr_batch_destroy(self.h)
            self.h = None


class Engine:
    """rt_Platform + rt_Scene over a generated scene (the user-facing API)."""

    def __init__(self, gen, x_res, y_res, fsaa=0, opts=OPTS_DEFAULT, depth=10, pton=0):
        self.gen = gen
        self.x_res, self.y_res = x_res, y_res
        # the frame buffer the scene renders into (rt_Scene's caller-owned
        # frame): render() returns it without a copy
        self.frame = np.zeros((y_res, x_res), dtype=np.uint32)
        self.h = lib().qrpy_scene_new(gen.h, x_res, y_res, fsaa, opts, depth,
                                      self.frame.ctypes.data_as(ctypes.c_void_p))
        if not self.h:
            raise RuntimeError("rt_Scene construction failed")
        self.pton = lib().qrpy_scene_set_pton(self.h, pton) if pton else 0

    def next_cam(self):
        """rt_Scene::next_cam"""
        return lib().qrpy_scene_next_cam(self.h)

    def update(self, time, action):
        """camera movement from user input (rt_Scene::update(time, action))"""
        lib().qrpy_scene_update(self.h, int(time), int(action))

    def set_device_update(self, on):
        """animated scenes updated on the device (default) or by the host
        update phases and an upload each render"""
        return lib().qrpy_scene_set_device_update(self.h, 1 if on else 0)

    def set_pton(self, pton):
        """Path-tracer samples per render (rt_Scene::set_pton); returns the
        value in effect (0 when the scene's options prohibit the tracer)."""
        self.pton = lib().qrpy_scene_set_pton(self.h, pton)
        return self.pton

    def render(self, time=0, out=None):
        """render frame `time` into the scene's frame buffer and return it
        (the next render overwrites it); with `out`, a copy goes there"""
        rc = lib().qrpy_scene_render(self.h, int(time), None)
        if rc != QR_OK:
            raise RuntimeError("render failed: %d" % rc)
        if out is None:
            return self.frame
        np.copyto(out, self.frame)
        return out

    def render_device(self, time, dev_ptr, stream=0):
        rc = lib().qrpy_scene_render_device(self.h, int(time), ctypes.c_void_p(dev_ptr),
                                            ctypes.c_void_p(stream))
        if rc != QR_OK:
            raise RuntimeError("render_device failed: %d" % rc)

    def close(self):
        if self.h:
            lib().qrpy_scene_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def build(verbose=False, force=False):
    """Compile the CUDA library (see build.py)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("qr_build", os.path.join(HERE, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(verbose=verbose, force=force)
