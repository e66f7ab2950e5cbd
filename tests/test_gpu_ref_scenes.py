"""The reference's own regression scenes (test/scenes/scn_test01-18.h)
rendered on the GPU through the C ABI: the scene as the host engine
flattens it from the unchanged header (tests/golden/scn_testNN_*.npz),
against the reference's frame (golden bar, and the reference's own
frame_cmp against its optimised run) and against the oracle bit for bit.
Scenes 17 and 18 are the reference's path-tracer scenes: the wavefront path
tracer at 256 samples a pixel agrees with the reference's own 256-sample
mean as closely as two independent frames of the estimator agree.
"""
import ctypes
import glob
import json
import os

import numpy as np
import pytest

from conftest import frame_cmp, load_qrsf
from test_oracle_golden import check_against_golden, pt_agreement

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SCENES = sorted(glob.glob(os.path.join(GOLDEN, "scn_test??_400x240.npz")))
PT = sorted(glob.glob(os.path.join(GOLDEN, "scn_test??_pt*.npz")))


@pytest.fixture(scope="module")
def ctx(qr):
    c = qr.Context(0)
    yield c
    c.close()


def _id(p):
    return os.path.basename(p)[:-4]


@pytest.mark.parametrize("path", SCENES, ids=[_id(p) for p in SCENES])
def test_gpu_renders_reference_scene(qr, oracle, ctx, path):
    z = np.load(path)
    d, fp, keep = load_qrsf(qr, z["qrsf"])
    sid = ctx.upload(d)
    img = ctx.render_host(sid, fp).copy()
    ctx.release(sid)
    meta = json.loads(str(z["meta"]))
    check_against_golden(img, z["frames"][0], meta)
    assert frame_cmp(img, z["frames_full"][0]) == 0
    out = np.zeros((fp.y_res, fp.x_row), dtype=np.uint32)
    oracle.qr_oracle_render(ctypes.addressof(d), ctypes.addressof(fp), out.ctypes.data,
                            0, fp.y_res, None)
    assert (img != out[:, :fp.x_res]).sum() == 0


@pytest.mark.parametrize("path", PT, ids=[_id(p) for p in PT])
def test_gpu_path_tracer_agrees_with_reference(qr, ctx, path):
    import torch
    z = np.load(path)
    meta = json.loads(str(z["meta"]))
    d, fp, keep = load_qrsf(qr, z["qrsf"])
    sid = ctx.upload(d)
    frames = []
    for seed in (21, 22):
        p = qr.QrFrameParams.from_buffer_copy(fp)
        p.pt_on, p.pts_c, p.seed, p.frame_idx = meta["samples"], 0.0, seed, 0
        fr = torch.zeros((p.y_res, p.x_row), dtype=torch.int32, device="cuda")
        acc = torch.zeros((p.y_res, p.x_row, 3), dtype=torch.float32, device="cuda")
        ctx.render_pt(sid, p, acc.data_ptr(), fr.data_ptr(),
                      torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        frames.append(fr.cpu().numpy().view(np.uint32)[:, :p.x_res].copy())
    ctx.release(sid)
    ratio, zz = pt_agreement(frames[0], frames[1], z["frames"][0])
    assert ratio < 1.35, ratio
    assert zz < 4.0, zz
