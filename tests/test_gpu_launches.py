"""The library's kernel-launch count (qr_kernel_launches), which the
benchmark reports as its launches in the timed region: a Whitted frame is
one kernel, a path-traced frame of the wavefront one chunk of (2 + 3 levels)
stage kernels plus the final and fallback kernels, a device update one
kernel, and a batch the kernels of its graph at every launch."""
import pytest

pytestmark = pytest.mark.gpu


def test_launch_counts(qr):
    import torch
    ctx = qr.Context(0)
    sp = torch.cuda.current_stream().cuda_stream
    g = qr.GenScene(qr.SCN_PLAIN, 1, 8, 0)
    f = qr.Flat(g, 96, 54, 0)
    desc, params = f.update(0, 4)
    sid = ctx.upload(desc)
    frame = torch.zeros((params.y_res, params.x_row), dtype=torch.int32, device="cuda")
    n0 = qr.kernel_launches()
    ctx.render_device(sid, params, frame.data_ptr(), sp)
    assert qr.kernel_launches() - n0 == 1

    g3 = qr.GenScene(qr.SCN_PT, 1, 8, 0)
    f3 = qr.Flat(g3, 96, 54, 0)
    desc3, p3 = f3.update(0, 8)
    sid3 = ctx.upload(desc3)
    acc = torch.zeros((p3.y_res, p3.x_row, 3), dtype=torch.float32, device="cuda")
    p3.pt_on, p3.pts_c, p3.seed, p3.frame_idx = 8, 0.0, 1, 0
    n0 = qr.kernel_launches()
    ctx.render_pt(sid3, p3, acc.data_ptr(), frame.data_ptr(), sp)
    # 12 x 14 tiles of 32 paths, 8 samples: one chunk of 9 levels (a tracing,
    # a shading and a folding kernel each)
    assert qr.kernel_launches() - n0 == (2 + 3 * 9) + 2
    p3.flags = p3.flags | qr.FP_PIXEL_PT
    n0 = qr.kernel_launches()
    ctx.render_pt(sid3, p3, acc.data_ptr(), frame.data_ptr(), sp)
    assert qr.kernel_launches() - n0 == 1

    frame3 = torch.zeros_like(frame)
    reqs = []
    for s, pp, fr in ((sid, params, frame), (sid3, p3, frame3)):
        r = qr.QrRequest()
        r.scene_id = s
        r.fp = qr.QrFrameParams.from_buffer_copy(pp)
        r.fp.flags = 0
        r.dev_frame = fr.data_ptr()
        r.dev_acc = acc.data_ptr() if pp.pt_on else None
        reqs.append(r)
    b = qr.Batch(ctx, 2)
    b.set(reqs)
    b.launch(sp)
    b.wait()
    n0 = qr.kernel_launches()
    b.launch(sp)
    torch.cuda.synchronize()
    # the Whitted batch kernel, the path-traced frame's kernels, its done mark
    assert qr.kernel_launches() - n0 == 1 + (2 + 3 * 9) + 2 + 1
    b.close()
    ctx.close()
