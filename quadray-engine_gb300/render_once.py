"""Render a few frames of one benchmark workload through the C ABI, and
nothing else: the launch list of such a run is the render's own (for a
profiler's capture; bench.py also runs instrumented, end-to-end and CPU
legs).

    python quadray-engine_gb300/render_once.py WORKLOAD [--frames N] [--spp S]
        [--flags F]

WORKLOAD is anim (1920x1080, 4x AA, the animated scene, depth 4), plain
(800x480, depth 10) or pt (1280x720, depth 8, the closed box); --spp sets
the path tracer's samples a pixel (default 64), --flags ORs bits into
qr_frame_params.flags (QR_FP_*).  Prints the frame's non-black pixel count.
"""
import argparse
import importlib
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

CASES = {
    "anim": dict(kind=2, seed=1, nq=64, w=1920, h=1080, fsaa=2, depth=4),
    "plain": dict(kind=1, seed=1, nq=16, w=800, h=480, fsaa=0, depth=10),
    "pt": dict(kind=3, seed=1, nq=32, w=1280, h=720, fsaa=0, depth=8),
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("workload", choices=sorted(CASES))
    ap.add_argument("--frames", type=int, default=2)
    ap.add_argument("--spp", type=int, default=64)
    ap.add_argument("--flags", type=int, default=0)
    args = ap.parse_args()
    c = CASES[args.workload]
    qr = importlib.import_module("quadray-engine_gb300")
    import torch
    ctx = qr.Context(0)
    g = qr.GenScene(c["kind"], c["seed"], c["nq"], 0)
    f = qr.Flat(g, c["w"], c["h"], c["fsaa"])
    desc, p = f.update(0, c["depth"])
    p.flags = p.flags | args.flags
    sid = ctx.upload(desc)
    frame = torch.zeros((c["h"], p.x_row), dtype=torch.int32, device="cuda")
    acc = torch.zeros((c["h"], p.x_row, 3), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for k in range(args.frames):
        if args.workload == "pt":
            p.pt_on, p.pts_c, p.seed, p.frame_idx = args.spp, 0.0, 1, k
            ctx.render_pt(sid, p, acc.data_ptr(), frame.data_ptr(), stream)
        else:
            ctx.render_device(sid, p, frame.data_ptr(), stream)
    torch.cuda.synchronize()
    print("frames %d, non-black pixels %d" % (args.frames, int((frame != 0).sum())))
    ctx.close()


if __name__ == "__main__":
    main()
