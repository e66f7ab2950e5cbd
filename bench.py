"""Benchmark of the GB300 QuadRay render path (rays/s, frames/s, latency).

A step renders one frame of the workload.  ``value`` is rays/s with the scene
resident in HBM and the frame written to device memory (CUDA events on the
launching stream, L2 flushed between steps).  For the animated workload every
step renders the next frame (t = 16 ms apart); the flattened scene of every
frame is uploaded before the timed region.  ``e2e`` is the same metric
through the engine API (rt_Scene::render) with a host frame buffer: host
update phases (animation, transforms, lists), scene upload, render and frame
download inside the timed region.  Rays are traced segments (primary +
shadow + reflected/refracted), counted per frame by an instrumented build of
the same kernel.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload anim|plain]
"""
import argparse
import ctypes
import importlib
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

# algorithmic FP32 operations per unit of work (div / sqrt count 1, FMA 2;
# the library is compiled without FMA contraction): per solver test,
# transform, clip evaluation, shaded hit, light evaluation, refraction and
# reflection
FLOPS = {
    "test_plane": 3, "test_quadric": 40, "test_twoplane": 28, "xform": 33,
    "clip_root": 12, "clip_custom": 15, "shade": 30, "light": 55,
    "refract": 40, "reflect": 25, "box_test": 12,
}
STAT_NAMES = ["ray_primary", "ray_shadow", "ray_secondary", "test_plane",
              "test_quadric", "test_twoplane", "xform", "clip_root",
              "clip_custom", "shade", "light", "refract", "reflect",
              "box_test", "far_walk"]

WORKLOADS = {
    # animated Whitted frame: 1920x1080, 4x AA, 64 quadrics cut by 1-2 planes
    # each plus 8 boolean-minus pairs, 3-level spinning hierarchy, 4 lights,
    # reflection + refraction with Fresnel to depth 4
    # (300 frames at t = 16 ms apart)
    "anim": dict(kind=2, seed=1, nq=64, w=1920, h=1080, fsaa=2, depth=4, anim=True,
                 frames=300),
    # plain Whitted frame: 800x480, 1 spp, 1 ground plane + 16 quadrics,
    # 2 lights, shadows
    "plain": dict(kind=1, seed=1, nq=16, w=800, h=480, fsaa=0, depth=10, anim=False),
    # path tracer: 1280x720, 64 samples a pixel per step, depth 8 (roulette
    # after 3 bounces), 32 quadrics in a closed box of 5 planes, light
    # cluster with an emitting sphere
    "pt": dict(kind=3, seed=1, nq=32, w=1280, h=720, fsaa=0, depth=8, anim=False, pt=64),
    # batched persistent launch: 256 requests (seeds 1000..1255), 8-512
    # quadrics (log-uniform), 320x240 / 640x480 / 1280x720 / 1920x1080,
    # Whitted depth 1-6 (plain scene) or path tracer 4-32 samples (box scene)
    "batch": dict(kind=0, seed=1000, nq=0, w=0, h=0, fsaa=0, depth=0, anim=False,
                  batch=256),
    "serve": dict(kind=0, seed=2000, nq=0, w=0, h=0, fsaa=0, depth=0, anim=True,
                  serve=(120, 500, 2000), seconds=60.0),
}

RESOLUTIONS = [(320, 240), (640, 480), (1280, 720), (1920, 1080)]

# served stream: 32 resident scenes (24 animated plain scenes with spinning
# quadrics, 16-256 quadrics; 8 path-traced box scenes), Poisson arrivals,
# 640x480 / 1280x720 / 1920x1080, 1-16 samples (Whitted: 1 sample or 4x AA;
# path tracer: that many samples), HBM budget 120 GB
SERVE_SIZES = [(640, 480), (1280, 720), (1920, 1080)]


def batch_requests(n, seed0):
    """the seeded request mix of the batched workload"""
    rng = np.random.default_rng(seed0)
    out = []
    for i in range(n):
        nq = int(round(math.exp(rng.uniform(math.log(8), math.log(512)))))
        w, h = RESOLUTIONS[int(rng.integers(0, 4))]
        if rng.uniform() < 0.5:
            out.append(dict(kind=1, seed=seed0 + i, nq=nq, w=w, h=h,
                            depth=int(rng.integers(1, 7)), spp=0))
        else:
            out.append(dict(kind=3, seed=seed0 + i, nq=nq, w=w, h=h, depth=8,
                            spp=int(rng.integers(4, 33))))
    return out


def anim_update_time(qr, ctx, seed):
    """device time of one update launch (qr_scene_anim_update) of a spinning
    scene of 256 quadrics and of the 512-quadric animated hierarchy, CUDA
    events around 200 launches on one stream; beside it the host update
    phases, hierarchy build and upload it replaces (wall clock)"""
    import time as _t
    import torch
    out = {}
    for name, kind, nq, flags in (("plain_spin_256", qr.SCN_PLAIN, 256, qr.GEN_SPIN),
                                  ("anim_512", qr.SCN_ANIM, 512, 0)):
        g = qr.GenScene(kind, seed, nq, flags)
        f = qr.Flat(g, 1920, 1080, 0)
        desc, _ = f.update(0, 4)
        sid = ctx.upload(desc)
        table = f.anim_table()
        ctx.anim_init(sid, desc, table)
        s = torch.cuda.Stream()
        params = [f.anim_params(16 * (k + 1))[1] for k in range(200)]
        for p in params[:5]:
            ctx.anim_update(sid, p, s.cuda_stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(s)
        for p in params:
            ctx.anim_update(sid, p, s.cuda_stream)
        e1.record(s)
        e1.synchronize()
        dev_us = 1000.0 * e0.elapsed_time(e1) / len(params)
        t0 = _t.perf_counter()
        for k in range(20):
            d2, _ = f.update(16 * (300 + k), 4)
            ctx.update(sid, d2)
        host_us = 1e6 * (_t.perf_counter() - t0) / 20
        t0 = _t.perf_counter()
        for k in range(200):
            rc, p = f.anim_params(16 * (400 + k))
        anim_host_us = 1e6 * (_t.perf_counter() - t0) / 200
        out[name] = {"entries": len(table), "device_update_us": dev_us,
                     "animators_host_us": anim_host_us,
                     "host_update_and_upload_us": host_us}
        ctx.release(sid)
    return out


def run_serve(args, wl, rank, world, dist, local):
    """served stream: rays/s sustained and latency at each arrival rate"""
    import torch
    qr = importlib.import_module("quadray-engine_gb300")
    serve = importlib.import_module("quadray-engine_gb300.serve")
    ctx = qr.Context(local)
    rng = np.random.default_rng(wl["seed"])
    scenes = []
    # 32 animated scenes with the features of the plain frame (16-256
    # quadrics, log-uniform); a request's spp > 1 asks for 4x AA
    for i in range(32):
        nq = int(round(math.exp(rng.uniform(math.log(16), math.log(256)))))
        scenes.append(dict(gen=qr.GenScene(qr.SCN_PLAIN, wl["seed"] + i, nq, qr.GEN_SPIN),
                           pt=False, depth=10, nq=nq, kind=1, anim=True))
    # rays per request class from instrumented frames at t = 0
    rays_of = {}

    def rays(req):
        sc = scenes[req.scene]
        fsaa = 0 if (sc["pt"] or req.spp <= 1) else 2
        key = (req.scene, req.w, req.h, fsaa)
        if key not in rays_of:
            g = qr.GenScene(sc["kind"], wl["seed"] + req.scene, sc["nq"],
                            0 if sc["pt"] else qr.GEN_SPIN)
            f = qr.Flat(g, req.w, req.h, fsaa)
            desc, params = f.update(0, sc["depth"])
            sid = ctx.upload(desc)
            if sc["pt"]:
                params.pt_on, params.pts_c = 1, 0.0
            counts = (ctypes.c_uint64 * len(STAT_NAMES))()
            host = np.zeros((params.y_res, params.x_row), dtype=np.uint32)
            rc = qr.lib().qr_render_stats(ctx.h, sid, ctypes.byref(params),
                                          host.ctypes.data_as(ctypes.c_void_p), counts)
            assert rc == 0, ctx.error()
            ctx.release(sid)
            rays_of[key] = int(counts[0]) + int(counts[1]) + int(counts[2])
        return rays_of[key] * (req.spp if sc["pt"] else 1)

    alone_ms = {}

    def alone(req):
        """device time of the request's frame rendered alone (its scene at
        t = 0, CUDA events, the median of 3)"""
        sc = scenes[req.scene]
        fsaa = 0 if (sc["pt"] or req.spp <= 1) else 2
        key = (req.scene, req.w, req.h, fsaa)
        if key not in alone_ms:
            g = qr.GenScene(sc["kind"], wl["seed"] + req.scene, sc["nq"], qr.GEN_SPIN)
            f = qr.Flat(g, req.w, req.h, fsaa)
            desc, params = f.update(0, sc["depth"])
            sid = ctx.upload(desc)
            fr = torch.empty((req.h, params.x_row), dtype=torch.int32, device="cuda")
            s = torch.cuda.current_stream()
            ts = []
            for _ in range(4):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(s)
                ctx.render_device(sid, params, fr.data_ptr(), s.cuda_stream)
                e1.record(s)
                e1.synchronize()
                ts.append(e0.elapsed_time(e1))
            ctx.release(sid)
            alone_ms[key] = float(np.median(ts[1:]))
        return alone_ms[key]

    urgent = None
    if args.serve_urgent:
        # 1080p Whitted frames, whose latency has a target, go first
        def urgent(r):
            return (r.w, r.h) == (1920, 1080) and not scenes[r.scene]["pt"]
    srv = serve.Server(qr, ctx, scenes, budget_bytes=120 << 30, max_batch=64,
                       max_batch_pixels=args.serve_batch_px, urgent=urgent,
                       urgent_batch_pixels=args.serve_urgent_px or None,
                       urgent_batches=args.serve_urgent_batches,
                       prep_threads=min(8, os.cpu_count() or 1),
                       device_anim=not args.serve_host_update)
    # warm-up: every scene once at every size
    warm = [serve.Request(i, s, 0, w, h, 1, 0.0)
            for i, (s, (w, h)) in enumerate((s, sz) for s in range(32) for sz in SERVE_SIZES)]
    srv.run(warm)
    results = []
    clocks = ClockSampler(local)
    clocks.start()
    rates = [float(x) for x in args.serve_rates.split(",")] if args.serve_rates else wl["serve"]
    seconds = args.serve_seconds or wl["seconds"]
    l0 = qr.kernel_launches()
    for rate in rates:
        reqs = serve.poisson_requests(32, rate, seconds, SERVE_SIZES, 16,
                                      wl["seed"] + int(rate))
        total = sum(rays(r) for r in reqs)
        done, wall = srv.run(reqs)
        lat = np.array([r.done - r.arrival for r in done]) * 1000.0
        big = np.array([r.done - r.arrival for r in done
                        if (r.w, r.h) == (1920, 1080) and not scenes[r.scene]["pt"]]) * 1000.0
        prep = np.array([r.prepared - r.arrival for r in done if r.prepared]) * 1000.0
        big_alone = np.array([alone(r) for r in done
                              if (r.w, r.h) == (1920, 1080) and not scenes[r.scene]["pt"]])
        results.append({"rate_per_s": rate, "requests": len(reqs), "seconds": wall,
                        "rays_per_s": total / wall,
                        "frames_per_s": len(reqs) / wall,
                        "latency_ms_p50": float(np.percentile(lat, 50)),
                        "latency_ms_p99": float(np.percentile(lat, 99)),
                        "whitted_1080p_ms_p50": float(np.percentile(big, 50)) if len(big) else None,
                        "whitted_1080p_ms_p99": float(np.percentile(big, 99)) if len(big) else None,
                        "whitted_1080p_alone_ms_p50": float(np.percentile(big_alone, 50))
                        if len(big_alone) else None,
                        "whitted_1080p_alone_ms_p99": float(np.percentile(big_alone, 99))
                        if len(big_alone) else None,
                        "prepared_ms_p99": float(np.percentile(prep, 99)) if len(prep) else None})
    ck = clocks.stop()
    launches = qr.kernel_launches() - l0
    counts = {"device_updates": srv.device_updates, "host_updates": srv.host_updates}
    srv.close()
    anim_us = anim_update_time(qr, ctx, wl["seed"])
    top = results[-1]
    line = {
        "metric": "rays_per_s", "value": top["rays_per_s"], "unit": "rays/s",
        "n_gpus": world, "steps": len(results), "warmup": 1,
        "ms_per_step": 1000.0 * top["seconds"] / max(1, top["requests"]),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": "serve", "scenes": 32, "animated_plain": 32,
                   "quadrics": [16, 256], "sizes": SERVE_SIZES, "spp": [1, 16],
                   "sampling": "spp 1: one camera ray a pixel; spp > 1: 4x AA",
                   "budget_bytes": 120 << 30, "seconds_per_rate": seconds,
                   "max_batch_pixels": args.serve_batch_px,
                   "urgent_first": "1080p Whitted" if args.serve_urgent else None,
                   "urgent_batch_pixels": (args.serve_urgent_px or args.serve_batch_px)
                   if args.serve_urgent else None,
                   "urgent_batches": args.serve_urgent_batches if args.serve_urgent else None,
                   "parallelism": "replicas" if world > 1 else "single"},
        "rates": results,
        "scene_updates": counts,
        "anim_update": anim_us,
        "e2e": {"value": top["rays_per_s"], "unit": "rays/s",
                "h2d_bytes_per_step": None, "d2h_bytes_per_step": 0,
                "note": "wall clock of the serving loop: animators on the host, "
                        "update phases on the device (host update phases and "
                        "uploads for a scene copy's first frame), batched "
                        "launches; frames stay on the device"},
        "gpu_launches": launches,
        "clocks": ck,
    }
    if rank == 0:
        print(json.dumps(line))
    ctx.close()


def run_batch(args, wl, rank, world, dist, local):
    import torch
    qr = importlib.import_module("quadray-engine_gb300")
    ctx = qr.Context(local)
    spec = batch_requests(wl["batch"], wl["seed"])
    keep, reqs, bufs = [], [], []
    rays = 0
    req_rays = []
    for i, rq in enumerate(spec):
        g = qr.GenScene(rq["kind"], rq["seed"], rq["nq"], 0)
        f = qr.Flat(g, rq["w"], rq["h"], 0)
        desc, params = f.update(0, rq["depth"])
        sid = ctx.upload(desc)
        r = qr.QrRequest()
        r.scene_id = sid
        r.fp = params
        r.fp.pt_on, r.fp.pts_c, r.fp.seed, r.fp.frame_idx = rq["spp"], 0.0, rq["seed"], 0
        fr = torch.empty((rq["h"], params.x_row), dtype=torch.int32, device="cuda")
        acc = (torch.empty((rq["h"], params.x_row, 3), dtype=torch.float32, device="cuda")
               if rq["spp"] else None)
        r.dev_frame = fr.data_ptr()
        r.dev_acc = acc.data_ptr() if acc is not None else None
        keep.append((g, f))
        bufs.append((fr, acc))
        reqs.append(r)
        counts = (ctypes.c_uint64 * len(STAT_NAMES))()
        host = np.zeros((params.y_res, params.x_row), dtype=np.uint32)
        rc = qr.lib().qr_render_stats(ctx.h, sid, ctypes.byref(r.fp),
                                      host.ctypes.data_as(ctypes.c_void_p), counts)
        assert rc == 0, ctx.error()
        req_rays.append(int(counts[0]) + int(counts[1]) + int(counts[2]))
        rays += req_rays[-1]
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream

    # the per-frame path: one launch per request, in order
    def per_frame():
        for r, (fr, acc) in zip(reqs, bufs):
            if r.fp.pt_on:
                ctx.render_pt(r.scene_id, r.fp, acc.data_ptr(), fr.data_ptr(), sp)
            else:
                ctx.render_device(r.scene_id, r.fp, fr.data_ptr(), sp)
    per_frame()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    per_frame()
    e1.record(stream)
    torch.cuda.synchronize()
    t_frames = e0.elapsed_time(e1) / 1000.0

    b = qr.Batch(ctx, len(reqs))
    b.set(reqs[:32])                # the autotuner times a 32-request sample
    tw, grab, tune_ms = b.tune()
    b.set(reqs)
    for _ in range(args.warmup):
        b.launch(sp)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    l0 = qr.kernel_launches()
    for i in range(args.steps):
        ev[i][0].record(stream)
        b.launch(sp)
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    launches = qr.kernel_launches() - l0
    ck = clocks.stop()
    ms = [a.elapsed_time(c) for a, c in ev]
    value, t_total = whole_job(rays, args.steps, sum(ms) / 1000.0, dist, "cuda")

    # each class alone (Whitted requests, path-traced requests): one batch
    # against one launch per request, device time of one pass after a warm-up
    classes = {}
    for name, pick in (("whitted", lambda r: not r.fp.pt_on), ("path_traced", lambda r: r.fp.pt_on)):
        idx = [i for i, r in enumerate(reqs) if pick(r)]
        sub = [reqs[i] for i in idx]
        bc = qr.Batch(ctx, len(sub))
        bc.config(tw, grab)
        bc.set(sub)
        bc.launch(sp)
        torch.cuda.synchronize()
        c0, c1, c2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        c0.record(stream)
        bc.launch(sp)
        c1.record(stream)
        for i in idx:
            r, (fr, acc) = reqs[i], bufs[i]
            if r.fp.pt_on:
                ctx.render_pt(r.scene_id, r.fp, acc.data_ptr(), fr.data_ptr(), sp)
            else:
                ctx.render_device(r.scene_id, r.fp, fr.data_ptr(), sp)
        c2.record(stream)
        torch.cuda.synchronize()
        bc.close()
        crays = sum(req_rays[i] for i in idx)
        tb, tf = c0.elapsed_time(c1) / 1000.0, c1.elapsed_time(c2) / 1000.0
        classes[name] = {"requests": len(idx), "rays": crays,
                         "batch_rays_per_s": crays / tb, "per_frame_rays_per_s": crays / tf,
                         "batch_over_per_frame": tf / tb}

    # end to end: request table in, batch, every frame out to pinned memory
    hosts = [torch.empty(fr.shape, dtype=torch.int32, pin_memory=True) for fr, _ in bufs]
    d2h = sum(h.numel() * 4 for h in hosts)
    h2d = ctypes.sizeof(qr.QrRequest) * len(reqs)
    lat = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        b.set(reqs)
        b.launch(sp)
        for (fr, _), hb in zip(bufs, hosts):
            hb.copy_(fr, non_blocking=True)
        torch.cuda.synchronize()
        if i >= args.warmup:
            lat.append(time.perf_counter() - t0)
    b.close()
    npx = sum(rq["w"] * rq["h"] for rq in spec)
    line = {
        "metric": "rays_per_s", "value": value, "unit": "rays/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * t_total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "classes": classes,
        "config": {"workload": "batch", "requests": len(reqs),
                   "whitted": sum(1 for q in spec if not q["spp"]),
                   "path_traced": sum(1 for q in spec if q["spp"]),
                   "pixels": npx, "rays_per_batch": rays, "seeds": [wl["seed"], wl["seed"] + len(reqs) - 1],
                   "tile": [tw, 32 // tw], "tiles_per_claim": grab,
                   "l2": "inputs (scenes, frames, sums) far larger than L2",
                   "parallelism": "replicas" if world > 1 else "single"},
        "per_frame_path": {"value": rays / t_frames, "unit": "rays/s",
                           "ms": 1000.0 * t_frames, "launches": len(reqs)},
        "batch_over_per_frame": (rays / (t_total / args.steps)) / (rays / t_frames),
        "e2e": {"value": rays * len(lat) / sum(lat), "unit": "rays/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_p50": 1000.0 * float(np.percentile(lat, 50))},
        "gpu_launches": launches,
        "clocks": ck,
    }
    if rank == 0:
        print(json.dumps(line))
    ctx.close()



def whole_job(units_per_step, steps, t_local, dist=None, device="cpu"):
    """Replicas: every rank renders its own frames; the job's time is the
    slowest rank's and its throughput counts the units of all ranks."""
    world = 1
    t = t_local
    if dist is not None and dist.is_initialized():
        import torch
        world = dist.get_world_size()
        tt = torch.tensor([t_local], dtype=torch.float64, device=device)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t = float(tt.item())
    return units_per_step * steps * world / t, t


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(qr, wl, seconds=12.0):
    """The CPU restatement of the reference tracer on the host cores, on a
    bounded sample of rows of the workload: rows in a stride order over the
    whole frame, and for the animated workload over 8 frames spread over its
    animation (frame k of the sample takes rows k, k + 8, ... of that
    order); returns rays/s and the setup."""
    import build as oracle_build
    O = oracle_build.load_oracle()
    nfr = wl.get("frames", 1)
    times = [16 * int((i + 0.5) * nfr / 8) for i in range(8)] if wl["anim"] else [0]
    spp = wl.get("pt", 0)
    frames = []
    for t in times:
        g = qr.GenScene(wl["kind"], wl["seed"], wl["nq"], 0)
        f = qr.Flat(g, wl["w"], wl["h"], wl["fsaa"])
        desc, params = f.update(t, wl["depth"])
        if spp:
            params.pt_on, params.pts_c, params.seed, params.frame_idx = spp, 0.0, 1, 0
        frames.append((g, f, desc, params))
    params = frames[0][3]
    acc = np.zeros((params.y_res, params.x_row, 3), dtype=np.float32)
    cores = os.cpu_count() or 1
    out = np.zeros((params.y_res, params.x_row), dtype=np.uint32)
    # rows in a stride order spread over the whole frame (the top rows of a
    # frame are mostly background and would flatter the CPU)
    stride = 7919
    while math.gcd(stride, params.y_res) != 1:
        stride += 2
    nxt = [0]
    rows_done = [0]
    rays = [0]
    lock = threading.Lock()
    t_end = time.perf_counter() + seconds

    def worker():
        while time.perf_counter() < t_end:
            with lock:
                i = nxt[0]
                nxt[0] += 1
            _, _, desc, prm = frames[i % len(frames)]
            yy = ((i // len(frames)) * stride) % prm.y_res
            nr = ctypes.c_uint64()
            if spp:
                O.qr_oracle_pt(ctypes.addressof(desc), ctypes.addressof(prm),
                               acc.ctypes.data, out.ctypes.data, yy, yy + 1,
                               ctypes.byref(nr))
            else:
                O.qr_oracle_render(ctypes.addressof(desc), ctypes.addressof(prm),
                                   out.ctypes.data, yy, yy + 1, ctypes.byref(nr))
            with lock:
                rows_done[0] += 1
                rays[0] += nr.value

    t0 = time.perf_counter()
    th = [threading.Thread(target=worker) for _ in range(cores)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    dt = time.perf_counter() - t0
    what = ("rows of %d frames spread over the %d-frame animation" % (len(frames), nfr)
            if wl["anim"] else "rows of the frame")
    return {"value": rays[0] / dt, "unit": "rays/s", "cores": cores, "kind": "port",
            "sample": "%d %s, %dx%d (%.1f s, %d threads)" % (
                rows_done[0], what, wl["w"], wl["h"], dt, cores)}


def run_reference(args, wl):
    qr = importlib.import_module("quadray-engine_gb300")
    vals = []
    cb = None
    for _ in range(args.warmup):
        cpu_baseline(qr, wl, seconds=1.0)
    for _ in range(args.steps):
        cb = cpu_baseline(qr, wl, seconds=max(2.0, 20.0 / max(1, args.steps)))
        vals.append(cb["value"])
    v = statistics.median(vals)
    line = {"impl": "reference", "metric": "rays_per_s", "value": v, "unit": "rays/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "dtype": "f32", "data": "synthetic",
            "config": line_config(args.workload, wl, "reference", 1),
            "cpu_baseline": {"value": v, "unit": "rays/s", "cores": cb["cores"],
                             "kind": cb["kind"], "sample": cb["sample"]},
            "e2e": {"value": v, "unit": "rays/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def line_config(name, wl, impl, world):
    """a line's config: the workload's identity (config_of, the same in
    both arms) and how the arm timed it"""
    cfg = config_of(name, wl)
    if impl == "reference":
        cfg.update({"l2": "none: the scalar port on the host cores", "parallelism": "single"})
    else:
        cfg.update({"l2": "256 MiB buffer written between timed steps",
                    "parallelism": "replicas" if world > 1 else "single"})
    return cfg


def config_of(name, wl):
    """the workload's identity, the same in both arms' lines"""
    spp = wl.get("pt", 0)
    return {"workload": name, "width": wl["w"], "height": wl["h"], "fsaa": wl["fsaa"],
            "quadrics": wl["nq"], "seed": wl["seed"], "depth": wl["depth"],
            "animated": wl["anim"], "frames": wl.get("frames", 1),
            "samples_per_pixel": spp if spp else (4 if wl["fsaa"] == 2 else 1)}


def frame_stats(qr, ctx, sid, params):
    """work counters of one frame (instrumented build of the same kernels)"""
    counts = (ctypes.c_uint64 * len(STAT_NAMES))()
    host = np.zeros((params.y_res, params.x_row), dtype=np.uint32)
    rc = qr.lib().qr_render_stats(ctx.h, sid, ctypes.byref(params),
                                  host.ctypes.data_as(ctypes.c_void_p), counts)
    assert rc == 0, ctx.error()
    return dict(zip(STAT_NAMES, (int(c) for c in counts)))


def rays_of(st):
    return st["ray_primary"] + st["ray_shadow"] + st["ray_secondary"]


def fp32_peaks(qr, local):
    """measured FP32 issue rates (TFLOP/s) of plain operations and of fused
    multiply-adds (qr_fp32_peak)"""
    out = {}
    for name, fma in (("plain", 0), ("fma", 1)):
        v = ctypes.c_double(0.0)
        rc = qr.lib().qr_fp32_peak(local, fma, ctypes.byref(v))
        out[name] = v.value if rc == 0 else None
    return out


REBUILD_EVERY = 32      # host update phases every 32nd frame of rt_Scene (engine.cpp)


def run_frames(args, wl, rank, world, dist, local):
    """one frame a step: the animated workload renders frames spread over its
    animation, each after its device-side update; plain and path-traced
    workloads render their frame"""
    import torch
    qr = importlib.import_module("quadray-engine_gb300")
    ctx = qr.Context(local)
    depth = wl["depth"]
    spp = wl.get("pt", 0)
    nfr = wl.get("frames", 1)
    K, W = args.steps, args.warmup

    def pt_params(p):
        if spp:
            p.pt_on, p.pts_c, p.seed, p.frame_idx = spp, 0.0, 1, 0
        return p

    # work counters of every frame of the workload (host update phases,
    # upload, instrumented render): rays per frame and algorithmic FLOPs
    sflat = qr.Flat(qr.GenScene(wl["kind"], wl["seed"], wl["nq"], 0), wl["w"], wl["h"],
                    wl["fsaa"])
    ssid = None
    per_frame = []
    scene_bytes = 0
    for j in range(nfr):
        desc, params = sflat.update(16 * j, depth)
        if ssid is None:
            ssid = ctx.upload(desc)
        else:
            ctx.update(ssid, desc)
        per_frame.append(frame_stats(qr, ctx, ssid, pt_params(params)))
        scene_bytes = (desc.nsrf * 256 + desc.nmat * 112 + desc.nlgt * 48 +
                       desc.nelem * 16 + desc.nlelem * 16 + desc.ntex * 4)
    nsrf = int(desc.nsrf)

    # timed frames: spread over the animation (the first warm-up frames
    # untimed); a frame j of an animated scene is rendered as rt_Scene does
    # in its steady state: the scene prepared by the host update phases at
    # the last rebuild frame j0 = 32 floor(j / 32) (untimed: the input
    # arriving), then the device-side update to frame j and the render
    timed = [int((i + 0.5) * nfr / K) for i in range(K)] if wl["anim"] else [0] * K
    warm = list(range(min(W, nfr))) if wl["anim"] else [0] * W
    warm += [warm[-1]] * (W - len(warm))
    dflat = qr.Flat(qr.GenScene(wl["kind"], wl["seed"], wl["nq"], 0), wl["w"], wl["h"],
                    wl["fsaa"])
    dsid = [None]
    if not wl["anim"]:
        desc, params = dflat.update(0, depth)
        dsid[0] = ctx.upload(desc)
        fixed = pt_params(qr.QrFrameParams.from_buffer_copy(params))

    def prepare(j):
        """untimed: the scene state of the last rebuild before frame j;
        returns the device update's parameters and the frame parameters"""
        if not wl["anim"]:
            return None, fixed
        # the in-place upload rewrites the scene's block: the previous
        # frame's render (on another stream) must have finished reading it
        torch.cuda.synchronize()
        j0 = REBUILD_EVERY * (j // REBUILD_EVERY)
        desc, _ = dflat.update(16 * j0, depth)
        table = dflat.anim_table()
        if dsid[0] is None:
            dsid[0] = ctx.anim_upload(desc, table)
        else:
            ctx.anim_init(dsid[0], desc, table)
        rc, prm = dflat.anim_params(16 * j)
        assert rc == 0, rc
        return prm, pt_params(dflat.frame_params())

    x_row = int(params.x_row)           # the same for every frame of the workload
    assert x_row >= wl["w"] and params.y_res == wl["h"]
    frame = torch.empty((wl["h"], x_row), dtype=torch.int32, device="cuda")
    acc = torch.empty((wl["h"], x_row, 3), dtype=torch.float32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream

    def step(prm, fp):
        assert fp.x_row == x_row and fp.y_res == wl["h"]
        if prm is not None:
            ctx.anim_update(dsid[0], prm, sp)
        if spp:
            ctx.render_pt(dsid[0], fp, acc.data_ptr(), frame.data_ptr(), sp)
        else:
            ctx.render_device(dsid[0], fp, frame.data_ptr(), sp)

    for j in warm:
        prm, fp = prepare(j)
        step(prm, fp)
    torch.cuda.synchronize()

    if dist is not None:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(K)]
    torch.cuda.synchronize()
    launches = 0                        # the library's kernels in the timed steps
    for i, j in enumerate(timed):
        prm, fp = prepare(j)
        flush.zero_()
        ev[i][0].record(stream)
        l0 = qr.kernel_launches()
        step(prm, fp)
        launches += qr.kernel_launches() - l0
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    ck = clocks.stop()
    ms = [a.elapsed_time(b) for a, b in ev]
    rays = sum(rays_of(per_frame[j]) for j in timed) / K          # per frame (mean)
    value, t_total = whole_job(rays, K, sum(ms) / 1000.0, dist, "cuda")
    if dist is not None:
        dist.barrier()
    fps = K * world / t_total
    anim_status = ctx.anim_status(dsid[0]) if wl["anim"] else None
    # the timed frames' work as rendered (the refitted hierarchy of a
    # device-updated frame tests more boxes than a fresh one; the traced
    # segments are the same)
    tstats = []
    for j in sorted(set(timed)):
        prm, fp = prepare(j)
        if prm is not None:
            ctx.anim_update(dsid[0], prm, sp)
            torch.cuda.synchronize()
        st = frame_stats(qr, ctx, dsid[0], fp)
        assert rays_of(st) == rays_of(per_frame[j]), j
        tstats += [st] * timed.count(j)
    stats = dict((k, sum(st[k] for st in tstats) / K) for k in STAT_NAMES)
    flops = sum(stats[k] * v for k, v in FLOPS.items())

    # end to end through the engine API (rt_Scene::render(time)) into the
    # caller's host frame: the animated workload renders its whole
    # animation in order and times every frame after the warm-up ones, so
    # the host rebuild of every 32nd frame and the loosening of the refitted
    # hierarchy between rebuilds are inside; other workloads render K frames
    eng = qr.Engine(qr.GenScene(wl["kind"], wl["seed"], wl["nq"], 0), wl["w"], wl["h"],
                    fsaa=wl["fsaa"], depth=depth, pton=spp)
    e2e_frames = list(range(nfr)) if wl["anim"] else [0] * (W + K)
    lat = []
    for n, j in enumerate(e2e_frames):
        t0 = time.perf_counter()
        eng.render(16 * j)                      # into the caller-owned host frame
        if n >= W:
            lat.append(time.perf_counter() - t0)
    eng.close()
    e2e_timed = e2e_frames[W:]
    e2e_rays = sum(rays_of(per_frame[j]) for j in e2e_timed)
    if wl["anim"]:
        nparams = len(dflat.anim_params(0)[1])
        # the animated transforms each frame (48 bytes each); the whole
        # scene on the frames of a host rebuild
        h2d = sum(scene_bytes if j % REBUILD_EVERY == 0 else 48 * nparams
                  for j in e2e_timed) / len(e2e_timed)
    else:
        h2d = 0                                 # the scene stays resident
    d2h = wl["w"] * wl["h"] * 4

    # FP32 issue rates measured on this device: the bit-exact arithmetic
    # issues no fused multiply-add, so the plain rate is the roofline; the
    # FMA rate is reported beside it
    pk = fp32_peaks(qr, local)
    achieved = flops * K / t_total / 1e12
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "dram_traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as fh:
            traffic = json.load(fh).get(args.workload, {}).get("bytes_per_launch")
    roof = {"bound": "fp32", "achieved": achieved, "peak": pk["plain"], "unit": "TFLOP/s",
            "frac": achieved / pk["plain"] if pk["plain"] else None, "traffic": traffic,
            "peak_fma": pk["fma"], "frac_fma": achieved / pk["fma"] if pk["fma"] else None,
            "peak_source": "measured on this device (qr_fp32_peak): FP32 additions, every "
                           "SM filled, CUDA events; peak_fma: fused multiply-adds as 2 ops",
            "flops_per_frame": flops}
    # config: the workload's identity (the reference arm's line carries the
    # same keys and values) and how it was timed; the measured workload
    # quantities go beside it
    cfg = line_config(args.workload, wl, "ours", world)
    line = {
        "metric": "rays_per_s", "value": value, "unit": "rays/s",
        "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": 1000.0 * t_total / K,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": cfg,
        "workload": {"surfaces": nsrf, "rays_per_frame": rays,
                     "timed_frames": timed if wl["anim"] else None},
        "step": ("device-side update of the animated transforms + render of the frame"
                 if wl["anim"] else "render of the frame"),
        "frames_per_s": fps,
        "frame_ms_p50": float(np.percentile(ms, 50)),
        "frame_ms_p99": float(np.percentile(ms, 99)),
        "e2e": {"value": e2e_rays / sum(lat), "unit": "rays/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "frames": len(lat),
                "host_rebuilds": sum(1 for j in e2e_timed if j % REBUILD_EVERY == 0)
                if wl["anim"] else 0,
                "frame_ms_p50": 1000.0 * float(np.percentile(lat, 50)),
                "frame_ms_p99": 1000.0 * float(np.percentile(lat, 99))},
        "roofline": roof,
        "work_per_frame": stats,
        "anim_status": anim_status,
        "gpu_launches": launches,
        "clocks": ck,
    }
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(qr, wl)
    if rank == 0:
        print(json.dumps(line))
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="anim", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--serve-rates", default="",
                    help="serve: arrival rates per second, comma-separated")
    ap.add_argument("--serve-seconds", type=float, default=0.0,
                    help="serve: seconds of arrivals per rate")
    ap.add_argument("--serve-batch-px", type=int, default=24 << 20,
                    help="serve: pixels of a batched launch at most")
    ap.add_argument("--serve-urgent", action="store_true",
                    help="serve: 1080p Whitted requests in batches of their own on a "
                         "high-priority stream")
    ap.add_argument("--serve-urgent-px", type=int, default=0,
                    help="serve: pixels of an urgent batch at most (default: as the others)")
    ap.add_argument("--serve-urgent-batches", type=int, default=2,
                    help="serve: urgent batches in flight at most")
    ap.add_argument("--serve-host-update", action="store_true",
                    help="serve: update animated scenes on the host (update phases, "
                         "hierarchy build and upload per request) instead of the device")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    wl = WORKLOADS[args.workload]

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank == 0:
            run_reference(args, wl)
        return

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    if wl.get("serve"):
        run_serve(args, wl, rank, world, dist, local)
        if dist is not None:
            dist.destroy_process_group()
        return
    if wl.get("batch"):
        run_batch(args, wl, rank, world, dist, local)
        if dist is not None:
            dist.destroy_process_group()
        return

    run_frames(args, wl, rank, world, dist, local)
    if dist is not None:
        dist.destroy_process_group()

if __name__ == "__main__":
    main()
