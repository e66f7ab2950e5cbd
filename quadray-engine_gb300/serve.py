"""Frame server: continuous batching of frame requests on device-resident
scenes.

The reference renders one frame per rt_Scene::render call on a CPU thread
pool (core/engine/engine.cpp:3014) and has no server.  This module serves
many clients from one GPU:

* scenes stay resident; each request names a scene, an animation time, a
  frame size and a sampling (Whitted: 1 sample or the reference's 4x AA;
  path tracer: pt_on samples);
* admission: a request is admitted when its device memory (frame, path-
  tracer sums, its version of the scene) fits the HBM budget; otherwise it
  waits;
* admitted requests are prepared on host threads: the scene's update phases
  at the request's time (animators, transforms, lists, the hierarchy) and an
  in-place upload into a pooled device copy of that scene; or, for animated
  scenes whose copy was prepared for it, only the animators on the host and
  the rest of the update phases on the device (qr_scene_anim_update_many:
  the scene updates of a batch in one launch on the serving stream, ahead
  of the batch);
* continuous batching: prepared requests go into the next batched launch
  (qr_batch_*), two batches in flight so the GPU never waits for the host;
  requests that arrive while a batch runs join the following one;
* a request completes when its own frame does (the batch's per-request
  completion words), not when its whole batch does;
* every frame equals the frame of the same request rendered alone.

Latency is arrival to completion (the request's completion word, seen by
polling).
"""
import collections
import ctypes
import threading
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np


class Request:
    """One frame request."""

    __slots__ = ("rid", "scene", "time", "w", "h", "spp", "arrival", "done",
                 "frame", "acc", "slot", "bytes", "fp", "flat_key", "prepared", "anim")

    def __init__(self, rid, scene, time_ms, w, h, spp, arrival):
        self.rid, self.scene, self.time = rid, scene, time_ms
        self.w, self.h, self.spp = w, h, spp
        self.arrival = arrival
        self.done = None
        self.prepared = None
        self.frame = self.acc = None
        self.slot = None
        self.bytes = 0
        self.fp = None
        self.flat_key = None
        self.anim = None                # animators' transforms for a device update


class Server:
    """Continuous-batching frame server over one context."""

    def __init__(self, qr, ctx, scenes, budget_bytes=120 << 30, max_batch=64,
                 max_batch_pixels=24 << 20, prep_threads=4, per_request=True,
                 device_anim=False, rebuild_every=32, urgent=None,
                 urgent_batch_pixels=None, urgent_batches=2):
        """scenes: list of dicts with keys gen (a GenScene), pt (path-traced
        scene), depth and anim (animated); per_request: complete each request
        when its frame is done (else when its batch is); device_anim: update
        animated scenes on the device (qr_scene_anim_*) where they allow it;
        urgent: a predicate on requests whose latency has a target (e.g.
        1080p Whitted frames): prepared urgent requests go into batches of
        their own (urgent_batches of them, of urgent_batch_pixels at most,
        default max_batch_pixels) on a stream of the highest priority"""
        self.per_request = per_request
        self.device_anim = device_anim
        self.tables = {}                # (scene, w, h, fsaa) -> update table or None
        # scene copies prepared for device updates -> device updates since:
        # the hierarchy keeps its first frame's tree and only refits its
        # boxes, which loosens as animated subtrees move, so every
        # rebuild_every updates the copy takes the host phases again
        self.anim_slots = {}
        self.rebuild_every = rebuild_every
        self.device_updates = self.host_updates = 0
        self.qr, self.ctx = qr, ctx
        self.scenes = scenes
        self.budget = budget_bytes
        self.used = 0
        self.max_batch = max_batch
        self.max_batch_pixels = max_batch_pixels
        self.pool = ThreadPoolExecutor(max_workers=prep_threads)
        self.locks = [threading.Lock() for _ in scenes]
        self.flats = {}                 # (scene, w, h, fsaa) -> Flat
        self.slots = [collections.deque() for _ in scenes]   # free scene copies
        self.slot_bytes = {}
        self.stream = self._new_stream()
        self.batches = [qr.Batch(ctx, max_batch), qr.Batch(ctx, max_batch)]
        self.free_batches = collections.deque(self.batches)
        # urgent requests: batches of their own on a stream of the highest
        # priority, so that their blocks take the SMs as soon as a running
        # batch frees them, ahead of the batches queued on the other stream
        self.ustream = self._new_stream(priority=-1) if urgent is not None else None
        self.ubatches = ([qr.Batch(ctx, max_batch) for _ in range(urgent_batches)]
                         if urgent is not None else [])
        self.urgent_batch_pixels = urgent_batch_pixels or max_batch_pixels
        self.free_ubatches = collections.deque(self.ubatches)
        if urgent is not None:
            # the other batches' blocks retire as they finish, so that an
            # urgent batch's blocks take their SMs at once
            for b in self.batches:
                b.persistent(False)
        self.waiting = collections.deque()      # arrived, not admitted
        self.preparing = []                      # futures
        self.ready = collections.deque()         # prepared, not launched
        self.ready_urgent = collections.deque()  # the same, urgent ones
        self.urgent = urgent
        self.inflight = collections.deque()      # (batch, [requests], words, pool)
        self.completed = []
        self.idle_sleep = 100e-6

    # ---- device memory ------------------------------------------------
    def _new_stream(self, priority=0):
        import torch
        return torch.cuda.Stream(priority=priority)

    def _alloc(self, req, pt):
        """the request's frame (and path-tracer sums) in device memory"""
        import torch
        req.frame = torch.empty((req.h, req.w), dtype=torch.int32, device="cuda")
        if pt:
            req.acc = torch.empty((req.h, req.w, 3), dtype=torch.float32, device="cuda")

    # ---- preparation --------------------------------------------------
    def _fsaa(self, req):
        return 0 if (self.scenes[req.scene]["pt"] or req.spp <= 1) else 2

    def _prepare(self, req):
        """the scene at the request's time in a device copy of its own: on
        the device (the animators' transforms and one update launch on the
        serving stream) when the copy was prepared for it, else by the host
        update phases and an upload"""
        qr = self.qr
        sc = self.scenes[req.scene]
        fsaa = self._fsaa(req)
        key = (req.scene, req.w, req.h, fsaa)
        dev = self.device_anim and sc.get("anim", False)
        with self.locks[req.scene]:
            flat = self.flats.get(key)
            if flat is None:
                flat = qr.Flat(sc["gen"], req.w, req.h, fsaa)
                self.flats[key] = flat
            fp = None
            refresh = False
            if dev and self.tables.get(key) is not None and req.slot in self.anim_slots \
                    and self.anim_slots[req.slot] < self.rebuild_every:
                rc, prm = flat.anim_params(req.time)
                refresh = rc != 0       # the table no longer fits the scene
                if rc == 0:
                    # the update runs with the others of the request's batch
                    req.anim = prm
                    fp = qr.QrFrameParams.from_buffer_copy(flat.frame_params())
                    self.device_updates += 1
                    self.anim_slots[req.slot] += 1
            if fp is None:
                desc, params = flat.update(req.time, sc["depth"])
                fp = qr.QrFrameParams.from_buffer_copy(params)
                table = None
                if dev:
                    if key not in self.tables or refresh:
                        try:
                            self.tables[key] = flat.anim_table()
                        except ValueError:
                            self.tables[key] = None
                    table = self.tables[key]
                if table is not None:
                    if req.slot is None:
                        req.slot = self.ctx.anim_upload(desc, table)
                    else:
                        self.ctx.anim_init(req.slot, desc, table)
                    self.anim_slots[req.slot] = 0
                else:
                    if req.slot is None:
                        req.slot = self.ctx.upload(desc)
                    else:
                        self.ctx.update(req.slot, desc)
                    self.anim_slots.pop(req.slot, None)
                self.host_updates += 1
        if sc["pt"]:
            fp.pt_on, fp.pts_c, fp.seed, fp.frame_idx = req.spp, 0.0, 0x5E, req.rid
        req.fp = fp
        return req

    def need_bytes(self, req):
        """device memory a request holds while in flight: frame, path-tracer
        sums, and (an allowance of 1 MiB for) its version of the scene"""
        pt = self.scenes[req.scene]["pt"]
        return req.w * req.h * 4 * (4 if pt else 1) + (1 << 20)

    def _admit(self):
        while self.waiting:
            req = self.waiting[0]
            pt = self.scenes[req.scene]["pt"]
            need = self.need_bytes(req)
            if self.used + need > self.budget:
                break
            self.waiting.popleft()
            self.used += need
            req.bytes = need
            self._alloc(req, pt)
            if self.slots[req.scene]:
                req.slot = self.slots[req.scene].popleft()
            self.preparing.append(self.pool.submit(self._prepare, req))

    def _collect_prepared(self, now_fn):
        keep = []
        for f in self.preparing:
            if f.done():
                r = f.result()
                r.prepared = now_fn()
                if self.urgent is not None and self.urgent(r):
                    self.ready_urgent.append(r)
                else:
                    self.ready.append(r)
            else:
                keep.append(f)
        self.preparing = keep

    # ---- batches ------------------------------------------------------
    def _launch(self):
        if self.urgent is None:
            self._launch_from((self.ready_urgent, self.ready), self.free_batches, self.stream,
                              self.max_batch_pixels)
        else:
            self._launch_from((self.ready_urgent,), self.free_ubatches, self.ustream,
                              self.urgent_batch_pixels)
            self._launch_from((self.ready,), self.free_batches, self.stream,
                              self.max_batch_pixels)

    def _launch_from(self, queues, free, stream, max_px):
        qr = self.qr
        while any(queues) and free:
            reqs, px = [], 0
            for q in queues:
                while q and len(reqs) < self.max_batch:
                    r = q[0]
                    if reqs and px + r.w * r.h > max_px:
                        break
                    q.popleft()
                    reqs.append(r)
                    px += r.w * r.h
            table = []
            for r in reqs:
                q = qr.QrRequest()
                q.scene_id = r.slot
                q.fp = r.fp
                q.fp.x_row = r.w
                q.dev_frame = r.frame.data_ptr()
                q.dev_acc = r.acc.data_ptr() if r.acc is not None else None
                table.append(q)
            b = free.popleft()
            b.set(table)
            ups = [(r.slot, r.anim) for r in reqs if r.anim is not None]
            if ups:
                # the batch's scene updates: one launch ahead of the batch
                self.ctx.anim_update_many(ups, stream.cuda_stream)
                for r in reqs:
                    r.anim = None
            b.launch(stream.cuda_stream)
            flags = np.frombuffer(b.done_flags(len(reqs)), dtype=np.uint32)
            self.inflight.append((b, reqs, flags, free))

    def _finish(self, r, t):
        r.done = t
        self.used -= r.bytes
        self.slots[r.scene].append(r.slot)
        self.completed.append(r)

    def _complete(self, now_fn):
        # each request completes when its own frame is done (the batch's
        # per-request completion words), its batch is recycled when all are
        t = None
        for b, reqs, flags, _ in (self.inflight if self.per_request else ()):
            if b is None:               # recycled: its words belong to a new launch
                continue
            for i in np.flatnonzero(flags.copy()):    # a snapshot: the device
                                                      # writes the words live
                r = reqs[i]
                if r.done is None:
                    if t is None:
                        t = now_fn()
                    self._finish(r, t)
        # batches are recycled in order per stream; either stream's batch at
        # the head of the in-flight list may finish first
        for k in range(len(self.inflight)):
            b, reqs, flags, free = self.inflight[k]
            if b is None or not b.poll():
                continue
            for r in reqs:
                if r.done is None:
                    self._finish(r, now_fn())
            free.append(b)
            self.inflight[k] = (None, reqs, flags, free)
        while self.inflight and self.inflight[0][0] is None:
            self.inflight.popleft()

    def step(self, now_fn):
        """one turn of the loop; returns whether anything moved"""
        def count():
            return (len(self.completed) + len(self.waiting) + len(self.ready) +
                    len(self.ready_urgent) + len(self.inflight))
        n = count()
        self._complete(now_fn)
        self._admit()
        self._collect_prepared(now_fn)
        self._launch()
        return n != count()

    def busy(self):
        return bool(self.waiting or self.preparing or self.ready or self.ready_urgent or
                    self.inflight)

    def run(self, arrivals, keep_frames=False):
        """serve a list of Requests (their arrival in seconds from the
        start); returns the completed requests"""
        for r in arrivals:
            if self.need_bytes(r) > self.budget:
                raise ValueError("request %d needs %d bytes, more than the budget"
                                 % (r.rid, self.need_bytes(r)))
        pending = collections.deque(sorted(arrivals, key=lambda r: r.arrival))
        t0 = time.perf_counter()

        def now():
            return time.perf_counter() - t0

        while pending or self.busy():
            t = now()
            while pending and pending[0].arrival <= t:
                self.waiting.append(pending.popleft())
            moved = self.step(now)
            if not keep_frames:
                for r in self.completed:
                    r.frame = r.acc = None
            if not moved:
                # idle turn: sleep briefly (up to the next arrival) so that the
                # preparation threads get the interpreter lock at once instead
                # of after the interpreter's switch interval
                wait = self.idle_sleep
                if pending:
                    wait = min(wait, max(0.0, pending[0].arrival - now()))
                time.sleep(wait)
        done, self.completed = self.completed, []
        return done, now()

    def close(self):
        for b in self.batches + self.ubatches:
            b.close()
        self.pool.shutdown()


def poisson_requests(n_scenes, rate, duration, sizes, spp_max, seed, pt_scenes=()):
    """Poisson arrivals at `rate` per second over `duration` seconds; each
    request picks a scene, the scene's next animation frame (16 ms apart), a
    size and a sampling uniformly"""
    rng = np.random.default_rng(seed)
    t, out, nxt = 0.0, [], [0] * n_scenes
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            break
        s = int(rng.integers(0, n_scenes))
        w, h = sizes[int(rng.integers(0, len(sizes)))]
        spp = int(rng.integers(1, spp_max + 1))
        out.append(Request(len(out), s, 16 * nxt[s], w, h, spp, t))
        nxt[s] += 1
    return out
