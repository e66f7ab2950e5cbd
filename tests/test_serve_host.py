"""Host logic of the frame server (quadray-engine_gb300/serve.py) on the CPU:
admission by the memory budget, continuous batching, completion of each
request on its own completion word, recycling of batches and scene copies.
The scene updates, uploads and batched launches are fakes; the device side is
covered by tests/test_gpu_serve.py."""
import ctypes
import importlib
import itertools

import pytest

serve = importlib.import_module("quadray-engine_gb300.serve")


class FakeParams:
    def __init__(self):
        self.pt_on, self.pts_c, self.seed, self.frame_idx, self.x_row = 0, 0.0, 0, 0, 0

    @classmethod
    def from_buffer_copy(cls, other):
        p = cls()
        p.__dict__.update(other.__dict__)
        return p


class FakeRequest:
    def __init__(self):
        self.scene_id = self.pad = 0
        self.fp = None
        self.dev_frame = self.dev_acc = None


class FakeFlat:
    def __init__(self, gen, w, h, fsaa):
        self.key = (gen, w, h, fsaa)

    def update(self, time, depth):
        return ("desc", time), FakeParams()


class FakeBatch:
    """each poll completes one more request, in the order given by the
    test's `order` function, and reports the batch done when all are (a
    test may hold it running with a non-index entry in `pending`)"""
    log = []

    def __init__(self, ctx, max_requests):
        self.max = max_requests
        self.flags = (ctypes.c_uint32 * max_requests)()
        self.table = []
        self.pending = []

    def set(self, table):
        assert len(table) <= self.max
        self.table = list(table)

    def persistent(self, on):
        self.is_persistent = on

    def launch(self, stream):
        for i in range(self.max):
            self.flags[i] = 0
        self.pending = FakeBatch.order(len(self.table))
        FakeBatch.log.append([q.scene_id for q in self.table])

    def done_flags(self, n):
        return (ctypes.c_uint32 * n).from_buffer(self.flags)

    def poll(self):
        if self.pending and isinstance(self.pending[0], int):
            self.flags[self.pending.pop(0)] = 1
        return not self.pending

    def close(self):
        pass


class FakeQr:
    QrFrameParams = FakeParams
    QrRequest = FakeRequest
    Flat = FakeFlat
    Batch = FakeBatch


class FakeCtx:
    def __init__(self):
        self.ids = itertools.count(1)
        self.uploads = self.updates = 0

    def upload(self, desc):
        self.uploads += 1
        return next(self.ids)

    def update(self, sid, desc):
        self.updates += 1


class FakeTensor:
    def data_ptr(self):
        return 0x1000


class HostServer(serve.Server):
    def _new_stream(self, priority=0):
        class S:
            cuda_stream = 1 if priority else 0
        return S()

    def _alloc(self, req, pt):
        req.frame = FakeTensor()
        req.acc = FakeTensor() if pt else None


def _server(budget, max_batch=4, per_request=True, urgent=None):
    scenes = [dict(gen="g%d" % i, pt=(i == 2), depth=4) for i in range(3)]
    return HostServer(FakeQr, FakeCtx(), scenes, budget_bytes=budget, max_batch=max_batch,
                      prep_threads=2, per_request=per_request, urgent=urgent)


def _requests(n, w=64, h=48, spp=1):
    return [serve.Request(i, i % 3, 16 * i, w, h, spp, 0.0005 * i) for i in range(n)]


def test_every_request_completes_once():
    FakeBatch.order = lambda n: list(range(n))
    srv = _server(1 << 30)
    reqs = _requests(20)
    done, wall = srv.run(reqs)
    assert sorted(r.rid for r in done) == list(range(20))
    assert all(r.done is not None and r.done >= r.arrival for r in done)
    assert all(r.prepared is not None and r.arrival <= r.prepared <= r.done for r in done)
    assert srv.used == 0 and not srv.busy()
    srv.close()


def test_budget_bounds_requests_in_flight():
    """a budget for two requests: never more than two hold memory, and
    requests are admitted in arrival order"""
    FakeBatch.order = lambda n: list(range(n))
    FakeBatch.log = []
    srv = _server(2 * (64 * 48 * 4 + (1 << 20)))
    peak = []
    orig = srv._admit

    def admit():
        orig()
        peak.append(srv.used)
    srv._admit = admit
    reqs = [serve.Request(i, 0, 16 * i, 64, 48, 1, 0.0) for i in range(7)]
    done, wall = srv.run(reqs)
    assert max(peak) <= 2 * (64 * 48 * 4 + (1 << 20))
    assert sorted(r.rid for r in done) == list(range(7))
    assert all(len(t) <= 2 for t in FakeBatch.log)
    srv.close()


def test_requests_complete_on_their_own_word():
    """a request of a running batch completes as soon as its word is set;
    with batch completion it waits for the whole batch"""
    import numpy as np
    for per_request in (True, False):
        srv = _server(1 << 30, max_batch=4, per_request=per_request)
        b = srv.free_batches.popleft()
        reqs = [serve.Request(i, 0, 0, 32, 24, 1, 0.0) for i in range(4)]
        for r in reqs:
            r.bytes, r.slot = 1000, 100 + r.rid
            srv.used += r.bytes
        b.pending = ["running"]                 # poll: not finished
        flags = np.frombuffer(b.done_flags(4), dtype=np.uint32)
        srv.inflight.append((b, reqs, flags, srv.free_batches))
        b.flags[2] = 1
        srv._complete(lambda: 1.0)
        assert [r.rid for r in srv.completed] == ([2] if per_request else [])
        b.pending = []
        for i in range(4):
            b.flags[i] = 1
        srv._complete(lambda: 2.0)
        assert sorted(r.rid for r in srv.completed) == [0, 1, 2, 3]
        assert {r.rid: r.done for r in reqs} == (
            {0: 2.0, 1: 2.0, 2: 1.0, 3: 2.0} if per_request else {i: 2.0 for i in range(4)})
        assert srv.used == 0 and not srv.inflight and b in srv.free_batches
        assert sorted(srv.slots[0]) == [100, 101, 102, 103]
        srv.close()


def test_urgent_requests_get_batches_of_their_own():
    """urgent requests go into batches of their own, launched on the
    high-priority stream ahead of the others; every request completes once
    and batches of both pools come back to their pools"""
    FakeBatch.order = lambda n: list(range(n))
    launched = []
    orig = FakeBatch.launch

    def launch(self, stream):
        launched.append((stream, [q.fp.urgent for q in self.table]))
        orig(self, stream)
    FakeBatch.launch = launch
    try:
        srv = _server(1 << 30, max_batch=4, urgent=lambda r: r.w == 128)
        reqs = [serve.Request(i, i % 2, 16 * i, 128 if i % 3 == 0 else 64, 48, 1, 0.0)
                for i in range(12)]
        orig_prep = srv._prepare

        def prepare(req):
            r = orig_prep(req)
            r.fp.urgent = req.w == 128
            return r
        srv._prepare = prepare
        done, wall = srv.run(reqs)
    finally:
        FakeBatch.launch = orig
    assert sorted(r.rid for r in done) == list(range(12))
    for stream, flags in launched:
        assert all(flags) if stream == 1 else not any(flags)
    assert any(s == 1 for s, _ in launched) and any(s == 0 for s, _ in launched)
    assert len(srv.free_batches) == 2 and len(srv.free_ubatches) == 2
    # the other batches yield their SMs between blocks
    assert all(b.is_persistent is False for b in srv.batches)
    assert srv.used == 0 and not srv.busy()
    srv.close()


def test_scene_copies_are_reused():
    """after the first round every scene copy comes back to its pool: later
    requests of a scene update a copy in place instead of uploading one"""
    FakeBatch.order = lambda n: list(range(n))
    srv = _server(1 << 30, max_batch=2)
    srv.run([serve.Request(i, 0, 16 * i, 32, 24, 1, 0.0) for i in range(2)])
    up = srv.ctx.uploads
    srv.run([serve.Request(10 + i, 0, 16 * i, 32, 24, 1, 0.0) for i in range(2)])
    assert srv.ctx.uploads == up and srv.ctx.updates >= 2
    srv.close()


def test_path_traced_requests_get_sums_and_their_samples():
    FakeBatch.order = lambda n: list(range(n))
    srv = _server(1 << 30)
    reqs = [serve.Request(i, 2, 0, 40, 30, 5, 0.0) for i in range(3)]
    done, wall = srv.run(reqs, keep_frames=True)
    for r in done:
        assert r.acc is not None and r.fp.pt_on == 5 and r.fp.frame_idx == r.rid
    srv.close()


def test_request_over_budget_is_refused():
    FakeBatch.order = lambda n: list(range(n))
    srv = _server(1 << 20)
    with pytest.raises(ValueError):
        srv.run([serve.Request(0, 0, 0, 1920, 1080, 1, 0.0)])
    srv.close()


class FakeAnimFlat(FakeFlat):
    """an animated scene: the table is taken after an update; the animators
    keep their free rotation until time `lose`"""
    lose = 10 ** 9

    def __init__(self, gen, w, h, fsaa):
        super().__init__(gen, w, h, fsaa)
        self.updated = False
        self.tables = 0

    def update(self, time, depth):
        self.updated = True
        return super().update(time, depth)

    def anim_table(self):
        assert self.updated
        self.tables += 1
        return ["entry"]

    def anim_params(self, time):
        return (1 if time >= FakeAnimFlat.lose else 0), ["param"]

    def frame_params(self):
        return FakeParams()


class FakeAnimCtx(FakeCtx):
    def __init__(self):
        super().__init__()
        self.inits = self.anim_updates = 0

    def anim_init(self, sid, desc, table):
        self.inits += 1

    def anim_upload(self, desc, table):
        self.inits += 1
        self.uploads += 1
        return next(self.ids)

    def anim_update_many(self, updates, stream):
        assert len(set(sid for sid, _ in updates)) == len(updates)
        self.anim_updates += len(updates)


class FakeAnimQr(FakeQr):
    Flat = FakeAnimFlat


def test_animated_scenes_update_on_the_device():
    """the first request of a scene copy runs the host update phases and
    prepares the copy for device updates; later requests on that copy run
    only the animators and one device update; when an animated transform
    loses its free rotation the host phases run again with a new table"""
    FakeBatch.order = lambda n: list(range(n))
    scenes = [dict(gen="g0", pt=False, depth=4, anim=True)]
    ctx = FakeAnimCtx()
    srv = HostServer(FakeAnimQr, ctx, scenes, budget_bytes=1 << 30, max_batch=1,
                     prep_threads=1, device_anim=True)
    # arrivals 20 ms apart: each request finds the previous one's copy free
    reqs = [serve.Request(i, 0, 16 * i, 32, 24, 1, 0.02 * i) for i in range(5)]
    done, _ = srv.run(reqs)
    assert sorted(r.rid for r in done) == list(range(5))
    assert ctx.uploads == 1 and ctx.inits == 1 and ctx.updates == 0
    assert ctx.anim_updates == 4 and srv.device_updates == 4 and srv.host_updates == 1
    FakeAnimFlat.lose = 16 * 7
    srv.run([serve.Request(10 + i, 0, 16 * (5 + i), 32, 24, 1, 0.02 * i) for i in range(4)])
    # times 80, 96 on the device; 112 loses the rotation: host phases and a
    # new table (which the fake accepts again), then 128 fails the same way
    assert ctx.anim_updates == 6 and srv.host_updates == 3 and ctx.inits == 3
    assert srv.flats[(0, 32, 24, 0)].tables == 3
    FakeAnimFlat.lose = 10 ** 9
    srv.close()


def test_device_updated_copies_are_rebuilt_periodically():
    FakeBatch.order = lambda n: list(range(n))
    scenes = [dict(gen="g0", pt=False, depth=4, anim=True)]
    ctx = FakeAnimCtx()
    srv = HostServer(FakeAnimQr, ctx, scenes, budget_bytes=1 << 30, max_batch=1,
                     prep_threads=1, device_anim=True, rebuild_every=3)
    srv.run([serve.Request(i, 0, 16 * i, 32, 24, 1, 0.02 * i) for i in range(9)])
    # host, 3 device, host, 3 device, host
    assert srv.host_updates == 3 and srv.device_updates == 6 and ctx.inits == 3
    srv.close()
