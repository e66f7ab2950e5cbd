"""Replica path of bench.py on CPU: world size 2 over gloo.

Multi-GPU runs are replicas only (every rank renders whole frames of its own
scene copy, no collective on the data path); the only exchange is the max of
the ranks' timed regions.  Here two gloo ranks each render rows of a frame
with the oracle (standing in for the device render) and agree on the job
throughput.
"""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    import sys
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import importlib
    import ctypes
    import numpy as np
    import bench
    import build as oracle_build
    qr = importlib.import_module("quadray-engine_gb300")
    O = oracle_build.load_oracle()
    g = qr.GenScene(qr.SCN_PLAIN, 1, 16)
    f = qr.Flat(g, 64, 40)
    desc, params = f.update(0, 10)
    out = np.zeros((params.y_res, params.x_row), dtype=np.uint32)
    nr = ctypes.c_uint64()
    O.qr_oracle_render(ctypes.addressof(desc), ctypes.addressof(params),
                       out.ctypes.data, 0, params.y_res, ctypes.byref(nr))
    # rank r reports a timed region of (1 + r) s
    value, t = bench.whole_job(nr.value, 3, 1.0 + rank, dist)
    digest = int(out[:, :params.x_res].astype(np.uint64).sum())
    q.put((rank, value, t, nr.value, digest))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_gloo():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    rays = res[0][3]
    assert rays > 0 and all(r[3] == rays for r in res)
    assert all(r[4] == res[0][4] for r in res)         # identical replica frames
    for _, value, t, _, _ in res:
        assert t == pytest.approx(2.0)                  # slowest rank
        assert value == pytest.approx(rays * 3 * world / 2.0)


def test_single_process_whole_job():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    v, t = bench.whole_job(100, 4, 2.0)
    assert t == 2.0 and v == 200.0
