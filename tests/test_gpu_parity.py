"""GPU tracer vs the CPU oracle, bit for bit, through the C ABI.

The oracle restates the reference's fp32 tracer and is pinned against the
reference's own frames (test_oracle_golden.py); here the CUDA kernel must
reproduce the oracle exactly (hit IDs and 8-bit colour) on the same
flattened scene.
"""
import numpy as np
import pytest

from conftest import oracle_render

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(qr):
    c = qr.Context(0)
    yield c
    c.close()


def _render_both(qr, oracle, ctx, kind, seed, nq, w, h, fsaa=0, flags=0, depth=10, t=0):
    g = qr.GenScene(kind, seed, nq, flags)
    f = qr.Flat(g, w, h, fsaa)
    desc, params = f.update(t, depth)
    sid = ctx.upload(desc)
    gpu = ctx.render_host(sid, params)
    cpu, _ = oracle_render(oracle, desc, params)
    return gpu, cpu


@pytest.mark.parametrize("seed", [1, 2, 3, 4, 5])
def test_plain_bit_exact(qr, oracle, ctx, seed):
    gpu, cpu = _render_both(qr, oracle, ctx, qr.SCN_PLAIN, seed, 16, 320, 192)
    assert (gpu != cpu).sum() == 0


@pytest.mark.parametrize("seed", [1, 6])
def test_plain_ids_bit_exact(qr, oracle, ctx, seed):
    gpu, cpu = _render_both(qr, oracle, ctx, qr.SCN_PLAIN, seed, 16, 320, 192,
                            flags=qr.GEN_IDS)
    assert (gpu != cpu).sum() == 0


def test_plain_aa4_bit_exact(qr, oracle, ctx):
    gpu, cpu = _render_both(qr, oracle, ctx, qr.SCN_PLAIN, 3, 16, 200, 120, fsaa=2)
    assert (gpu != cpu).sum() == 0


def test_plain_full_size(qr, oracle, ctx):
    gpu, cpu = _render_both(qr, oracle, ctx, qr.SCN_PLAIN, 1, 16, 800, 480)
    assert (gpu != cpu).sum() == 0


def test_engine_api_matches_c_abi(qr, oracle):
    g = qr.GenScene(qr.SCN_PLAIN, 2, 16, 0)
    eng = qr.Engine(g, 256, 160)
    a = eng.render(0).copy()
    eng.close()
    g2 = qr.GenScene(qr.SCN_PLAIN, 2, 16, 0)
    f = qr.Flat(g2, 256, 160)
    desc, params = f.update(0, 10)
    cpu, _ = oracle_render(oracle, desc, params)
    assert (a != cpu).sum() == 0


def test_tiny_and_ragged_frames(qr, oracle, ctx):
    for (w, h) in [(1, 1), (7, 3), (33, 17), (129, 65)]:
        gpu, cpu = _render_both(qr, oracle, ctx, qr.SCN_PLAIN, 4, 16, w, h)
        assert (gpu != cpu).sum() == 0, (w, h)
