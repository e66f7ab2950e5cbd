"""Shared fixtures: the package, the CPU oracle, and the gpu marker."""
import ctypes
import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
ORACLE_DIR = os.path.join(ROOT, "oracle")
if ORACLE_DIR not in sys.path:
    sys.path.insert(0, ORACLE_DIR)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def qr():
    mod = importlib.import_module("quadray-engine_gb300")
    if not os.path.exists(mod.LIB_PATH):
        mod.build()
    return mod


@pytest.fixture(scope="session")
def oracle():
    import build as oracle_build
    return oracle_build.load_oracle()


def oracle_render(oracle, desc, params, y0=0, y1=None):
    """Render a frame with the CPU oracle; returns (frame, traced rays)."""
    y1 = params.y_res if y1 is None else y1
    out = np.zeros((params.y_res, params.x_row), dtype=np.uint32)
    nr = ctypes.c_uint64()
    rc = oracle.qr_oracle_render(ctypes.addressof(desc), ctypes.addressof(params),
                                 out.ctypes.data, y0, y1, ctypes.byref(nr))
    assert rc == 0
    return out[:, :params.x_res], nr.value


_ORACLE64 = []


def boundary_mask(desc, params):
    """the hit-ID exclusion mask of a frame (qr_oracle_boundary of the FP64
    oracle): 1 where a camera ray meets a solver or clipper decision within
    1e-5 relative of its boundary no farther than its hit"""
    if not _ORACLE64:
        import build as oracle_build
        L = oracle_build.load_oracle(fp64=True)
        L.qr_oracle_boundary.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_int, ctypes.c_int]
        _ORACLE64.append(L)
    mask = np.zeros((params.y_res, params.x_res), dtype=np.uint8)
    rc = _ORACLE64[0].qr_oracle_boundary(ctypes.addressof(desc), ctypes.addressof(params),
                                         mask.ctypes.data, 0, params.y_res)
    assert rc == 0
    return mask.astype(bool)


def oracle_render_par(oracle, desc, params, y0=0, y1=None, threads=None):
    """oracle_render over row bands on all host cores (the oracle call
    releases the interpreter lock); returns (frame, traced rays)"""
    import threading
    y1 = params.y_res if y1 is None else y1
    out = np.zeros((params.y_res, params.x_row), dtype=np.uint32)
    nt = max(1, min(threads or (os.cpu_count() or 1), y1 - y0))
    # interleaved bands of 4 rows even out the work of dense and empty rows
    rows = list(range(y0, y1, 4))
    counts = [0] * nt
    rcs = [0] * nt

    def work(t):
        for r0 in rows[t::nt]:
            nr = ctypes.c_uint64()
            rc = oracle.qr_oracle_render(ctypes.addressof(desc), ctypes.addressof(params),
                                         out.ctypes.data, r0, min(r0 + 4, y1),
                                         ctypes.byref(nr))
            rcs[t] |= rc
            counts[t] += nr.value

    th = [threading.Thread(target=work, args=(t,)) for t in range(nt)]
    [t.start() for t in th]
    [t.join() for t in th]
    assert not any(rcs)
    return out[:, :params.x_res], sum(counts)


def oracle_pt_par(oracle, desc, params, y0, y1, threads=None):
    """the oracle's path tracer over rows [y0, y1) on all host cores;
    returns (frame, running sums)"""
    import threading
    out = np.zeros((params.y_res, params.x_row), dtype=np.uint32)
    acc = np.zeros((params.y_res, params.x_row, 3), dtype=np.float32)
    nt = max(1, min(threads or (os.cpu_count() or 1), y1 - y0))
    rows = list(range(y0, y1))
    rcs = [0] * nt

    def work(t):
        for r in rows[t::nt]:
            rcs[t] |= oracle.qr_oracle_pt(ctypes.addressof(desc), ctypes.addressof(params),
                                          acc.ctypes.data, out.ctypes.data, r, r + 1, None)

    th = [threading.Thread(target=work, args=(t,)) for t in range(nt)]
    [t.start() for t in th]
    [t.join() for t in th]
    assert not any(rcs)
    return out[:, :params.x_res], acc[:, :params.x_res]


def load_qrsf(qr, raw):
    """a flattened scene written by tests/golden/scene_fixture.cpp (QRSF):
    returns (QrSceneDesc, QrFrameParams, arrays the descriptor points into)"""
    b = bytes(raw)
    hdr = np.frombuffer(b[:40], dtype="<i4")
    assert hdr[0] == 0x46535251 and hdr[1] == 1
    ns, nm, nl, ne, nle, nt, co, cn = (int(x) for x in hdr[2:])
    off, arrs = 40, []
    for n, sz in ((ns, 256), (nm, 112), (nl, 48), (ne, 16), (nle, 16), (nt, 4)):
        a = np.frombuffer(b[off:off + n * sz], dtype=np.uint8).copy()
        arrs.append(a if a.size else np.zeros(16, dtype=np.uint8))
        off += n * sz
    fp = qr.QrFrameParams.from_buffer_copy(b[off:off + ctypes.sizeof(qr.QrFrameParams)])
    d = qr.QrSceneDesc()
    d.nsrf, d.nmat, d.nlgt, d.nelem, d.nlelem, d.ntex = ns, nm, nl, ne, nle, nt
    d.cam_off, d.cam_num = co, cn
    d.srf, d.mat, d.lgt, d.elems, d.lelems, d.texels = (a.ctypes.data for a in arrs)
    return d, fp, arrs


def frame_cmp(a, b, t_diff=3):
    """the reference's own frame comparison (test/core_test.cpp:98-148): a
    pixel differs when a channel differs by more than t_diff, and a
    differing pixel counts only when one of its 8 neighbours differs too;
    returns the count of such pixels"""
    bad = max_channel_diff(a, b) > t_diff
    h, w = bad.shape
    p = np.pad(bad, 1)
    nb = sum(p[1 + dy:1 + dy + h, 1 + dx:1 + dx + w]
             for dy in (-1, 0, 1) for dx in (-1, 0, 1) if dy or dx)
    return int((bad & (nb > 0)).sum())


def channels(frame):
    f = frame.astype(np.int64)
    return np.stack([(f >> 16) & 255, (f >> 8) & 255, f & 255], axis=-1)


def max_channel_diff(a, b):
    return np.abs(channels(a) - channels(b)).max(axis=-1)
