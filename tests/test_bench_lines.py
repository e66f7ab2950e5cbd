"""The bench's JSON lines (bench.py): both arms carry the same config keys,
with the same workload identity, for every frame workload."""
import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.mark.parametrize("name", ["anim", "plain", "pt"])
def test_arms_share_config(name):
    b = _bench()
    wl = b.WORKLOADS[name]
    ours = b.line_config(name, wl, "ours", 1)
    ref = b.line_config(name, wl, "reference", 1)
    assert set(ours) == set(ref)
    ident = b.config_of(name, wl)
    for k, v in ident.items():
        assert ours[k] == v and ref[k] == v
    assert ours["workload"] == name
    assert ours["depth"] == wl["depth"] and ours["animated"] == wl["anim"]
