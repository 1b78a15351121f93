"""Host-side pieces of the serving layer (no GPU): size classes, slot
memory footprint, latency statistics."""
import numpy as np

from dxtb_gb300 import serve


def test_size_class_capacity_covers_chno():
    from dxtb_gb300 import molgen, params

    raw = params.raw()["elements"]
    for n in (8, 50, 200, 400):
        nsh, nao = serve.size_class_capacity(n)
        num, _ = molgen.grow(n, 11)
        shells = sum(len(raw[str(int(z))]["shells"]) for z in num)
        aos = sum(2 * s["l"] + 1 for z in num for s in raw[str(int(z))]["shells"])
        assert shells <= nsh and aos <= nao


def test_slot_bytes_grows_quadratically():
    b = [serve.slot_bytes(n) for n in (32, 64, 128)]
    assert b[0] < b[1] < b[2]
    assert 3.5 < b[2] / b[1] < 4.5


def test_latency_summary():
    reqs = []
    for k in range(100):
        r = serve.Request(k, np.array([1, 1]), np.zeros((2, 3)), t_submit=0.0)
        r.t_done = (k + 1) * 1e-3
        reqs.append(r)
    s = serve.latency_summary(reqs)
    assert abs(s["p50_ms"] - 50.5) < 1e-9
    assert 99.0 <= s["p99_ms"] <= 100.0
