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


def test_orbital_padding_of_the_calculator():
    """The host-side padding of per-orbital values (get_charges): ragged in
    plan order -> (B, nao_max) with zeros, or (nao,) for one molecule."""
    import numpy as np

    from dxtb_gb300.calculator import GFN1Calculator

    calc = GFN1Calculator.__new__(GFN1Calculator)  # no device needed for the padding
    calc._numbers_ragged = np.array([8, 1, 1, 6, 1, 1, 1, 1])  # H2O, CH4
    calc._counts = np.array([3, 5])
    calc._offsets = np.array([0, 3, 8])
    calc.batched = True
    assert calc._orbital_counts().tolist() == [8, 12]
    ragged = np.arange(20.0)
    out = calc._pad_orbitals(ragged)
    assert out.shape == (2, 12)
    assert out[0, :8].tolist() == list(range(8)) and np.all(out[0, 8:] == 0)
    assert out[1].tolist() == list(range(8, 20))
    single = GFN1Calculator.__new__(GFN1Calculator)
    single._numbers_ragged = np.array([8, 1, 1])
    single._counts = np.array([3])
    single._offsets = np.array([0, 3])
    single.batched = False
    assert single._pad_orbitals(np.ones(8)).shape == (8,)
    import pytest

    with pytest.raises(ValueError):
        calc._pad_orbitals(np.ones(19))
