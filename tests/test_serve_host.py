"""Host-side pieces of the serving layer (no GPU): size classes, slot
memory footprint, latency statistics, and the admission and step logic of
``Server`` over stand-in pools."""
import time

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


class _FakePool:
    """Stands in for a slot pool: a fixed number of slots; a launched step
    ends the molecules whose remaining pass count reaches 0."""

    def __init__(self, max_atoms, nslots, passes=2):
        self.max_atoms, self.nslots, self.passes = max_atoms, nslots, passes
        self.cap_sh, self.cap_ao = serve.size_class_capacity(max_atoms)
        self.requests = {}
        self.left = {}
        self.launched = False
        self.iterating = 0

    fits = serve._Pool.fits

    def evict(self, slot):
        self.left.pop(slot)
        return self.requests.pop(slot)

    def free(self):
        return self.nslots - len(self.requests)

    def admit(self, req):
        if self.free() == 0:
            return False
        slot = min(set(range(self.nslots)) - set(self.requests))
        self.requests[slot] = req
        self.left[slot] = self.passes
        return True

    def launch(self):
        self.launched = True

    def ready(self):
        return True

    def finish(self):
        self.launched = False
        done = []
        for slot in list(self.requests):
            self.left[slot] -= 1
            if self.left[slot] == 0:
                req = self.requests.pop(slot)
                req.energy, req.status, req.iterations = -1.0, 0, self.passes
                req.t_left = time.perf_counter()  # the slot is free from here on
                done.append(req)
        return done

    @property
    def busy(self):
        return bool(self.requests)


def _server_with_fake_pools(classes, evict_after=None, slow=(), passes=2):
    srv = serve.Server.__new__(serve.Server)
    srv.pools = [_FakePool(a, n, passes) for a, n in classes]
    srv.slow = [_FakePool(a, n, passes) for a, n in slow]
    srv.evict_after = evict_after
    srv.queue = serve.deque()
    srv.slow_queue = serve.deque()
    srv.completed = []
    srv._next_id = 0
    srv.steps = 0
    srv.device = 0
    return srv


def test_requests_go_to_the_smallest_class_that_fits_and_wait_when_full():
    srv = _server_with_fake_pools([(10, 1), (40, 2)])
    sizes = [5, 30, 8, 35, 3]
    for n in sizes:
        srv.submit(np.ones(n, dtype=np.int64), np.zeros((n, 3)))
    srv.step(wait=False)
    # the 5-atom one in the small class, 30 and 8 in the large class (the
    # small class is full), 35 and 3 wait
    placed = {r.id: r.size_class for p in srv.pools for r in p.requests.values()}
    assert placed == {0: 0, 1: 1, 2: 1}
    assert [r.id for r in srv.queue] == [3, 4]
    srv.run_until_idle()
    assert srv.idle
    assert sorted(r.id for r in srv.completed) == list(range(len(sizes)))
    assert all(r.status == 0 and r.latency is not None for r in srv.completed)
    # the waiting requests took slots that others had left: continuous batching
    by_id = {r.id: r for r in srv.completed}
    first_left = min(by_id[k].t_left for k in (0, 1, 2))
    assert by_id[3].t_admit >= first_left and by_id[4].t_admit >= first_left


def test_oversized_request_is_refused_on_the_host():
    import pytest

    srv = _server_with_fake_pools([(10, 1)])
    with pytest.raises(ValueError):
        srv.submit(np.ones(11, dtype=np.int64), np.zeros((11, 3)))


def test_request_that_fits_no_class_by_orbitals_is_refused():
    """A molecule within the atom capacity whose d-shell elements need more
    orbitals than the largest class holds is refused, not left waiting."""
    import pytest

    srv = _server_with_fake_pools([(10, 1)])
    srv.submit(np.array([6] * 10), np.zeros((10, 3)))  # 40 AOs: fits
    with pytest.raises(ValueError, match="orbitals"):
        srv.submit(np.array([35] * 10), np.zeros((10, 3)))  # Br: s, p, d shells


def test_stragglers_move_to_the_straggler_pool():
    """With evict_after = 3 passes and molecules needing 5: the first
    molecule leaves its main slot after 3 passes because the second waits
    for it, restarts in the straggler pool and finishes there; the second
    takes the main slot meanwhile and, with nothing waiting behind it, keeps
    it to the end."""
    srv = _server_with_fake_pools([(40, 1)], evict_after=3, slow=[(40, 1)], passes=5)
    for n in (5, 6):
        srv.submit(np.ones(n, dtype=np.int64), np.zeros((n, 3)))
    srv.run_until_idle()
    assert srv.idle
    assert sorted(r.id for r in srv.completed) == [0, 1]
    by_id = {r.id: r for r in srv.completed}
    assert by_id[0].evicted and not by_id[1].evicted
    assert all(r.status == 0 for r in srv.completed)
    # request 1 entered the main slot while request 0 finished in the straggler pool
    assert by_id[1].t_admit < by_id[0].t_done


def test_eviction_only_for_waiting_requests():
    """Three long molecules in three slots, two requests waiting: the two
    longest-running stragglers leave (one per waiting request), the third
    keeps its slot; a waiting request of another class evicts nothing."""
    srv = _server_with_fake_pools([(10, 1), (40, 3)], evict_after=2, slow=[(10, 1), (40, 3)], passes=50)
    for n in (30, 31, 32):
        srv.submit(np.ones(n, dtype=np.int64), np.zeros((n, 3)))
    srv.step(wait=False)
    for _ in range(3):
        srv.step(wait=False)
    assert not any(r.evicted for p in srv.pools for r in p.requests.values())
    srv.pools[1].requests[0].passes += 1  # slot 0 has run longest
    srv.submit(np.ones(5, dtype=np.int64), np.zeros((5, 3)))  # small class: free slot
    srv.submit(np.ones(33, dtype=np.int64), np.zeros((33, 3)))
    srv.submit(np.ones(34, dtype=np.int64), np.zeros((34, 3)))
    srv.step(wait=False)
    evicted = sorted(r.id for r in srv.slow_queue) + sorted(r.id for p in srv.slow for r in p.requests.values())
    assert evicted == [0, 1] or evicted == [0, 2]
    assert 0 in evicted
    assert sum(1 for r in srv.pools[1].requests.values() if r.id in (0, 1, 2)) == 1
