"""Admission, reuse and eviction of the request loop, on the CPU with a fake
session (no GPU): requests wait while the HBM budget is held, resident
geometries are reused, idle sessions are evicted least-recently-used first,
and an oversized request fails at once."""
import threading
import time

import numpy as np
import pytest

from ion_gym_gb300.serve import FieldServer, poisson_schedule, percentile


class FakeSession:
    opened = []
    closed = []
    lock = threading.Lock()
    running = 0
    peak = 0
    hold = 0.05

    def __init__(self, metal, n):
        self.nbytes = 100 * n
        self.shape = metal.shape
        with FakeSession.lock:
            FakeSession.opened.append(self)

    def solve_bases(self, masks, v_basis, accuracy):
        with FakeSession.lock:
            FakeSession.running += 1
            FakeSession.peak = max(FakeSession.peak, FakeSession.running)
        time.sleep(FakeSession.hold)
        with FakeSession.lock:
            FakeSession.running -= 1
        return np.stack([np.where(np.asarray(m), v_basis, 0.0) for m in masks])

    def close(self):
        FakeSession.closed.append(self)


def _deck(seed, n_bases, shape=(6, 5, 4)):
    rng = np.random.default_rng(seed)
    return {i + 1: rng.random(shape) < 0.2 for i in range(n_bases)}


@pytest.fixture(autouse=True)
def _reset():
    FakeSession.opened, FakeSession.closed = [], []
    FakeSession.running = FakeSession.peak = 0
    yield


def _server(workers, budget):
    return FieldServer(workers=workers, hbm_budget=budget, device=None,
                       session_factory=FakeSession,
                       bytes_fn=lambda shape, n: 100 * n)


def test_budget_limits_concurrency():
    srv = _server(workers=4, budget=450)       # two 2-basis decks fit at once
    futs = [srv.submit(_deck(s, 2)) for s in range(6)]
    for f in futs:
        assert sorted(f.result(timeout=10)) == [1, 2]
    srv.close()
    assert FakeSession.peak <= 2
    assert len(srv.completed) == 6


def test_resident_geometry_is_reused_and_lru_evicted():
    srv = _server(workers=1, budget=400)
    a, b = _deck(1, 2), _deck(2, 2)
    srv.submit(a).result(timeout=10)
    srv.submit(a).result(timeout=10)           # same metal: reuse
    assert len(FakeSession.opened) == 1
    srv.submit(b).result(timeout=10)           # fits beside a (400)
    assert len(FakeSession.opened) == 2 and not FakeSession.closed
    srv.submit(_deck(3, 3)).result(timeout=10)  # 300: evicts both idle decks
    assert len(FakeSession.closed) == 2
    srv.close()


def test_oversized_request_fails_fast():
    srv = _server(workers=1, budget=150)
    with pytest.raises(MemoryError):
        srv.submit(_deck(1, 2)).result(timeout=10)
    srv.close()


def test_schedule_and_percentiles():
    t = poisson_schedule(50.0, 20.0, seed=3)
    assert 800 < len(t) < 1200 and all(np.diff(t) > 0)
    assert percentile([1, 2, 3, 4], 50) == 2.5
    assert percentile([], 99) is None


def test_unknown_results_kind_is_refused():
    with pytest.raises(ValueError, match="results"):
        FieldServer(workers=1, hbm_budget=100, device=None,
                    session_factory=FakeSession, results="disk")


def test_caller_keys_identify_geometries():
    """A deck submitted with the caller's geometry key is matched to a
    resident session by that key (no pass over its masks); another key is
    another geometry, and keyed and unkeyed submissions do not mix."""
    srv = _server(workers=1, budget=1000)
    a, b = _deck(1, 2), _deck(2, 2)
    srv.submit(a, key="deck-a").result(timeout=10)
    srv.submit(a, key="deck-a").result(timeout=10)
    assert len(FakeSession.opened) == 1
    srv.submit(b, key="deck-b").result(timeout=10)
    assert len(FakeSession.opened) == 2
    srv.submit(a).result(timeout=10)           # hashed key: a new session
    assert len(FakeSession.opened) == 3
    srv.submit(a).result(timeout=10)
    assert len(FakeSession.opened) == 3
    srv.close()


def test_finished_requests_keep_no_results():
    """A finished request keeps its timing only: the result lives in the
    caller's future alone (device results would otherwise stay in HBM for
    the life of the server)."""
    import gc
    import weakref
    srv = _server(workers=1, budget=1000)
    f = srv.submit(_deck(4, 2))
    res = f.result(timeout=10)
    probe = weakref.ref(next(iter(res.values())).base)
    (r,) = srv.completed
    assert r.future is None and r.masks is None and r.end >= r.start
    del f, res
    gc.collect()
    assert probe() is None
    srv.close()


class RebindingSession(FakeSession):
    rebinds = []

    def __init__(self, metal, n):
        super().__init__(metal, n)
        self.max_problems = n

    def rebind(self, metal):
        RebindingSession.rebinds.append(np.asarray(metal).shape)
        return self


def test_new_geometry_of_a_resident_shape_rebinds_an_idle_session():
    """A request whose geometry is not resident takes over an idle session
    of the same grid shape and basis count (rebound to its metal) instead
    of opening one; another shape or basis count opens a new session."""
    RebindingSession.rebinds = []
    srv = FieldServer(workers=1, hbm_budget=10000, device=None,
                      session_factory=RebindingSession,
                      bytes_fn=lambda shape, n: 100 * n)
    srv.submit(_deck(1, 2)).result(timeout=10)
    srv.submit(_deck(2, 2)).result(timeout=10)           # same shape, new metal
    assert len(FakeSession.opened) == 1
    assert RebindingSession.rebinds == [(6, 5, 4)]
    srv.submit(_deck(2, 2)).result(timeout=10)           # now resident: reuse
    assert len(FakeSession.opened) == 1 and len(RebindingSession.rebinds) == 1
    srv.submit(_deck(3, 3)).result(timeout=10)           # other basis count
    srv.submit(_deck(4, 2, shape=(7, 5, 4))).result(timeout=10)  # other shape
    assert len(FakeSession.opened) == 3 and len(RebindingSession.rebinds) == 1
    srv.close()


def test_sessions_keep_the_cheaper_smoothing():
    """auto_cycle: a session's second solve tries the other smoothing and
    the session keeps whichever moved fewer algorithmic bytes (a fake
    whose bytes depend on the cycle): one geometry cheaper with three
    pairs keeps three, one cheaper with two returns to two."""

    class CycleSession(FakeSession):
        def __init__(self, metal, n):
            super().__init__(metal, n)
            self.cycle = {"nu1": 2, "nu2": 2, "cg_iters": 3}
            self.prefer3 = bool(metal[0, 0, 0])
            self.calls = []

        def set_cycle(self, nu1, nu2, cg_iters):
            self.calls.append((nu1, nu2, cg_iters))
            self.cycle = {"nu1": nu1, "nu2": nu2, "cg_iters": cg_iters}

        def solve_bytes(self):
            three = self.cycle["nu1"] == 3
            return 80.0 if three == self.prefer3 else 100.0

    srv = FieldServer(workers=1, hbm_budget=10_000, device=None,
                      session_factory=CycleSession,
                      bytes_fn=lambda shape, n: 100 * n, auto_cycle=True)
    a = _deck(1, 2)
    a[1][0, 0, 0] = True                      # this geometry prefers three
    b = _deck(2, 2)
    b[1][0, 0, 0] = b[2][0, 0, 0] = False     # this one prefers two
    for _ in range(3):
        srv.submit(a, key="a").result(10)
        srv.submit(b, key="b").result(10)
    srv.close()
    sa, sb = [s for s in CycleSession.opened]
    assert sa.cycle["nu1"] == 3 and sa.calls == [(3, 3, 3)]
    assert sb.cycle["nu1"] == 2 and sb.calls == [(3, 3, 3), (2, 2, 3)]
