"""Host-side serving logic on the CPU: memory-based admission, slots,
rejection, cancellation and launch failures, with a fake executor (failures
are injected on the host; no GPU is involved)."""
import numpy as np

from shenfun_gb300 import serving as S


class FakeExecutor:
    """Completes a launched request after `lag` polls; may fail launches."""

    def __init__(self, lag=2, fail_ids=(), cache_budget=1 << 40):
        self.lag = lag
        self.fail_ids = set(fail_ids)
        self.inflight = {}
        self.cache = {}
        self.cache_budget = cache_budget
        self.launched = []

    def cache_bytes(self):
        return sum(self.cache.values())

    def factor_cost(self, req):
        return 0 if req.key in self.cache else S.factor_bytes(req.N, req.family)

    def shrink_cache(self, room):
        while self.cache and self.cache_bytes() > max(room, 0):
            self.cache.pop(next(iter(self.cache)))

    def launch(self, req):
        if req.id in self.fail_ids:
            raise RuntimeError("injected launch failure")
        self.cache.setdefault(req.key, S.factor_bytes(req.N, req.family))
        self.inflight[req.id] = self.lag
        self.launched.append(req.id)
        req.result = np.zeros(1)

    def poll(self):
        done = []
        for rid in list(self.inflight):
            self.inflight[rid] -= 1
            if self.inflight[rid] <= 0:
                done.append(rid)
                del self.inflight[rid]
        return done


def mk(i, N=(16, 16, 17), fam="chebyshev", c=1.0):
    return S.Request(i, N, fam, c, None, 0.0)


def drain(sched, limit=1000):
    t = [0.0]

    def now():
        t[0] += 1.0
        return t[0]
    for _ in range(limit):
        sched.step(now)
        if sched.idle():
            return
    raise AssertionError("scheduler did not drain")


def test_slots_bound_concurrency():
    ex = FakeExecutor(lag=3)
    sched = S.Scheduler(ex, max_slots=2, mem_budget=1 << 40)
    for i in range(7):
        sched.submit(mk(i))
    peak = 0
    t = [0.0]
    while not sched.idle():
        t[0] += 1
        sched.step(lambda: t[0])
        peak = max(peak, len(sched.running))
    assert peak == 2
    assert sorted(r.id for r in sched.finished) == list(range(7))
    assert all(r.state == S.DONE and r.latency > 0 for r in sched.finished)


def test_memory_admission_and_no_head_of_line_blocking():
    ex = FakeExecutor(lag=2)
    big = (64, 64, 65)
    small = (16, 16, 17)
    budget = S.request_bytes(big) + S.factor_bytes(big, "chebyshev") + 1000
    sched = S.Scheduler(ex, max_slots=4, mem_budget=budget)
    sched.submit(mk(0, big))
    sched.submit(mk(1, big, c=2.0))     # must wait for request 0
    sched.submit(mk(2, small))          # fits next to request 0? only if memory allows
    t = [0.0]
    t[0] += 1
    sched.step(lambda: t[0])
    assert 0 in sched.running and 1 not in sched.running
    drain(sched)
    assert {r.id: r.state for r in sched.finished} == {0: S.DONE, 1: S.DONE, 2: S.DONE}
    assert sched.mem_used == 0


def test_oversized_request_rejected():
    ex = FakeExecutor()
    sched = S.Scheduler(ex, max_slots=2, mem_budget=1 << 20)
    assert not sched.submit(mk(0, (256, 256, 257)))
    assert sched.finished[0].state == S.REJECTED and "budget" in sched.finished[0].error
    assert sched.idle()


def test_cancel_queued_and_running():
    ex = FakeExecutor(lag=5)
    sched = S.Scheduler(ex, max_slots=1, mem_budget=1 << 40)
    for i in range(3):
        sched.submit(mk(i))
    t = [1.0]
    sched.step(lambda: t[0])
    assert sched.cancel(0)          # running: result discarded
    assert sched.cancel(2)          # queued: dropped
    assert not sched.cancel(99)
    drain(sched)
    st = {r.id: r.state for r in sched.finished}
    assert st == {0: S.CANCELLED, 1: S.DONE, 2: S.CANCELLED}
    assert 2 not in ex.launched
    assert next(r for r in sched.finished if r.id == 0).result is None


def test_launch_failure_is_reported_and_loop_continues():
    ex = FakeExecutor(lag=1, fail_ids={1})
    sched = S.Scheduler(ex, max_slots=2, mem_budget=1 << 40)
    for i in range(4):
        sched.submit(mk(i))
    drain(sched)
    st = {r.id: r.state for r in sched.finished}
    assert st[1] == S.FAILED and "injected" in next(r.error for r in sched.finished if r.id == 1)
    assert all(st[i] == S.DONE for i in (0, 2, 3))
    assert sched.mem_used == 0 and sorted(sched.free_slots) == [0, 1]


def test_cache_eviction_under_memory_pressure():
    ex = FakeExecutor(lag=1)
    N = (32, 32, 33)
    one = S.request_bytes(N) + S.factor_bytes(N, "chebyshev")
    sched = S.Scheduler(ex, max_slots=1, mem_budget=one + S.factor_bytes(N, "chebyshev") // 2)
    for i in range(4):
        sched.submit(mk(i, N, c=float(i)))  # distinct keys: every request needs a new factor
    drain(sched)
    assert all(r.state == S.DONE for r in sched.finished)
    assert len(ex.cache) == 1


def test_stream_generator():
    st = S.make_stream(200, seed=3, rate=100.0)
    assert len(st) == 200
    dims = {len(N) for N, *_ in st}
    assert dims == {2, 3}
    assert all(32 <= n <= 512 for N, *_ in st for n in N)
    arr = [t for *_, t, _ in st]
    assert all(b >= a for a, b in zip(arr, arr[1:]))
    cs = np.array([c for _, _, c, _, _ in st])
    assert cs.min() >= 0.1 and cs.max() <= 1e4
