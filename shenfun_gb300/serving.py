"""Continuous-batching request loop for Helmholtz solves on one GPU.

Requests (2D or 3D grids, Chebyshev or Legendre Dirichlet axis, shift c)
arrive over time.  The ``Scheduler`` admits them as slots and device memory
free up (memory-based admission, no head-of-line blocking behind a request
that does not fit yet), the ``GpuExecutor`` runs each admitted request on one
of several CUDA streams so that work from different requests overlaps on the
device, and completions are detected with CUDA events and retired while new
requests keep arriving.  Factorised problems are cached on the device, keyed
by (grid, family, c, form), with least-recently-used eviction under a byte
budget; a problem whose key is new is built on a worker thread while the
loop keeps launching other requests, and every request of that key starts
once it is ready.  Results do not depend on what else is in flight: every request runs
its own deterministic kernels on its own buffers (no atomics, no shared
scratch), which tests/test_gpu_serving.py checks bit for bit.

Failure handling is host-side: a request larger than the whole memory budget
is rejected with an error, a cancelled request is dropped before launch (or
its result discarded after), and a request that raises during launch, or
whose problem fails to build, is marked failed without stopping the loop.
"""
import collections
import time

import numpy as np

QUEUED, RUNNING, DONE, FAILED, CANCELLED, REJECTED = "queued", "running", "done", "failed", \
    "cancelled", "rejected"


class Request:
    __slots__ = ("id", "N", "family", "c", "f", "arrival", "state", "result", "t_admit", "t_done",
                 "error", "nbytes", "slot")

    def __init__(self, rid, N, family, c, f, arrival=0.0):
        self.id = rid
        self.N = tuple(int(n) for n in N)
        self.family = family
        self.c = float(c)
        self.f = f
        self.arrival = float(arrival)
        self.state = QUEUED
        self.result = None
        self.t_admit = None
        self.t_done = None
        self.error = None
        self.nbytes = 0
        self.slot = None

    @property
    def key(self):
        return (self.N, self.family, self.c)

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.arrival


def array_bytes(N):
    n = 1
    for v in N:
        n *= int(v)
    return 8 * n


def request_bytes(N):
    """Device bytes one in-flight request holds: RHS + solution + scratch
    (real physical array + complex spectral array + the mixed form's split
    copy of the physical array, 14 bytes per padded point, bounded by 16 per
    point with the padding of the last axis to a multiple of 32)."""
    spec = list(N)
    spec[-2 if len(N) == 3 else 0] = spec[-2 if len(N) == 3 else 0] // 2 + 1
    nspec = 1
    for v in spec:
        nspec *= v
    npad = array_bytes(N[:-1]) // 8 * (-(-N[-1] // 32) * 32)
    return 3 * array_bytes(N) + 16 * nspec + 16 * npad + 1024


def factor_bytes(N, family):
    """Device bytes of a cached problem (factor arrays and plan tables)."""
    nd = N[-1]
    spec = list(N)
    spec[-2 if len(N) == 3 else 0] = spec[-2 if len(N) == 3 else 0] // 2 + 1
    nsys = 1
    for v in spec[:-1]:
        nsys *= v
    if family == "chebyshev":
        return 8 * (4 * (nd - 2) + 2) * nsys + 64 * sum(N)
    return 8 * (7 * nd + 4) * nsys + 16 * nd * nd + 64 * sum(N)


class Scheduler:
    """Admission and retirement; independent of the device (tests drive it
    with a fake executor on the CPU)."""

    def __init__(self, executor, max_slots=8, mem_budget=8 << 30, lookahead=16):
        self.ex = executor
        self.max_slots = max_slots
        self.mem_budget = int(mem_budget)
        self.lookahead = lookahead
        self.queue = collections.deque()
        self.running = {}
        self.finished = []
        self.mem_used = 0
        self.free_slots = list(range(max_slots))

    def submit(self, req):
        need = request_bytes(req.N) + self.ex.factor_cost(req)
        req.nbytes = request_bytes(req.N)
        if need > self.mem_budget:
            req.state = REJECTED
            req.error = f"needs {need} bytes, budget {self.mem_budget}"
            self.finished.append(req)
            return False
        self.queue.append(req)
        return True

    def cancel(self, rid):
        for r in list(self.queue):
            if r.id == rid:
                self.queue.remove(r)
                r.state = CANCELLED
                self.finished.append(r)
                return True
        r = self.running.get(rid)
        if r is not None:
            r.state = CANCELLED   # result discarded at retirement
            return True
        return False

    def _retire(self, now):
        for rid in self.ex.poll():
            r = self.running.pop(rid, None)
            if r is None:
                continue
            self.mem_used -= r.nbytes
            self.free_slots.append(r.slot)
            if r.state == CANCELLED:
                r.result = None
            elif r.state != FAILED:
                r.state = DONE
            r.t_done = now()
            self.finished.append(r)

    def _admit(self, now):
        scanned = 0
        i = 0
        while self.free_slots and i < len(self.queue) and scanned < self.lookahead:
            r = self.queue[i]
            scanned += 1
            need = r.nbytes + self.ex.factor_cost(r)
            if self.mem_used + self.ex.cache_bytes() + need > self.mem_budget:
                # evict cached factorisations (least recently used) to make room
                self.ex.shrink_cache(self.mem_budget - self.mem_used - need)
                if self.mem_used + self.ex.cache_bytes() + need > self.mem_budget:
                    i += 1   # does not fit yet: look further down the queue
                    continue
            del self.queue[i]
            r.slot = self.free_slots.pop()
            r.t_admit = now()
            r.state = RUNNING
            self.mem_used += r.nbytes
            self.running[r.id] = r
            try:
                self.ex.launch(r)
            except Exception as e:  # launch failure: report, keep serving
                r.state = FAILED
                r.error = repr(e)
                self.running.pop(r.id, None)
                self.mem_used -= r.nbytes
                self.free_slots.append(r.slot)
                r.t_done = now()
                self.finished.append(r)

    def step(self, now=time.perf_counter):
        self._retire(now)
        self._admit(now)

    def idle(self):
        return not self.queue and not self.running


class GpuExecutor:
    """Runs requests on a pool of CUDA streams with a device-resident,
    byte-budgeted LRU cache of factorised problems."""

    def __init__(self, nstreams=4, cache_budget=4 << 30, form="mixed", keep_results=True, prep_workers=4):
        import torch
        from .problem import HelmholtzProblem
        self.torch = torch
        self.Problem = HelmholtzProblem
        self.streams = [torch.cuda.Stream() for _ in range(nstreams)]
        self.cache = collections.OrderedDict()
        self._cbytes = 0  # bytes of the cached problems, kept with every insertion and eviction
        self.cache_budget = int(cache_budget)
        self.form = form
        self.inflight = {}
        self.keep_results = keep_results
        self.hits = 0
        self.misses = 0
        # problems of new keys are built on worker threads (plan tables and
        # matrices are host work; the library releases the GIL), so that the
        # loop keeps launching requests whose problems are cached
        self.pool = None
        if prep_workers > 0:
            from concurrent.futures import ThreadPoolExecutor
            self.pool = ThreadPoolExecutor(max_workers=prep_workers)
        # worker threads build on streams of their own: work a thread enqueues
        # into a stream that another thread is capturing into a CUDA graph
        # would become part of that graph; the serving streams wait for a
        # build through the event recorded after it
        self.build_streams = [torch.cuda.Stream() for _ in range(max(prep_workers, 1))]
        self._nbuild = 0
        self.pending = {}   # key -> (future, creation stream)
        self.waiting = {}   # request id -> request whose problem is being built
        self.failed = []    # request ids whose problem could not be built

    def _build_stream(self):
        self._nbuild += 1
        return self.build_streams[self._nbuild % len(self.build_streams)]

    # -- factorisation cache ---------------------------------------------
    def cache_bytes(self):
        return self._cbytes

    def _cache_put(self, key, p, nbytes, ready):
        old = self.cache.get(key)
        if old is not None:
            self._cbytes -= old[1]
        self.cache[key] = (p, nbytes, ready)
        self._cbytes += nbytes

    def _cache_evict_oldest(self):
        _, ent = self.cache.popitem(last=False)
        self._cbytes -= ent[1]

    def factor_cost(self, req):
        return 0 if req.key in self.cache else factor_bytes(req.N, req.family)

    def shrink_cache(self, room):
        while self.cache and self.cache_bytes() > max(0, min(room, self.cache_budget)):
            key, _ = next(iter(self.cache.items()))
            if any(r.key == key for r, _, _ in self.inflight.values()) or \
                    any(r.key == key for r in self.waiting.values()):
                break  # still in use
            self._cache_evict_oldest()

    def problem(self, req, stream):
        """Cached problem for `req`, ready for use on `stream`.  A miss is
        created stream-ordered on `stream` (no device synchronisation); a hit
        created on another stream makes `stream` wait for its factorisation."""
        ent = self.cache.get(req.key)
        if ent is not None:
            self.cache.move_to_end(req.key)
            self.hits += 1
            p, _, ready = ent
            if ready is not None and ready[1] is not stream:
                stream.wait_event(ready[0])
            return p
        self.misses += 1
        p = self.Problem(req.N, req.family, req.c, self.form, stream=stream)
        ev = self.torch.cuda.Event()
        ev.record(stream)
        self._cache_put(req.key, p, factor_bytes(req.N, req.family), (ev, stream))
        self.shrink_cache(self.cache_budget)
        return p

    def prepare(self, f):
        """Host input as page-locked memory, so that its copy to the device
        is asynchronous on the request's stream (a pageable source makes the
        copy wait on the host)."""
        torch = self.torch
        t = f if isinstance(f, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(f))
        return t if t.is_pinned() else t.pin_memory()

    def _cached(self, req, stream):
        """The cached problem of `req` for use on `stream` (a hit)."""
        self.cache.move_to_end(req.key)
        p, nb, ready = self.cache[req.key]
        if ready is not None and ready[1] is not stream:
            if ready[0].query():
                self.cache[req.key] = (p, nb, None)  # factorised: no later request needs to wait
            else:
                stream.wait_event(ready[0])
        return p

    def _collect(self):
        """Move finished builds into the cache and start the requests that
        wait for them; a failed build fails its waiting requests."""
        for key, (fut, cs) in list(self.pending.items()):
            if not fut.done():
                continue
            del self.pending[key]
            err = fut.exception()
            if err is None:
                ev = self.torch.cuda.Event()
                ev.record(cs)  # after the build's factorisation on its stream
                self._cache_put(key, fut.result(), factor_bytes(key[0], key[1]), (ev, cs))
                self.shrink_cache(self.cache_budget)
            for rid, r in list(self.waiting.items()):
                if r.key != key:
                    continue
                del self.waiting[rid]
                if err is not None:
                    r.state = FAILED
                    r.error = repr(err)
                    self.failed.append(rid)
                else:
                    s = self.streams[r.slot % len(self.streams)]
                    try:
                        self._start(r, self._cached(r, s), s)
                    except Exception as e:  # launch failure: report, keep serving
                        r.state = FAILED
                        r.error = repr(e)
                        self.failed.append(rid)

    # -- execution ----------------------------------------------------------
    def launch(self, req):
        s = self.streams[req.slot % len(self.streams)]
        if self.pool is None or req.key in self.cache:
            self._start(req, self.problem(req, s), s)
            return
        if req.key in self.pending:
            self.hits += 1  # built once for every request of the key
        else:
            self.misses += 1
            bs = self._build_stream()
            fut = self.pool.submit(self.Problem, req.N, req.family, req.c, self.form, stream=bs)
            self.pending[req.key] = (fut, bs)
        self.waiting[req.id] = req

    def _start(self, req, p, s):
        torch = self.torch
        with torch.cuda.stream(s):
            f_host = req.f if isinstance(req.f, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(req.f))
            d_f = torch.empty(p.phys_shape, dtype=torch.float64, device="cuda")
            d_f.copy_(f_host, non_blocking=True)
            d_u = torch.empty_like(d_f)
            work = p.new_workspace()
            p.solve(d_f, d_u, work, stream=s)
            out = torch.empty(p.phys_shape, dtype=torch.float64, pin_memory=True) if self.keep_results else None
            if out is not None:
                out.copy_(d_u, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(s)
        # keep buffers alive until the event completes
        self.inflight[req.id] = (req, ev, (d_f, d_u, work, out, f_host))
        req.result = out

    def poll(self):
        self._collect()
        done, self.failed = list(self.failed), []
        for rid, (req, ev, bufs) in list(self.inflight.items()):
            if ev.query():
                done.append(rid)
                del self.inflight[rid]
        return done


class BatchExecutor(GpuExecutor):
    """Continuous batching across requests: admitted requests wait per shape
    class (grid, family); whenever a stream is free, the class with the
    oldest waiting request is launched as one batch of up to ``max_batch``
    requests (any shifts) through a CUDA graph of the batched step
    (problem.BatchRunner: one launch per transform pass and one solve launch
    for all members, each member with its own cached factorisation).  While
    the streams are busy, arrivals accumulate into larger batches.  Graph
    runners are cached per (class, batch size), batch sizes rounded up to a
    power of two; a batch's members stay independent (per-line transforms,
    per-system solves), so results are the same alone and in a batch."""

    def __init__(self, nstreams=4, cache_budget=4 << 30, form="mixed", keep_results=True, prep_workers=4,
                 max_batch=16, batch_bytes=1 << 30, graphs=True, tune=False, runner_budget=8 << 30):
        GpuExecutor.__init__(self, nstreams=nstreams, cache_budget=cache_budget, form=form,
                             keep_results=keep_results, prep_workers=prep_workers)
        # factorisations and graph runners have budgets of their own, so that
        # a full factorisation cache does not evict the runners (and their
        # captured graphs) batch after batch
        self.runner_budget = int(runner_budget)
        self.max_batch = int(max_batch)
        self.batch_bytes = int(batch_bytes)
        self.graphs = graphs
        self.tune = tune
        self.tuned = {}  # class -> variants the autotuner picked for its plans
        self.ready = collections.OrderedDict()  # class -> deque of requests whose problem is cached
        self.runners = collections.OrderedDict()  # (class, K) -> [BatchRunner], least recently used first
        self._rbytes = 0  # bytes of the runners' staging buffers
        self.busy = {}  # stream index -> batch id in flight
        self.batches = 0
        self.batch_sizes = collections.Counter()
        self._bid = 0

    @staticmethod
    def _class(req):
        return (req.N, req.family)

    def cache_bytes(self):
        return self._cbytes + self._rbytes

    def _kmax(self, req):
        per = 3 * request_bytes(req.N)
        return max(1, min(self.max_batch, self.batch_bytes // max(per, 1)))

    def launch(self, req):
        if req.key in self.cache:
            self.hits += 1
            self.ready.setdefault(self._class(req), collections.deque()).append(req)
            self._flush()
            return
        if req.key in self.pending:
            self.hits += 1
        else:
            self.misses += 1
            s = self._build_stream()
            fut = self.pool.submit(self.Problem, req.N, req.family, req.c, self.form, stream=s) if self.pool else None
            if fut is None:
                p = self.Problem(req.N, req.family, req.c, self.form, stream=s)
                ev = self.torch.cuda.Event()
                ev.record(s)
                self._cache_put(req.key, p, factor_bytes(req.N, req.family), (ev, s))
                self.ready.setdefault(self._class(req), collections.deque()).append(req)
                self._flush()
                return
            self.pending[req.key] = (fut, s)
        self.waiting[req.id] = req

    def _collect(self):
        for key, (fut, cs) in list(self.pending.items()):
            if not fut.done():
                continue
            del self.pending[key]
            err = fut.exception()
            if err is None:
                ev = self.torch.cuda.Event()
                ev.record(cs)
                self._cache_put(key, fut.result(), factor_bytes(key[0], key[1]), (ev, cs))
                self.shrink_cache(self.cache_budget)
            for rid, r in list(self.waiting.items()):
                if r.key != key:
                    continue
                del self.waiting[rid]
                if err is not None:
                    r.state = FAILED
                    r.error = repr(err)
                    self.failed.append(rid)
                else:
                    self.ready.setdefault(self._class(r), collections.deque()).append(r)

    def _runner(self, cls, K, proto, si):
        """A runner of class `cls` and size K that no batch in flight uses
        (its graph replays on whichever stream the batch runs on)."""
        from .problem import BatchRunner
        key = (cls, K)
        busy = self._busy_runners()
        pool = self.runners.get(key)
        if pool is not None:
            self.runners.move_to_end(key)
            for r in pool:
                if id(r) not in busy:
                    return r
        if self.tune and cls not in self.tuned:
            from . import autotune
            self.streams[si].synchronize()
            self.tuned[cls] = autotune.tune_problem(proto)  # before the graph captures the variants
        # a runner's first batch runs as plain launches, later ones replay
        # the graph captured at its second batch
        r = BatchRunner(proto, K, self.streams[si], graph=self.graphs, capture_after=1)
        r.bytes = r.f.numel() * 16 + r.work.numel()
        self.runners.setdefault(key, []).append(r)
        self.runners.move_to_end(key)
        self._rbytes += r.bytes
        self._trim_runners(self.runner_budget, busy | {id(r)})
        return r

    def _flush(self):
        torch = self.torch
        while self.ready:
            free = [i for i in range(len(self.streams)) if i not in self.busy]
            if not free:
                return
            cls = next(iter(self.ready))
            q = self.ready[cls]
            if not q:
                del self.ready[cls]
                continue
            si = free[0]
            s = self.streams[si]
            kmax = self._kmax(q[0])
            reqs = [q.popleft() for _ in range(min(kmax, len(q)))]
            if not q:
                del self.ready[cls]
            else:
                self.ready.move_to_end(cls)
            K = 1
            while K < len(reqs):
                K *= 2
            K = min(K, kmax) if kmax >= len(reqs) else len(reqs)
            try:
                probs = [self._cached(r, s) for r in reqs]
                run = self._runner(cls, K, probs[0], si)
                with torch.cuda.stream(s):
                    for k, r in enumerate(reqs):
                        src = r.f if isinstance(r.f, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(r.f))
                        run.f[k].copy_(src.reshape(run.f[k].shape), non_blocking=True)
                    run.run(probs, stream=s)
                    outs = []
                    for k, r in enumerate(reqs):
                        out = torch.empty(run.u.shape[1:], dtype=torch.float64, pin_memory=True) \
                            if self.keep_results else None
                        if out is not None:
                            out.copy_(run.u[k], non_blocking=True)
                        r.result = out
                        outs.append(out)
                    ev = torch.cuda.Event()
                    ev.record(s)
            except Exception as e:  # launch failure: report, keep serving
                for r in reqs:
                    r.state = FAILED
                    r.error = repr(e)
                    self.failed.append(r.id)
                continue
            self._bid += 1
            self.busy[si] = self._bid
            self.inflight[("batch", self._bid)] = (reqs, ev, (outs, run, si))
            self.batches += 1
            self.batch_sizes[len(reqs)] += 1

    def _busy_runners(self):
        return {id(v[2][1]) for v in self.inflight.values()}

    def _trim_runners(self, limit, busy):
        """Drop idle runners, least recently used classes first, until the
        runners hold at most `limit` bytes."""
        for key in list(self.runners):
            if self._rbytes <= limit:
                return
            pool = self.runners[key]
            keep = []
            for r in pool:
                if self._rbytes > limit and id(r) not in busy:
                    self._rbytes -= r.bytes
                else:
                    keep.append(r)
            if keep:
                self.runners[key] = keep
            else:
                del self.runners[key]

    def shrink_cache(self, room):
        """Keep the runners within their budget and the factorisations within
        theirs and within `room` (bytes the caches may hold), least recently
        used first; entries in use stay."""
        busy_runners = self._busy_runners()
        self._trim_runners(self.runner_budget, busy_runners)
        flimit = max(0, min(room - self._rbytes, self.cache_budget))
        if self._cbytes > flimit:
            busy_keys = {r.key for reqs, _, _ in self.inflight.values() for r in reqs}
            busy_keys |= {r.key for q in self.ready.values() for r in q}
            busy_keys |= {r.key for r in self.waiting.values()}
            while self.cache and self._cbytes > flimit:
                key, _ = next(iter(self.cache.items()))
                if key in busy_keys:
                    break  # still in use
                self._cache_evict_oldest()
        if self.cache_bytes() > room:
            self._trim_runners(max(0, room - self._cbytes), busy_runners)

    def poll(self):
        self._collect()
        done, self.failed = list(self.failed), []
        for bid, (reqs, ev, bufs) in list(self.inflight.items()):
            if ev.query():
                del self.inflight[bid]
                self.busy.pop(bufs[2], None)
                done.extend(r.id for r in reqs)
        self._flush()
        return done


def make_stream(n, seed=0, rate=None, nmin=32, nmax=512, max_points=2 ** 24, families=("chebyshev", "legendre"),
                sizes=None, shifts=None):
    """Synthetic request stream: dim in {2, 3} (50/50), N per axis log-uniform
    in [nmin, nmax], family uniform, shift c log-uniform in [0.1, 1e4],
    Poisson arrivals at `rate` requests/s (all at t = 0 when rate is None).
    Grids with more than `max_points` points are redrawn (device memory).
    With `sizes` / `shifts` (sequences), N per axis and c are drawn
    log-uniformly from those discrete values instead, so that keys repeat
    (a serving population of fixed configurations with new right-hand
    sides)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    while len(out) < n:
        dim = 2 if rng.random() < 0.5 else 3
        if sizes is not None:
            N = tuple(int(sizes[int(rng.integers(len(sizes)))]) for _ in range(dim))
        else:
            N = tuple(int(round(np.exp(rng.uniform(np.log(nmin), np.log(nmax))))) for _ in range(dim))
        N = N[:-1] + (max(N[-1], 8),)
        if np.prod(N) > max_points:
            continue
        fam = families[int(rng.integers(len(families)))]
        if shifts is not None:
            c = float(shifts[int(rng.integers(len(shifts)))])
        else:
            c = float(np.exp(rng.uniform(np.log(0.1), np.log(1e4))))
        if rate:
            t += rng.exponential(1.0 / rate)
        out.append((N, fam, c, t, int(rng.integers(1 << 31))))
    return out


class RhsPool:
    """Right-hand sides of a synthetic stream: `per_shape` seeded N(0, 1)
    arrays per grid shape, page-locked, made on first use and shared by the
    requests of that shape (request i of a shape gets array i mod
    `per_shape`), so that a stream of thousands of requests holds a bounded
    amount of host memory."""

    def __init__(self, per_shape=2, seed=0, pinned=True):
        self.per_shape = int(per_shape)
        self.seed = int(seed)
        self.pinned = pinned
        self.arrays = {}

    def __call__(self, N, seed):
        N = tuple(int(n) for n in N)
        k = (N, int(seed) % self.per_shape)
        a = self.arrays.get(k)
        if a is None:
            f = np.random.default_rng([self.seed, k[1]] + list(N)).standard_normal(N)
            if self.pinned:
                import torch
                a = torch.from_numpy(f).pin_memory()
            else:
                a = f
            self.arrays[k] = a
        return a

    @property
    def nbytes(self):
        return sum(int(a.nbytes) if hasattr(a, "nbytes") else a.numel() * 8 for a in self.arrays.values())


def run_stream(stream, executor, max_slots=8, mem_budget=8 << 30, poll_sleep=0.0, rhs=None):
    """Drive a stream through the scheduler in wall-clock time; returns the
    finished requests and the elapsed seconds.  `rhs(N, seed)` gives a
    request's right-hand side (default: a fresh seeded N(0, 1) array)."""
    sched = Scheduler(executor, max_slots=max_slots, mem_budget=mem_budget)
    reqs = []
    prepare = getattr(executor, "prepare", None)
    for i, (N, fam, c, t, seed) in enumerate(stream):
        f = rhs(N, seed) if rhs is not None else np.random.default_rng(seed).standard_normal(N)
        reqs.append(Request(i, N, fam, c, prepare(f) if prepare else f, t))
    t0 = time.perf_counter()
    now = lambda: time.perf_counter() - t0  # noqa: E731
    nxt = 0
    while nxt < len(reqs) or not sched.idle():
        tn = now()
        while nxt < len(reqs) and reqs[nxt].arrival <= tn:
            sched.submit(reqs[nxt])
            nxt += 1
        sched.step(now)
        if poll_sleep:
            time.sleep(poll_sleep)
    return sched.finished, now()
