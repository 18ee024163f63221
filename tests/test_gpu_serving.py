"""GPU: the one-call Helmholtz problem against the oracle, and the serving
loop: every result in a concurrent mix equals the same request run alone."""
import numpy as np
import pytest
import torch

from oracle import problems as P, spectral as S, la as OL

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg():
    from shenfun_gb300 import build
    build.build()
    import shenfun_gb300
    return shenfun_gb300


def rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def oracle_roundtrip(f, N, family, c):
    if len(N) == 2:
        bases = [("fourier", "R2C", N[0]), (family, "SD", N[1])]
    else:
        bases = [("fourier", "C2C", N[0]), ("fourier", "R2C", N[1]), (family, "SD", N[2])]
    ax = len(N) - 1
    fh = P.scalar_product(f, bases)
    if family == "chebyshev":
        uh = P.helmholtz_solve(fh, bases, c, ax)
    else:
        beta = (P.fourier_k2(bases, ax) + c).reshape(-1)
        fs, shp = P._systems(fh, ax)
        uh = np.moveaxis(OL.leg_helmholtz_solve(fs, np.ones_like(beta), beta).reshape(shp), -1, ax)
    return P.backward(uh, bases)


@pytest.mark.parametrize("N,family,c", [((16, 12, 24), "chebyshev", 1000.0),
                                         ((32, 33), "chebyshev", 0.5),
                                         ((8, 10, 20), "legendre", 7.0),
                                         ((24, 31), "legendre", 100.0)])
@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_problem_roundtrip(sg, N, family, c, form):
    from shenfun_gb300.problem import HelmholtzProblem
    p = HelmholtzProblem(N, family, c, form)
    f = np.random.default_rng(1).standard_normal(N)
    u = p.solve(torch.as_tensor(f, device="cuda")).cpu().numpy()
    tol = 1e-12 if form == "plain" else 1e-10
    assert rel(u, oracle_roundtrip(f, N, family, c)) < tol


def test_serving_mix_equals_alone(sg):
    from shenfun_gb300 import serving as SV
    stream = SV.make_stream(24, seed=11, rate=None, nmin=16, nmax=96)
    # alone: one request at a time (one slot, one stream)
    ex1 = SV.GpuExecutor(nstreams=1)
    alone, _ = SV.run_stream(stream, ex1, max_slots=1)
    # in the mix: many slots, several streams, a tight cache budget
    ex2 = SV.GpuExecutor(nstreams=4, cache_budget=16 << 20)
    mix, _ = SV.run_stream(stream, ex2, max_slots=8)
    torch.cuda.synchronize()
    a = {r.id: r for r in alone}
    m = {r.id: r for r in mix}
    assert len(a) == len(m) == 24
    for i in range(24):
        assert a[i].state == SV.DONE and m[i].state == SV.DONE, (a[i].error, m[i].error)
        # identical kernels on private buffers: bit-for-bit equal
        assert torch.equal(a[i].result, m[i].result), i
    # and correct: a sample against the oracle (the executor's default is the
    # mixed form, bound 1e-10)
    for i in range(0, 24, 6):
        N, fam, c, _, seed = stream[i]
        f = np.random.default_rng(seed).standard_normal(N)
        assert rel(m[i].result.numpy(), oracle_roundtrip(f, N, fam, c)) < 1e-10


@pytest.mark.parametrize("N,family", [((16, 12, 24), "chebyshev"), ((24, 31), "legendre")])
def test_stream_ordered_create_equals_plain(sg, N, family):
    """A problem created stream-ordered (shared plans, factorisation queued on
    a side stream) gives bit-for-bit the result of the synchronous creation."""
    from shenfun_gb300.problem import HelmholtzProblem
    f = torch.as_tensor(np.random.default_rng(3).standard_normal(N), device="cuda")
    u0 = HelmholtzProblem(N, family, 3.0).solve(f)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    p = HelmholtzProblem(N, family, 3.0, stream=s)
    with torch.cuda.stream(s):
        f.record_stream(s)
        u1 = p.solve(f, stream=s)
    s.synchronize()
    assert torch.equal(u0, u1)


def test_serving_shared_keys_across_streams(sg):
    """Requests that share a cached problem run on other streams than the one
    that created it: each must wait for the factorisation, and every result
    equals the request run alone."""
    from shenfun_gb300 import serving as SV
    keys = [((24, 20, 32), "chebyshev", 10.0), ((40, 48), "legendre", 2.0),
            ((16, 16, 64), "chebyshev", 0.3)]
    stream = [(keys[i % 3][0], keys[i % 3][1], keys[i % 3][2], 0.0, 100 + i) for i in range(18)]
    alone, _ = SV.run_stream(stream, SV.GpuExecutor(nstreams=1), max_slots=1)
    ex = SV.GpuExecutor(nstreams=4)
    mix, _ = SV.run_stream(stream, ex, max_slots=8)
    torch.cuda.synchronize()
    assert ex.misses == 3 and ex.hits == 15
    a = {r.id: r for r in alone}
    for r in mix:
        assert r.state == SV.DONE, r.error
        assert torch.equal(a[r.id].result, r.result), r.id


def test_background_build_failure_fails_only_its_requests(sg):
    """A problem the library refuses to build (Dirichlet axis shorter than 8)
    fails, on its worker thread, the two requests of its key; the others
    finish and equal their runs alone."""
    from shenfun_gb300 import serving as SV
    good = [((24, 20, 32), "chebyshev", 10.0), ((40, 48), "legendre", 2.0)]
    bad = ((16, 4), "chebyshev", 1.0)
    stream = []
    for i in range(8):
        N, fam, c = bad if i in (2, 5) else good[i % 2]
        stream.append((N, fam, c, 0.0, 300 + i))
    ex = SV.GpuExecutor(nstreams=4)
    fin, _ = SV.run_stream(stream, ex, max_slots=4)
    torch.cuda.synchronize()
    by = {r.id: r for r in fin}
    assert len(by) == 8
    for i in range(8):
        if i in (2, 5):
            assert by[i].state == SV.FAILED and "SgpuError" in by[i].error
        else:
            assert by[i].state == SV.DONE, by[i].error
    alone, _ = SV.run_stream([stream[i] for i in (0, 1)], SV.GpuExecutor(nstreams=1, prep_workers=0),
                             max_slots=1)
    for r in alone:
        assert torch.equal(r.result, by[r.id].result)


# (96, 96, 33): 4,704 systems, above the one-CTA-per-system solve, so the
# single solve runs one thread per (system, parity, component)
@pytest.mark.parametrize("N,family", [((16, 12, 24), "chebyshev"), ((24, 31), "legendre"),
                                      ((32, 33), "chebyshev"), ((8, 10, 20), "legendre"),
                                      ((96, 96, 33), "chebyshev")])
@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_batched_step_equals_single_solves(sg, N, family, form):
    """sgpu_helmholtz_solve_batch over K problems of one shape (different
    shifts): the same bits as K single solves, eager and as a graph replay."""
    from shenfun_gb300.problem import HelmholtzProblem, BatchRunner
    shifts = [0.5, 3.0, 1000.0]
    probs = [HelmholtzProblem(N, family, c, form) for c in shifts]
    g = np.random.default_rng(9)
    fs = [torch.as_tensor(g.standard_normal(N), device="cuda") for _ in shifts]
    single = [p.solve(f) for p, f in zip(probs, fs)]
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    for graph in (False, True):
        run = BatchRunner(probs[0], 4, s, graph=graph)  # one slot unused
        with torch.cuda.stream(s):
            for k, f in enumerate(fs):
                run.f[k].copy_(f)
            run.run(probs)
        s.synchronize()
        for k in range(len(shifts)):
            assert torch.equal(run.u[k], single[k]), (graph, k)


def test_batch_executor_mix_equals_alone(sg):
    """The batching executor: requests batched per shape class through graph
    replays give the bits of the same requests run alone, and repeated keys
    hit the factorisation cache."""
    from shenfun_gb300 import serving as SV
    stream = SV.make_stream(40, seed=21, rate=None, sizes=(16, 24, 32), shifts=(0.5, 10.0, 1e3))
    alone, _ = SV.run_stream(stream, SV.GpuExecutor(nstreams=1), max_slots=1)
    ex = SV.BatchExecutor(nstreams=2, max_batch=8)
    mix, _ = SV.run_stream(stream, ex, max_slots=64)
    torch.cuda.synchronize()
    a = {r.id: r for r in alone}
    assert len(mix) == 40
    for r in mix:
        assert r.state == SV.DONE, r.error
        assert torch.equal(a[r.id].result, r.result), r.id
    assert ex.hits > 0 and max(ex.batch_sizes) > 1
