"""The allocation-free whole-step entry point, sgpu_helmholtz_solve_noalloc.

It exists for callers that cannot give the library a scratch buffer or let it
allocate one: programs whose device memory is owned by another allocator, thin
FFI callers that only hold their input and output arrays, loops that must not
allocate during a step.  It runs the same step as sgpu_helmholtz_solve, using
a 64 MiB scratch array built into the library instead of caller scratch.

Checked through the C ABI: two calls in a row, each against the scratch-taking
entry point on the same input (relative error <= 1e-12), no device memory
change on the second call, and the size limit; in both arithmetic forms, and
for the mixed form with two problems of different sizes in a row (the
tensor-core contraction's scratch, the Legendre digit copy included, reused
from the built-in array).  Collected last
on purpose (file name) so that a run stopping at the first failure has run
every other test first; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture(scope="module")
def lib():
    from shenfun_gb300 import build, _lib
    build.build()
    return _lib.load()


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("N,family,form", [((64, 48, 65), "chebyshev", "plain"), ((96, 97), "legendre", "plain"),
                                           ((64, 48, 65), "chebyshev", "mixed")])
def test_noalloc_matches_scratch_entry(lib, N, family, form):
    from shenfun_gb300.problem import HelmholtzProblem
    prob = HelmholtzProblem(N, family, c=1000.0, form=form)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    work = torch.empty(prob.workspace_bytes, dtype=torch.uint8, device="cuda")
    rng = np.random.default_rng(3)
    for call in range(2):
        f = torch.as_tensor(rng.standard_normal(N), device="cuda")
        ref = torch.empty_like(f)
        st = lib.sgpu_helmholtz_solve(prob._h, _p(f), _p(ref), _p(work),
                                      ctypes.c_size_t(work.numel()), stream)
        assert st == 0
        got = torch.full_like(f, float("nan"))
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        st = lib.sgpu_helmholtz_solve_noalloc(prob._h, _p(f), _p(got), stream)
        assert st == 0, lib.sgpu_status_string(st)
        torch.cuda.synchronize()
        if call == 1:
            assert torch.cuda.mem_get_info()[0] == free_before
        err = ((got - ref).abs().max() / ref.abs().max()).item()
        assert err <= TOL, (call, err)


def test_noalloc_mixed_form_two_sizes_in_a_row(lib):
    """Mixed form: a Chebyshev (32, 32, 33) and a Legendre (96, 97) problem
    alternate on the built-in array; each call against the scratch-taking
    entry point with a fresh workspace."""
    from shenfun_gb300.problem import HelmholtzProblem
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    probs = [(HelmholtzProblem((32, 32, 33), "chebyshev", c=10.0, form="mixed"), (32, 32, 33)),
             (HelmholtzProblem((96, 97), "legendre", c=10.0, form="mixed"), (96, 97))]
    rng = np.random.default_rng(7)
    for rep in range(2):
        for prob, N in probs:
            assert prob.workspace_bytes <= (64 << 20)
            f = torch.as_tensor(rng.standard_normal(N), device="cuda")
            work = torch.empty(prob.workspace_bytes, dtype=torch.uint8, device="cuda")
            ref = torch.empty_like(f)
            assert lib.sgpu_helmholtz_solve(prob._h, _p(f), _p(ref), _p(work),
                                            ctypes.c_size_t(work.numel()), stream) == 0
            got = torch.full_like(f, float("nan"))
            st = lib.sgpu_helmholtz_solve_noalloc(prob._h, _p(f), _p(got), stream)
            assert st == 0, lib.sgpu_status_string(st)
            torch.cuda.synchronize()
            err = ((got - ref).abs().max() / ref.abs().max()).item()
            assert err <= TOL, (rep, N, err)


def test_noalloc_rejects_problems_beyond_its_scratch(lib):
    from shenfun_gb300 import _lib
    from shenfun_gb300.problem import HelmholtzProblem
    prob = HelmholtzProblem((256, 256, 65), "chebyshev", c=1.0)
    assert prob.workspace_bytes > (64 << 20)
    f = torch.zeros((256, 256, 65), dtype=torch.float64, device="cuda")
    u = torch.zeros_like(f)
    st = lib.sgpu_helmholtz_solve_noalloc(prob._h, _p(f), _p(u),
                                          ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == _lib.ERR_SCRATCH_LIMIT
    assert b"64 MiB" in lib.sgpu_status_string(st)
