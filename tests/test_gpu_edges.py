"""GPU edge cases through the C ABI: empty batches (no lines, no systems)
return OK without touching the output, out-of-range sizes are rejected with
SGPU_ERR_ARG / SGPU_ERR_UNSUPPORTED before any launch, and the largest
supported lengths run (reference tests: empty and ragged inputs, maximum
sizes)."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import spectral as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from shenfun_gb300 import build, _lib
    build.build()
    lb = _lib.load()
    assert lb.sgpu_device_ok() == 1
    return lb


def P(t):
    return ctypes.c_void_p(t.data_ptr())


def test_empty_batches(lib):
    from shenfun_gb300 import _lib
    sentinel = torch.full((64,), 7.0, dtype=torch.float64, device="cuda")
    buf = torch.zeros(64, dtype=torch.float64, device="cuda")
    s = None
    h = ctypes.c_void_p()
    assert lib.sgpu_plan_create(ctypes.byref(h), _lib.XF_CHEB_FORWARD, 17, _lib.BASIS_SD, 0) == 0
    assert lib.sgpu_plan_execute(h, P(buf), P(sentinel), 0, 1, 0, ctypes.c_double(1.0), s) == 0
    lib.sgpu_plan_destroy(h)
    assert lib.sgpu_TDMA_Solve(P(sentinel), P(buf), 0, 16, 1, 0, s) == 0
    assert lib.sgpu_helmholtz_solve_cached(P(buf), P(sentinel), P(buf), 0, 0, 17, 1, 0, 0, s) == 0
    assert lib.sgpu_Poisson_Solve_ADD(P(buf), P(sentinel), ctypes.c_double(1.0), 0, 16, 1, 0, s) == 0
    assert lib.sgpu_bc_apply(P(sentinel), None, None, None, None, P(buf), 0, 16, 1, 1, 0, s) == 0
    assert lib.sgpu_fourier_pad(P(buf), P(sentinel), 0, 8, 12, 1, _lib.XF_C2C_BWD, s) == 0
    lp = ctypes.c_void_p()
    assert lib.sgpu_legendre_plan_create(ctypes.byref(lp), 64, _lib.BASIS_SD, _lib.MIXED_DF) == 0
    assert lib.sgpu_legendre_execute(lp, 2, P(buf), P(sentinel), 0, 1, 0, s) == 0
    lib.sgpu_legendre_plan_destroy(lp)
    torch.cuda.synchronize()
    assert torch.all(sentinel == 7.0)


def test_size_limits(lib):
    from shenfun_gb300 import _lib
    h = ctypes.c_void_p()
    assert lib.sgpu_plan_create(ctypes.byref(h), _lib.XF_R2C, (1 << 20) + 1, 0, 0) == _lib.ERR_ARG
    assert lib.sgpu_plan_create(ctypes.byref(h), _lib.XF_CHEB_SCALAR, 3, _lib.BASIS_SD, 0) == _lib.ERR_ARG
    assert lib.sgpu_plan_create(ctypes.byref(h), _lib.XF_CHEB_SCALAR, 16, _lib.BASIS_SB | _lib.BASIS_BC,
                                0) == _lib.ERR_ARG
    lp = ctypes.c_void_p()
    assert lib.sgpu_legendre_plan_create(ctypes.byref(lp), 8193, _lib.BASIS_SD, 0) == _lib.ERR_ARG
    assert lib.sgpu_legendre_plan_create(ctypes.byref(lp), 64, _lib.BASIS_SN, 0) == _lib.ERR_ARG
    buf = torch.zeros(64, dtype=torch.float64, device="cuda")
    assert lib.sgpu_fourier_pad(P(buf), P(buf), 1, 8, 12, 1, _lib.XF_C2C_BWD, None) == _lib.ERR_ARG  # aliasing
    assert lib.sgpu_fourier_pad(P(buf), None, 1, 12, 8, 1, _lib.XF_C2C_BWD, None) == _lib.ERR_ARG


@pytest.mark.parametrize("n", [2, 3, 1024, 4096, 4093])
def test_extreme_fourier_lengths(lib, n):
    """Shortest lengths, a register-FFT length, the largest power of two and
    a large prime (Rader) of the shared-memory line kernels on one line
    (a line's three staging buffers must fit one CTA's shared memory)."""
    from shenfun_gb300.spaces import C2C
    rng = np.random.default_rng(n)
    x = rng.standard_normal((1, n)) + 1j * rng.standard_normal((1, n))
    y = C2C(n).forward(torch.as_tensor(x, device="cuda"), axis=1)
    ref = S.c2c_forward(x, axis=1)
    assert np.abs(y.cpu().numpy() - ref).max() / np.abs(ref).max() < 1e-12


def test_single_line_chebyshev_large(lib):
    """A Chebyshev ShenDirichlet line of 4097 points (plain, and the
    double-float form above the tensor-core range); longer lines than the
    shared memory holds are rejected."""
    from shenfun_gb300 import _lib
    from shenfun_gb300.spaces import ChebyshevShenDirichlet
    h = ctypes.c_void_p()
    assert lib.sgpu_plan_create(ctypes.byref(h), _lib.XF_CHEB_FORWARD, 8193, _lib.BASIS_SD, 0) == \
        _lib.ERR_UNSUPPORTED
    n = 4097
    x = np.random.default_rng(1).standard_normal((2, n))
    for form in (_lib.PLAIN_F64, _lib.MIXED_DF):
        V = ChebyshevShenDirichlet(n)
        V.form = form
        y = V.forward(torch.as_tensor(x, device="cuda"), axis=1)
        ref = S.cheb_forward(x, "SD", 1)
        assert np.abs(y.cpu().numpy() - ref).max() / np.abs(ref).max() < 1e-10
