"""GPU: Legendre transforms in the mixed form (BF16 digit slices on the
tensor cores, tcgen05) against the oracle and the reference's golden
fixtures.  Tolerance of the mixed form: normwise relative 1e-10 (the scheme
keeps about 48 bits; the measured error is near 1e-13)."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import spectral as S

pytestmark = pytest.mark.gpu

TOL = 1e-10


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else a
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def dev(a):
    return torch.as_tensor(np.ascontiguousarray(a), device="cuda")


@pytest.fixture(scope="module")
def L():
    from shenfun_gb300 import build
    build.build()
    from shenfun_gb300 import legendre
    return legendre


def space(L, basis, N):
    cls = {"L": L.LegendreOrthogonal, "SD": L.LegendreShenDirichlet, "SB": L.LegendreShenBiharmonic}[basis]
    return cls(N, form="mixed")


def timeouts():
    from shenfun_gb300 import _lib
    c = ctypes.c_uint()
    _lib.call("sgpu_wait_timeouts", ctypes.byref(c))
    return c.value


@pytest.mark.parametrize("N", [16, 33, 64])
@pytest.mark.parametrize("kind", ["recursive", "vandermonde"])
def test_golden_mixed(L, golden, N, kind):
    d = golden("legendre")
    for tag, basis in (("L", "L"), ("LD", "SD")):
        V = space(L, basis, N)
        assert rel(V.scalar_product(dev(d[f"{tag}{N}_f"]), kind=kind), d[f"{tag}{N}_sp_{kind}"]) < TOL
        assert rel(V.backward(dev(d[f"{tag}{N}_uh"]), kind=kind), d[f"{tag}{N}_bw_{kind}"]) < TOL
        assert rel(V.forward(dev(d[f"{tag}{N}_f"]), kind=kind), d[f"{tag}{N}_fw_{kind}"]) < TOL
    assert timeouts() == 0


@pytest.mark.parametrize("N", [12, 40, 129, 256])
@pytest.mark.parametrize("basis", ["L", "SD", "SB"])
@pytest.mark.parametrize("cplx", [False, True])
def test_axis_mixed(L, N, basis, cplx):
    V = space(L, basis, N)
    rng = np.random.default_rng(N)
    # 300 x 3 lines: three 128-row tiles, the last one ragged; and a middle axis
    for shape, axis in (((300, 3, N), 2), ((4, N, 37), 1)):
        x = rng.standard_normal(shape)
        if cplx:
            x = x + 1j * rng.standard_normal(shape)
        assert rel(V.scalar_product(dev(x), axis=axis), S.leg_scalar_product(x, basis, axis)) < TOL
        fw = S.leg_forward(x, basis, axis)
        assert rel(V.forward(dev(x), axis=axis), fw) < (TOL if basis != "SB" else 1e-9)
        assert rel(V.backward(dev(fw), axis=axis), S.leg_backward(fw, basis, axis)) < TOL
    assert timeouts() == 0


@pytest.mark.parametrize("N,lines", [(512, 4096), (1024, 1000), (1100, 700), (2048, 500)])
def test_mixed_vs_plain_large(L, N, lines):
    """cfg-size lines with k^-2-decaying coefficients: backward then forward
    in both forms; the mixed form within 1e-10 of the FP64 one, and the round
    trip returns the coefficients."""
    rng = np.random.default_rng(0)
    c = rng.uniform(-1, 1, (lines, N)) * (np.arange(N) + 1.0) ** -2
    c[:, -2:] = 0
    cd = dev(c)
    Vp = L.LegendreShenDirichlet(N)
    Vm = space(L, "SD", N)
    up = Vp.backward(cd, axis=1)
    um = Vm.backward(cd, axis=1)
    assert rel(um, up.cpu().numpy()) < TOL
    cm = Vm.forward(um, axis=1)
    assert rel(cm, c) < TOL
    assert rel(Vm.scalar_product(up, axis=1), Vp.scalar_product(up, axis=1).cpu().numpy()) < TOL
    assert timeouts() == 0


def test_mixed_limits(L):
    """Above 1024 the contraction runs in exact K chunks of 1024 (one GEMM
    launch each); lengths beyond 8192 are rejected."""
    from shenfun_gb300 import _lib
    with pytest.raises(_lib.SgpuError):
        L.get_plan(8200, _lib.BASIS_SD, _lib.MIXED_DF)


def test_mixed_chunked_golden_oracle(L):
    """N = 1500 (two K chunks): the mixed backward / scalar product against
    the oracle's FP64 Vandermonde evaluation."""
    N = 1500
    rng = np.random.default_rng(3)
    c = rng.uniform(-1, 1, (64, N)) * (np.arange(N) + 1.0) ** -2
    c[:, -2:] = 0
    V = space(L, "SD", N)
    u = V.backward(dev(c), axis=1)
    ref = S.leg_backward(c, "SD", axis=1, kind="vandermonde")
    assert rel(u, ref) < TOL
    f = rng.standard_normal((64, N))
    assert rel(V.scalar_product(dev(f), axis=1), S.leg_scalar_product(f, "SD", axis=1)) < TOL
    assert timeouts() == 0


@pytest.mark.parametrize("n", [16, 17, 64, 129, 257])
@pytest.mark.parametrize("basis", ["T", "SD", "SB"])
@pytest.mark.parametrize("cplx", [False, True])
def test_chebyshev_mixed_tensor(L, n, basis, cplx):
    """The mixed form's Chebyshev scalar product / forward / backward run as
    tensor-core contractions with the FP64 transform's matrix: within 1e-10
    of the oracle, on contiguous and strided axes, 300+ lines."""
    from shenfun_gb300 import _lib
    from shenfun_gb300.spaces import ChebyshevOrthogonal, ChebyshevShenDirichlet, ChebyshevShenBiharmonic
    V = {"T": ChebyshevOrthogonal, "SD": ChebyshevShenDirichlet, "SB": ChebyshevShenBiharmonic}[basis](n)
    V.form = _lib.MIXED_DF
    rng = np.random.default_rng(n)
    for shape, axis in (((100, 3, n), 2), ((3, n, 41), 1)):
        x = rng.standard_normal(shape)
        if cplx:
            x = x + 1j * rng.standard_normal(shape)
        assert rel(V.scalar_product(dev(x), axis=axis), S.cheb_scalar_product(x, basis, axis)) < TOL
        fw = V.forward(dev(x), axis=axis)
        assert rel(fw, S.cheb_forward(x, basis, axis)) < TOL
        fwn = fw.cpu().numpy()
        assert rel(V.backward(fw, axis=axis), S.cheb_backward(fwn, basis, axis)) < TOL
        # in place (the contraction reads its split copy of the input)
        y = dev(x).clone()
        V.scalar_product(y, y, axis=axis)
        assert rel(y, S.cheb_scalar_product(x, basis, axis)) < TOL
    assert timeouts() == 0
