"""The per-axis plan objects with the FFTW plan interface the reference's
bases use (shenfun_gb300.fftw): FFTW's unnormalised conventions against
scipy.fft (whose norm=None DCTs are FFTW's REDFT10/REDFT01), the
input_array / output_array / __call__ / get_normalization protocol, and the
forward/backward pairing of a basis' plan() (chebyshev/bases.py:407-469,
fourier/bases.py:218-279).  FP64 form: 1e-13 of the largest output."""
import numpy as np
import pytest
import scipy.fft as sfft
import torch

pytestmark = pytest.mark.gpu

TOL = 1e-13


def rel(a, b):
    a = a.cpu().numpy() if isinstance(a, torch.Tensor) else a
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.fixture
def F():
    from shenfun_gb300 import fftw
    return fftw


SHAPES = [((5, 33, 3), 1), ((40,), 0), ((7, 64), -1), ((64, 6), 0), ((4, 257, 2), 1)]


@pytest.mark.parametrize("shape,axis", SHAPES)
@pytest.mark.parametrize("dct_type", [2, 3])
@pytest.mark.parametrize("cplx", [False, True])
def test_dctn(F, shape, axis, dct_type, cplx):
    r = np.random.default_rng(len(shape) + dct_type)
    x = r.standard_normal(shape) + (1j * r.standard_normal(shape) if cplx else 0)
    U = F.aligned(shape, dtype=x.dtype)
    p = F.dctn(U, axes=(axis,), type=dct_type)
    assert p.input_array is U and p.output_array.shape == U.shape
    U.copy_(torch.as_tensor(x))
    y = p()
    assert y is p.output_array
    ref = sfft.dct(x.real, type=dct_type, axis=axis) + (1j * sfft.dct(x.imag, type=dct_type, axis=axis) if cplx else 0)
    assert rel(y, ref) < TOL
    n = shape[axis]
    assert p.get_normalization() == 1.0 / (2 * n)
    assert rel(p(normalize=True), ref / (2 * n)) < TOL


@pytest.mark.parametrize("shape,axis", SHAPES)
def test_complex_dfts(F, shape, axis):
    r = np.random.default_rng(7)
    x = r.standard_normal(shape) + 1j * r.standard_normal(shape)
    n = shape[axis]
    for plan, ref in ((F.fftn, np.fft.fft(x, axis=axis)), (F.ifftn, np.fft.ifft(x, axis=axis) * n)):
        U = F.aligned(shape, dtype=complex)
        p = plan(U, axes=(axis,))
        out = np.zeros(shape, dtype=complex)
        got = p(input_array=torch.as_tensor(x, device="cuda"), output_array=out)  # copies in and out
        assert got is out
        assert rel(out, ref) < TOL
        assert p.get_normalization() == 1.0 / n


@pytest.mark.parametrize("shape,axis", SHAPES)
def test_real_dfts_and_plan_pairing(F, shape, axis):
    """rfftn's output array is irfftn's input, irfftn writes back into the
    forward plan's input (a basis' plan()); backward(forward(x)) = N x."""
    r = np.random.default_rng(8)
    x = r.standard_normal(shape)
    n = shape[axis]
    U = F.aligned(shape, dtype=float)
    fwd = F.rfftn(U, axes=(axis,))
    V = fwd.output_array
    bck = F.irfftn(V, axes=(axis,), s=(n,), output_array=U)
    assert bck.output_array is U and V.shape[axis] == n // 2 + 1
    U.copy_(torch.as_tensor(x))
    assert rel(fwd(), np.fft.rfft(x, axis=axis)) < TOL
    assert rel(bck(), x * n) < TOL
    assert rel(fwd(normalize=True), np.fft.rfft(x * n, axis=axis) / n) < TOL


def test_aligned_like(F):
    z = np.zeros((3, 8), dtype=complex)
    a = F.aligned_like(z, fill=1.0)
    assert a.is_cuda and a.dtype == torch.complex128 and tuple(a.shape) == (3, 8)
    assert bool((a == 1).all())
    b = F.aligned_like(a)
    assert b.is_cuda and b.shape == a.shape and b.dtype == a.dtype


def test_unsupported_kinds(F):
    from shenfun_gb300 import _lib
    U = F.aligned((4, 16))
    for call in (lambda: F.dctn(U, type=1), lambda: F.dctn(U, axes=(0, 1)),
                 lambda: F.irfftn(F.aligned((4, 9), dtype=complex), s=(20,)),
                 lambda: F.fftn(U), lambda: F.rfftn(F.aligned((4, 16), dtype=complex))):
        with pytest.raises(_lib.SgpuError):
            call()
