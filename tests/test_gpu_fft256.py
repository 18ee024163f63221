"""The strided length-256 Fourier kernel (variant 1 of length-256 Fourier
plans) against the generic line programs (variant 2) and the oracle, on the
channel grid's layouts and on ragged ones, in both arithmetic forms."""
import numpy as np
import pytest
import torch

from oracle import spectral as S

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else a
    return float(np.abs(a - b).max() / np.abs(b).max())


def run(kind, form, x, axis, n_out, variant, scale):
    from shenfun_gb300 import _lib
    from shenfun_gb300.plans import LinePlan
    p = LinePlan(kind, 256, form=form)
    p.variant = variant
    assert p.variant == variant
    shape = list(x.shape)
    shape[axis] = n_out
    dt = torch.float64 if kind == _lib.XF_C2R else torch.complex128
    out = torch.empty(shape, dtype=dt, device="cuda")
    p(x, out, axis, scale)
    torch.cuda.synchronize()
    return out


SHAPES = [((256, 129, 257), 0), ((256, 256, 257), 1), ((7, 256, 37), 1), ((256, 33), 0), ((3, 256, 16), 1)]


@pytest.mark.parametrize("form", ["plain", "mixed"])
@pytest.mark.parametrize("shape,axis", SHAPES, ids=[f"{s}-ax{a}" for s, a in SHAPES])
def test_fft256_variants_and_oracle(form, shape, axis):
    from shenfun_gb300 import _lib
    f = _lib.FORMS[form]
    g = np.random.default_rng(sum(shape) + axis)
    small = int(np.prod(shape)) <= 2_000_000
    tol = 1e-13 if form == "plain" else 2e-13
    # C2C forward / backward
    xc = g.standard_normal(shape) + 1j * g.standard_normal(shape)
    xd = torch.as_tensor(xc, device="cuda")
    for kind, scale in ((_lib.XF_C2C_FWD, 1.0 / 256), (_lib.XF_C2C_BWD, 1.0)):
        a = run(kind, f, xd, axis, 256, 1, scale)
        b = run(kind, f, xd, axis, 256, 2, scale)
        assert rel(a, b.cpu().numpy()) < tol
        for v in (3, 4):  # the strided kernel at 2 and 3 CTAs per SM: the same arithmetic
            assert torch.equal(run(kind, f, xd, axis, 256, v, scale), a)
        if small:
            ref = S.c2c_forward(xc, axis=axis) if kind == _lib.XF_C2C_FWD else S.c2c_backward(xc, axis=axis)
            assert rel(a, ref) < tol
    # R2C, then C2R of its output
    xr = g.standard_normal(shape)
    xrd = torch.as_tensor(xr, device="cuda")
    a = run(_lib.XF_R2C, f, xrd, axis, 129, 1, 1.0 / 256)
    b = run(_lib.XF_R2C, f, xrd, axis, 129, 2, 1.0 / 256)
    assert rel(a, b.cpu().numpy()) < tol
    if small:
        assert rel(a, S.r2c_forward(xr, axis=axis)) < tol
    c1 = run(_lib.XF_C2R, f, a, axis, 256, 1, 1.0)
    c2 = run(_lib.XF_C2R, f, a, axis, 256, 2, 1.0)
    assert rel(c1, c2.cpu().numpy()) < tol
    assert rel(c1, xr) < tol  # inverse of the normalised forward


def test_fft256_in_place_c2c():
    from shenfun_gb300 import _lib
    from shenfun_gb300.plans import LinePlan
    g = np.random.default_rng(5)
    xc = g.standard_normal((256, 40, 3)) + 1j * g.standard_normal((256, 40, 3))
    for form in (_lib.PLAIN_F64, _lib.MIXED_DF):
        p = LinePlan(_lib.XF_C2C_FWD, 256, form=form)
        x = torch.as_tensor(xc, device="cuda")
        p(x, x, 0, 1.0 / 256)
        assert rel(x, S.c2c_forward(xc, axis=0)) < 2e-13
