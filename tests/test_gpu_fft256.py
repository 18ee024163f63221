"""The strided length-256 Fourier kernel (variant 1 of length-256 Fourier
plans: FP64, or the mixed form in 64-bit fixed point) against the generic
line programs (variant 2), the double-float kernels (variants 3 / 4) and the
oracle, on the channel grid's layouts and on ragged ones."""
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
        # the strided kernel at 2 and 3 CTAs per SM: the same arithmetic (the
        # mixed form's default is the fixed-point pair 5 / 6, FP64's is 3 / 4)
        pair = (5, 6) if form == "mixed" else (3, 4)
        for v in pair:
            assert torch.equal(run(kind, f, xd, axis, 256, v, scale), a)
        if form == "mixed":
            d3 = run(kind, f, xd, axis, 256, 3, scale)
            assert torch.equal(run(kind, f, xd, axis, 256, 4, scale), d3)
            assert rel(d3, b.cpu().numpy()) < tol
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


@pytest.mark.parametrize("shape,axis", SHAPES, ids=[f"{s}-ax{a}" for s, a in SHAPES])
def test_fft256_fixed_point_variants(shape, axis):
    """Variants 5 and 6 (the mixed form in 64-bit fixed point, 2 and 3 CTAs
    per SM): the same bits at both occupancies, every line to ~1e-15 of its
    own largest entry with line magnitudes spread over 2^-200 .. 2^200, and
    R2C -> C2R returns the input."""
    from shenfun_gb300 import _lib
    f = _lib.MIXED_DF
    g = np.random.default_rng(sum(shape) + 3 * axis)
    small = int(np.prod(shape)) <= 2_000_000
    mshape = [1] * len(shape)
    for d in range(len(shape)):
        if d != axis:
            mshape[d] = shape[d]
    mag = np.exp2(g.integers(-200, 200, mshape).astype(float))

    def line_rel(a, ref):
        a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else a
        err = np.abs(a - ref).max(axis=axis)
        sc = np.abs(ref).max(axis=axis)
        return float((err / np.where(sc > 0, sc, 1.0)).max())

    xc = (g.standard_normal(shape) + 1j * g.standard_normal(shape)) * mag
    xd = torch.as_tensor(xc, device="cuda")
    for kind, scale in ((_lib.XF_C2C_FWD, 1.0 / 256), (_lib.XF_C2C_BWD, 1.0)):
        a = run(kind, f, xd, axis, 256, 5, scale)
        assert torch.equal(run(kind, f, xd, axis, 256, 6, scale), a)
        # variant 7: the input tile of each CTA by one tensor copy (where a
        # CTA's lines lie in one outer block), the same bits
        assert torch.equal(run(kind, f, xd, axis, 256, 7, scale), a)
        if small:
            ref = S.c2c_forward(xc, axis=axis) if kind == _lib.XF_C2C_FWD else S.c2c_backward(xc, axis=axis)
            assert line_rel(a, ref) < 4e-15
    xr = g.standard_normal(shape) * mag
    xrd = torch.as_tensor(xr, device="cuda")
    a = run(_lib.XF_R2C, f, xrd, axis, 129, 5, 1.0 / 256)
    assert torch.equal(run(_lib.XF_R2C, f, xrd, axis, 129, 6, 1.0 / 256), a)
    if small:
        assert line_rel(a, S.r2c_forward(xr, axis=axis)) < 4e-15
    c1 = run(_lib.XF_C2R, f, a, axis, 256, 5, 1.0)
    assert torch.equal(run(_lib.XF_C2R, f, a, axis, 256, 6, 1.0), c1)
    assert line_rel(c1, xr) < 1e-14


def test_fft256_fixed_point_is_mixed_only():
    from shenfun_gb300 import _lib
    from shenfun_gb300.plans import LinePlan
    p = LinePlan(_lib.XF_C2C_FWD, 256, form=_lib.PLAIN_F64)
    with pytest.raises(_lib.SgpuError):
        p.variant = 5
    q = LinePlan(_lib.XF_R2C, 256, form=_lib.MIXED_DF)
    with pytest.raises(_lib.SgpuError):
        q.variant = 7  # the tensor-copy input is a C2C variant


def test_fft256_tensor_copy_waits_complete():
    """The tensor-copy C2C kernel on the channel grid's x axis: no bounded
    wait gave up."""
    import ctypes
    from shenfun_gb300 import _lib
    x = torch.randn(256, 129, 257, dtype=torch.complex128, device="cuda")
    run(_lib.XF_C2C_FWD, _lib.MIXED_DF, x, 0, 256, 7, 1.0 / 256)
    c = ctypes.c_uint()
    _lib.call("sgpu_wait_timeouts", ctypes.byref(c))
    assert c.value == 0


def test_fft256_fixed_point_unaligned_complex_falls_back():
    """Complex arrays that are not 16-byte aligned (reachable through the C
    ABI) run the generic programs instead of the fixed-point kernel's 16-byte
    loads and stores, with the same results to rounding."""
    import ctypes
    from shenfun_gb300 import _lib
    from shenfun_gb300.plans import LinePlan
    from shenfun_gb300.device import stream_handle
    g = np.random.default_rng(11)
    outer, inner = 3, 40
    xc = g.standard_normal((outer, 256, inner)) + 1j * g.standard_normal((outer, 256, inner))
    n = xc.size
    buf_in = torch.zeros(2 * n + 1, dtype=torch.float64, device="cuda")
    buf_out = torch.zeros(2 * n + 1, dtype=torch.float64, device="cuda")
    buf_in[1:].copy_(torch.as_tensor(xc.view(np.float64).ravel(), device="cuda"))
    p = LinePlan(_lib.XF_C2C_FWD, 256, form=_lib.MIXED_DF)
    _lib.call("sgpu_plan_execute", p._h, ctypes.c_void_p(buf_in.data_ptr() + 8),
              ctypes.c_void_p(buf_out.data_ptr() + 8), outer, inner, _lib.COMPLEX, 1.0 / 256, stream_handle())
    torch.cuda.synchronize()
    got = buf_out[1:].cpu().numpy().view(np.complex128).reshape(xc.shape)
    assert rel(got, S.c2c_forward(xc, axis=1)) < 2e-13


@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_small_launch_same_bits_as_large(form):
    """A small array runs the line programs with fewer lines per CTA (so that
    it spreads over more SMs); its lines come out with the bits they get
    inside a large array."""
    from shenfun_gb300 import _lib
    from shenfun_gb300.plans import LinePlan
    f = _lib.FORMS[form]
    g = np.random.default_rng(21)
    big = g.standard_normal((4096, 64))
    small = big[:40].copy()
    for kind, basis, n_out in ((_lib.XF_R2C, _lib.BASIS_ORTHO, 33), (_lib.XF_CHEB_SCALAR, _lib.BASIS_SD, 64)):
        p = LinePlan(kind, 64, basis=basis, form=f)
        dt = torch.complex128 if kind == _lib.XF_R2C else torch.float64
        yb = torch.empty((4096, n_out), dtype=dt, device="cuda")
        ys = torch.empty((40, n_out), dtype=dt, device="cuda")
        scale = 1.0 / 64 if kind == _lib.XF_R2C else 1.0
        p(torch.as_tensor(big, device="cuda"), yb, 1, scale)
        p(torch.as_tensor(small, device="cuda"), ys, 1, scale)
        torch.cuda.synchronize()
        assert torch.equal(ys, yb[:40])
