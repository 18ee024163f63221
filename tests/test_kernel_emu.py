"""CPU run of the CUDA block programs (index math, buffer bounds, numerics).

The library's kernel bodies are __host__ __device__ block programs; the
harness tests/kernel_emu/emu.cpp runs them on the CPU (one emulated thread per
block) under AddressSanitizer/UBSan on exactly-sized buffers and compares the
results with the oracle.  This checks every index and every buffer bound of
each kernel before the code runs on a GPU.  No GPU needed.
"""
import hashlib
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

from oracle import spectral as S, la

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EMU_DIR = os.path.join(REPO, "tests", "kernel_emu")
EMU = os.path.join(EMU_DIR, "_build", "emu")
CSRC = os.path.join(REPO, "shenfun_gb300", "csrc")

# transform kinds / bases (include/shenfun_gb300.h)
R2C, C2R, C2C_FWD, C2C_BWD, DCT2, DCT3, CHEB_SCALAR, CHEB_FORWARD, CHEB_BACKWARD = range(1, 10)
BASIS = {"T": 0, "SD": 1, "SB": 2, "SN": 3}


def _emu_stamp():
    h = hashlib.sha256()
    for d in (CSRC, EMU_DIR, os.path.join(REPO, "include")):
        for f in sorted(os.listdir(d)):
            p = os.path.join(d, f)
            if os.path.isfile(p) and f.endswith((".cuh", ".cpp", ".h")):
                h.update(open(p, "rb").read())
    return h.hexdigest()


@pytest.fixture(scope="module")
def emu():
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    os.makedirs(os.path.dirname(EMU), exist_ok=True)
    stamp = _emu_stamp()
    sf = EMU + ".stamp"
    if not (os.path.exists(EMU) and os.path.exists(sf) and open(sf).read() == stamp):
        cuda_inc = "/usr/local/cuda/include"
        cmd = ["g++", "-O1", "-g", "-std=c++17", "-fsanitize=address,undefined",
               "-fno-sanitize-recover=all", "-fno-omit-frame-pointer",
               "-I" + cuda_inc, "-I" + os.path.join(REPO, "include"),
               os.path.join(EMU_DIR, "emu.cpp"), "-o", EMU]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        open(sf, "w").write(stamp)
    return EMU


def run(emu, args, inputs, out_count):
    with tempfile.TemporaryDirectory() as td:
        paths = []
        for i, arr in enumerate(inputs):
            p = os.path.join(td, f"in{i}.bin")
            np.ascontiguousarray(arr).view(np.float64).ravel().tofile(p)
            paths.append(p)
        outp = os.path.join(td, "out.bin")
        env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0:abort_on_error=1")
        r = subprocess.run([emu] + [str(a) for a in args] + paths + [outp], capture_output=True,
                           text=True, env=env)
        assert r.returncode == 0, r.stderr[-3000:]
        return np.fromfile(outp, dtype=np.float64, count=out_count)


def xform(emu, kind, n, basis, arr, axis, data_complex, scale=1.0, n_out=None):
    """Run a transform along `axis` of arr (C-contiguous) through the emulator."""
    arr = np.ascontiguousarray(arr)
    outer = int(np.prod(arr.shape[:axis]))
    inner = int(np.prod(arr.shape[axis + 1:]))
    n_out = n_out if n_out is not None else arr.shape[axis]
    out_complex = {R2C: True, C2R: False}.get(kind, data_complex)
    shape = list(arr.shape)
    shape[axis] = n_out
    cnt = int(np.prod(shape)) * (2 if out_complex else 1)
    res = run(emu, ["xform", kind, n, basis, outer, inner, 1 if data_complex else 0, repr(scale)],
              [arr], cnt)
    if out_complex:
        res = res.view(np.complex128)
    return res.reshape(shape)


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


rng = np.random.default_rng(7)


@pytest.mark.parametrize("n", [2, 3, 4, 5, 6, 8, 12, 16, 17, 30, 43, 45, 64, 97, 128, 129, 256, 257])
def test_fourier_r2c_c2r(emu, n):
    x = rng.standard_normal((3, n, 5))
    y = xform(emu, R2C, n, 0, x, 1, False, 1.0 / n, n // 2 + 1)
    assert rel(y, S.r2c_forward(x, axis=1)) < 1e-13
    z = xform(emu, C2R, n, 0, y, 1, True, 1.0, n)
    assert rel(z, S.r2c_backward(y, n, axis=1)) < 1e-13
    # contiguous axis, odd number of lines
    x2 = rng.standard_normal((7, n))
    y2 = xform(emu, R2C, n, 0, x2, 1, False, 1.0, n // 2 + 1)
    assert rel(y2, np.fft.rfft(x2, axis=1)) < 1e-13


@pytest.mark.parametrize("n", [2, 3, 7, 8, 11, 16, 43, 60, 64, 129, 256, 257])
def test_fourier_c2c(emu, n):
    x = rng.standard_normal((n, 6)) + 1j * rng.standard_normal((n, 6))
    y = xform(emu, C2C_FWD, n, 0, x, 0, True, 1.0 / n)
    assert rel(y, S.c2c_forward(x, axis=0)) < 1e-13
    z = xform(emu, C2C_BWD, n, 0, y, 0, True, 1.0)
    assert rel(z, S.c2c_backward(y, axis=0)) < 1e-13


@pytest.mark.parametrize("n", [4, 5, 8, 9, 16, 17, 33, 64, 129, 257])
@pytest.mark.parametrize("cplx", [False, True])
def test_raw_dct(emu, n, cplx):
    import scipy.fft as sfft
    x = rng.standard_normal((5, n))
    if cplx:
        x = x + 1j * rng.standard_normal((5, n))
    y = xform(emu, DCT2, n, 0, x, 1, cplx, 1.0)
    ref = sfft.dct(x.real, 2, axis=1) + (1j * sfft.dct(x.imag, 2, axis=1) if cplx else 0)
    assert rel(y, ref) < 1e-13
    y3 = xform(emu, DCT3, n, 0, x, 1, cplx, 0.5)
    ref3 = (sfft.dct(x.real, 3, axis=1) + (1j * sfft.dct(x.imag, 3, axis=1) if cplx else 0)) * 0.5
    assert rel(y3, ref3) < 1e-13


@pytest.mark.parametrize("n", [12, 16, 17, 33, 64, 129, 257])
@pytest.mark.parametrize("basis", ["T", "SD", "SB", "SN"])
@pytest.mark.parametrize("layout", ["last", "middle"])
@pytest.mark.parametrize("cplx", [False, True])
def test_chebyshev(emu, n, basis, layout, cplx):
    shape = (3, 4, n) if layout == "last" else (2, n, 5)
    axis = 2 if layout == "last" else 1
    x = rng.standard_normal(shape)
    if cplx:
        x = x + 1j * rng.standard_normal(shape)
    b = BASIS[basis]
    sp_ = xform(emu, CHEB_SCALAR, n, b, x, axis, cplx)
    assert rel(sp_, S.cheb_scalar_product(x, basis, axis)) < 1e-13
    fw = xform(emu, CHEB_FORWARD, n, b, x, axis, cplx)
    # The ShenBiharmonic mass solve amplifies input rounding by ~1e3 at
    # n = 129..257 (a 1e-16 relative input perturbation moves the oracle's own
    # output by 4e-14..2e-13), so its bound is wider.
    tol = 1e-12 if basis != "SB" else 5e-11
    assert rel(fw, S.cheb_forward(x, basis, axis)) < tol
    bw = xform(emu, CHEB_BACKWARD, n, b, fw, axis, cplx)
    assert rel(bw, S.cheb_backward(fw, basis, axis)) < 1e-13


@pytest.mark.parametrize("N,outer,inner", [(8, 1, 3), (17, 4, 1), (33, 2, 5), (64, 3, 1), (257, 2, 3)])
@pytest.mark.parametrize("cplx", [False, True])
def test_helmholtz(emu, N, outer, inner, cplx):
    ns = outer * inner
    alfa = -np.ones(ns)
    beta = rng.uniform(0.5, 2000.0, ns)
    fac = run(emu, ["hlu", N, outer, inner], [alfa, beta], 4 * outer * N * inner)
    fac = fac.reshape(4, outer, N, inner)
    d0, d1, d2, L = la.helmholtz_lu(N, alfa, beta)
    to_sys = lambda a: np.moveaxis(a, 1, -1).reshape(ns, N)  # noqa: E731
    for got, ref in zip(fac, (d0, d1, d2, L)):
        assert rel(to_sys(got), ref) < 1e-14
    f = rng.standard_normal((outer, N, inner))
    if cplx:
        f = f + 1j * rng.standard_normal((outer, N, inner))
    cnt = outer * N * inner * (2 if cplx else 1)
    u = run(emu, ["hsolve", N, outer, inner, int(cplx)], [f, fac], cnt)
    u = u.view(np.complex128) if cplx else u
    u = u.reshape(outer, N, inner)
    uref = la.helmholtz_solve(to_sys(f), d0, d1, d2, L)
    assert rel(to_sys(u)[:, :N - 2], uref[:, :N - 2]) < 1e-13
    mv = run(emu, ["hmatvec", N, outer, inner, int(cplx)], [u, alfa, beta], cnt)
    mv = (mv.view(np.complex128) if cplx else mv).reshape(outer, N, inner)
    assert rel(to_sys(mv), la.helmholtz_matvec(to_sys(u), alfa, beta)) < 1e-13
    # the matvec undoes the solve on the dofs
    assert rel(to_sys(mv)[:, :N - 2], to_sys(f)[:, :N - 2]) < 1e-11


@pytest.mark.parametrize("n,outer,inner", [(14, 1, 4), (30, 3, 1), (255, 2, 2)])
@pytest.mark.parametrize("which", ["tdma", "pdma"])
@pytest.mark.parametrize("cplx", [False, True])
def test_banded(emu, n, outer, inner, which, cplx):
    rows = 3 if which == "tdma" else 5
    raw = np.zeros((rows, n))
    raw[rows // 2] = 4.0 + rng.uniform(0, 1, n)
    for r in range(rows):
        if r != rows // 2:
            raw[r] = rng.uniform(-1, 1, n)
    u = rng.standard_normal((outer, n, inner))
    if cplx:
        u = u + 1j * rng.standard_normal((outer, n, inner))
    cnt = outer * n * inner * (2 if cplx else 1)
    got = run(emu, [which, n, outer, inner, int(cplx)], [raw, u], cnt)
    got = (got.view(np.complex128) if cplx else got).reshape(outer, n, inner)
    data = raw.copy()
    if which == "tdma":
        la.tdma_lu(data)
        ref = la.tdma_solve(u, data, axis=1)
    else:
        la.pdma_lu(data)
        ref = la.pdma_solve(u, data, axis=1)
    assert rel(got, ref) < 1e-13


# --------------------------------------------------------------------------
# mixed (double-float) form
def test_df_conversions_and_ops(emu):
    n = 20000
    # magnitudes 1e-15..1e15; below 2^-75 the low word degrades gradually and
    # below 2^-120 values flush to zero, which the mixed form accepts
    x = rng.standard_normal(n) * 10.0 ** rng.uniform(-15, 15, n)
    y = rng.standard_normal(n) * 10.0 ** rng.uniform(-3, 3, n)
    x[:5] = [0.0, -0.0, 1.0, -1.0, 3.0]
    y[:5] = [1.0, 2.0, -1.0, 0.0, 1e-20]
    out = run(emu, ["dfops", n], [x, y], 4 * n).reshape(n, 4)
    eps = 2.0 ** -46  # df carries ~46-48 significant bits (truncating split, sloppy product)
    assert np.all(np.abs(out[:, 0] - x) <= eps * np.abs(x))
    for j, ref in ((1, x + y), (2, x - y), (3, x * y)):
        scale = np.maximum(np.abs(x), np.abs(y)) if j < 3 else np.abs(x * y)
        assert np.all(np.abs(out[:, j] - ref) <= 8 * eps * scale + 1e-300), j


def xform_df(emu, *a, **k):
    os.environ["SGPU_EMU_FORM"] = "1"
    try:
        return xform(emu, *a, **k)
    finally:
        del os.environ["SGPU_EMU_FORM"]


DF_TOL = 1e-12


@pytest.mark.parametrize("n", [8, 16, 17, 43, 129, 256, 257])
def test_df_fourier(emu, n):
    x = rng.standard_normal((3, n, 5))
    y = xform_df(emu, R2C, n, 0, x, 1, False, 1.0 / n, n // 2 + 1)
    assert rel(y, S.r2c_forward(x, axis=1)) < DF_TOL
    z = xform_df(emu, C2R, n, 0, y, 1, True, 1.0, n)
    assert rel(z, S.r2c_backward(y, n, axis=1)) < DF_TOL
    xc = rng.standard_normal((n, 4)) + 1j * rng.standard_normal((n, 4))
    yc = xform_df(emu, C2C_FWD, n, 0, xc, 0, True, 1.0 / n)
    assert rel(yc, S.c2c_forward(xc, axis=0)) < DF_TOL
    assert rel(xform_df(emu, C2C_BWD, n, 0, yc, 0, True, 1.0), xc) < DF_TOL


@pytest.mark.parametrize("n", [16, 17, 64, 129, 257])
@pytest.mark.parametrize("basis", ["T", "SD", "SB", "SN"])
@pytest.mark.parametrize("cplx", [False, True])
def test_df_chebyshev(emu, n, basis, cplx):
    x = rng.standard_normal((3, 2, n))
    if cplx:
        x = x + 1j * rng.standard_normal(x.shape)
    b = BASIS[basis]
    assert rel(xform_df(emu, CHEB_SCALAR, n, b, x, 2, cplx), S.cheb_scalar_product(x, basis, 2)) < DF_TOL
    fw = S.cheb_forward(x, basis, 2)
    assert rel(xform_df(emu, CHEB_BACKWARD, n, b, fw, 2, cplx), S.cheb_backward(fw, basis, 2)) < DF_TOL


@pytest.mark.parametrize("N,outer,inner", [(8, 1, 3), (17, 4, 1), (33, 2, 5), (257, 3, 2)])
@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("form", [0, 1, 2, 3])
def test_helmholtz_cached(emu, N, outer, inner, cplx, form):
    """Cached solves: FP64 (form 0), double-float (1), FP32 sweeps refined by
    an FP64 (2) or double-float (3) residual, against the oracle's FP64 LU."""
    ns = outer * inner
    alfa = -np.ones(ns)
    beta = rng.uniform(0.5, 2000.0, ns)
    f = rng.standard_normal((outer, N, inner))
    if cplx:
        f = f + 1j * rng.standard_normal(f.shape)
    cnt = outer * N * inner * (2 if cplx else 1)
    u = run(emu, ["hcached", N, outer, inner, int(cplx), form], [alfa, beta, f], cnt)
    u = (u.view(np.complex128) if cplx else u).reshape(outer, N, inner)
    to_sys = lambda a: np.moveaxis(a, 1, -1).reshape(ns, N)  # noqa: E731
    uref = la.helmholtz_solve(to_sys(f), *la.helmholtz_lu(N, alfa, beta))
    tol = {0: 1e-13, 1: 1e-12, 2: 1e-12, 3: 1e-12}[form]
    assert rel(to_sys(u)[:, :N - 2], uref[:, :N - 2]) < tol


@pytest.mark.parametrize("N,nlines,inner,cplx,precise", [(40, 130, 1, 0, 0), (130, 70, 1, 0, 0),
                                                         (33, 50, 5, 1, 0), (24, 300, 3, 0, 0),
                                                         (64, 129, 1, 1, 0), (100, 40, 2, 1, 0),
                                                         (40, 130, 1, 0, 1), (90, 60, 3, 1, 1),
                                                         (90, 60, 3, 1, 2), (130, 70, 1, 0, 2)])
def test_ozaki_contraction(emu, N, nlines, inner, cplx, precise):
    """Split-BF16 tensor-core contraction (row exponents, digit split, slice
    tiles, MMA operand addressing from the descriptors, integer epilogue)
    against the FP64 product: normwise relative error below 5e-13 with 7
    digits, 5e-15 with 8 digits and a fifth exact group."""
    r = np.random.default_rng(N + nlines)
    outer = nlines // inner
    nlines = outer * inner
    shape = (outer, N, inner)
    # coefficients decaying like (k+1)^-2, one zero line, one line of huge range
    x = r.uniform(-1, 1, shape) / (np.arange(N)[None, :, None] + 1.0) ** 2
    if cplx:
        x = x + 1j * r.uniform(-1, 1, shape)
    x[0, :, 0] = 0
    x[-1, :, -1] *= np.logspace(0, -30, N)
    M = r.standard_normal((N, N)) * np.logspace(0, -3, N)[None, :]
    res = run(emu, ["ozaki", N, nlines, inner, cplx, precise], [x, M], x.size * (2 if cplx else 1))
    if cplx:
        res = res.view(np.complex128)
    res = res.reshape(shape)
    ref = np.einsum("ojl,jk->okl", x, M)
    # per output column the error is relative to |x| |M[:, k]|
    scale = np.einsum("ojl,jk->okl", np.abs(x), np.abs(M)).max()
    assert np.abs(res - ref).max() / scale < (5e-15 if precise else 5e-13)
    # and the all-zero line stays exactly zero
    assert np.all(res[0, :, 0] == 0)


@pytest.mark.parametrize("N,nlines,cplx,bn", [(257, 70, 0, 64), (257, 40, 1, 32), (129, 100, 0, 64),
                                              (130, 33, 1, 32), (64, 65, 0, 64), (200, 20, 1, 64),
                                              (300, 20, 0, 32), (339, 30, 0, 64), (16, 7, 0, 32)])
def test_fused_contraction(emu, N, nlines, cplx, bn):
    """Fused split-BF16 contraction (the cluster's row shares, the B-stage
    offsets of every rank, the MMAs of each 128-output tile from their
    descriptors, the FP64 dot-product outputs past the last full tile, the
    integer epilogue) against the FP64 product: normwise error below 1e-14 of
    |x| |M| (the 36-product contraction it replaces measures 5e-15 - 6e-15 on
    the same data), tail tiles and zero lines included."""
    r = np.random.default_rng(N + nlines)
    x = r.uniform(-1, 1, (nlines, N)) / (np.arange(N)[None, :] + 1.0) ** 2
    if cplx:
        x = x + 1j * r.uniform(-1, 1, (nlines, N))
    x[0] = 0
    x[-1] *= np.logspace(0, -30, N)
    M = r.standard_normal((N, N)) * np.logspace(0, -3, N)[None, :]
    res = run(emu, ["lcf", N, nlines, int(cplx), bn], [x, M], x.size * (2 if cplx else 1))
    if cplx:
        res = res.view(np.complex128)
    res = res.reshape(x.shape)
    ref = x @ M
    scale = (np.abs(x) @ np.abs(M)).max()
    assert np.abs(res - ref).max() / scale < 1e-14
    assert np.all(res[0] == 0)


@pytest.mark.parametrize("N", [257, 129])
def test_fused_contraction_ignored_rows(emu, N):
    """K < N (the backward transform ignores the two boundary dofs): large
    values there neither set the line scale nor enter the product."""
    nlines = 40
    r = np.random.default_rng(N)
    x = r.standard_normal((nlines, N)) * 1e-4
    x[:, -2:] = 1e6
    M = r.standard_normal((N, N))
    M[-2:, :] = 0
    res = run(emu, ["lcf", N, nlines, 0, 64], [x, M], x.size).reshape(x.shape)
    ref = x[:, :-2] @ M[:-2, :]
    assert np.abs(res - ref).max() / np.abs(ref).max() < 1e-14


@pytest.mark.parametrize("N,precise", [(53, 0), (65, 0), (97, 1), (257, 1)])
def test_ozaki_ignored_tail_rows(emu, N, precise):
    """A matrix whose last rows are zero (a backward transform ignores the
    boundary dofs) must not let large values there set the line's scale;
    the contraction then runs over the active K blocks only (N = 65, 97,
    257: one K block fewer than the matrix tiles hold)."""
    nlines = 40
    r = np.random.default_rng(5)
    x = r.standard_normal((nlines, N)) * 1e-4
    x[:, -2:] = 1e6  # ignored entries, far larger than the used ones
    M = r.standard_normal((N, N))
    M[-2:, :] = 0
    res = run(emu, ["ozaki", N, nlines, 1, 0, precise], [x, M], x.size).reshape(x.shape)
    ref = x[:, :-2] @ M[:-2, :]
    assert np.abs(res - ref).max() / np.abs(ref).max() < (5e-15 if precise else 5e-13)


# --------------------------------------------------------------------------
# Chebyshev ShenNeumann: Helmholtz Neumann branch, Neumann matvec, Poisson
# ADD / ANN solves (la.pyx:735-751, 907-912; chebyshev/la.py:11-128)
@pytest.mark.parametrize("N,outer,inner", [(8, 1, 3), (17, 4, 1), (33, 2, 5), (257, 2, 3)])
@pytest.mark.parametrize("cplx", [False, True])
def test_helmholtz_neumann(emu, N, outer, inner, cplx):
    ns = outer * inner
    alfa = -np.ones(ns)
    beta = rng.uniform(0.5, 2000.0, ns)
    beta[0] = 0.0  # the pure-stiffness (zero-mode) system
    fac = run(emu, ["nlu", N, outer, inner], [alfa, beta], 4 * outer * N * inner)
    fac = fac.reshape(4, outer, N, inner)
    d0, d1, d2, L = la.helmholtz_lu(N, alfa, beta, neumann=True)
    to_sys = lambda a: np.moveaxis(a, 1, -1).reshape(ns, N)  # noqa: E731
    for got, ref in zip(fac, (d0, d1, d2, L)):
        assert rel(to_sys(got), ref) < 1e-14
    f = rng.standard_normal((outer, N, inner))
    if cplx:
        f = f + 1j * rng.standard_normal((outer, N, inner))
    cnt = outer * N * inner * (2 if cplx else 1)
    uref = la.helmholtz_solve(to_sys(f), d0, d1, d2, L, neumann=True)
    u = run(emu, ["nsolve", N, outer, inner, int(cplx)], [f, fac], cnt)
    u = (u.view(np.complex128) if cplx else u).reshape(outer, N, inner)
    assert rel(to_sys(u)[:, :N - 2], uref[:, :N - 2]) < 1e-13
    for form in (0, 1):
        uc = run(emu, ["ncached", N, outer, inner, int(cplx), form], [alfa, beta, f], cnt)
        uc = (uc.view(np.complex128) if cplx else uc).reshape(outer, N, inner)
        assert rel(to_sys(uc)[:, :N - 2], uref[:, :N - 2]) < (1e-13 if form == 0 else 1e-12)
    mv = run(emu, ["nmatvec", N, outer, inner, int(cplx)], [u, alfa, beta], cnt)
    mv = (mv.view(np.complex128) if cplx else mv).reshape(outer, N, inner)
    ref = la.helmholtz_neumann_matvec(to_sys(u), alfa, beta)
    assert rel(to_sys(mv), ref) < 1e-13
    # the matvec undoes the solve on the dofs of the regular systems
    assert rel(to_sys(mv)[1:, :N - 2], to_sys(f)[1:, :N - 2]) < 1e-11


@pytest.mark.parametrize("N,outer,inner", [(8, 1, 1), (17, 3, 2), (32, 2, 5), (257, 1, 3)])
@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("which", ["padd", "pann"])
def test_poisson(emu, N, outer, inner, cplx, which):
    b = rng.standard_normal((outer, N, inner))
    if cplx:
        b = b + 1j * rng.standard_normal(b.shape)
    scale = -1.0
    cnt = outer * N * inner * (2 if cplx else 1)
    u = run(emu, [which, N, outer, inner, int(cplx), repr(scale)], [b], cnt)
    u = (u.view(np.complex128) if cplx else u).reshape(outer, N, inner)
    if which == "padd":
        A = la.cheb_sd_stiffness(N)
        ref = la.add_solve(b, A[0], -4 * np.pi * (np.arange(N - 4) + 1.0), scale, axis=1)
    else:
        A = la.cheb_sn_stiffness(N)
        ref = la.ann_solve(b, A[0], A[2], scale, axis=1)
    assert rel(u, ref) < 1e-13


# --------------------------------------------------------------------------
# non-homogeneous boundary values: the backward flag (boundary functions in
# to_ortho) and the dof correction / boundary dofs program
@pytest.mark.parametrize("basis", ["SD", "SN"])
@pytest.mark.parametrize("n", [12, 17, 64, 257])
@pytest.mark.parametrize("cplx", [False, True])
def test_backward_boundary_functions(emu, basis, n, cplx):
    from oracle import bcs as BC
    x = rng.standard_normal((3, n, 4))
    if cplx:
        x = x + 1j * rng.standard_normal(x.shape)
    flagged = BASIS[basis] | 0x10
    got = xform(emu, CHEB_BACKWARD, n, flagged, x, 1, cplx)
    assert rel(got, BC.backward_1d(x, basis, axis=1)) < 1e-13
    got_df = xform_df(emu, CHEB_BACKWARD, n, flagged, x, 1, cplx)
    assert rel(got_df, BC.backward_1d(x, basis, axis=1)) < DF_TOL
    # scalar product / forward plans ignore the flag
    f = rng.standard_normal((3, n, 4))
    assert rel(xform(emu, CHEB_FORWARD, n, flagged, f, 1, False), S.cheb_forward(f, basis, 1)) < 1e-12


@pytest.mark.parametrize("N,outer,inner", [(12, 1, 1), (17, 3, 4), (33, 2, 1)])
@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("tables,set_dofs", [(0, 1), (1, 0), (2, 1), (3, 1)])
def test_bc_apply(emu, N, outer, inner, cplx, tables, set_dofs):
    u = rng.standard_normal((outer, N, inner))
    g = rng.standard_normal((outer, 2, inner))
    g[:, :, 0] = 0.0  # lines with zero boundary values are left alone
    if cplx:
        u = u + 1j * rng.standard_normal(u.shape)
        g = g + 1j * rng.standard_normal(g.shape)
        g[:, :, 0] = 0.0
    CA = rng.standard_normal((N - 2, 2))
    CB = rng.standard_normal((N - 2, 2))
    al = rng.standard_normal(outer * inner)
    be = rng.standard_normal(outer * inner)
    cnt = u.size * (2 if cplx else 1)
    got = run(emu, ["bcapply", N, outer, inner, int(cplx), set_dofs, tables], [u, CA, al, CB, be, g], cnt)
    got = (got.view(np.complex128) if cplx else got).reshape(u.shape)
    ref = u.copy()
    for o in range(outer):
        for i in range(inner):
            s = o * inner + i
            C = np.zeros((N - 2, 2))
            if tables & 1:
                C += al[s] * CA
            if tables & 2:
                C += be[s] * CB
            if np.any(g[o, :, i] != 0):
                ref[o, :N - 2, i] -= C @ g[o, :, i]
            if set_dofs:
                ref[o, N - 2:, i] = g[o, :, i]
    assert rel(got, ref) < 1e-14


@pytest.mark.parametrize("N,nlines,kchunk,precise", [(150, 70, 2, 0), (200, 40, 3, 1), (97, 50, 1, 0)])
def test_ozaki_k_chunks(emu, N, nlines, kchunk, precise):
    """Contractions longer than one exact K chunk run as one GEMM launch per
    chunk, each adding its FP64 result to the previous ones (the GPU's chunk
    is 1024; small chunks here exercise the same launch sequence)."""
    r = np.random.default_rng(N)
    x = r.uniform(-1, 1, (nlines, N, 1)) / (np.arange(N)[None, :, None] + 1.0)
    M = r.standard_normal((N, N))
    res = run(emu, ["ozakic", N, nlines, 1, 0, precise, kchunk], [x, M], x.size).reshape(x.shape)
    ref = np.einsum("ojl,jk->okl", x, M)
    scale = np.einsum("ojl,jk->okl", np.abs(x), np.abs(M)).max()
    # the chunks' FP64 sums add a few ulps of the partial results
    tol = 2e-14 if precise else 5e-13
    assert np.abs(res - ref).max() / scale < tol
    one = run(emu, ["ozaki", N, nlines, 1, 0, precise], [x, M], x.size).reshape(x.shape)
    assert np.abs(res - one).max() / scale < tol


# --------------------------------------------------------------------------
# the general banded LU / solve (DiagMA, TwoDMA, ThreeDMA, FDMA, HeptaDMA)
@pytest.mark.parametrize("offsets", [(0,), (0, 2), (0, 2, 4), (-2, 0, 2, 4), (-4, -2, 0, 2, 4, 6, 8)])
@pytest.mark.parametrize("n,outer,inner", [(12, 1, 3), (17, 4, 1), (33, 2, 5)])
@pytest.mark.parametrize("cplx", [False, True])
def test_general_banded(emu, offsets, n, outer, inner, cplx):
    raw = np.zeros((len(offsets), n))
    for r, o in enumerate(offsets):
        lo, hi = max(0, o), n + min(0, o)
        raw[r, lo:hi] = (4.0 + rng.uniform(0, 1, hi - lo)) if o == 0 else rng.uniform(-0.5, 0.5, hi - lo)
    u = rng.standard_normal((outer, n, inner))
    if cplx:
        u = u + 1j * rng.standard_normal(u.shape)
    cnt = u.size * (2 if cplx else 1)
    got = run(emu, ["banded", n, len(offsets), outer, inner, int(cplx)],
              [np.array(offsets, dtype=float), raw, u], cnt)
    got = (got.view(np.complex128) if cplx else got).reshape(u.shape)
    data = raw.copy()
    la.banded_lu(data, offsets)
    assert rel(got, la.banded_solve(u, data, offsets, axis=1)) < 1e-14
    ref = np.einsum("ij,ojk->oik", np.linalg.inv(la.dia_dense(raw, offsets)), u)
    assert rel(got, ref) < 1e-12


# ---- reference-signature programs (ref_progs.cuh) ---------------------------
from oracle import refabi as RA  # noqa: E402

_BIH_SHORT = (0, 2, 4, 2, 0, 2, 4, 2, 0, 2, 4)


def _bih_diags(g, n):
    """Random diagonals with a dominant main diagonal, lengths n - short."""
    out = []
    for q, short in enumerate(_BIH_SHORT):
        main = q in (0, 4, 8)
        out.append((3.0 + g.uniform(0, 1, n - short)) if main else g.uniform(-0.5, 0.5, n - short))
    return out


@pytest.mark.parametrize("M,outer,inner,cplx", [(5, 2, 1, 0), (6, 1, 3, 1), (9, 3, 2, 1), (33, 2, 5, 0)])
def test_biharmonic_reference_layout(emu, M, outer, inner, cplx):
    g = np.random.default_rng(M * 7 + inner)
    n, N = 2 * M, 2 * M + 4
    diags = _bih_diags(g, n)
    a0 = 1.0
    alfa = g.uniform(-3, 3, outer * inner)
    beta = g.uniform(0.5, 4, outer * inner)
    shape = (outer, N, inner)
    f = g.standard_normal(shape) + (1j * g.standard_normal(shape) if cplx else 0)
    res = run(emu, ["bih", outer, M, inner, cplx, repr(a0)], [alfa, beta] + diags + [f],
              7 * 2 * outer * inner * M + f.size * (2 if cplx else 1))
    fsz = 2 * outer * M * inner
    got = [res[q * fsz:(q + 1) * fsz].reshape(2, outer, M, inner) for q in range(7)]
    u = res[7 * fsz:]
    u = (u.view(np.complex128) if cplx else u).reshape(shape)
    ref = [np.zeros((2, outer, M, inner)) for _ in range(7)]
    RA.lu_biharmonic(a0, alfa.reshape(outer, 1, inner), beta.reshape(outer, 1, inner), *diags, *ref[:5], axis=1)
    RA.biharmonic_factor_pr(ref[5], ref[6], ref[3], ref[4], axis=1)
    for q in range(7):
        assert rel(got[q], ref[q]) < 1e-13, q
    uo = f.copy()
    RA.biharmonic_solve(f, uo, *ref, a0, axis=1)
    assert rel(u, uo) < 1e-12
    assert np.array_equal(u[:, n:], f[:, n:])  # entries past the dofs untouched


@pytest.mark.parametrize("N,outer,inner,cplx", [(14, 1, 1, 0), (20, 2, 3, 1), (37, 3, 1, 1)])
def test_biharmonic_matvec_reference_layout(emu, N, outer, inner, cplx):
    g = np.random.default_rng(N)
    M = N - 4
    diags = _bih_diags(g, M)
    alfa = g.uniform(-3, 3, outer * inner)
    beta = g.uniform(0.5, 4, outer * inner)
    shape = (outer, N, inner)
    v = g.standard_normal(shape) + (1j * g.standard_normal(shape) if cplx else 0)
    res = run(emu, ["bihmv", outer, N, inner, cplx, repr(1.5)], [alfa, beta] + diags + [v], v.size * (2 if cplx else 1))
    b = (res.view(np.complex128) if cplx else res).reshape(shape)
    ref = np.zeros_like(v)
    RA.biharmonic_matvec(v, ref, 1.5, alfa.reshape(outer, 1, inner), beta.reshape(outer, 1, inner), *diags, axis=1)
    assert rel(b, ref) < 1e-13


_DMA = {"DiagMA": (0, 1), "TwoDMA": (1, 2), "ThreeDMA": (2, 3), "TDMA": (3, 3), "TDMA_O": (4, 3), "PDMA": (5, 5),
        "FDMA": (6, 4), "HeptaDMA": (7, 7)}


@pytest.mark.parametrize("name", list(_DMA))
@pytest.mark.parametrize("per,skip", [(0, 0), (1, 1)])
def test_dma_solves_reference_layout(emu, name, per, skip):
    kind, rows = _DMA[name]
    g = np.random.default_rng(kind * 11 + per)
    outer, N, inner, cols = 3, 15, 2, 13
    nsys = outer * inner
    data = g.uniform(-0.3, 0.3, (nsys if per else 1, rows, cols))
    mid = {"DiagMA": 0, "TwoDMA": 0, "ThreeDMA": 0, "TDMA": 1, "TDMA_O": 1, "PDMA": 2, "FDMA": 1, "HeptaDMA": 2}[name]
    data[:, mid] = 2.0 + g.uniform(0, 1, (data.shape[0], cols))
    u = g.standard_normal((outer, N, inner)) + 1j * g.standard_normal((outer, N, inner))
    res = run(emu, ["dma", kind, rows, cols, outer, N, inner, 1, per, skip], [data, u], u.size * 2)
    got = res.view(np.complex128).reshape(u.shape)
    ref = u.copy()
    lines = np.moveaxis(ref, 1, -1).reshape(-1, N)
    for s in range(nsys):
        if skip and s == 0:
            continue
        line = lines[s].copy()
        RA.inner_solve(name, line, data[s if per else 0])
        lines[s] = line
    ref = np.moveaxis(lines.reshape(outer, inner, N), -1, 1)
    assert rel(got, ref) < 1e-13


@pytest.mark.parametrize("n,npts,rows", [(12, 12, 2), (17, 17, 3), (9, 20, 2)])
@pytest.mark.parametrize("scalar", [0, 1])
def test_legendre_recursion_matrix(emu, n, npts, rows, scalar):
    if scalar and n != npts:
        pytest.skip("the scalar product takes as many points as degrees")
    g = np.random.default_rng(n + npts)
    x = np.sort(g.uniform(-1, 1, npts))
    w = g.uniform(0.1, 1, npts)
    cols = max(n, npts) + 3
    k = np.arange(cols, dtype=float)
    # the Legendre recursion x L_k = k/(2k+1) L_{k-1} + (k+1)/(2k+1) L_{k+1} in DIA rows
    a = np.zeros((rows, cols))
    a[0] = (k + 1) / (2 * k + 1)
    a[-1] = k / (2 * k + 1)
    if rows == 3:
        a[1] = g.uniform(-0.1, 0.1, cols)
    res = run(emu, ["legrec", scalar, n, npts, rows, cols], [x, w, a], n * npts)
    P = RA.legendre_matrix(x, a, n)
    ref = (P * w).T if scalar else P
    assert rel(res.reshape(ref.shape), ref) < 1e-14


# ---- strided length-256 Fourier passes (fft256.cuh) ---------------------------
@pytest.mark.parametrize("form", [0, 1])
@pytest.mark.parametrize("kind,outer,inner", [(C2C_FWD, 1, 37), (C2C_BWD, 2, 20), (R2C, 3, 19), (R2C, 1, 33),
                                              (C2R, 2, 17), (C2R, 1, 33)])
def test_fft256_strided(emu, kind, outer, inner, form, monkeypatch):
    monkeypatch.setenv("SGPU_EMU_FORM", str(form))
    g = np.random.default_rng(kind * 100 + inner)
    n = 256
    if kind in (C2C_FWD, C2C_BWD):
        x = g.standard_normal((outer, n, inner)) + 1j * g.standard_normal((outer, n, inner))
        scl = 1.0 / n if kind == C2C_FWD else 1.0
        res = run(emu, ["f256", kind, outer, inner, repr(scl)], [x], x.size * 2).view(np.complex128)
        ref = S.c2c_forward(x, axis=1) if kind == C2C_FWD else S.c2c_backward(x, axis=1)
        got = res.reshape(x.shape)
    elif kind == R2C:
        x = g.standard_normal((outer, n, inner))
        res = run(emu, ["f256", kind, outer, inner, repr(1.0 / n)], [x], outer * 129 * inner * 2)
        got = res.view(np.complex128).reshape(outer, 129, inner)
        ref = S.r2c_forward(x, axis=1)
    else:
        y = g.standard_normal((outer, 129, inner)) + 1j * g.standard_normal((outer, 129, inner))
        res = run(emu, ["f256", kind, outer, inner, repr(1.0)], [y], outer * n * inner)
        got = res.reshape(outer, n, inner)
        ref = S.r2c_backward(y, n, axis=1)
    assert np.isfinite(got).all()
    assert rel(got, ref) < 1e-13


# ---- the same passes in 64-bit fixed point (fft256_fx.cuh) ------------------------
def _line_rel(got, ref, axis=1):
    """max over lines of the line's error / the line's largest entry"""
    err = np.abs(got - ref).max(axis=axis)
    scale = np.abs(ref).max(axis=axis)
    return float((err / np.where(scale > 0, scale, 1.0)).max())


@pytest.mark.parametrize("kind,outer,inner", [(C2C_FWD, 1, 37), (C2C_BWD, 2, 20), (R2C, 3, 19), (R2C, 1, 33),
                                              (C2R, 2, 17), (C2R, 1, 33)])
def test_fft256_fixed_point(emu, kind, outer, inner, monkeypatch):
    """Every line (every real line of a pair) to ~2^-53 of its own largest
    entry, with line magnitudes spread over 2^-300 .. 2^300 so that paired
    lines differ by many orders of magnitude."""
    monkeypatch.setenv("SGPU_EMU_FORM", "1")
    monkeypatch.setenv("SGPU_EMU_FX", "1")
    g = np.random.default_rng(kind * 100 + inner + 7)
    n = 256
    mag = np.exp2(g.integers(-300, 300, (outer, 1, inner)).astype(float))
    if kind in (C2C_FWD, C2C_BWD):
        x = (g.standard_normal((outer, n, inner)) + 1j * g.standard_normal((outer, n, inner))) * mag
        scl = 1.0 / n if kind == C2C_FWD else 1.0
        res = run(emu, ["f256", kind, outer, inner, repr(scl)], [x], x.size * 2).view(np.complex128)
        ref = S.c2c_forward(x, axis=1) if kind == C2C_FWD else S.c2c_backward(x, axis=1)
        got = res.reshape(x.shape)
    elif kind == R2C:
        x = g.standard_normal((outer, n, inner)) * mag
        res = run(emu, ["f256", kind, outer, inner, repr(1.0 / n)], [x], outer * 129 * inner * 2)
        got = res.view(np.complex128).reshape(outer, 129, inner)
        ref = S.r2c_forward(x, axis=1)
    else:
        y = (g.standard_normal((outer, 129, inner)) + 1j * g.standard_normal((outer, 129, inner))) * mag
        res = run(emu, ["f256", kind, outer, inner, repr(1.0)], [y], outer * n * inner)
        got = res.reshape(outer, n, inner)
        ref = S.r2c_backward(y, n, axis=1)
    assert np.isfinite(got).all()
    assert _line_rel(got, ref) < 4e-15


@pytest.mark.parametrize("kind,outer,inner", [(C2C_FWD, 1, 37), (C2C_BWD, 1, 16), (C2C_FWD, 2, 32),
                                              (C2C_BWD, 3, 16)])
def test_fft256_fixed_point_tensor_copy_tile(emu, kind, outer, inner, monkeypatch):
    """The C2C kernel whose input arrives as one tensor copy per CTA (the box
    of its 16 lines x 256 points, row-major, zeros past the array) gives the
    bits of the kernel that loads its own values."""
    monkeypatch.setenv("SGPU_EMU_FORM", "1")
    monkeypatch.setenv("SGPU_EMU_FX", "1")
    g = np.random.default_rng(outer * 100 + inner)
    n = 256
    x = (g.standard_normal((outer, n, inner)) + 1j * g.standard_normal((outer, n, inner))) \
        * np.exp2(g.integers(-30, 30, (outer, 1, inner)))
    outs = []
    for tile in ("0", "1"):
        monkeypatch.setenv("SGPU_EMU_TILE", tile)
        outs.append(run(emu, ["f256", kind, outer, inner, repr(1.0 / n)], [x], x.size * 2))
    assert np.array_equal(outs[0].view(np.int64), outs[1].view(np.int64))
    ref = S.c2c_forward(x, axis=1) if kind == C2C_FWD else S.c2c_backward(x, axis=1) / n
    assert _line_rel(outs[1].view(np.complex128).reshape(x.shape), ref) < 4e-15


@pytest.mark.parametrize("kind", [C2C_FWD, R2C, C2R])
def test_fft256_fixed_point_nan_scale_and_zero_lines(emu, kind, monkeypatch):
    """A line holding NaN comes out NaN (its pair partner does not), a zero
    line stays zero, and a scale that is not a power of two applies."""
    monkeypatch.setenv("SGPU_EMU_FORM", "1")
    monkeypatch.setenv("SGPU_EMU_FX", "1")
    g = np.random.default_rng(kind)
    n, outer, inner = 256, 1, 18
    scl = 0.3
    if kind == C2C_FWD:
        x = g.standard_normal((outer, n, inner)) + 1j * g.standard_normal((outer, n, inner))
        x[0, 5, 3] = np.nan
        x[0, :, 4] = 0
        got = run(emu, ["f256", kind, outer, inner, repr(scl)], [x], x.size * 2).view(np.complex128)
        got = got.reshape(x.shape)
        ref = S.c2c_forward(x, axis=1) * n * scl
    elif kind == R2C:
        x = g.standard_normal((outer, n, inner))
        x[0, 7, 2] = np.inf
        x[0, :, 5] = 0
        got = run(emu, ["f256", kind, outer, inner, repr(scl)], [x], outer * 129 * inner * 2)
        got = got.view(np.complex128).reshape(outer, 129, inner)
        ref = S.r2c_forward(x, axis=1) * n * scl
    else:
        x = g.standard_normal((outer, 129, inner)) + 1j * g.standard_normal((outer, 129, inner))
        x[0, 9, 2] = np.nan
        x[0, :, 5] = 0
        got = run(emu, ["f256", kind, outer, inner, repr(scl)], [x], outer * n * inner).reshape(outer, n, inner)
        ref = S.r2c_backward(x, n, axis=1) * scl
    bad = 3 if kind == C2C_FWD else 2
    assert np.isnan(got[0, :, bad]).all()
    ok = [i for i in range(inner) if i != bad]
    assert np.isfinite(got[0][:, ok]).all()
    assert np.all(got[0, :, 4 if kind == C2C_FWD else 5] == 0)
    assert _line_rel(got[:, :, ok], ref[:, :, ok]) < 4e-15


# ---- pairing blocks: a stack of arrays transformed at once gives each array's bits
@pytest.mark.parametrize("kind,n,basis", [(R2C, 24, 0), (R2C, 256, 0), (C2R, 24, 0), (C2R, 256, 0),
                                          (CHEB_SCALAR, 17, BASIS["SD"]), (CHEB_BACKWARD, 17, BASIS["SD"])])
@pytest.mark.parametrize("inner", [1, 31])
@pytest.mark.parametrize("fx_form", [0, 1])
def test_pair_blocks_stack_equals_alone(emu, kind, n, basis, inner, fx_form, monkeypatch):
    g = np.random.default_rng(n + inner)
    K, outer = 3, 3  # outer x inner lines per member: odd when inner is odd
    if kind == C2R:
        nin = n // 2 + 1
        x = g.standard_normal((K * outer, nin, inner)) + 1j * g.standard_normal((K * outer, nin, inner))
        n_out, cplx = n, True
    else:
        x = g.standard_normal((K * outer, n, inner))
        n_out = n // 2 + 1 if kind == R2C else n
        cplx = False
    if n == 256 and inner >= 16 and kind in (R2C, C2R):
        mode = ["f256", kind, K * outer, inner, repr(1.0)]
        count_out = K * outer * n_out * inner * (2 if kind == R2C else 1)
        runner = lambda arr, o: run(emu, ["f256", kind, o, inner, repr(1.0)], [arr],  # noqa: E731
                                    o * n_out * inner * (2 if kind == R2C else 1))
    else:
        runner = lambda arr, o: xform(emu, kind, n, basis, arr, 1, cplx, 1.0, n_out).reshape(-1)  # noqa: E731
    if n == 256 and inner >= 16 and kind in (R2C, C2R):
        monkeypatch.setenv("SGPU_EMU_FORM", str(fx_form))
        monkeypatch.setenv("SGPU_EMU_FX", "1" if fx_form else "0")
    monkeypatch.setenv("SGPU_EMU_PB", str(outer * inner))
    stacked = runner(x, K * outer)
    monkeypatch.delenv("SGPU_EMU_PB")
    per = stacked.size // K
    for k in range(K):
        alone = runner(x[k * outer:(k + 1) * outer], outer)
        assert np.array_equal(stacked[k * per:(k + 1) * per], alone), k


# ---------------------------------------------------------------------------
# plan tables built in double-double: every FP64 twiddle is the correctly
# rounded value of its exact expression (mpmath at 60 digits), and every
# double-float pair carries the value to ~2^-48
@pytest.mark.parametrize("kind,n,basis", [(C2C_FWD, 256, 0), (C2C_FWD, 257, 0), (R2C, 96, 0),
                                          (CHEB_SCALAR, 65, 1), (C2C_FWD, 31, 0)])
def test_plan_tables_correctly_rounded(emu, kind, n, basis):
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.dps = 60
    rader = n >= 11 and all(n % d for d in range(2, int(n ** 0.5) + 1))
    m = n - 1 if rader else n
    cheb = kind >= DCT2
    nrk = m if rader else 0
    npost = n if cheb else 0
    cnt = 2 * (m + nrk + npost) + 4 * (m + nrk + npost)
    with tempfile.TemporaryDirectory() as td:
        outp = os.path.join(td, "t.bin")
        env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0:abort_on_error=1")
        r = subprocess.run([emu, "tables", str(kind), str(n), str(basis), outp], capture_output=True,
                           text=True, env=env)
        assert r.returncode == 0, r.stderr[-2000:]
        o = np.fromfile(outp, dtype=np.float64)
    assert o.size == cnt
    exact = []
    for e in range(m):  # exp(-2 pi i e / m)
        a = -2 * mpmath.pi * e / m
        exact.append((mpmath.cos(a), mpmath.sin(a)))
    if rader:
        g = next(g for g in range(2, n) if all(pow(g, (n - 1) // q, n) != 1 for q in range(2, n)
                                                if (n - 1) % q == 0 and all(q % d for d in range(2, q))))
        ginv = pow(g, n - 2, n)
        b = [mpmath.exp(-2j * mpmath.pi * pow(ginv, q, n) / n) for q in range(m)]
        for s in range(m):
            v = mpmath.fsum(b[q] * mpmath.exp(-2j * mpmath.pi * q * s / m) for q in range(m)) / m
            exact.append((mpmath.re(v), mpmath.im(v)))
    if cheb:
        for k in range(n):
            a = -mpmath.pi * k / (2 * n)
            exact.append((mpmath.cos(a), mpmath.sin(a)))
    fp = o[:2 * len(exact)].reshape(-1, 2)
    pairs = o[2 * len(exact):].reshape(-1, 4)
    for i, (cr, ci) in enumerate(exact):
        for j, ex in enumerate((cr, ci)):
            got = fp[i, j]
            rounded = float(ex)  # mpmath rounds to nearest
            # (an exact zero of the Rader spectrum comes out of a 256-term
            # double-double sum as ~1e-33: absolute slack 1e-30)
            assert got == rounded or abs(mpmath.mpf(got) - ex) <= abs(mpmath.mpf(rounded) - ex) * (1 + 1e-9) + 1e-30, \
                (i, j, got, rounded)
            hi, lo = pairs[i, 2 * j], pairs[i, 2 * j + 1]
            assert abs(mpmath.mpf(hi) + mpmath.mpf(lo) - ex) <= 2.0 ** -47 * max(abs(ex), 2.0 ** -20)


# ---- small launches run fewer lines per CTA: the same bits -------------------------
@pytest.mark.parametrize("kind,n,basis,cplx", [(R2C, 64, 0, False), (C2R, 64, 0, True), (C2C_FWD, 48, 0, True),
                                               (CHEB_SCALAR, 64, BASIS["SD"], False),
                                               (CHEB_FORWARD, 33, BASIS["SD"], True),
                                               (CHEB_BACKWARD, 64, BASIS["SD"], False),
                                               (CHEB_SCALAR, 17, BASIS["SB"], False)])
@pytest.mark.parametrize("inner", [1, 7])
@pytest.mark.parametrize("form", [0, 1])
def test_fewer_lines_per_cta_same_bits(emu, kind, n, basis, cplx, inner, form, monkeypatch):
    monkeypatch.setenv("SGPU_EMU_FORM", str(form))
    g = np.random.default_rng(n * 10 + inner)
    outer = 5
    if kind == C2R:
        nin = n // 2 + 1
        x = g.standard_normal((outer, nin, inner)) + 1j * g.standard_normal((outer, nin, inner))
        n_out = n
    else:
        x = g.standard_normal((outer, n, inner))
        if cplx:
            x = x + 1j * g.standard_normal((outer, n, inner))
        n_out = n // 2 + 1 if kind == R2C else n
    ref = xform(emu, kind, n, basis, x, 1, cplx, 1.0, n_out)
    for t in (1, 2, 4):
        monkeypatch.setenv("SGPU_EMU_TLC", str(t))
        got = xform(emu, kind, n, basis, x, 1, cplx, 1.0, n_out)
        assert np.array_equal(got, ref), t
    monkeypatch.delenv("SGPU_EMU_TLC")


def test_fused_epilogue_combine(emu):
    """The fused contraction's epilogue (combine8, the device's eight-output
    form) against its scalar statement (combine) and against exact integer
    arithmetic: the group sums weighted into one 64-bit fixed-point value,
    rounded to FP64 to nearest-even (ties included: about one output in 2048
    has them), subnormal and overflowing scales included; bit for bit."""
    import math
    r = np.random.default_rng(11)
    nb = 20000
    n = 8 * nb
    mag = 2.0 ** r.uniform(0, 24, (n, 7))
    G = np.trunc(r.choice([-1.0, 1.0], (n, 7)) * mag)
    G = np.clip(G, -(2 ** 24 - 1), 2 ** 24 - 1)
    G[:, 0] = np.clip(G[:, 0], -(2 ** 20), 2 ** 20)
    G[: n // 16] = 0.0                      # zero outputs
    G[n // 16: n // 8, :3] = 0.0            # few significant bits: no rounding
    ex = r.integers(-520, 520, n)
    em = np.repeat(r.integers(-520, 520, nb), 8)
    ex[-n // 10:] = r.integers(-1060, 1060, n // 10)   # subnormal / overflow results
    sc = np.stack([ex, em], axis=1).astype(float)
    out = run(emu, ["lccombine", n], [G, sc], 2 * n)
    o8, o1 = out[:n], out[n:]
    assert np.array_equal(o8.view(np.int64), o1.view(np.int64))
    Gi = G.astype(np.int64)
    ref = np.empty(n)
    for i in range(n):
        g = [int(v) for v in Gi[i]]
        T = (g[0] * 256 + g[1]) * 2 ** 33 + g[2] * 2 ** 25 + g[3] * 2 ** 17 + g[4] * 2 ** 9 + g[5] * 2 \
            + ((g[6] + 64) >> 7)
        E = int(ex[i]) + int(em[i]) + 8 * 12 - 2 * 54 - 41
        try:
            ref[i] = math.ldexp(float(T), E)
        except OverflowError:
            ref[i] = math.copysign(math.inf, T)
    assert np.array_equal(o8.view(np.int64), ref.view(np.int64))
