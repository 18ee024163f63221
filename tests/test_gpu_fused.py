"""GPU: the fused split-BF16 contraction (one kernel per mixed-form Chebyshev
pass over contiguous lines: digits split inside the tensor-core kernel,
clusters of CTAs sharing them) against the oracle, the FP64 plan and itself.

Tolerances: 1e-12 normwise against the oracle (the kernel keeps 54 bits;
the emulator measures ~5e-15 of |x| |M|), and bit-for-bit equality between
a line computed alone and in a batch."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import spectral as S

pytestmark = pytest.mark.gpu

TOL = 1e-12


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = b.detach().cpu().numpy() if isinstance(b, torch.Tensor) else np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def dev(a):
    return torch.as_tensor(np.ascontiguousarray(a), device="cuda")


@pytest.fixture(scope="module")
def lib():
    from shenfun_gb300 import build
    build.build()
    from shenfun_gb300 import _lib
    assert _lib.load().sgpu_device_ok() == 1
    return _lib


def timeouts(lib):
    c = ctypes.c_uint()
    lib.call("sgpu_wait_timeouts", ctypes.byref(c))
    return c.value


def space(lib, basis, n):
    from shenfun_gb300.spaces import ChebyshevOrthogonal, ChebyshevShenDirichlet, ChebyshevShenBiharmonic
    V = {"T": ChebyshevOrthogonal, "SD": ChebyshevShenDirichlet, "SB": ChebyshevShenBiharmonic}[basis](n)
    V.form = lib.MIXED_DF
    return V


# n = 130, 258: two outputs past the last 128-row tile (FP64 dot products);
# n = 300, 339: three CTAs per cluster with a partial third tile
@pytest.mark.parametrize("n", [16, 64, 129, 130, 257, 258, 300, 339])
@pytest.mark.parametrize("basis", ["T", "SD"])
@pytest.mark.parametrize("cplx", [False, True])
def test_fused_against_oracle(lib, n, basis, cplx):
    V = space(lib, basis, n)
    rng = np.random.default_rng(n + 7 * cplx)
    x = rng.standard_normal((3, 67, n))  # 201 lines: a partial last tile
    if cplx:
        x = x + 1j * rng.standard_normal(x.shape)
    sp = V.scalar_product(dev(x), axis=2)
    assert rel(sp, S.cheb_scalar_product(x, basis, 2)) < TOL
    fw = V.forward(dev(x), axis=2)
    assert rel(fw, S.cheb_forward(x, basis, 2)) < TOL
    fwn = fw.cpu().numpy()
    assert rel(V.backward(fw, axis=2), S.cheb_backward(fwn, basis, 2)) < TOL
    # in place: a tile's outputs are written after the tile has been read
    y = dev(x).clone()
    V.scalar_product(y, y, axis=2)
    assert torch.equal(y, sp)
    assert timeouts(lib) == 0


@pytest.mark.parametrize("n", [129, 257, 300])
def test_fused_many_tiles_per_cluster(lib, n):
    """65,536 lines: every persistent cluster runs many tiles (rings wrap,
    scale slots and the accumulator set are reused) against the FP64 plan."""
    from shenfun_gb300.spaces import ChebyshevShenDirichlet
    Vm = space(lib, "SD", n)
    Vp = ChebyshevShenDirichlet(n)
    x = torch.randn(65536 + 37, n, dtype=torch.float64, device="cuda")
    assert rel(Vm.scalar_product(x, axis=1), Vp.scalar_product(x, axis=1)) < TOL
    assert timeouts(lib) == 0


@pytest.mark.parametrize("n", [129, 257, 300])
def test_fused_tile_widths(lib, n):
    """64-line tiles (one accumulator set) and 32-line tiles (two sets) give
    the same bits for every output on the tensor cores (the digit groups are
    exact sums); the FP64 dot-product outputs past the last 128-row tile
    (n = 129, 257) sum different partials and agree to rounding."""
    from shenfun_gb300.plans import get_plan
    V = space(lib, "SD", n)
    p = get_plan(lib.XF_CHEB_SCALAR, n, lib.BASIS_SD, lib.MIXED_DF)
    x = dev(np.random.default_rng(n).standard_normal((5000, n)))
    outs = []
    for v in (1, 2):
        lib.call("sgpu_plan_set_variant", p._h, v)
        outs.append(V.scalar_product(x, axis=1))
    lib.call("sgpu_plan_set_variant", p._h, 0)
    nmma = n - (n % 128 if n % 128 <= 2 else 0)
    assert torch.equal(outs[0][:, :nmma], outs[1][:, :nmma])
    assert rel(outs[0], outs[1]) < 1e-15
    assert rel(outs[1], S.cheb_scalar_product(x.cpu().numpy(), "SD", 1)) < TOL
    assert timeouts(lib) == 0


def test_fused_line_alone_equals_batch(lib):
    """A line's result does not depend on the other lines of the launch (the
    serving engine's mix-versus-alone guarantee at kernel level)."""
    n = 257
    V = space(lib, "SD", n)
    x = dev(np.random.default_rng(1).standard_normal((4099, n)))
    full = V.scalar_product(x, axis=1)
    for i in (0, 63, 64, 4098):
        one = V.scalar_product(x[i:i + 1].contiguous(), axis=1)
        assert torch.equal(one[0], full[i])


def test_fused_channel_grid_full_size(lib):
    """The channel grid's z pass (65,536 lines of 257) in both directions
    against the FP64 plan, normwise 1e-12."""
    from shenfun_gb300.spaces import ChebyshevShenDirichlet
    n = 257
    Vm = space(lib, "SD", n)
    Vp = ChebyshevShenDirichlet(n)
    x = torch.randn(256, 256, n, dtype=torch.float64, device="cuda")
    a = Vm.scalar_product(x, axis=2)
    b = Vp.scalar_product(x, axis=2)
    assert rel(a, b) < TOL
    c = Vm.backward(b, axis=2)
    d = Vp.backward(b, axis=2)
    assert rel(c, d) < TOL
    assert timeouts(lib) == 0


def test_fused_small_scratch(lib):
    """Contiguous lines need 4 bytes of scratch per line (their scales),
    instead of the 14 bytes per entry of the digit copy that strided lines
    still use."""
    from shenfun_gb300.plans import get_plan
    p = get_plan(7, 257, 1, lib.MIXED_DF)
    nb = ctypes.c_size_t()
    lib.call("sgpu_plan_workspace_size", p._h, 1024, 1, lib.REAL, ctypes.byref(nb))
    assert nb.value == 1024 * 4
    lib.call("sgpu_plan_workspace_size", p._h, 10, 7, lib.REAL, ctypes.byref(nb))
    assert nb.value > 70 * 257 * 14


def test_fused_scales_unaligned_input(lib):
    """Lines starting off a 16-byte boundary (an 8-byte-aligned view) give
    the bits of the same lines in an aligned array (333 lines: an odd count,
    a partial last tile)."""
    V = space(lib, "SD", 257)
    rng = np.random.default_rng(31)
    x = rng.standard_normal((333, 257)) * np.exp2(rng.integers(-40, 40, (333, 1)))
    a = dev(x)
    buf = torch.empty(a.numel() + 1, dtype=a.dtype, device="cuda")
    u = buf[1:].view(a.shape)
    u.copy_(a)
    assert a.data_ptr() % 16 == 0 and u.data_ptr() % 16 == 8
    ya = V.scalar_product(a, axis=1)
    yu = V.scalar_product(u, axis=1)
    assert torch.equal(ya, yu)
    assert rel(ya, S.cheb_scalar_product(x, "SD", 1)) < TOL
