"""A shenfun optimization mode whose kernels run on the GPU.

shenfun dispatches its hot-path kernels by name (optimization/__init__.py:
37-84 of the reference): ``optimizer(func)`` looks the function's name (or
``Class_method``) up in the module of ``config['optimization']['mode']``, and
the recursive Legendre transforms import ``shenfun.optimization.<mode>.
transforms`` (spectralbase.py:485-491, 551-558).  This package provides those
names with the reference's signatures and argument meaning
(optimization/cython/la.pyx, Matvec.pyx, transforms.pyx), forwarding each
call to the library's C ABI:

* numpy arrays (what shenfun passes) are copied to the GPU and the arrays the
  kernel writes are copied back in place, so shenfun's own classes
  (``la.TDMA``, ``chebyshev.la.Helmholtz``, ``chebyshev.la.Biharmonic``,
  ``la.SolverGeneric1ND``, Legendre ``kind='recursive'``) run unchanged;
* CUDA tensors are used in place (no copies).

Errors raise ``SgpuError`` (the compiled kernels of the reference report
nothing).  ``install()`` routes an imported, unmodified shenfun's 'cython'
mode through this module for the names it provides.
"""
import ctypes
import sys
import types

import numpy as np
import torch

from .. import _lib
from ..device import require_cuda, stream_handle, view3

__all__ = [
    "TDMA_LU", "TDMA_Solve", "PDMA_LU", "PDMA_Solve", "TDMA_O_LU", "TDMA_O_Solve", "FDMA_LU", "FDMA_Solve",
    "TwoDMA_Solve", "ThreeDMA_Solve", "DiagMA_Solve", "HeptaDMA_LU", "HeptaDMA_Solve",
    "TDMA_inner_solve", "TDMA_O_inner_solve", "PDMA_inner_solve", "FDMA_inner_solve", "TwoDMA_inner_solve",
    "ThreeDMA_inner_solve", "DiagMA_inner_solve", "HeptaDMA_inner_solve", "SolverGeneric1ND_solve_data",
    "LU_Helmholtz", "Solve_Helmholtz", "Helmholtz_matvec", "Helmholtz_Neumann_matvec",
    "LU_Biharmonic", "Biharmonic_factor_pr", "Biharmonic_Solve", "Biharmonic_matvec", "install",
]

# *_inner_solve names -> SGPU_SOL_* (la.pyx:307-325)
SOL = {"DiagMA": 0, "TwoDMA": 1, "ThreeDMA": 2, "TDMA": 3, "TDMA_O": 4, "PDMA": 5, "FDMA": 6, "HeptaDMA": 7}
_SOL_ROWS = {"DiagMA": 1, "TwoDMA": 2, "ThreeDMA": 3, "TDMA": 3, "TDMA_O": 3, "PDMA": 5, "FDMA": 4, "HeptaDMA": 7}
_LU_OFFSETS = {"FDMA": (-2, 0, 2, 4), "TDMA_O": (-1, 0, 1), "HeptaDMA": (-4, -2, 0, 2, 4, 6, 8)}


# ---- argument plumbing -------------------------------------------------------
class _Dev:
    """Device copy of one argument: numpy arrays are uploaded, CUDA tensors
    used in place; ``back()`` writes the device result into the caller's
    array."""

    def __init__(self, a, dtype=None):
        require_cuda()
        self.orig = a
        if isinstance(a, torch.Tensor):
            if not a.is_cuda:
                raise _lib.SgpuError(_lib.ERR_ARG, "tensor arguments must be on a CUDA device")
            t = a if dtype is None else a.to(dtype)
            self.t = t.contiguous()
            self.copy = self.t.data_ptr() != a.data_ptr()
        else:
            arr = np.asarray(a)
            if dtype is not None:
                arr = arr.astype({torch.float64: np.float64, torch.complex128: np.complex128}[dtype], copy=False)
            self.t = torch.from_numpy(np.ascontiguousarray(arr)).to("cuda")
            self.copy = True
        if self.t.dtype not in (torch.float64, torch.complex128):
            raise _lib.SgpuError(_lib.ERR_ARG, f"unsupported dtype {self.t.dtype}")

    @property
    def ptr(self):
        return self.t.data_ptr()

    @property
    def kind(self):
        return _lib.COMPLEX if self.t.is_complex() else _lib.REAL

    def back(self):
        if not self.copy:
            return
        if isinstance(self.orig, torch.Tensor):
            self.orig.copy_(self.t)
        else:
            torch.cuda.current_stream().synchronize()
            np.copyto(self.orig, self.t.cpu().numpy())


def _f64(a):
    return _Dev(a, torch.float64)


def _systems(scale, shape, axis):
    """A scale argument broadcast to one value per system: ``shape`` with the
    solve axis collapsed, in (outer, inner) order."""
    sys_shape = list(shape)
    sys_shape[axis] = 1
    if isinstance(scale, torch.Tensor):
        scale = scale.detach().cpu().numpy()
    s = np.broadcast_to(np.asarray(scale, dtype=np.float64), tuple(sys_shape))
    return torch.from_numpy(np.array(s, dtype=np.float64).reshape(-1)).to("cuda")


def _shape(a):
    return tuple(a.shape)


def _call(name, *args):
    require_cuda()
    _lib.call(name, *args)


# ---- banded solvers (la.pyx:61-613) -----------------------------------------
def _lu(entry, data, offsets=None):
    d = _f64(data)
    n = d.t.shape[-1]
    if offsets is None:
        _call(entry, d.ptr, n, stream_handle())
    else:
        offs = (ctypes.c_int * len(offsets))(*offsets)
        _call("sgpu_banded_LU", d.ptr, len(offsets), offs, n, stream_handle())
    d.back()


def _dma_solve(name, u, data, axis):
    if _shape(data)[0] < _SOL_ROWS[name]:
        raise _lib.SgpuError(_lib.ERR_ARG, f"{name}: data needs {_SOL_ROWS[name]} rows")
    ud, dd = _Dev(u), _f64(data)
    outer, N, inner = view3(_shape(ud.t), axis)
    rows, cols = dd.t.shape
    _call("sgpu_DMA_Solve", SOL[name], ud.ptr, dd.ptr, rows, cols, outer, N, inner, ud.kind, stream_handle())
    ud.back()
    return u


def TDMA_LU(data):
    """la.pyx:243 TDMA_LU(data) (la.py:344-354)"""
    _lu("sgpu_TDMA_LU", data)


def PDMA_LU(data):
    """la.pyx:213 PDMA_LU(data) (la.py:480-516)"""
    _lu("sgpu_PDMA_LU", data)


def TDMA_O_LU(data):
    """la.pyx:254 TDMA_O_LU(data) (la.py:416-426)"""
    _lu(None, data, _LU_OFFSETS["TDMA_O"])


def FDMA_LU(data):
    """la.pyx:199 FDMA_LU(data) (la.py:565-589)"""
    _lu(None, data, _LU_OFFSETS["FDMA"])


def HeptaDMA_LU(data):
    """la.pyx:265 HeptaDMA_LU(data) (la.py:744-787)"""
    _lu(None, data, _LU_OFFSETS["HeptaDMA"])


def TDMA_Solve(u, data, axis=0):
    """la.pyx:77 TDMA_Solve(u, data, axis) (la.py:387-393)"""
    return _dma_solve("TDMA", u, data, axis)


def PDMA_Solve(u, data, axis=0):
    """la.pyx:61 PDMA_Solve(u, data, axis) (la.py:537-543)"""
    return _dma_solve("PDMA", u, data, axis)


def TDMA_O_Solve(u, data, axis=0):
    """la.pyx:93 TDMA_O_Solve(u, data, axis) (la.py:441-447)"""
    return _dma_solve("TDMA_O", u, data, axis)


def FDMA_Solve(u, data, axis=0):
    """la.pyx:165 FDMA_Solve(u, data, axis) (la.py:607-613)"""
    return _dma_solve("FDMA", u, data, axis)


def TwoDMA_Solve(u, data, axis=0):
    """la.pyx:45 TwoDMA_Solve(u, data, axis) (la.py:653-659)"""
    return _dma_solve("TwoDMA", u, data, axis)


def ThreeDMA_Solve(u, data, axis=0):
    """la.pyx:29 ThreeDMA_Solve(u, data, axis) (la.py:703-709)"""
    return _dma_solve("ThreeDMA", u, data, axis)


def DiagMA_Solve(u, data, axis=0):
    """la.pyx:109 DiagMA_Solve(u, data, axis) (la.py:323-329)"""
    return _dma_solve("DiagMA", u, data, axis)


def HeptaDMA_Solve(u, data, axis=0):
    """la.pyx:181 HeptaDMA_Solve(u, data, axis) (la.py:814-820)"""
    return _dma_solve("HeptaDMA", u, data, axis)


def _inner(name):
    def inner_solve(u, data):
        return _dma_solve(name, u, data, 0)

    inner_solve.__name__ = inner_solve.__qualname__ = name + "_inner_solve"
    inner_solve.__doc__ = f"la.pyx {name}_inner_solve(u, data): one line (la.pyx:466-613)"
    return inner_solve


TDMA_inner_solve = _inner("TDMA")
TDMA_O_inner_solve = _inner("TDMA_O")
PDMA_inner_solve = _inner("PDMA")
FDMA_inner_solve = _inner("FDMA")
TwoDMA_inner_solve = _inner("TwoDMA")
ThreeDMA_inner_solve = _inner("ThreeDMA")
DiagMA_inner_solve = _inner("DiagMA")
HeptaDMA_inner_solve = _inner("HeptaDMA")


def SolverGeneric1ND_solve_data(u, data, sol, naxes, is_zero_index):
    """la.pyx:371-383: solve every (Fourier) system of u along axis naxes with
    its own LU'd matrix data[i(, j)]; sol is the *_inner_solve function,
    resolved by name; system 0 is skipped when is_zero_index."""
    name = getattr(sol, "__name__", str(sol))
    if not name.endswith("_inner_solve") or name[:-len("_inner_solve")] not in SOL:
        raise _lib.SgpuError(_lib.ERR_ARG, f"SolverGeneric1ND_solve_data: unknown solver {name}")
    kind = name[:-len("_inner_solve")]
    ud, dd = _Dev(u), _f64(data)
    shape = _shape(ud.t)
    if len(shape) not in (2, 3):
        raise _lib.SgpuError(_lib.ERR_ARG, "SolverGeneric1ND_solve_data: 2D or 3D arrays")
    outer, N, inner = view3(shape, naxes)
    rows, cols = dd.t.shape[-2:]
    if int(np.prod(dd.t.shape[:-2])) != outer * inner or rows < _SOL_ROWS[kind]:
        raise _lib.SgpuError(_lib.ERR_ARG, "SolverGeneric1ND_solve_data: data does not match the systems")
    _call("sgpu_SolverGeneric1ND_solve_data", ud.ptr, dd.ptr, SOL[kind], int(bool(is_zero_index)), outer, N,
          inner, rows, cols, ud.kind, stream_handle())
    ud.back()
    return u


# ---- Chebyshev Helmholtz (la.pyx:708-960, Matvec.pyx:656-800) ----------------
def _diag(mat, k):
    d = mat.get(k) if hasattr(mat, "get") else mat[k]
    return np.atleast_1d(np.asarray(d, dtype=np.float64))


def _check_helmholtz_matrices(A, B, N, neumann):
    """The kernels use the closed forms of ASDSD / BSDSD (ASNSN / BSNSN for
    Neumann); refuse other matrices instead of solving the wrong system."""
    if A is None or B is None:
        return
    k = np.arange(N - 2, dtype=np.float64)
    if neumann:
        a0 = -2 * np.pi * k ** 2 * (k + 1) / (k + 2)
    else:
        a0 = -2 * np.pi * (k + 1) * (k + 2)
    got = _diag(A, 0)
    if got.size == 1:
        got = np.broadcast_to(got, a0.shape)
    if got.shape != a0.shape or not np.allclose(got, a0, rtol=1e-12, atol=0):
        raise _lib.SgpuError(_lib.ERR_UNSUPPORTED,
                             "Helmholtz kernels: A must be the reference's ASDSD (or ASNSN) matrix")


def LU_Helmholtz(A, B, As, Bs, neumann, u0, u1, u2, L, axis=0):
    """la.pyx:708 LU_Helmholtz(A, B, A_s, B_s, neumann, d0, d1, d2, L, axis)"""
    d = [_f64(x) for x in (u0, u1, u2, L)]
    shape = _shape(d[0].t)
    outer, N, inner = view3(shape, axis)
    _check_helmholtz_matrices(A, B, N, bool(neumann))
    alfa, beta = _systems(As, shape, axis), _systems(Bs, shape, axis)
    _call("sgpu_LU_Helmholtz", N, alfa.data_ptr(), beta.data_ptr(), int(bool(neumann)),
          *[x.ptr for x in d], outer, inner, stream_handle())
    for x in d:
        x.back()


def Solve_Helmholtz(b, u, neumann, u0, u1, u2, L, axis=0):
    """la.pyx:845 Solve_Helmholtz(b, u, neumann, d0, d1, d2, L, axis)"""
    bd = _Dev(b)
    ud = bd if u is b else _Dev(u, bd.t.dtype)
    d = [_f64(x) for x in (u0, u1, u2, L)]
    outer, N, inner = view3(_shape(bd.t), axis)
    _call("sgpu_Solve_Helmholtz", bd.ptr, ud.ptr, int(bool(neumann)), *[x.ptr for x in d], outer, N, inner,
          bd.kind, stream_handle())
    ud.back()
    return u


def _helmholtz_matvec(entry, v, b, alfa, beta, axis):
    vd = _Dev(v)
    bd = _Dev(b, vd.t.dtype)
    shape = _shape(vd.t)
    outer, N, inner = view3(shape, axis)
    a, c = _systems(alfa, shape, axis), _systems(beta, shape, axis)
    _call(entry, vd.ptr, bd.ptr, a.data_ptr(), c.data_ptr(), outer, N, inner, vd.kind, stream_handle())
    bd.back()
    return b


def Helmholtz_matvec(v, b, alfa, beta, A, B, axis=0):
    """Matvec.pyx:697 Helmholtz_matvec(v, b, alfa, beta, A, B, axis)"""
    _check_helmholtz_matrices(A, B, _shape(v)[axis], False)
    return _helmholtz_matvec("sgpu_Helmholtz_matvec", v, b, alfa, beta, axis)


def Helmholtz_Neumann_matvec(v, b, alfa, beta, A, B, axis=0):
    """Matvec.pyx:769 Helmholtz_Neumann_matvec(v, b, alfa, beta, A, B, axis)"""
    _check_helmholtz_matrices(A, B, _shape(v)[axis], True)
    return _helmholtz_matvec("sgpu_Helmholtz_Neumann_matvec", v, b, alfa, beta, axis)


# ---- Chebyshev biharmonic (la.pyx:975-1290, Matvec.pyx:820-920) -------------
_BIH_LEN = (("sii", 0), ("siu", 2), ("siuu", 4), ("ail", 2), ("aii", 0), ("aiu", 2),
            ("bill", 4), ("bil", 2), ("bii", 0), ("biu", 2), ("biuu", 4))


def _bih_diags(n, diags):
    """Device copies of the 11 diagonals, checked against the lengths the
    kernels read (n dofs: n, n - 2 or n - 4 entries)."""
    out = []
    for (name, short), d in zip(_BIH_LEN, diags):
        t = _f64(np.atleast_1d(np.asarray(d, dtype=np.float64)) if not isinstance(d, torch.Tensor) else d).t
        if t.dim() != 1 or t.numel() < n - short:
            raise _lib.SgpuError(_lib.ERR_ARG, f"biharmonic: diagonal {name} shorter than {n - short}")
        out.append(t)
    return out


def LU_Biharmonic(a0, alfa, beta, sii, siu, siuu, ail, aii, aiu, bill, bil, bii, biu, biuu, u0, u1, u2, l0, l1,
                  axis=0):
    """la.pyx:975 LU_Biharmonic: factors u0, u1, u2, l0, l1 of shape
    (2,) + (the systems' shape with M along axis)"""
    f = [_f64(x) for x in (u0, u1, u2, l0, l1)]
    shape = _shape(f[0].t)[1:]
    outer, M, inner = view3(shape, axis)
    diags = _bih_diags(2 * M, (sii, siu, siuu, ail, aii, aiu, bill, bil, bii, biu, biuu))
    a, c = _systems(alfa, shape, axis), _systems(beta, shape, axis)
    _call("sgpu_LU_Biharmonic", float(np.asarray(a0).reshape(-1)[0]), a.data_ptr(), c.data_ptr(),
          *[t.data_ptr() for t in diags], *[x.ptr for x in f], outer, M, inner, stream_handle())
    for x in f:
        x.back()


def Biharmonic_factor_pr(ak, bk, l0, l1, axis=0):
    """la.pyx:1195 Biharmonic_factor_pr(a, b, l0, l1, axis)"""
    f = [_f64(x) for x in (ak, bk, l0, l1)]
    outer, M, inner = view3(_shape(f[0].t)[1:], axis)
    _call("sgpu_Biharmonic_factor_pr", *[x.ptr for x in f], outer, M, inner, stream_handle())
    f[0].back()
    f[1].back()


def Biharmonic_Solve(b, u, u0, u1, u2, l0, l1, ak, bk, a0, axis=0):
    """la.pyx:1235 Biharmonic_Solve(b, u, u0, u1, u2, l0, l1, ak, bk, a0, axis)"""
    bd = _Dev(b)
    ud = bd if u is b else _Dev(u, bd.t.dtype)
    f = [_f64(x) for x in (u0, u1, u2, l0, l1, ak, bk)]
    outer, N, inner = view3(_shape(bd.t), axis)
    M = _shape(f[0].t)[1:][axis]
    _call("sgpu_Biharmonic_Solve", bd.ptr, ud.ptr, *[x.ptr for x in f], float(np.asarray(a0).reshape(-1)[0]),
          outer, N, inner, M, bd.kind, stream_handle())
    ud.back()
    return u


def Biharmonic_matvec(v, b, a0, alfa, beta, sii, siu, siuu, ail, aii, aiu, bill, bil, bii, biu, biuu, axis=0):
    """Matvec.pyx:908 Biharmonic_matvec: b[:M] = (a0 S + alfa A + beta B) v"""
    vd = _Dev(v)
    bd = _Dev(b, vd.t.dtype)
    shape = _shape(vd.t)
    outer, N, inner = view3(shape, axis)
    M = int(np.asarray(sii).shape[0]) if not isinstance(sii, torch.Tensor) else sii.numel()
    diags = _bih_diags(M, (sii, siu, siuu, ail, aii, aiu, bill, bil, bii, biu, biuu))
    a, c = _systems(alfa, shape, axis), _systems(beta, shape, axis)
    _call("sgpu_Biharmonic_matvec", vd.ptr, bd.ptr, float(np.asarray(a0).reshape(-1)[0]), a.data_ptr(),
          c.data_ptr(), *[t.data_ptr() for t in diags], outer, N, inner, M, vd.kind, stream_handle())
    bd.back()
    return b


# ---- routing an unmodified shenfun through this module -----------------------
class _Routed(types.ModuleType):
    """A module that answers with this package's functions and falls back to
    the module it replaces for every other name."""

    def __init__(self, name, mine, fallback):
        super().__init__(name)
        self.__dict__["_mine"] = mine
        self.__dict__["_fallback"] = fallback

    def __getattr__(self, name):
        mine = self.__dict__["_mine"]
        if name in getattr(mine, "__all__", ()) and name != "install":
            return getattr(mine, name)
        return getattr(self.__dict__["_fallback"], name)


def install():
    """Route an imported shenfun's 'cython' optimization mode through this
    module: every kernel named here (the solvers, matvecs and the recursive
    Legendre transforms) runs on the GPU, every other name stays the compiled
    one.  Sets config['optimization']['mode'] to 'cython'.  (A shenfun that
    lists a 'gb300' mode in its optimizer imports this package directly.)"""
    from . import transforms
    opt = sys.modules.get("shenfun.optimization")
    if opt is None:
        raise ImportError("import shenfun first")
    cy = opt.cython
    if isinstance(cy, _Routed):
        return cy
    routed = _Routed("shenfun.optimization.cython", sys.modules[__name__], cy)
    routed.__path__ = getattr(cy, "__path__", [])
    tr_orig = sys.modules.get("shenfun.optimization.cython.transforms") or getattr(cy, "transforms", None)
    routed.__dict__["transforms"] = _Routed("shenfun.optimization.cython.transforms", transforms, tr_orig)
    opt.cython = routed
    sys.modules["shenfun.optimization.cython"] = routed
    sys.modules["shenfun.optimization.cython.transforms"] = routed.__dict__["transforms"]
    from shenfun.config import config
    config["optimization"]["mode"] = "cython"
    return routed
