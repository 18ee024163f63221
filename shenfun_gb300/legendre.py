"""Legendre spaces with Gauss-Legendre quadrature on the GPU path
(legendre/bases.py:76-572 of the reference).

Transforms are dense contractions (``sgpu_legendre_execute_ws``) with the
Shen stencil folded into the matrix; the nodes and weights come from the
library's host routine ``sgpu_leggauss``.  ``form='mixed'`` runs them on the
tensor cores with BF16 digit slices (about 48 bits, N <= 8192; above 1024 in
exact K chunks of 1024 whose results are added).  ``kind='vandermonde'`` zeroes the tail rows of
the composite scalar product (spectralbase.py:1466-1469); the default
('recursive', the reference's default for Legendre) keeps the orthogonal
coefficients there, as the reference's stencil product does.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .device import require_cuda, ptr, stream_handle, view3, data_kind
from .spaces import SpectralBase, Domain

_plans = {}


def leggauss(N):
    """Gauss-Legendre nodes (ascending) and weights (host, FP64)."""
    x = np.zeros(N)
    w = np.zeros(N)
    _lib.call("sgpu_leggauss", int(N), x.ctypes.data, w.ctypes.data)
    return x, w


class _Plan:
    def __init__(self, N, basis, form):
        h = ctypes.c_void_p()
        _lib.call("sgpu_legendre_plan_create", ctypes.byref(h), N, basis, form)
        self._h = h

    def __del__(self):
        try:
            if self._h:
                _lib.load().sgpu_legendre_plan_destroy(self._h)
                self._h = None
        except Exception:
            pass

    def workspace_bytes(self, outer, inner, kind):
        nb = ctypes.c_size_t()
        _lib.call("sgpu_legendre_workspace_size", self._h, outer, inner, kind, ctypes.byref(nb))
        return int(nb.value)

    def __call__(self, direction, inp, out, axis, stream=None, work=None):
        outer, n, inner = view3(tuple(inp.shape), axis)
        kind = data_kind(inp)
        nb = self.workspace_bytes(outer, inner, kind)
        if nb and (work is None or work.numel() < nb):
            # torch's caching allocator: 512-byte aligned, reused across calls
            work = torch.empty(nb, dtype=torch.uint8, device=inp.device)
        _lib.call("sgpu_legendre_execute_ws", self._h, direction, ptr(inp), ptr(out), outer, inner,
                  kind, work.data_ptr() if nb else None, nb, stream_handle(stream))
        return out


def get_plan(N, basis, form=_lib.PLAIN_F64):
    key = (N, basis, form)
    p = _plans.get(key)
    if p is None:
        p = _Plan(N, basis, form)
        _plans[key] = p
    return p


class LegendreBase(SpectralBase):
    family_name = "legendre"
    basis_id = _lib.BASIS_ORTHO
    quad = "LG"
    inplace_ok = False   # the contraction reads whole lines: never in place

    def __init__(self, N, quad="LG", domain=(-1.0, 1.0), dtype=float, **kw):
        if quad != "LG":
            raise NotImplementedError("only Legendre-Gauss quadrature is on the GPU path")
        SpectralBase.__init__(self, N, dtype)
        self.domain = Domain(domain)
        if kw.get("form") is not None:
            self.form = _lib.FORMS[kw["form"]]

    def domain_factor(self):
        a, b = self.domain
        return 2.0 / (b - a)

    def points_and_weights(self, N=None, map_true_domain=False, **kw):
        N = self.N if N is None else N
        x, w = leggauss(N)
        if map_true_domain:
            a, b = self.domain
            x = (x + 1) * (b - a) / 2 + a
        return x, w

    def mesh(self, bcast=True, map_true_domain=True):
        return self.points_and_weights(map_true_domain=map_true_domain)[0]

    def dim(self):
        return self.N - self.num_bcs()

    def _run(self, direction, input_array, output_array, axis, kind):
        require_cuda()
        if self.domain_factor() != 1:
            raise NotImplementedError("only the reference domain [-1, 1] is on the GPU path")
        ax = self.axis if axis is None else axis
        out = self._out(input_array, True, output_array, ax)
        if out.data_ptr() == input_array.data_ptr():
            raise _lib.SgpuError(_lib.ERR_ARG, "Legendre transforms cannot run in place")
        get_plan(self.N, self.basis_id, self.form)(direction, input_array, out, ax)
        if direction == 0 and kind == "vandermonde" and self.num_bcs():
            out.narrow(ax % out.dim(), self.dim(), self.num_bcs()).zero_()
        return out

    def scalar_product(self, input_array, output_array=None, axis=None, kind="recursive"):
        return self._run(0, input_array, output_array, axis, kind)

    def forward(self, input_array, output_array=None, axis=None, kind="recursive"):
        return self._run(1, input_array, output_array, axis, kind)

    def backward(self, input_array, output_array=None, axis=None, kind="recursive"):
        return self._run(2, input_array, output_array, axis, kind)


class LegendreOrthogonal(LegendreBase):
    @staticmethod
    def short_name():
        return "L"

    @staticmethod
    def boundary_condition():
        return ""


class LegendreShenDirichlet(LegendreBase):
    """phi_k = L_k - L_{k+2} (legendre/bases.py:319-384)."""

    basis_id = _lib.BASIS_SD

    def num_bcs(self):
        return 2

    @staticmethod
    def short_name():
        return "SD"

    @staticmethod
    def boundary_condition():
        return "Dirichlet"


class LegendreShenBiharmonic(LegendreBase):
    """legendre/bases.py:513-572."""

    basis_id = _lib.BASIS_SB

    def num_bcs(self):
        return 4

    @staticmethod
    def short_name():
        return "SB"

    @staticmethod
    def boundary_condition():
        return "Biharmonic"


def space(N, nbcs, quad="LG", domain=(-1.0, 1.0)):
    cls = {0: LegendreOrthogonal, 2: LegendreShenDirichlet, 4: LegendreShenBiharmonic}.get(nbcs)
    if cls is None:
        raise NotImplementedError(f"Legendre space with {nbcs} boundary conditions")
    return cls(N, quad=quad, domain=domain)
