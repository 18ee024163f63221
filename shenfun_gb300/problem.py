"""Helmholtz problems as native objects: one call = the whole hot-path step.

``HelmholtzProblem((Nx, Ny, Nz), 'chebyshev', c)`` owns the transform plans
and the factorised per-wavenumber systems of (-lap + c) u = f on a
Fourier x ... x ShenDirichlet grid (Dirichlet axis last); ``solve(f)`` runs
scalar product -> banded solves -> backward in one C-ABI call
(``sgpu_helmholtz_solve``) on the caller's stream, with a reusable scratch
buffer.  This is the unit the serving engine caches and schedules.
"""
import ctypes

import torch

from . import _lib
from .device import require_cuda, ptr, stream_handle

FAMILIES = {"chebyshev": 1, "legendre": 2}


class HelmholtzProblem:
    def __init__(self, N, family="chebyshev", c=0.0, form="plain", stream=None):
        """With `stream`, creation is stream-ordered (shared per-axis plans,
        factorisation queued on that stream, no device synchronisation)."""
        require_cuda()
        self.N = tuple(int(n) for n in N)
        self.family = family
        self.c = float(c)
        self.form = _lib.FORMS[form]
        h = ctypes.c_void_p()
        arr = (ctypes.c_int64 * len(self.N))(*self.N)
        if stream is None:
            _lib.call("sgpu_helmholtz_create", ctypes.byref(h), len(self.N),
                      ctypes.cast(arr, ctypes.c_void_p), FAMILIES[family], self.c, self.form)
        else:
            _lib.call("sgpu_helmholtz_create_on", ctypes.byref(h), len(self.N),
                      ctypes.cast(arr, ctypes.c_void_p), FAMILIES[family], self.c, self.form,
                      stream_handle(stream))
        self._h = h
        phys = (ctypes.c_int64 * 3)()
        spec = (ctypes.c_int64 * 3)()
        _lib.call("sgpu_helmholtz_shape", self._h, ctypes.cast(phys, ctypes.c_void_p),
                  ctypes.cast(spec, ctypes.c_void_p))
        self.phys_shape = tuple(phys[i] for i in range(len(self.N)))
        self.spec_shape = tuple(spec[i] for i in range(len(self.N)))
        nb = ctypes.c_size_t()
        _lib.call("sgpu_helmholtz_workspace_size", self._h, ctypes.byref(nb))
        self.workspace_bytes = int(nb.value)
        self._work = None
        self._fac = None

    @property
    def factor_ptr(self):
        """Device address of the problem's factor block (what a batched
        step's pointer table holds for this member)."""
        if self._fac is None:
            q = ctypes.c_void_p()
            _lib.call("sgpu_helmholtz_factor_ptr", self._h, ctypes.byref(q))
            self._fac = q.value
        return self._fac

    def __del__(self):
        try:
            if self._h:
                _lib.load().sgpu_helmholtz_destroy(self._h)
                self._h = None
        except Exception:
            pass

    @property
    def array_bytes(self):
        n = 1
        for v in self.phys_shape:
            n *= v
        return 8 * n

    def new_workspace(self, device=None):
        # 256-byte aligned: torch's caching allocator returns 512-byte aligned blocks
        return torch.empty(self.workspace_bytes, dtype=torch.uint8, device=device or "cuda")

    def solve(self, f, u=None, work=None, stream=None):
        """u = solution of (-lap + c) u = f on the quadrature grid (FP64)."""
        if u is None:
            u = torch.empty_like(f)
        if work is None:
            if self._work is None:
                self._work = self.new_workspace(f.device)
            work = self._work
        if tuple(f.shape) != self.phys_shape or tuple(u.shape) != self.phys_shape:
            raise _lib.SgpuError(_lib.ERR_ARG, f"arrays must have shape {self.phys_shape}")
        _lib.call("sgpu_helmholtz_solve", self._h, ptr(f), ptr(u), work.data_ptr(),
                  work.numel(), stream_handle(stream))
        return u


class BatchRunner:
    """K problems of one shape class (N, family, form), different shifts,
    solved with one launch per stage (sgpu_helmholtz_solve_batch) on fixed
    staging buffers, captured as a CUDA graph and replayed: per batch the
    members' right-hand sides are copied into the input slots, the
    factor-pointer table is updated, the graph is replayed and the solutions
    are read from the output slots.  The graph allocates nothing and reads
    the table at replay time, so any K problems of the class (any shifts) can
    share it.

    With ``capture_after=0`` the graph is captured at construction (after one
    warm-up launch); with ``capture_after=n`` the first n batches run as
    plain launches and the graph is captured at the next one, so that a
    runner used once costs no capture.  Capture neither synchronises the
    device nor touches torch's allocator (the capture of torch.cuda.graph
    does both), so a serving loop can capture while other streams work."""

    def __init__(self, proto, K, stream, graph=True, capture_after=0):
        self.proto = proto
        self.K = int(K)
        self.stream = stream
        shape = (self.K,) + proto.phys_shape
        with torch.cuda.stream(stream):
            self.f = torch.zeros(shape, dtype=torch.float64, device="cuda")
            self.u = torch.zeros(shape, dtype=torch.float64, device="cuda")
            nb = ctypes.c_size_t()
            _lib.call("sgpu_helmholtz_batch_workspace_size", proto._h, self.K, ctypes.byref(nb))
            self.work = torch.empty(max(int(nb.value), 256), dtype=torch.uint8, device="cuda")
            self.table = torch.zeros(self.K, dtype=torch.int64, device="cuda")
        self.graph = None
        self.use_graph = bool(graph)
        self.capture_after = int(capture_after)
        self.runs = 0
        if self.use_graph and self.capture_after == 0:
            self._set_table([proto.factor_ptr] * self.K)  # valid pointers for the warm-up launch
            with torch.cuda.stream(stream):
                self._launch()  # warm-up outside the capture (plan attributes, lazy state)
            self._capture()

    def _launch(self, stream=None):
        _lib.call("sgpu_helmholtz_solve_batch", self.proto._h, self.K, self.table.data_ptr(), self.f.data_ptr(),
                  self.u.data_ptr(), self.work.data_ptr(), self.work.numel(), stream_handle(stream or self.stream))

    def _set_table(self, ptrs, stream=None):
        # a fresh page-locked source per batch: the previous batch's copy may
        # still be queued (torch's host allocator keeps it until that copy ran)
        host = torch.tensor(ptrs, dtype=torch.int64).pin_memory()
        with torch.cuda.stream(stream or self.stream):
            self.table.copy_(host, non_blocking=True)

    def _capture(self):
        g = torch.cuda.CUDAGraph()
        # thread-local capture mode: worker threads keep creating problems
        # (stream-ordered allocations) while this thread captures
        with torch.cuda.stream(self.stream):
            g.capture_begin(capture_error_mode="thread_local")
            try:
                self._launch()
            finally:
                g.capture_end()
        self.graph = g

    def run(self, problems, stream=None):
        """Queue the batch of `problems` (at most K, all of the class) whose
        right-hand sides are already in self.f[:len(problems)] on `stream`
        (default: the runner's own); the solutions land in self.u.  Unused
        slots repeat the last member.  The graph (captured on the runner's
        stream) replays on `stream`; a runner serves one batch at a time."""
        s = stream or self.stream
        ptrs = [p.factor_ptr for p in problems]
        ptrs += [ptrs[-1]] * (self.K - len(ptrs))
        self._set_table(ptrs, s)
        if self.graph is None and self.use_graph and self.runs >= self.capture_after:
            self._capture()  # records the launches only: nothing runs on the capture stream
        with torch.cuda.stream(s):
            if self.graph is not None:
                self.graph.replay()
            else:
                self._launch(s)
        self.runs += 1
