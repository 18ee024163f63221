"""Autotuner of the library's kernel variants, with an on-disk cache.

Several plans have more than one kernel for the same result
(``sgpu_plan_set_variant``): the fused Chebyshev contraction runs 64- or
32-line tiles, the length-256 Fourier passes run the strided register-FFT
kernel at two or three CTAs per SM (the mixed form in double-float or in
64-bit fixed point) or the generic line programs.  Which is
fastest depends on the layout and the size.  ``tune_plan`` times every
variant of a plan on the call's own layout (CUDA events, the median of a few
repetitions after warm-up), checks that the candidates agree with the
default to 1e-12 (relative, max norm), and records the fastest under a key
(device, kind, n, basis, form, data kind, layout class, size class).  The
records live in a JSON file (``SGPU_TUNE_CACHE``, default
``~/.cache/shenfun_gb300/tuning.json``), written atomically, so that a
process reuses what earlier ones measured.  ``tune_problem`` tunes the plans
of a Helmholtz problem's step (the serving engine calls it once per shape
class when tuning is enabled); ``enable()`` makes ``plans.LinePlan`` look up
(and, on a miss, tune) its variant on every new layout.  No counterpart in
the reference (FFTW's planner flags are the closest: measure, then reuse the
choice through wisdom files).
"""
import ctypes
import json
import math
import os
import tempfile
import threading

import numpy as np
import torch

from . import _lib

_lock = threading.Lock()
_records = None
_enabled = os.environ.get("SGPU_AUTOTUNE", "0") not in ("", "0")

FOURIER = (_lib.XF_R2C, _lib.XF_C2R, _lib.XF_C2C_FWD, _lib.XF_C2C_BWD)
CHEB_TENSOR = (_lib.XF_CHEB_SCALAR, _lib.XF_CHEB_FORWARD, _lib.XF_CHEB_BACKWARD)


def cache_path():
    p = os.environ.get("SGPU_TUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "shenfun_gb300", "tuning.json")


def enable(on=True):
    """Let plans look up (and on a miss, tune) their kernel variant."""
    global _enabled
    _enabled = bool(on)


def enabled():
    return _enabled


def _load():
    global _records
    if _records is None:
        try:
            with open(cache_path()) as fh:
                _records = json.load(fh)
        except (OSError, ValueError):
            _records = {}
    return _records


def _save():
    path = cache_path()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    fd, tmp = tempfile.mkstemp(dir=os.path.dirname(path), prefix=".tuning")
    with os.fdopen(fd, "w") as fh:
        json.dump(_records, fh, indent=1, sort_keys=True)
    os.replace(tmp, path)


def candidates(kind, n, form, inner):
    """Variants that exist for this plan and layout (the default first)."""
    if kind in FOURIER and n == 256 and inner >= 16:
        if form != _lib.MIXED_DF:
            return [1, 2, 3, 4]
        # 7: the fixed-point C2C kernel with a tensor-copy input tile
        return [1, 2, 3, 4, 5, 6, 7] if kind in (_lib.XF_C2C_FWD, _lib.XF_C2C_BWD) else [1, 2, 3, 4, 5, 6]
    if form == _lib.MIXED_DF and kind in CHEB_TENSOR and inner == 1 and 16 <= n <= 341:
        return [1, 2]
    return []


def key(plan, outer, inner, data_kind):
    dev = torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"
    lines = max(1, int(outer) * int(inner))
    layout = "contiguous" if inner == 1 else "strided"
    return "|".join(str(x) for x in (dev, plan.kind, plan.n, plan.basis, plan.form, data_kind, layout,
                                     int(math.log2(lines))))


def lookup(plan, outer, inner, data_kind):
    with _lock:
        rec = _load().get(key(plan, outer, inner, data_kind))
    return None if rec is None else int(rec["variant"])


def _shapes(plan, outer, inner, data_kind):
    """(input, output) tensors of one call of `plan` on (outer, n, inner)."""
    n_in = n_out = plan.n
    cin = cout = data_kind == _lib.COMPLEX
    if plan.kind == _lib.XF_R2C:
        n_out, cin, cout = plan.n // 2 + 1, False, True
    elif plan.kind == _lib.XF_C2R:
        n_in, cin, cout = plan.n // 2 + 1, True, False
    elif plan.kind in (_lib.XF_C2C_FWD, _lib.XF_C2C_BWD):
        cin = cout = True
    g = torch.Generator(device="cuda").manual_seed(7)
    dt_in = torch.complex128 if cin else torch.float64
    x = torch.randn((outer, n_in, inner), dtype=dt_in, device="cuda", generator=g)
    y = torch.empty((outer, n_out, inner), dtype=torch.complex128 if cout else torch.float64, device="cuda")
    return x, y


def tune_plan(plan, outer, inner, data_kind, reps=5, warmup=2, save=True):
    """Time every variant of `plan` on (outer, n, inner) lines; returns the
    fastest (recorded under the layout's key), or None without variants."""
    cands = candidates(plan.kind, plan.n, plan.form, inner)
    if not cands:
        return None
    x, y = _shapes(plan, outer, inner, data_kind)
    scale = 1.0 / plan.n if plan.kind in (_lib.XF_R2C, _lib.XF_C2C_FWD) else 1.0
    times, ref = {}, None
    old = plan.variant
    try:
        for v in cands:
            try:
                plan.variant = v
            except _lib.SgpuError:
                continue
            for _ in range(warmup):
                plan(x, y, 1, scale)
            torch.cuda.synchronize()
            ts = []
            for _ in range(reps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                plan(x, y, 1, scale)
                e1.record()
                e1.synchronize()
                ts.append(e0.elapsed_time(e1) * 1e3)
            out = y.clone()
            if ref is None:
                ref = out
            else:
                err = float((out - ref).abs().max() / ref.abs().max().clamp_min(1e-300))
                if not err <= 1e-12:
                    raise _lib.SgpuError(_lib.ERR_CUDA, f"variant {v} disagrees with the default ({err:.1e})")
            times[v] = float(np.median(ts))
    finally:
        plan.variant = old
    best = min(times, key=times.get)
    with _lock:
        _load()[key(plan, outer, inner, data_kind)] = {"variant": best, "us": {str(k): round(t, 2)
                                                                             for k, t in times.items()}}
        if save:
            _save()
    return best


def apply(plan, outer, inner, data_kind):
    """Set `plan`'s variant for this layout from the records, tuning on a
    miss (a no-op for plans without variants)."""
    if not candidates(plan.kind, plan.n, plan.form, inner):
        return None
    v = lookup(plan, outer, inner, data_kind)
    if v is None:
        v = tune_plan(plan, outer, inner, data_kind)
    if v is not None and plan.variant != v:
        plan.variant = v
    return v


class _Handle:
    """A borrowed sgpu_plan handle (owned by the library's plan cache)."""

    def __init__(self, h, kind, n, basis, form):
        self._h = ctypes.c_void_p(h)
        self.kind, self.n, self.basis, self.form = kind, n, basis, form

    @property
    def variant(self):
        v = ctypes.c_int()
        _lib.call("sgpu_plan_get_variant", self._h, ctypes.byref(v))
        return v.value

    @variant.setter
    def variant(self, v):
        _lib.call("sgpu_plan_set_variant", self._h, int(v))

    def __call__(self, x, y, axis, scale):
        from .device import view3, data_kind, stream_handle
        outer, _, inner = view3(tuple(x.shape), axis)
        nb = ctypes.c_size_t()
        _lib.call("sgpu_plan_workspace_size", self._h, outer, inner, data_kind(x), ctypes.byref(nb))
        work = torch.empty(max(int(nb.value), 1), dtype=torch.uint8, device="cuda") if nb.value else None
        _lib.call("sgpu_plan_execute_ws", self._h, x.data_ptr(), y.data_ptr(), outer, inner, data_kind(x),
                  float(scale), work.data_ptr() if work is not None else None, nb.value, stream_handle())


def tune_problem(problem):
    """Tune and set the variants of the plans of a HelmholtzProblem's step
    (their layouts in that step); returns {pass: variant}."""
    hs = (ctypes.c_void_p * 6)()
    lines = (ctypes.c_int64 * 12)()
    _lib.call("sgpu_helmholtz_plan_handles", problem._h, ctypes.cast(hs, ctypes.c_void_p),
              ctypes.cast(lines, ctypes.c_void_p))
    nd = len(problem.N)
    Nd = problem.N[-1]
    Nr = problem.N[0] if nd == 2 else problem.N[1]
    cheb = _lib.BASIS_SD
    desc = [("dirichlet_scalar", _lib.XF_CHEB_SCALAR, Nd, cheb, _lib.REAL),
            ("r2c", _lib.XF_R2C, Nr, _lib.BASIS_ORTHO, _lib.REAL),
            ("c2c_fwd", _lib.XF_C2C_FWD, problem.N[0], _lib.BASIS_ORTHO, _lib.COMPLEX),
            ("c2c_bwd", _lib.XF_C2C_BWD, problem.N[0], _lib.BASIS_ORTHO, _lib.COMPLEX),
            ("c2r", _lib.XF_C2R, Nr, _lib.BASIS_ORTHO, _lib.COMPLEX),
            ("dirichlet_backward", _lib.XF_CHEB_BACKWARD, Nd, cheb, _lib.REAL)]
    out = {}
    for i, (name, kind, n, basis, dk) in enumerate(desc):
        if not hs[i]:
            continue
        h = _Handle(hs[i], kind, n, basis, problem.form)
        outer, inner = int(lines[2 * i]), int(lines[2 * i + 1])
        v = apply(h, outer, inner, dk)
        if v is not None:
            out[name] = v
    return out
