"""The gb300 optimization mode against the reference's kernel dispatch, on
the CPU: the oracle replays every call recorded from the unmodified
reference (pinning its restatements of the biharmonic, banded, generic and
recursive-Legendre kernels), the module exposes every recorded name with a
signature that takes the recorded arguments, and install() routes an
imported, unmodified reference through it.  The GPU replays of the same
records are in test_gpu_optimization_mode.py."""
import inspect
import os
import subprocess
import sys

import numpy as np
import pytest

import optmode_replay as R
from oracle import la as OL, refabi as RA

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SOLVE_KINDS = ("TDMA", "PDMA", "FDMA", "TwoDMA", "ThreeDMA", "DiagMA", "HeptaDMA", "TDMA_O")
LU_OFFSETS = {"TDMA": (-2, 0, 2), "PDMA": (-4, -2, 0, 2, 4), "FDMA": (-2, 0, 2, 4), "TDMA_O": (-1, 0, 1),
              "HeptaDMA": (-4, -2, 0, 2, 4, 6, 8)}


def _systems(a, axis):
    return np.moveaxis(a, axis, -1).reshape(-1, a.shape[axis])


def oracle_call(rec):
    """Run one recorded call through the oracle; returns nothing (in place)."""
    name, a = rec.name, rec.args
    if name.endswith("_LU") and name[:-3] in LU_OFFSETS:
        kind = name[:-3]
        if kind == "TDMA":
            OL.tdma_lu(a[0])
        elif kind == "PDMA":
            OL.pdma_lu(a[0])
        else:
            OL.banded_lu(a[0], LU_OFFSETS[kind])
    elif name.endswith("_Solve") and name[:-6] in SOLVE_KINDS:
        u, data, axis = a
        v = np.moveaxis(u, axis, -1)
        lines = v.reshape(-1, v.shape[-1])
        for s in range(lines.shape[0]):
            line = lines[s].copy()
            RA.inner_solve(name[:-6], line, data)
            lines[s] = line
        v[...] = lines.reshape(v.shape)
    elif name == "SolverGeneric1ND_solve_data":
        u, data, sol, naxes, zero = a
        RA.solve_data(u, data, sol[:-len("_inner_solve")], int(naxes), zero)
    elif name == "LU_Helmholtz":
        A, B, As, Bs, neumann, d0, d1, d2, L, axis = a
        shape = list(d0.shape)
        shape[axis] = 1
        al = np.broadcast_to(As, shape).reshape(-1)
        be = np.broadcast_to(Bs, shape).reshape(-1)
        res = OL.helmholtz_lu(d0.shape[axis], al, be, neumann)
        for arr, r in zip((d0, d1, d2, L), res):
            np.moveaxis(arr, axis, -1)[...] = r.reshape(np.moveaxis(arr, axis, -1).shape)
    elif name == "Solve_Helmholtz":
        b, u, neumann, d0, d1, d2, L, axis = a
        f = _systems(b, axis)
        res = OL.helmholtz_solve(f, *[_systems(x, axis) for x in (d0, d1, d2, L)], neumann=neumann)
        np.moveaxis(u, axis, -1)[...] = res.reshape(np.moveaxis(u, axis, -1).shape)
    elif name == "Helmholtz_matvec":
        v, b, alfa, beta, A, B, axis = a
        shape = list(v.shape)
        shape[axis] = 1
        res = OL.helmholtz_matvec(_systems(v, axis), np.broadcast_to(alfa, shape).reshape(-1),
                                  np.broadcast_to(beta, shape).reshape(-1))
        np.moveaxis(b, axis, -1)[...] = res.reshape(np.moveaxis(b, axis, -1).shape)
    elif name == "LU_Biharmonic":
        RA.lu_biharmonic(*a[:-1], axis=int(a[-1]))
    elif name == "Biharmonic_factor_pr":
        RA.biharmonic_factor_pr(*a[:-1], axis=int(a[-1]))
    elif name == "Biharmonic_Solve":
        RA.biharmonic_solve(*a[:-1], axis=int(a[-1]))
    elif name == "Biharmonic_matvec":
        RA.biharmonic_matvec(*a[:-1], axis=int(a[-1]))
    elif name == "transforms.scalar_product":
        RA.scalar_product(*a)
    elif name == "transforms.evaluate_expansion_all":
        RA.evaluate_expansion_all(*a)
    else:
        raise KeyError(name)


RECORDS = R.calls()


@pytest.mark.parametrize("i", range(len(RECORDS)), ids=[f"{i}-{r.name}" for i, r in enumerate(RECORDS)])
def test_oracle_replays_reference_dispatch(i):
    rec = R.calls()[i]
    oracle_call(rec)
    errs = rec.rel_errors()
    assert errs, "the record wrote nothing"
    for j, e in errs.items():
        assert e < 1e-13, (rec.name, j, e)


def test_every_dispatched_name_is_covered():
    names = {r.name for r in RECORDS}
    # every kernel family of the reference's dispatch list on this path
    for n in ("TDMA_LU", "TDMA_Solve", "PDMA_LU", "PDMA_Solve", "FDMA_LU", "FDMA_Solve", "TwoDMA_Solve",
              "ThreeDMA_Solve", "DiagMA_Solve", "HeptaDMA_LU", "HeptaDMA_Solve", "TDMA_O_LU", "TDMA_O_Solve",
              "SolverGeneric1ND_solve_data", "LU_Helmholtz", "Solve_Helmholtz", "Helmholtz_matvec",
              "LU_Biharmonic", "Biharmonic_factor_pr", "Biharmonic_Solve", "Biharmonic_matvec",
              "transforms.scalar_product", "transforms.evaluate_expansion_all"):
        assert n in names, n


def test_module_exposes_recorded_names_and_signatures():
    import shenfun_gb300.optimization as opt
    import shenfun_gb300.optimization.transforms as tr
    for rec in RECORDS:
        fn = getattr(tr, rec.name.split(".", 1)[1]) if rec.name.startswith("transforms.") else getattr(opt, rec.name)
        inspect.signature(fn).bind(*rec.args)  # raises TypeError when the arguments do not fit
    for kind in SOLVE_KINDS:
        fn = getattr(opt, kind + "_inner_solve")
        assert fn.__name__ == kind + "_inner_solve"  # SolverGeneric1ND_solve_data resolves sol by name
    assert "inner_solve" not in dir(opt)  # optimizer() must fall through to the Class_method name


def test_no_gpu_means_an_error_not_a_fallback():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import shenfun_gb300.optimization as opt
    from shenfun_gb300 import SgpuError
    rec = R.calls(names={"TDMA_LU"})[0]
    with pytest.raises((SgpuError, RuntimeError, AssertionError)):
        opt.TDMA_LU(rec.args[0])


ROUTE_CHECK = r"""
import importlib, sys
sys.path.insert(0, {golden!r}); sys.path.insert(0, {repo!r})
from refimport import import_reference
import_reference()
import shenfun
from shenfun import la, chebyshev
from shenfun.optimization import optimizer
import shenfun_gb300.optimization as gb
import shenfun_gb300.optimization.transforms as gbt
gb.install()
def resolve(static):
    return optimizer(static.func, False)
checks = {{
    "TDMA.LU": (la.TDMA.LU, gb.TDMA_LU), "TDMA.Solve": (la.TDMA.Solve, gb.TDMA_Solve),
    "PDMA.LU": (la.PDMA.LU, gb.PDMA_LU), "PDMA.Solve": (la.PDMA.Solve, gb.PDMA_Solve),
    "FDMA.Solve": (la.FDMA.Solve, gb.FDMA_Solve), "TwoDMA.Solve": (la.TwoDMA.Solve, gb.TwoDMA_Solve),
    "ThreeDMA.Solve": (la.ThreeDMA.Solve, gb.ThreeDMA_Solve), "HeptaDMA.Solve": (la.HeptaDMA.Solve, gb.HeptaDMA_Solve),
    "TDMA_O.Solve": (la.TDMA_O.Solve, gb.TDMA_O_Solve), "DiagMA.Solve": (la.DiagMA.Solve, gb.DiagMA_Solve),
    "SolverGeneric1ND.solve_data": (la.SolverGeneric1ND.solve_data, gb.SolverGeneric1ND_solve_data),
    "Helmholtz.LU_Helmholtz": (chebyshev.la.Helmholtz.LU_Helmholtz, gb.LU_Helmholtz),
    "Helmholtz.Solve_Helmholtz": (chebyshev.la.Helmholtz.Solve_Helmholtz, gb.Solve_Helmholtz),
    "Helmholtz.Helmholtz_matvec": (chebyshev.la.Helmholtz.Helmholtz_matvec, gb.Helmholtz_matvec),
    "Biharmonic.LU_Biharmonic": (chebyshev.la.Biharmonic.LU_Biharmonic, gb.LU_Biharmonic),
    "Biharmonic.Biharmonic_factor_pr": (chebyshev.la.Biharmonic.Biharmonic_factor_pr, gb.Biharmonic_factor_pr),
    "Biharmonic.Biharmonic_Solve": (chebyshev.la.Biharmonic.Biharmonic_Solve, gb.Biharmonic_Solve),
    "Biharmonic.Biharmonic_matvec": (chebyshev.la.Biharmonic.Biharmonic_matvec, gb.Biharmonic_matvec),
}}
for k, (static, mine) in checks.items():
    got = resolve(static)
    assert got is mine, (k, got)
# the inner solves SolverGeneric1ND.fast_solve passes as `sol`
assert optimizer(la.TDMA.inner_solve, False) is gb.TDMA_inner_solve
assert optimizer(la.PDMA.inner_solve, False) is gb.PDMA_inner_solve
tr = importlib.import_module("shenfun.optimization.cython.transforms")
assert tr.scalar_product is gbt.scalar_product and tr.evaluate_expansion_all is gbt.evaluate_expansion_all
# names off the path keep the compiled kernels
assert not getattr(tr.leg2cheb, "__module__", "").startswith("shenfun_gb300")
print("ROUTED", len(checks))
"""


def test_install_routes_the_unmodified_reference():
    ref = os.environ.get("REFERENCE_ROOT") or os.path.normpath(os.path.join(REPO, os.pardir, "reference"))
    if not os.path.isdir(os.path.join(ref, "shenfun")):
        pytest.skip("reference checkout not present")
    refdir = os.path.join(REPO, "oracle", "_ref")
    if not os.path.isdir(refdir) or not any(f.startswith("la.") and f.endswith(".so") for f in os.listdir(refdir)):
        pytest.skip("reference kernels not built")
    code = ROUTE_CHECK.format(golden=os.path.join(REPO, "tests", "golden"), repo=REPO)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "ROUTED" in r.stdout, r.stderr[-3000:]
