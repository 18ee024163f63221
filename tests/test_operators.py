"""Host operators of projections and linear forms (shenfun_gb300/operators.py)
against the reference's own results (tests/golden/project.npz), applied with
numpy on the CPU exactly as sgpu_line_gemm applies them on the GPU."""
import numpy as np
import pytest

import shenfun_gb300 as sg
from shenfun_gb300.operators import expr_plan


def apply(plan, u):
    ax, out_shape, cplx, terms = plan
    out = np.zeros(out_shape, dtype=complex if cplx else float)
    um = np.moveaxis(np.asarray(u, dtype=complex if cplx else float), ax, -1)
    om = np.moveaxis(out, ax, -1)
    lines_in = um.reshape(-1, um.shape[-1])
    lines_out = om.reshape(-1, om.shape[-1])
    for M, scale in terms:
        s = scale.view(complex) if cplx else scale
        lines_out += s[:, None] * (lines_in @ M)
    return np.moveaxis(lines_out.reshape(om.shape), -1, ax)


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def D(*d):
    return tuple(d)


CASES = [
    # (fixture key, test space, trial space, input key, terms, solve)
    ("sd_dx_T", ("C", None, 14), ("C", (0, 0), 14), "sd_u", [(1.0, D(1))], True),
    ("sd_dxx_SD", ("C", (0, 0), 14), ("C", (0, 0), 14), "sd_u", [(1.0, D(2))], True),
    ("sd_u_T", ("C", None, 14), ("C", (0, 0), 14), "sd_u", [(1.0, D(0))], True),
    ("sd_inner_dxx", ("C", (0, 0), 14), ("C", (0, 0), 14), "sd_u", [(1.0, D(2))], False),
    ("sd_inner_u_T", ("C", None, 14), ("C", (0, 0), 14), "sd_u", [(1.0, D(0))], False),
    ("sb_d3_T", ("C", None, 16), ("C", (0, 0, 0, 0), 16), "sb_u", [(1.0, D(3))], True),
    ("sb_lap_SB", ("C", (0, 0, 0, 0), 16), ("C", (0, 0, 0, 0), 16), "sb_u", [(1.0, D(2))], True),
    ("sn_dx_T", ("C", None, 14), ("C", {"left": {"N": 0}, "right": {"N": 0}}, 14), "sn_u", [(1.0, D(1))], True),
    ("l_dx_L", ("L", None, 14), ("L", (0, 0), 14), "l_u", [(1.0, D(1))], True),
    ("l_dxx_SD", ("L", (0, 0), 14), ("L", (0, 0), 14), "l_u", [(1.0, D(2))], True),
]


def space(spec):
    fam, bc, N = spec
    return sg.FunctionSpace(N, fam, bc=bc) if bc is not None else sg.FunctionSpace(N, fam)


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_operator_1d(golden, case):
    key, ts, us, ukey, terms, solve = case
    d = golden("project")
    plan = expr_plan(space(ts), space(us), terms, solve, False)
    assert rel(apply(plan, d[ukey]), d[key]) < 1e-12


def test_operator_tensor_product(golden):
    d = golden("project")
    F0 = sg.FunctionSpace(6, "F", dtype="D")
    F1 = sg.FunctionSpace(8, "F", dtype="d")
    SD, T14 = sg.FunctionSpace(14, "C", bc=(0, 0)), sg.FunctionSpace(14, "C")
    T3 = sg.TensorProductSpace(sg.comm, (F0, F1, SD))
    T3o = sg.TensorProductSpace(sg.comm, (F0, F1, T14))
    u = d["t3_u"]
    assert rel(apply(expr_plan(T3o, T3, [(1.0, (0, 0, 1))], True, True), u), d["t3_dz_T"]) < 1e-12
    lap = [(1.0, (2, 0, 0)), (1.0, (0, 2, 0)), (1.0, (0, 0, 2))]
    assert rel(apply(expr_plan(T3, T3, lap, True, True), u), d["t3_lap"]) < 1e-12
    assert rel(apply(expr_plan(T3, T3, lap, False, True), u), d["t3_inner_lap"]) < 1e-12
    mix = [(1.0, (1, 0, 0)), (2.0, (0, 2, 0))]
    assert rel(apply(expr_plan(T3, T3, mix, True, True), u), d["t3_mix"]) < 1e-12
    FF = sg.TensorProductSpace(sg.comm, (F0, F1))
    ff = [(1.0, (0, 1)), (-1.0, (2, 0))]
    assert rel(apply(expr_plan(FF, FF, ff, True, True), d["ff_u"]), d["ff_d"]) < 1e-12
