"""The C-ABI library loads and exports every symbol the header declares (CPU)."""
import ctypes
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "shenfun_gb300.h")


def header_symbols():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+char\s*\*|int)\s+(sgpu_\w+)\s*\(", txt, re.M)))


@pytest.fixture(scope="module")
def lib():
    from shenfun_gb300 import build, _lib
    build.build()
    return _lib.load()


def test_exports_every_declared_symbol(lib):
    syms = header_symbols()
    assert len(syms) >= 12
    for s in syms:
        assert hasattr(lib, s), s


def test_python_binding_covers_header():
    from shenfun_gb300 import _lib
    assert set(header_symbols()) <= set(_lib.SIGNATURES)


def test_status_strings(lib):
    for st in range(8):
        assert lib.sgpu_status_string(st)
    assert lib.sgpu_version() >= 100


def test_argument_checks_without_device(lib):
    from shenfun_gb300 import _lib
    h = ctypes.c_void_p()
    # invalid kind / length / basis are rejected before any CUDA call
    assert lib.sgpu_plan_create(ctypes.byref(h), 99, 16, 0, 0) == _lib.ERR_ARG
    assert lib.sgpu_plan_create(ctypes.byref(h), _lib.XF_R2C, 1, 0, 0) == _lib.ERR_ARG
    assert lib.sgpu_plan_create(ctypes.byref(h), _lib.XF_CHEB_SCALAR, 16, 7, 0) == _lib.ERR_ARG
    assert lib.sgpu_plan_create(ctypes.byref(h), _lib.XF_R2C, 16, 0, 5) == _lib.ERR_UNSUPPORTED
    assert lib.sgpu_LU_Helmholtz(16, None, None, 1, None, None, None, None, 1, 1, None) == \
        _lib.ERR_ARG
    # neumann must be 0 or 1; Poisson solves need a nonzero scale
    buf = (ctypes.c_double * 64)()
    assert lib.sgpu_LU_Helmholtz(16, buf, buf, 2, buf, buf, buf, buf, 1, 1, None) == _lib.ERR_ARG
    assert lib.sgpu_Poisson_Solve_ADD(buf, buf, ctypes.c_double(0.0), 1, 16, 1, 0, None) == _lib.ERR_ARG
    assert lib.sgpu_Poisson_Solve_ANN(buf, buf, ctypes.c_double(1.0), ctypes.c_double(0.0), 1, 4, 1, 0,
                                      None) == _lib.ERR_ARG
    assert lib.sgpu_plan_create(ctypes.byref(h), _lib.XF_CHEB_SCALAR, 16, 4, 0) == _lib.ERR_ARG
    assert lib.sgpu_Solve_Helmholtz(None, None, 0, None, None, None, None, 1, 16, 1, 1, None) == \
        _lib.ERR_ARG
    assert lib.sgpu_TDMA_Solve(None, None, 1, 16, 1, 0, None) == _lib.ERR_ARG


def test_no_device_means_no_compute():
    import torch
    from shenfun_gb300 import device, SgpuError
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    with pytest.raises(SgpuError):
        device.require_cuda()
