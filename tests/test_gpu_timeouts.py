"""GPU: a bounded device wait that runs out is reported, not silent, and the
library stays usable afterwards.

The fused tensor-core contraction's pipeline waits get a 1 ns limit, so that
the first wait that is not satisfied at once gives up.  The kernel then
records the event, waits for the copies and MMAs it already issued (with the
standard limit) and returns: no trap, no hang.  sgpu_last_error reports
SGPU_ERR_TIMEOUT; with the limit restored the same call is correct again."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from shenfun_gb300 import build
    build.build()
    from shenfun_gb300 import _lib
    assert _lib.load().sgpu_device_ok() == 1
    return _lib


def test_wait_that_runs_out_is_reported(lib):
    from shenfun_gb300.spaces import ChebyshevShenDirichlet
    n = 257
    Vm = ChebyshevShenDirichlet(n)
    Vm.form = lib.MIXED_DF
    Vp = ChebyshevShenDirichlet(n)
    x = torch.randn(8192, n, dtype=torch.float64, device="cuda")
    ref = Vp.scalar_product(x, axis=1)
    Vm.scalar_product(x, axis=1)
    lib.check_device()  # clean so far
    try:
        lib.call("sgpu_set_wait_limit_ns", 1)
        Vm.scalar_product(x, axis=1)
        with pytest.raises(lib.SgpuError) as e:
            lib.check_device()
        assert e.value.status == lib.ERR_TIMEOUT
    finally:
        lib.call("sgpu_set_wait_limit_ns", 0)
    # the context is intact and the next call is right
    y = Vm.scalar_product(x, axis=1)
    lib.check_device()
    err = (y - ref).abs().max().item() / ref.abs().max().item()
    assert err < 1e-12
