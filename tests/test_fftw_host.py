"""Host-side logic of the FFTW-style plan objects (shenfun_gb300.fftw): the
planner flags, axis and dtype handling, and that making device arrays
without a GPU fails loudly (no CPU fallback)."""
import numpy as np
import pytest
import torch

from shenfun_gb300 import _lib, fftw as F


def test_flags_are_fftw_values():
    assert F.flag_dict["FFTW_MEASURE"] == 0 and F.flag_dict["FFTW_ESTIMATE"] == 64
    assert F.flag_dict["FFTW_DESTROY_INPUT"] == 1 and F.flag_dict["FFTW_PRESERVE_INPUT"] == 16


def test_one_axis_per_plan():
    x = torch.zeros(2, 3, 4)
    assert F._axis(x, (-1,)) == 2 and F._axis(x, 1) == 1
    with pytest.raises(_lib.SgpuError):
        F._axis(x, (0, 1))


def test_dtypes():
    assert F._tdtype(float) is torch.float64 and F._tdtype(np.complex128) is torch.complex128
    assert F._tdtype(torch.float64) is torch.float64
    with pytest.raises(_lib.SgpuError):
        F._tdtype(np.float32)


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the no-device path")
def test_no_device_fails_loudly():
    with pytest.raises(_lib.SgpuError):
        F.aligned((4, 4))
    with pytest.raises(_lib.SgpuError):
        F.dctn(torch.zeros(4, 16))
