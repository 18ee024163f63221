"""The autotuner's records on the CPU: candidate variants per plan and
layout, keys, and the on-disk cache (atomic write, reload)."""
import json

import pytest

from shenfun_gb300 import _lib, autotune


class FakePlan:
    def __init__(self, kind, n, basis=0, form=_lib.MIXED_DF):
        self.kind, self.n, self.basis, self.form = kind, n, basis, form
        self.variant = 0


def test_candidates():
    assert autotune.candidates(_lib.XF_C2C_FWD, 256, _lib.MIXED_DF, 33153) == [1, 2, 3, 4, 5, 6, 7]
    assert autotune.candidates(_lib.XF_R2C, 256, _lib.MIXED_DF, 257) == [1, 2, 3, 4, 5, 6]
    assert autotune.candidates(_lib.XF_R2C, 256, _lib.PLAIN_F64, 257) == [1, 2, 3, 4]
    assert autotune.candidates(_lib.XF_R2C, 256, _lib.MIXED_DF, 1) == []      # contiguous lines: one kernel
    assert autotune.candidates(_lib.XF_R2C, 128, _lib.MIXED_DF, 257) == []    # not the strided kernel's length
    assert autotune.candidates(_lib.XF_CHEB_SCALAR, 257, _lib.MIXED_DF, 1) == [1, 2]
    assert autotune.candidates(_lib.XF_CHEB_SCALAR, 257, _lib.PLAIN_F64, 1) == []
    assert autotune.candidates(_lib.XF_CHEB_SCALAR, 257, _lib.MIXED_DF, 4) == []


def test_records_roundtrip(tmp_path, monkeypatch):
    path = tmp_path / "t.json"
    monkeypatch.setenv("SGPU_TUNE_CACHE", str(path))
    monkeypatch.setattr(autotune, "_records", None)
    p = FakePlan(_lib.XF_C2C_FWD, 256)
    k = autotune.key(p, 1, 33153, _lib.COMPLEX)
    assert "|strided|" in k and k.endswith("|15")
    assert autotune.lookup(p, 1, 33153, _lib.COMPLEX) is None
    with autotune._lock:
        autotune._load()[k] = {"variant": 4, "us": {"1": 220.0, "4": 210.0}}
        autotune._save()
    monkeypatch.setattr(autotune, "_records", None)  # a new process reads the file
    assert autotune.lookup(p, 1, 33153, _lib.COMPLEX) == 4
    assert json.loads(path.read_text())[k]["variant"] == 4
    assert not list(tmp_path.glob(".tuning*"))  # the temporary file was renamed into place


def test_apply_without_variants_is_a_no_op():
    assert autotune.apply(FakePlan(_lib.XF_R2C, 100), 4, 4, _lib.REAL) is None
