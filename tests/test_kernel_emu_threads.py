"""Thread decompositions of the block programs cover every element exactly once
for the CTA sizes the kernels launch with (CPU)."""
import os
import subprocess
import tempfile

from test_kernel_emu import emu  # noqa: F401  (fixture: builds the harness)


def test_loop_decompositions(emu):  # noqa: F811
    with tempfile.TemporaryDirectory() as td:
        r = subprocess.run([emu, "lkcheck", os.path.join(td, "o")], capture_output=True, text=True,
                           env=dict(os.environ, ASAN_OPTIONS="detect_leaks=0"))
        assert r.returncode == 0, r.stderr
