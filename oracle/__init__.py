"""CPU oracle for the spectral-Galerkin forward / banded-solve / backward path.

TEST INFRASTRUCTURE ONLY.  This package is the checker: only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py`` may import
it.  The product (``shenfun_gb300``) never imports, links or calls anything
here, and it has no CPU fallback.

It is a numpy restatement of the reference algorithms (shenfun 4.3.0), each
function citing the reference file:line it follows.  It is pinned against
golden fixtures recorded from the unmodified reference (``tests/golden``), see
``tests/test_oracle_golden.py``.  FFTW (used by the reference through
mpi4py-fft, unpinned version) is restated with scipy.fft using FFTW's
unnormalised REDFT10/REDFT01/DFT conventions.

Modules:
  spectral  - 1D transforms along an axis (Chebyshev GC, Fourier R2C/C2C,
              Legendre LG recursive/Vandermonde), Shen stencils, mass matrices
  la        - banded LU/solves (TDMA, PDMA), Chebyshev Helmholtz LU/solve/matvec,
              biharmonic and generic per-wavenumber solves
  problems  - tensor-product round trips used by tests and the CPU baseline
"""
from . import spectral, la, problems  # noqa: F401
