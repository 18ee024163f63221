"""Chebyshev namespace mirroring ``shenfun.chebyshev`` (bases + la)."""
from ..spaces import (ChebyshevOrthogonal as Orthogonal,  # noqa: F401
                      ChebyshevShenDirichlet as ShenDirichlet,
                      ChebyshevShenBiharmonic as ShenBiharmonic,
                      ChebyshevShenNeumann as ShenNeumann)
from . import la  # noqa: F401
