"""``shenfun.chebyshev.la`` counterpart: tailored Chebyshev solvers."""
from ..la import Helmholtz, Biharmonic  # noqa: F401
