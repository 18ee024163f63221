"""``shenfun.chebyshev.la`` counterpart: tailored Chebyshev solvers."""
from ..la import Helmholtz  # noqa: F401
