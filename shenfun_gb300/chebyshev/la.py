"""``shenfun.chebyshev.la`` counterpart: tailored Chebyshev solvers."""
from ..la import Helmholtz, Biharmonic, ADDSolver, ANNSolver  # noqa: F401
