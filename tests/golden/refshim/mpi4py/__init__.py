"""Single-rank stand-in for mpi4py (the reference imports MPI unconditionally)."""
from . import MPI  # noqa: F401
