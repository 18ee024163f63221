"""Single-rank stand-in for mpi4py-fft (not installed here): serial FFT plan
objects with FFTW's unnormalised conventions, trivial pencils/transfers and a
numpy-backed DistArray."""
from . import fftw  # noqa: F401
from .distarray import DistArray, newDistArray  # noqa: F401
from .mpifft import PFFT, Transform  # noqa: F401
from . import pencil  # noqa: F401
from . import io  # noqa: F401
