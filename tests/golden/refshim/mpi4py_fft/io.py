"""File I/O is not on the solve path; these classes only need to exist."""


class HDF5File:
    def __init__(self, *a, **k):
        raise NotImplementedError("HDF5 output is not available in the shim")


class NCFile(HDF5File):
    pass
