"""One-process communicator with the subset of mpi4py.MPI the reference uses."""
import copy as _copy

SUM = "sum"
MAX = "max"
MIN = "min"
PROD = "prod"
IN_PLACE = "in_place"
UNDEFINED = -32766


class Comm:
    rank = 0
    size = 1

    def Get_rank(self):
        return 0

    def Get_size(self):
        return 1

    def allreduce(self, x, op=SUM):
        return _copy.copy(x)

    def Allreduce(self, a, b=None, op=SUM):
        if a is IN_PLACE:
            return
        if b is not None:
            b[...] = a

    def reduce(self, x, op=SUM, root=0):
        return _copy.copy(x)

    def Reduce(self, a, b=None, op=SUM, root=0):
        if b is not None and a is not IN_PLACE:
            b[...] = a

    def bcast(self, x, root=0):
        return x

    def Bcast(self, a, root=0):
        return None

    def gather(self, x, root=0):
        return [x]

    def allgather(self, x):
        return [x]

    def scatter(self, x, root=0):
        return x[0]

    def Barrier(self):
        return None

    barrier = Barrier

    def Split(self, color=0, key=0):
        return Comm()

    def Create_cart(self, dims, periods=None, reorder=False):
        return Cartcomm(dims)

    def Free(self):
        return None

    def Dup(self):
        return Comm()

    def Get_topology(self):
        return ([1], [0], [0])


class Cartcomm(Comm):
    def __init__(self, dims=(1,)):
        self.dims = list(dims)

    def Sub(self, remain):
        return Cartcomm([1] * sum(bool(r) for r in remain))

    def Get_coords(self, rank):
        return [0] * len(self.dims)


COMM_WORLD = Comm()
COMM_SELF = Comm()


def Compute_dims(size, dims):
    return [1 if d == 0 else d for d in dims]
