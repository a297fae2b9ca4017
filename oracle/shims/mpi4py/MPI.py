"""Single-rank stand-in for ``mpi4py.MPI`` used to import the reference pylbm.

Oracle test infrastructure only.  It implements what pylbm touches on one
process: a periodic Cartesian communicator, sub-array datatypes and
tag-matched ``Isend``/``Irecv`` pairs that copy slabs of the same array,
which is exactly the periodic ghost refresh pylbm performs with one rank
(pylbm/storage.py, ``Array.update``).
"""
import time

import numpy as np

SUM = "sum"
MAX = "max"
MIN = "min"


def Wtime():
    return time.perf_counter()


def Compute_dims(size, ndim):
    return [1] * ndim


class _Subarray:
    def __init__(self, sizes, subsizes, starts):
        self.sizes = list(sizes)
        self.subsizes = list(subsizes)
        self.starts = list(starts)

    def Commit(self):
        return self

    def Free(self):
        pass

    def slices(self):
        return tuple(slice(s, s + n) for s, n in zip(self.starts, self.subsizes))


class _Datatype:
    def Create_subarray(self, sizes, subsizes, starts, order=None):
        return _Subarray(sizes, subsizes, starts)


DOUBLE = _Datatype()
INT = _Datatype()


class _Request:
    def __init__(self, comm, kind, array, dtype, tag):
        self.comm = comm
        self.kind = kind
        self.array = array
        self.dtype = dtype
        self.tag = tag
        self.data = None
        if kind == "send":
            self.data = np.array(array[dtype.slices()], copy=True)

    def Wait(self):
        Request.Waitall([self])


class Request:
    @staticmethod
    def Waitall(requests):
        sends = {r.tag: r for r in requests if r.kind == "send"}
        for r in requests:
            if r.kind == "recv":
                s = sends.get(r.tag)
                if s is None:
                    s = r.comm._pending_sends.pop(r.tag, None)
                if s is None:
                    raise RuntimeError("single-rank MPI shim: unmatched receive")
                r.array[r.dtype.slices()] = s.data
        for r in requests:
            if r.kind == "send":
                r.comm._pending_sends.pop(r.tag, None)


class Comm:
    def __init__(self, ndim=0, periods=None):
        self.ndim = ndim
        self.periods = periods
        self._pending_sends = {}

    def Get_rank(self):
        return 0

    def Get_size(self):
        return 1

    def allreduce(self, sendobj=None, op=SUM):
        return sendobj

    def reduce(self, sendobj=None, op=SUM, root=0):
        return sendobj

    def bcast(self, obj=None, root=0):
        return obj

    def gather(self, sendobj=None, root=0):
        return [sendobj]

    def Barrier(self):
        pass

    def barrier(self):
        pass

    def Create_cart(self, dims, periods=None, reorder=False):
        return Comm(len(dims), periods)

    def Get_topo(self):
        return ([1] * self.ndim, self.periods, [0] * self.ndim)

    def Get_coords(self, rank):
        return [0] * self.ndim

    def Get_cart_rank(self, coords):
        return 0

    def Sub(self, remain_dims):
        return Comm(sum(1 for r in remain_dims if r), None)

    def Free(self):
        pass

    def Isend(self, buf, dest=0, tag=0):
        array, dtype = buf
        req = _Request(self, "send", array, dtype, tag)
        self._pending_sends[tag] = req
        return req

    def Irecv(self, buf, source=0, tag=0):
        array, dtype = buf
        return _Request(self, "recv", array, dtype, tag)

    def Send(self, *args, **kwargs):
        raise RuntimeError("single-rank MPI shim: Send is not supported")

    def Recv(self, *args, **kwargs):
        raise RuntimeError("single-rank MPI shim: Recv is not supported")


COMM_WORLD = Comm()
