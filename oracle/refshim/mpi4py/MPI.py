"""Single-rank MPI communicator (rank 0 of 1)."""
import numpy as _np

INT = "int"
FLOAT = "float"
DOUBLE = "double"
MAX = "max"
SUM = "sum"


class Request:
    @staticmethod
    def Waitall(reqs):
        return None


class _Comm:
    def Get_rank(self):
        return 0

    def Get_size(self):
        return 1

    def barrier(self):
        return None

    Barrier = barrier

    def bcast(self, obj, root=0):
        return obj

    def allgather(self, obj):
        return [obj]

    def Allgather(self, sendbuf, recvbuf):
        s = sendbuf[0] if isinstance(sendbuf, (list, tuple)) else sendbuf
        r = recvbuf[0] if isinstance(recvbuf, (list, tuple)) else recvbuf
        _np.asarray(r).reshape(-1)[: _np.asarray(s).size] = _np.asarray(s).reshape(-1)

    def Allreduce(self, sendbuf, recvbuf, op=None):
        _np.copyto(recvbuf, sendbuf)

    def Gatherv(self, sendbuf, recvbuf, root=0):
        s = sendbuf[0] if isinstance(sendbuf, (list, tuple)) else sendbuf
        r = recvbuf[0] if isinstance(recvbuf, (list, tuple)) else recvbuf
        _np.asarray(r).reshape(-1)[: _np.asarray(s).size] = _np.asarray(s).reshape(-1)

    def Alltoall(self, sendbuf, recvbuf):
        _np.copyto(recvbuf, sendbuf)


COMM_WORLD = _Comm()
