"""Single-rank ``MPI.COMM_WORLD`` stand-in: rank 0 of size 1.

Collectives degenerate to identities: ``bcast``/``reduce`` return the object,
``Reduce`` copies the send buffer into the receive buffer, ``Bcast`` is a no-op.
"""

import numpy as _np


class _Comm:
    rank = 0
    size = 1

    def Get_rank(self):
        return 0

    def Get_size(self):
        return 1

    def bcast(self, obj, root=0):
        return obj

    def reduce(self, obj, op=None, root=0):
        return obj

    def allreduce(self, obj, op=None):
        return obj

    def Reduce(self, sendbuf, recvbuf, op=None, root=0):
        _np.copyto(recvbuf, sendbuf)

    def Bcast(self, buf, root=0):
        return None

    def send(self, obj, dest=0, tag=0):
        raise RuntimeError("single-rank stand-in: send is unreachable")

    def recv(self, source=0, tag=0):
        raise RuntimeError("single-rank stand-in: recv is unreachable")

    def Barrier(self):
        return None


COMM_WORLD = _Comm()
SUM = "sum"
