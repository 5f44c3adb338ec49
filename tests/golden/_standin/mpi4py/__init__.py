"""Single-rank stand-in for ``mpi4py``, used only to run the reference's own
``bin/assemble.py`` in this repository's fixture generator.

The reference assembles its pencil under MPI (``bin/assemble.py:46-67`` scatter of
the l lists, ``:548,1128`` allgather of local lengths, ``:574-576,1156-1158`` gather
of COO triplets to rank 0, ``:596,1176`` barriers). With one rank every collective
is a copy, which is all this module implements. It is test infrastructure: no
product code imports it.
"""


def _buf(x):
    # mpi4py accepts either an array or a [array, datatype] pair
    if isinstance(x, (list, tuple)):
        return x[0]
    return x


class _Comm:
    def Get_size(self):
        return 1

    def Get_rank(self):
        return 0

    def Scatter(self, sendbuf, recvbuf, root=0):
        s, r = _buf(sendbuf), _buf(recvbuf)
        r[...] = s[: r.shape[0]]

    def Gather(self, sendbuf, recvbuf, root=0):
        s, r = _buf(sendbuf), _buf(recvbuf)
        r[: s.shape[0]] = s

    def allgather(self, x):
        return [x]

    def Barrier(self):
        pass


class MPI:
    COMM_WORLD = _Comm()
    DOUBLE_COMPLEX = "DOUBLE_COMPLEX"
    DOUBLE = "DOUBLE"
