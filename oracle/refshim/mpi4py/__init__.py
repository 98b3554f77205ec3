"""Single-rank stand-in for mpi4py, imported by the reference's adFVM/parallel.py:28-36.

Reductions return their input (one rank); MAX/MIN/SUM exist so that parallel.min/max/sum
(adFVM/parallel.py:103-110) work. Test infrastructure only."""


class _Comm(object):
    def Get_size(self): return 1
    def Get_rank(self): return 0
    def gather(self, x, root=0): return [x]
    def bcast(self, x, root=0): return x
    def Bcast(self, x, root=0): return None
    def Barrier(self): return None
    def scatter(self, x, root=0): return x[0]
    def allreduce(self, x, op=None): return x
    def Abort(self, code=1): raise RuntimeError('MPI Abort requested by the reference (NaN check)')


class _MPI(object):
    COMM_WORLD = _Comm()
    MAX, MIN, SUM, MINLOC = 'max', 'min', 'sum', 'minloc'

    @staticmethod
    def Get_processor_name():
        return 'localhost'


MPI = _MPI()
