/* Single-rank stand-in for the MPI header included by the reference's
 * adFVM/cpp/include/parallel.hpp. Provides only what adFVM/cpp/mesh.cpp and that header
 * use when compiled for one process. Test infrastructure only. */
#ifndef AFVM_REFSHIM_MPI_H
#define AFVM_REFSHIM_MPI_H
typedef int MPI_Comm;
typedef int MPI_Datatype;
#define MPI_COMM_WORLD 0
#define MPI_FLOAT 1
#define MPI_DOUBLE 2
static inline int MPI_Comm_rank(MPI_Comm c, int* r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int* s) { (void)c; *s = 1; return 0; }
#endif
