// Single-rank stand-in for <mpi.h> -- TEST INFRASTRUCTURE ONLY.
//
// Lets the reference's own src/kmeans.cpp compile and run as one MPI rank without an MPI
// library: every collective of a one-process communicator degenerates to a copy (Scatter,
// Scatterv, Gather, Gatherv, Allreduce) or to nothing (Bcast, Barrier), and the rank is 0.
#ifndef THC_REF_MPI_STUB_H
#define THC_REF_MPI_STUB_H

#include <cstring>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_SUM 1
#define MPI_MAX 2
// Datatype handles encode the element size in bytes.
#define MPI_INT ((MPI_Datatype)sizeof(int))
#define MPI_UNSIGNED ((MPI_Datatype)sizeof(unsigned))
#define MPI_DOUBLE ((MPI_Datatype)sizeof(double))
#define MPI_UNSIGNED_LONG_LONG ((MPI_Datatype)sizeof(unsigned long long))
#define MPI_DOUBLE_COMPLEX ((MPI_Datatype)(2 * sizeof(double)))
#define MPI_CHAR ((MPI_Datatype)1)

inline int thc_mpi_copy(const void* src, void* dst, long long count, MPI_Datatype t)
{
  if (src != dst && count > 0) std::memmove(dst, src, (size_t)count * (size_t)t);
  return MPI_SUCCESS;
}

inline int MPI_Init(int*, char***) { return MPI_SUCCESS; }
inline int MPI_Finalize() { return MPI_SUCCESS; }
inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return MPI_SUCCESS; }
inline int MPI_Comm_size(MPI_Comm, int* n) { *n = 1; return MPI_SUCCESS; }
inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm)
{
  return thc_mpi_copy(s, r, n, t);
}
inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm)
{
  return thc_mpi_copy(s, r, n, t);
}
inline int MPI_Scatter(const void* s, int n, MPI_Datatype t, void* r, int, MPI_Datatype, int,
                       MPI_Comm)
{
  return thc_mpi_copy(s, r, n, t);
}
inline int MPI_Scatterv(const void* s, const int* counts, const int* displs, MPI_Datatype t,
                        void* r, int, MPI_Datatype, int, MPI_Comm)
{
  return thc_mpi_copy((const char*)s + (size_t)displs[0] * t, r, counts[0], t);
}
inline int MPI_Gather(const void* s, int n, MPI_Datatype t, void* r, int, MPI_Datatype, int,
                      MPI_Comm)
{
  return thc_mpi_copy(s, r, n, t);
}
inline int MPI_Gatherv(const void* s, int n, MPI_Datatype t, void* r, const int*,
                       const int* displs, MPI_Datatype, int, MPI_Comm)
{
  return thc_mpi_copy(s, (char*)r + (size_t)displs[0] * t, n, t);
}

#endif
