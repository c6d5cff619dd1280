/*
 * Single-rank stand-in for <mpi.h>, used ONLY to compile the reference's
 * unmodified C++ sources into the test oracle (oracle/_ref).  It is test
 * infrastructure: nothing in the product links it.
 *
 * The reference's MPI path (src/simulation/my_mpi.cpp) is reached only when a
 * communicator is handed in through set_mpi_comm(); the oracle harness never
 * does that, so every function below is a no-op that reports a world of one
 * rank.
 */
#ifndef ORACLE_STUB_MPI_H_
#define ORACLE_STUB_MPI_H_

#include <cstdlib>

typedef int MPI_Comm;
typedef int MPI_Request;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct {
   int MPI_SOURCE;
   int MPI_TAG;
   int MPI_ERROR;
} MPI_Status;

#define MPI_REQUEST_NULL 0
#define MPI_PROC_NULL (-2)
#define MPI_UNDEFINED (-32766)
#define MPI_ANY_SOURCE (-1)
#define MPI_DOUBLE 1
#define MPI_INT 2
#define MPI_SUM 1
#define MPI_MAX 2

inline int MPI_Abort(MPI_Comm, int code) { std::exit(code); }
inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
inline int MPI_Comm_size(MPI_Comm, int *s) { *s = 1; return 0; }
inline int MPI_Cart_create(MPI_Comm c, int, const int *, const int *, int,
                           MPI_Comm *out) { *out = c; return 0; }
inline int MPI_Cart_coords(MPI_Comm, int, int n, int *coords) {
   for (int i = 0; i < n; i++) coords[i] = 0;
   return 0;
}
inline int MPI_Cart_shift(MPI_Comm, int, int, int *src, int *dst) {
   *src = MPI_PROC_NULL;
   *dst = MPI_PROC_NULL;
   return 0;
}
inline int MPI_Issend(const void *, int, MPI_Datatype, int, int, MPI_Comm,
                      MPI_Request *) { return 0; }
inline int MPI_Probe(int, int, MPI_Comm, MPI_Status *) { return 0; }
inline int MPI_Get_count(const MPI_Status *, MPI_Datatype, int *c) {
   *c = 0;
   return 0;
}
inline int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm,
                    MPI_Status *) { return 0; }
inline int MPI_Allreduce(const void *, void *, int, MPI_Datatype, MPI_Op,
                         MPI_Comm) { return 0; }

#endif
