/* Single-rank stand-in for the MPI interface used by the reference FEM solvers.
 * Oracle test infrastructure only: it lets the unmodified reference sources
 * compile and run as one rank with dims = (1,1,1).  With one rank every pair
 * communicator holds one process, so an allreduce is a copy. */
#pragma once
#include <cstring>
#include <chrono>
typedef int MPI_Comm;
typedef int MPI_Request;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Status;
#define MPI_COMM_WORLD 0
#define MPI_REQUEST_NULL 0
#define MPI_DOUBLE 8
#define MPI_SUM 1
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
inline int MPI_Init(int *, char ***) { return 0; }
inline int MPI_Finalize() { return 0; }
inline int MPI_Comm_size(MPI_Comm, int *s) { *s = 1; return 0; }
inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
inline int MPI_Comm_split(MPI_Comm, int, int, MPI_Comm *out) { *out = 0; return 0; }
inline int MPI_Comm_free(MPI_Comm *) { return 0; }
inline int MPI_Iallreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm, MPI_Request *q)
{ std::memmove(r, s, (size_t)n * (size_t)t); *q = 0; return 0; }
inline int MPI_Waitall(int, MPI_Request *, MPI_Status *) { return 0; }
inline double MPI_Wtime()
{ return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count(); }
