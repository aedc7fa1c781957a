// Build shim: the reference headers include <mpi.h> unconditionally. This single-rank
// stand-in declares only what they name; point-to-point and collective calls abort,
// since the contraction / SVD / QR path never reaches them. Test infrastructure only.
#pragma once
#include <cstdio>
#include <cstdlib>
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
struct MPI_Status { int MPI_SOURCE; int MPI_TAG; int MPI_ERROR; };
#define MPI_SUCCESS 0
#define MPI_MAX_ERROR_STRING 256
#define MPI_COMM_WORLD 0
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_IN_PLACE ((void*)1)
#define MPI_THREAD_MULTIPLE 3
enum { MPI_CHAR = 1, MPI_INT, MPI_UNSIGNED, MPI_UNSIGNED_LONG, MPI_UNSIGNED_LONG_LONG, MPI_DOUBLE,
       MPI_FLOAT, MPI_CXX_BOOL, MPI_CXX_DOUBLE_COMPLEX, MPI_CXX_FLOAT_COMPLEX };
enum { MPI_SUM = 1, MPI_MIN, MPI_MAX };
[[noreturn]] inline void qltg_mpi_shim_abort(const char* f) {
  std::fprintf(stderr, "single-rank MPI shim: %s is not available\n", f);
  std::abort();
}
inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
inline int MPI_Barrier(MPI_Comm) { return 0; }
inline int MPI_Error_string(int, char* s, int* l) { s[0] = 0; *l = 0; return 0; }
inline int MPI_Init_thread(int*, char***, int, int* p) { *p = MPI_THREAD_MULTIPLE; return 0; }
inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return 0; }
inline int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) { qltg_mpi_shim_abort("MPI_Send"); }
inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) { qltg_mpi_shim_abort("MPI_Recv"); }
inline int MPI_Allreduce(const void*, void*, int, MPI_Datatype, MPI_Op, MPI_Comm) { qltg_mpi_shim_abort("MPI_Allreduce"); }
inline int MPI_Reduce(const void*, void*, int, MPI_Datatype, MPI_Op, int, MPI_Comm) { qltg_mpi_shim_abort("MPI_Reduce"); }
inline int MPI_Allgather(const void*, int, MPI_Datatype, void*, int, MPI_Datatype, MPI_Comm) { qltg_mpi_shim_abort("MPI_Allgather"); }
inline int MPI_Allgatherv(const void*, int, MPI_Datatype, void*, const int*, const int*, MPI_Datatype, MPI_Comm) { qltg_mpi_shim_abort("MPI_Allgatherv"); }
inline int MPI_Gather(const void*, int, MPI_Datatype, void*, int, MPI_Datatype, int, MPI_Comm) { qltg_mpi_shim_abort("MPI_Gather"); }
