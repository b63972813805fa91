/*
 * Single-process stand-in for the MPI interface, used only to compile the
 * reference's own hot-path translation units into the CPU checker
 * (oracle/_ref).  There is no MPI on this machine; with one rank every
 * collective is a local copy and point-to-point traffic never happens.
 *
 * Datatype handles encode their size in bytes, so collectives can copy
 * `count * size` bytes without a type table.  Point-to-point calls abort:
 * with a communicator of size one the reference never issues them.
 */
#ifndef SEMO_ORACLE_MPI_SHIM_H
#define SEMO_ORACLE_MPI_SHIM_H

#include <cstdio>
#include <cstdlib>
#include <cstring>

#define MPI_VERSION 3
#define MPI_SUBVERSION 1

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
struct MPI_Status { int MPI_SOURCE; int MPI_TAG; int MPI_ERROR; };

#define MPI_COMM_NULL 0
#define MPI_COMM_WORLD 1
#define MPI_UNDEFINED (-32766)
#define MPI_SUCCESS 0
#define MPI_THREAD_MULTIPLE 3
#define MPI_REQUEST_NULL 0

#define MPI_CHAR ((MPI_Datatype)1)
#define MPI_BYTE ((MPI_Datatype)1)
#define MPI_C_BOOL ((MPI_Datatype)sizeof(bool))
#define MPI_INT ((MPI_Datatype)4)
#define MPI_INTEGER ((MPI_Datatype)4)
#define MPI_UNSIGNED ((MPI_Datatype)4)
#define MPI_FLOAT ((MPI_Datatype)4)
#define MPI_DOUBLE ((MPI_Datatype)8)
#define MPI_LONG_LONG_INT ((MPI_Datatype)8)
#define MPI_UNSIGNED_LONG_LONG ((MPI_Datatype)8)
#define MPI_LONG_DOUBLE ((MPI_Datatype)sizeof(long double))

#define MPI_SUM 1
#define MPI_MIN 2
#define MPI_MAX 3
#define MPI_PROD 4

#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_IN_PLACE ((void*)1)

inline void semo_mpi_copy(const void* s, void* r, int count, MPI_Datatype t) {
    if (s == MPI_IN_PLACE || s == r || count <= 0) return;
    std::memmove(r, s, (size_t)count * (size_t)t);
}
inline void semo_mpi_p2p(const char* what) {
    std::fprintf(stderr, "mpi shim: %s called with one rank\n", what);
    std::abort();
}

inline int MPI_Init(int*, char***) { return 0; }
inline int MPI_Init_thread(int*, char***, int, int* provided) { if (provided) *provided = MPI_THREAD_MULTIPLE; return 0; }
inline int MPI_Finalize() { return 0; }
inline int MPI_Abort(MPI_Comm, int code) { std::exit(code); return 0; }
inline int MPI_Barrier(MPI_Comm) { return 0; }
inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
inline int MPI_Comm_split(MPI_Comm, int color, int, MPI_Comm* out) {
    *out = (color == MPI_UNDEFINED) ? MPI_COMM_NULL : MPI_COMM_WORLD; return 0;
}
inline int MPI_Comm_free(MPI_Comm* c) { *c = MPI_COMM_NULL; return 0; }
inline int MPI_Type_contiguous(int n, MPI_Datatype old, MPI_Datatype* out) { *out = n * old; return 0; }
inline int MPI_Type_commit(MPI_Datatype*) { return 0; }
inline int MPI_Type_free(MPI_Datatype*) { return 0; }

inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) { semo_mpi_copy(s, r, n, t); return 0; }
inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) { semo_mpi_copy(s, r, n, t); return 0; }
inline int MPI_Exscan(const void*, void*, int, MPI_Datatype, MPI_Op, MPI_Comm) { return 0; }
inline int MPI_Scan(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) { semo_mpi_copy(s, r, n, t); return 0; }
inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return 0; }
inline int MPI_Allgather(const void* s, int sn, MPI_Datatype st, void* r, int, MPI_Datatype, MPI_Comm) { semo_mpi_copy(s, r, sn, st); return 0; }
inline int MPI_Gather(const void* s, int sn, MPI_Datatype st, void* r, int, MPI_Datatype, int, MPI_Comm) { semo_mpi_copy(s, r, sn, st); return 0; }
inline int MPI_Scatter(const void* s, int sn, MPI_Datatype st, void* r, int, MPI_Datatype, int, MPI_Comm) { semo_mpi_copy(s, r, sn, st); return 0; }
inline int MPI_Allgatherv(const void* s, int sn, MPI_Datatype st, void* r, const int*, const int* displs, MPI_Datatype rt, MPI_Comm) {
    semo_mpi_copy(s, (char*)r + (size_t)displs[0] * (size_t)rt, sn, st); return 0;
}
inline int MPI_Gatherv(const void* s, int sn, MPI_Datatype st, void* r, const int*, const int* displs, MPI_Datatype rt, int, MPI_Comm) {
    semo_mpi_copy(s, (char*)r + (size_t)displs[0] * (size_t)rt, sn, st); return 0;
}
inline int MPI_Scatterv(const void* s, const int* counts, const int* displs, MPI_Datatype st, void* r, int, MPI_Datatype, int, MPI_Comm) {
    semo_mpi_copy((const char*)s + (size_t)displs[0] * (size_t)st, r, counts[0], st); return 0;
}
inline int MPI_Alltoall(const void* s, int sn, MPI_Datatype st, void* r, int, MPI_Datatype, MPI_Comm) { semo_mpi_copy(s, r, sn, st); return 0; }
inline int MPI_Alltoallv(const void* s, const int* sc, const int* sd, MPI_Datatype st, void* r, const int*, const int* rd, MPI_Datatype rt, MPI_Comm) {
    semo_mpi_copy((const char*)s + (size_t)sd[0] * (size_t)st, (char*)r + (size_t)rd[0] * (size_t)rt, sc[0], st); return 0;
}
inline int MPI_Ialltoall(const void* s, int sn, MPI_Datatype st, void* r, int, MPI_Datatype, MPI_Comm, MPI_Request* q) {
    semo_mpi_copy(s, r, sn, st); *q = MPI_REQUEST_NULL; return 0;
}

inline int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) { semo_mpi_p2p("MPI_Send"); return 0; }
inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) { semo_mpi_p2p("MPI_Recv"); return 0; }
inline int MPI_Isend(const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*) { semo_mpi_p2p("MPI_Isend"); return 0; }
inline int MPI_Irecv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*) { semo_mpi_p2p("MPI_Irecv"); return 0; }
inline int MPI_Wait(MPI_Request*, MPI_Status*) { return 0; }
inline int MPI_Waitall(int, MPI_Request*, MPI_Status*) { return 0; }

/* the C++ binding subset the reference uses: COMM_WORLD rank/size, Init, Status */
namespace MPI {
struct Intracomm_ {
    int Get_rank() const { return 0; }
    int Get_size() const { return 1; }
};
static const Intracomm_ COMM_WORLD = {};
inline void Init() {}
inline void Init(int&, char**&) {}
inline void Finalize() {}
typedef ::MPI_Status Status;
}

#endif
