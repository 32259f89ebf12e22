/* Single-process stand-in for the MPI calls the reference's CPU sources name
 * (oracle build only). Point-to-point calls are no-ops; a reduction over one
 * rank copies its input. */
#pragma once
#include <string.h>
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Info;
typedef int MPI_Request;
typedef int MPI_Op;
typedef long long MPI_Offset;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
#define MPI_SUCCESS 0
#define MPI_COMM_WORLD 0
#define MPI_INFO_NULL 0
#define MPI_DOUBLE 8
#define MPI_FLOAT 4
#define MPI_INT 40
#define MPI_LONG 41
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_MAX_LIBRARY_VERSION_STRING 64
static inline int MPI_Init(int*, char***) { return 0; }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
static inline int MPI_Comm_split(MPI_Comm c, int, int, MPI_Comm* o) { *o = c; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Isend(const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request* r) { *r = 0; return 0; }
static inline int MPI_Irecv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request* r) { *r = 0; return 0; }
static inline int MPI_Wait(MPI_Request*, MPI_Status*) { return 0; }
static inline int MPI_Waitall(int, MPI_Request*, MPI_Status*) { return 0; }
static inline int MPI_Get_library_version(char* v, int* l) { strcpy(v, "stub"); *l = 4; return 0; }
static inline int MPI_Type_size(MPI_Datatype t, int* s) { *s = (t == MPI_DOUBLE) ? 8 : 4; return 0; }
static inline int MPI_Reduce(const void* in, void* out, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
    int s; MPI_Type_size(t, &s); memcpy(out, in, (size_t)n * (size_t)s); return 0; }
static inline int MPI_Allreduce(const void* in, void* out, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
    int s; MPI_Type_size(t, &s); memcpy(out, in, (size_t)n * (size_t)s); return 0; }
static inline int MPI_Allgather(const void* in, int n, MPI_Datatype t, void* out, int, MPI_Datatype, MPI_Comm) {
    int s; MPI_Type_size(t, &s); memcpy(out, in, (size_t)n * (size_t)s); return 0; }
static inline int MPI_Type_free(MPI_Datatype*) { return 0; }
static inline int MPI_Type_commit(MPI_Datatype*) { return 0; }
static inline int MPI_Type_indexed(int, const int*, const int*, MPI_Datatype o, MPI_Datatype* n) { *n = o; return 0; }
