/*
 * Single-rank stand-in for the MPI interface, used only to compile the
 * reference library as a test oracle on machines without an MPI install.
 * Every call behaves as it would on a communicator of size 1: rank 0,
 * reductions copy input to output, point-to-point calls never match.
 * This header is test infrastructure; nothing in the shipped library uses it.
 */
#ifndef NSEM_ORACLE_MPI_STUB_H
#define NSEM_ORACLE_MPI_STUB_H

#include <string.h>

typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef int MPI_Comm;
typedef struct { int MPI_SOURCE; int MPI_TAG; } MPI_Status;

/* datatype handles are their element sizes in bytes */
#define MPI_INT       4
#define MPI_UNSIGNED  4
#define MPI_FLOAT     4
#define MPI_DOUBLE    8
#define MPI_MAX   1
#define MPI_MIN   2
#define MPI_SUM   3
#define MPI_PROD  4
#define MPI_COMM_WORLD 0
#define MPI_ANY_SOURCE (-1)
#define MPI_BOTTOM ((void*)0)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_MAX_PROCESSOR_NAME 64

static inline int MPI_Init(int*, char***) { return 0; }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int MPI_Get_processor_name(char* n, int* len) {
    strcpy(n, "localhost"); *len = 9; return 0;
}
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) { return 0; }
static inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) { return 0; }
static inline int MPI_Isend(const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request* r) { *r = 0; return 0; }
static inline int MPI_Irecv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request* r) { *r = 0; return 0; }
static inline int MPI_Waitall(int, MPI_Request*, MPI_Status*) { return 0; }
static inline int MPI_Iprobe(int, int, MPI_Comm, int* flag, MPI_Status*) { *flag = 0; return 0; }
static inline int MPI_Allreduce(const void* s, void* r, int count, MPI_Datatype t, MPI_Op, MPI_Comm) {
    if (s != r) memmove(r, s, (size_t)count * (size_t)t);
    return 0;
}
static inline int MPI_Reduce(const void* s, void* r, int count, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
    if (s != r) memmove(r, s, (size_t)count * (size_t)t);
    return 0;
}

#endif
