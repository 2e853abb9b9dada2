/* Single-process stand-in for <mpi.h>: TEST INFRASTRUCTURE ONLY.
 *
 * Lets the reference's own basis, Hamiltonian-build and observable code,
 * which reaches MPI only through its MpiWrapper, compile into oracle/_ref as
 * one rank of a one-rank communicator.  Collectives over one rank copy the
 * send buffer to the receive buffer; point-to-point calls have no partner
 * with one rank and abort if reached.  A datatype's value is its size in
 * bytes, which is all a one-rank copy needs. */
#ifndef ORACLE_REF_STUB_MPI_H
#define ORACLE_REF_STUB_MPI_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Fint;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD ((MPI_Comm)0)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_SUCCESS 0
#define MPI_MAX_PROCESSOR_NAME 256
#define MPI_SUM ((MPI_Op)1)
#define MPI_MAX ((MPI_Op)2)
#define MPI_MIN ((MPI_Op)3)
#define MPI_LOR ((MPI_Op)4)
#define MPI_LAND ((MPI_Op)5)

#define MPI_CHAR ((MPI_Datatype)1)
#define MPI_UNSIGNED_CHAR ((MPI_Datatype)1)
#define MPI_C_BOOL ((MPI_Datatype)1)
#define MPI_INT8_T ((MPI_Datatype)1)
#define MPI_UINT8_T ((MPI_Datatype)1)
#define MPI_SHORT ((MPI_Datatype)2)
#define MPI_UNSIGNED_SHORT ((MPI_Datatype)2)
#define MPI_INT16_T ((MPI_Datatype)2)
#define MPI_UINT16_T ((MPI_Datatype)2)
#define MPI_INT ((MPI_Datatype)4)
#define MPI_UNSIGNED ((MPI_Datatype)4)
#define MPI_INT32_T ((MPI_Datatype)4)
#define MPI_UINT32_T ((MPI_Datatype)4)
#define MPI_FLOAT ((MPI_Datatype)4)
#define MPI_LONG ((MPI_Datatype)8)
#define MPI_UNSIGNED_LONG ((MPI_Datatype)8)
#define MPI_INT64_T ((MPI_Datatype)8)
#define MPI_UINT64_T ((MPI_Datatype)8)
#define MPI_DOUBLE ((MPI_Datatype)8)
#define MPI_DOUBLE_COMPLEX ((MPI_Datatype)16)

static inline int orstub_copy_(const void* s, void* r, int count, MPI_Datatype t)
{
    if (s && r && s != r && count > 0) memmove(r, s, (size_t)count * (size_t)t);
    return MPI_SUCCESS;
}
static inline int orstub_no_peer_(const char* what)
{
    fprintf(stderr, "one-rank MPI stand-in: %s has no peer\n", what);
    abort();
    return 1;
}

static inline int MPI_Init(int* argc, char*** argv) { (void)argc; (void)argv; return MPI_SUCCESS; }
static inline int MPI_Finalize(void) { return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm c, int* r) { (void)c; *r = 0; return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm c, int* s) { (void)c; *s = 1; return MPI_SUCCESS; }
static inline int MPI_Comm_split(MPI_Comm c, int color, int key, MPI_Comm* out)
{
    (void)color; (void)key; *out = c; return MPI_SUCCESS;
}
static inline MPI_Fint MPI_Comm_c2f(MPI_Comm c) { return (MPI_Fint)c; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return MPI_SUCCESS; }
static inline int MPI_Bcast(void* b, int n, MPI_Datatype t, int root, MPI_Comm c)
{
    (void)b; (void)n; (void)t; (void)root; (void)c; return MPI_SUCCESS;
}
static inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c)
{
    (void)op; (void)root; (void)c; return orstub_copy_(s, r, n, t);
}
static inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c)
{
    (void)op; (void)c; return orstub_copy_(s, r, n, t);
}
static inline int MPI_Gather(const void* s, int ns, MPI_Datatype ts, void* r, int nr, MPI_Datatype tr, int root,
                             MPI_Comm c)
{
    (void)nr; (void)tr; (void)root; (void)c; return orstub_copy_(s, r, ns, ts);
}
static inline int MPI_Allgather(const void* s, int ns, MPI_Datatype ts, void* r, int nr, MPI_Datatype tr, MPI_Comm c)
{
    (void)nr; (void)tr; (void)c; return orstub_copy_(s, r, ns, ts);
}
static inline int MPI_Scatter(const void* s, int ns, MPI_Datatype ts, void* r, int nr, MPI_Datatype tr, int root,
                              MPI_Comm c)
{
    (void)ns; (void)ts; (void)root; (void)c; return orstub_copy_(s, r, nr, tr);
}
static inline int MPI_Send(const void* b, int n, MPI_Datatype t, int dest, int tag, MPI_Comm c)
{
    (void)b; (void)n; (void)t; (void)dest; (void)tag; (void)c; return orstub_no_peer_("MPI_Send");
}
static inline int MPI_Recv(void* b, int n, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Status* st)
{
    (void)b; (void)n; (void)t; (void)src; (void)tag; (void)c; (void)st; return orstub_no_peer_("MPI_Recv");
}
static inline int MPI_Get_processor_name(char* name, int* len)
{
    strcpy(name, "oracle"); *len = 6; return MPI_SUCCESS;
}

#endif
