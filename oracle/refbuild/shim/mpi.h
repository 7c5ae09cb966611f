/*
 * Single-rank stand-in for <mpi.h>, used ONLY to compile the unmodified reference
 * sources into oracle/_ref/ so that they can serve as a checker (test infrastructure,
 * never part of the product).
 *
 * Semantics: MPI_COMM_WORLD has exactly one rank (rank 0, size 1). Every collective is
 * therefore a local copy (send buffer -> receive buffer, honouring MPI_IN_PLACE and the
 * v-variants' displacements) or a no-op. A datatype handle is its extent in bytes, so
 * derived types built with MPI_Type_create_struct / vector / contiguous compute their
 * extent from the arguments. Point-to-point calls only occur in the reference when a
 * group has more than one rank, which cannot happen here; they abort if reached.
 *
 * Written from the MPI-3.1 standard's definitions of these calls; no MPI implementation
 * source was consulted.
 */
#ifndef CAC_ORACLE_SINGLE_RANK_MPI_H
#define CAC_ORACLE_SINGLE_RANK_MPI_H

#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#include <stddef.h>
#include <stdint.h>

typedef long MPI_Datatype; /* extent in bytes */
typedef int MPI_Comm;
typedef int MPI_Op;
typedef ptrdiff_t MPI_Aint;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_SUCCESS 0
#define MPI_COMM_WORLD ((MPI_Comm)1)
#define MPI_COMM_NULL ((MPI_Comm)0)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_IN_PLACE ((void *)1)
#define MPI_BSEND_OVERHEAD 96

#define MPI_CHAR ((MPI_Datatype)sizeof(char))
#define MPI_INT ((MPI_Datatype)sizeof(int))
#define MPI_UNSIGNED ((MPI_Datatype)sizeof(unsigned))
#define MPI_LONG ((MPI_Datatype)sizeof(long))
#define MPI_UNSIGNED_LONG ((MPI_Datatype)sizeof(unsigned long))
#define MPI_UNSIGNED_LONG_LONG ((MPI_Datatype)sizeof(unsigned long long))
#define MPI_LONG_LONG ((MPI_Datatype)sizeof(long long))
#define MPI_DOUBLE ((MPI_Datatype)sizeof(double))
#define MPI_FLOAT ((MPI_Datatype)sizeof(float))
#define MPI_UINT32_T ((MPI_Datatype)sizeof(uint32_t))
#define MPI_UINT64_T ((MPI_Datatype)sizeof(uint64_t))
#define MPI_2INT ((MPI_Datatype)(2 * sizeof(int)))

#define MPI_MAX ((MPI_Op)1)
#define MPI_MIN ((MPI_Op)2)
#define MPI_SUM ((MPI_Op)3)

static inline void cac_mpi_shim_unreachable(const char *what) {
    fprintf(stderr, "single-rank MPI stand-in: %s needs more than one rank\n", what);
    abort();
}

static inline void cac_mpi_copy(const void *send, void *recv, size_t bytes) {
    if (send == MPI_IN_PLACE || send == recv || bytes == 0 || recv == NULL || send == NULL) return;
    memmove(recv, send, bytes);
}

static inline int MPI_Init(int *, char ***) { return MPI_SUCCESS; }
static inline int MPI_Finalize(void) { return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm, int *rank) { *rank = 0; return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm, int *size) { *size = 1; return MPI_SUCCESS; }
static inline int MPI_Comm_split(MPI_Comm comm, int, int, MPI_Comm *out) { *out = comm; return MPI_SUCCESS; }
static inline int MPI_Comm_free(MPI_Comm *c) { *c = MPI_COMM_NULL; return MPI_SUCCESS; }
static inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }

static inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
    cac_mpi_copy(s, r, (size_t)n * (size_t)t); return MPI_SUCCESS;
}
static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
    cac_mpi_copy(s, r, (size_t)n * (size_t)t); return MPI_SUCCESS;
}
static inline int MPI_Scan(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
    cac_mpi_copy(s, r, (size_t)n * (size_t)t); return MPI_SUCCESS;
}
static inline int MPI_Gather(const void *s, int sn, MPI_Datatype st, void *r, int, MPI_Datatype, int, MPI_Comm) {
    cac_mpi_copy(s, r, (size_t)sn * (size_t)st); return MPI_SUCCESS;
}
static inline int MPI_Allgather(const void *s, int sn, MPI_Datatype st, void *r, int, MPI_Datatype, MPI_Comm) {
    cac_mpi_copy(s, r, (size_t)sn * (size_t)st); return MPI_SUCCESS;
}
static inline int MPI_Scatter(const void *s, int sn, MPI_Datatype st, void *r, int, MPI_Datatype, int, MPI_Comm) {
    if (r == MPI_IN_PLACE) return MPI_SUCCESS;
    cac_mpi_copy(s, r, (size_t)sn * (size_t)st); return MPI_SUCCESS;
}
static inline int MPI_Gatherv(const void *s, int sn, MPI_Datatype st, void *r, const int *, const int *displs,
                              MPI_Datatype rt, int, MPI_Comm) {
    if (r == NULL) return MPI_SUCCESS;
    cac_mpi_copy(s, (char *)r + (size_t)displs[0] * (size_t)rt, (size_t)sn * (size_t)st); return MPI_SUCCESS;
}
static inline int MPI_Allgatherv(const void *s, int sn, MPI_Datatype st, void *r, const int *, const int *displs,
                                 MPI_Datatype rt, MPI_Comm) {
    cac_mpi_copy(s, (char *)r + (size_t)displs[0] * (size_t)rt, (size_t)sn * (size_t)st); return MPI_SUCCESS;
}
static inline int MPI_Alltoall(const void *s, int sn, MPI_Datatype st, void *r, int, MPI_Datatype, MPI_Comm) {
    cac_mpi_copy(s, r, (size_t)sn * (size_t)st); return MPI_SUCCESS;
}
static inline int MPI_Alltoallv(const void *s, const int *sc, const int *sd, MPI_Datatype st, void *r, const int *,
                                const int *rd, MPI_Datatype rt, MPI_Comm) {
    cac_mpi_copy((const char *)s + (size_t)sd[0] * (size_t)st, (char *)r + (size_t)rd[0] * (size_t)rt,
                 (size_t)sc[0] * (size_t)st);
    return MPI_SUCCESS;
}

static inline int MPI_Isend(const void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) {
    cac_mpi_shim_unreachable("MPI_Isend"); return 1;
}
static inline int MPI_Ibsend(const void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) {
    cac_mpi_shim_unreachable("MPI_Ibsend"); return 1;
}
static inline int MPI_Irecv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) {
    cac_mpi_shim_unreachable("MPI_Irecv"); return 1;
}
static inline int MPI_Wait(MPI_Request *, MPI_Status *) { return MPI_SUCCESS; }
static inline int MPI_Buffer_attach(void *, int) { return MPI_SUCCESS; }
static inline int MPI_Buffer_detach(void *b, int *n) { *(void **)b = NULL; *n = 0; return MPI_SUCCESS; }
static inline int MPI_Pack_size(int n, MPI_Datatype t, MPI_Comm, int *size) { *size = (int)(n * t); return MPI_SUCCESS; }

static inline int MPI_Type_create_struct(int count, const int *lens, const MPI_Aint *offs, const MPI_Datatype *types,
                                         MPI_Datatype *out) {
    MPI_Aint extent = 0, align = 1;
    for (int i = 0; i < count; i++) {
        MPI_Aint end = offs[i] + (MPI_Aint)lens[i] * (MPI_Aint)types[i];
        if (end > extent) extent = end;
        if ((MPI_Aint)types[i] > align && types[i] <= 8) align = types[i];
    }
    extent = (extent + align - 1) / align * align;
    *out = (MPI_Datatype)extent;
    return MPI_SUCCESS;
}
static inline int MPI_Type_contiguous(int n, MPI_Datatype t, MPI_Datatype *out) { *out = n * t; return MPI_SUCCESS; }
static inline int MPI_Type_vector(int count, int blocklen, int stride, MPI_Datatype t, MPI_Datatype *out) {
    *out = (MPI_Datatype)((count > 0 ? (count - 1) * stride + blocklen : 0) * t); return MPI_SUCCESS;
}
static inline int MPI_Type_create_hvector(int count, int blocklen, MPI_Aint stride, MPI_Datatype t, MPI_Datatype *out) {
    *out = (MPI_Datatype)(count > 0 ? (count - 1) * stride + blocklen * t : 0); return MPI_SUCCESS;
}
static inline int MPI_Type_create_resized(MPI_Datatype, MPI_Aint, MPI_Aint extent, MPI_Datatype *out) {
    *out = (MPI_Datatype)extent; return MPI_SUCCESS;
}
static inline int MPI_Type_get_extent(MPI_Datatype t, MPI_Aint *lb, MPI_Aint *extent) { *lb = 0; *extent = t; return MPI_SUCCESS; }
static inline int MPI_Type_size(MPI_Datatype t, int *size) { *size = (int)t; return MPI_SUCCESS; }
static inline int MPI_Type_commit(MPI_Datatype *) { return MPI_SUCCESS; }
static inline int MPI_Type_free(MPI_Datatype *) { return MPI_SUCCESS; }

#endif
