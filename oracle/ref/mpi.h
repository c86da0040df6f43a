/*
 * Single-rank stand-in for the MPI interface, written for this project so
 * that the unchanged CitcomCU sources compile and run as one process on a
 * machine without an MPI installation.
 *
 * Only the calls CitcomCU makes are provided.  With one rank every
 * collective is a copy of the send buffer into the receive buffer, point to
 * point traffic never happens (the reference only posts it between distinct
 * ranks), and communicator/group management is bookkeeping-free.
 *
 * A datatype is represented by its element size in bytes, evaluated where
 * the macro is expanded.  This matters for the FP64-promoted oracle build,
 * which compiles the reference with -Dfloat=double: there MPI_FLOAT expands
 * to sizeof(double), matching the promoted arrays it describes.
 *
 * This header is test infrastructure (it builds the oracle binary) and is
 * never part of the GPU library.
 */
#ifndef CITCOM_GB300_SINGLE_RANK_MPI_H
#define CITCOM_GB300_SINGLE_RANK_MPI_H

#include <string.h>
#include <time.h>

typedef int MPI_Comm;
typedef int MPI_Group;
typedef int MPI_Request;
typedef int MPI_Op;
typedef long MPI_Datatype;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD ((MPI_Comm)0)
#define MPI_SUCCESS 0
#define MPI_SUM ((MPI_Op)1)
#define MPI_MAX ((MPI_Op)2)
#define MPI_MIN ((MPI_Op)3)
#define MPI_INT ((MPI_Datatype)sizeof(int))
#define MPI_FLOAT ((MPI_Datatype)sizeof(float))
#define MPI_DOUBLE ((MPI_Datatype)sizeof(double))
#define MPI_CHAR ((MPI_Datatype)sizeof(char))
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)

static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }

static inline int MPI_Allreduce(const void *sb, void *rb, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c)
{
	(void)op; (void)c;
	if(sb != rb)
		memmove(rb, sb, (size_t)n * (size_t)t);
	return 0;
}

static inline int MPI_Bcast(void *b, int n, MPI_Datatype t, int root, MPI_Comm c)
{
	(void)b; (void)n; (void)t; (void)root; (void)c;
	return 0;
}

static inline int MPI_Comm_group(MPI_Comm c, MPI_Group *g) { (void)c; *g = 0; return 0; }
static inline int MPI_Group_incl(MPI_Group g, int n, int *r, MPI_Group *ng) { (void)g; (void)n; (void)r; *ng = 0; return 0; }
static inline int MPI_Comm_create(MPI_Comm c, MPI_Group g, MPI_Comm *nc) { (void)c; (void)g; *nc = 0; return 0; }
static inline int MPI_Comm_free(MPI_Comm *c) { (void)c; return 0; }
static inline int MPI_Group_free(MPI_Group *g) { (void)g; return 0; }

static inline int MPI_Isend(void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c, MPI_Request *r)
{ (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; *r = 0; return 0; }
static inline int MPI_Irecv(void *b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Request *r)
{ (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; *r = 0; return 0; }
static inline int MPI_Send(void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c)
{ (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; return 0; }
static inline int MPI_Recv(void *b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Status *st)
{ (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)st; return 0; }
static inline int MPI_Waitall(int n, MPI_Request *r, MPI_Status *st) { (void)n; (void)r; (void)st; return 0; }

static inline double MPI_Wtime(void)
{
	struct timespec ts;
	clock_gettime(CLOCK_MONOTONIC, &ts);
	return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

#endif
