/*
 * Minimal stand-in for <mpi.h>, used ONLY to compile the reference's
 * unmodified src/fluid.c and src/hash.c into the test oracle (oracle/_ref).
 * No MPI library exists on either build machine.  Every function declared
 * here is a no-op defined in oracle/ref_stubs.c; the oracle harness never
 * reaches the reference code paths that call them (it drives the step
 * functions directly, not start_simulation()).
 *
 * Only the names the reference's fluid.c / communication.h use are declared
 * (types, constants and the calls in fluid.c:51-364).
 */
#pragma once

typedef int MPI_Datatype;
typedef int MPI_Comm;
typedef int MPI_Group;
typedef int MPI_Request;
typedef long MPI_Aint;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; int count; } MPI_Status;

#define MPI_COMM_WORLD     ((MPI_Comm)0)
#define MPI_SHORT          ((MPI_Datatype)1)
#define MPI_FLOAT          ((MPI_Datatype)2)
#define MPI_INT            ((MPI_Datatype)3)
#define MPI_CHAR           ((MPI_Datatype)4)
#define MPI_REQUEST_NULL   ((MPI_Request)-1)
#define MPI_STATUS_IGNORE  ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Bcast(void *buf, int count, MPI_Datatype t, int root, MPI_Comm comm);
int MPI_Send(const void *buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm);
int MPI_Isend(const void *buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm,
              MPI_Request *req);
int MPI_Wait(MPI_Request *req, MPI_Status *status);
int MPI_Gatherv(const void *sbuf, int scount, MPI_Datatype st, void *rbuf, const int *rcounts,
                const int *displs, MPI_Datatype rt, int root, MPI_Comm comm);
int MPI_Scatterv(const void *sbuf, const int *scounts, const int *displs, MPI_Datatype st,
                 void *rbuf, int rcount, MPI_Datatype rt, int root, MPI_Comm comm);
