/*
 * mpi.h -- an in-process stand-in for the handful of MPI calls the
 * reference's halo exchange makes (lulesh-comm.cc, lulesh-init.cc), so that
 * those unchanged sources can run several ranks' Domains inside one process
 * (oracle/halo_ref_driver.cc).  Test infrastructure only: it is not MPI.
 *
 * Semantics: MPI_Comm_rank returns the rank the driver has made current;
 * MPI_Isend copies the message into an in-process mailbox at once; MPI_Irecv
 * records where the message goes; MPI_Wait takes the matching message (same
 * source, destination and tag) from the mailbox and copies it there.  A
 * driver therefore posts every rank's receives and sends before any rank
 * waits.  Anything unexpected (no matching message, a size mismatch) aborts
 * the process.
 */
#ifndef LG_MPI_STUB_H
#define LG_MPI_STUB_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Request;
typedef int MPI_Op;
typedef struct { int source, tag; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_FLOAT 4
#define MPI_DOUBLE 8
#define MPI_REQUEST_NULL (-1)
#define MPI_MIN 1
#define MPI_MAX 2
#define MPI_THREAD_SINGLE 0
#define MPI_THREAD_FUNNELED 1

int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Isend(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm,
              MPI_Request *req);
int MPI_Irecv(void *buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm comm,
              MPI_Request *req);
int MPI_Wait(MPI_Request *req, MPI_Status *status);
int MPI_Waitall(int n, MPI_Request *reqs, MPI_Status *statuses);
int MPI_Abort(MPI_Comm comm, int code);

/* Named by the reference's main program and time step, which the halo driver
 * links but never runs: each of these aborts if it is ever called. */
int MPI_Init(int *argc, char ***argv);
int MPI_Init_thread(int *argc, char ***argv, int required, int *provided);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Barrier(MPI_Comm comm);
int MPI_Finalize(void);
double MPI_Wtime(void);
int MPI_Allreduce(const void *in, void *out, int count, MPI_Datatype type, MPI_Op op,
                  MPI_Comm comm);
int MPI_Reduce(const void *in, void *out, int count, MPI_Datatype type, MPI_Op op, int root,
               MPI_Comm comm);

#ifdef __cplusplus
}
#endif

#endif
