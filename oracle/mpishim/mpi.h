/*
 * Thread-MPI shim -- TEST INFRASTRUCTURE ONLY (part of the oracle).
 *
 * Lets the reference grid2grid library (kabicm/grid2grid, src/grid2grid/*.cpp)
 * compile and run unmodified with its P MPI ranks played by P threads of one
 * process. It declares exactly the MPI surface the reference's transform path
 * uses: MPI_Comm_rank/size (transform.cpp:131,154,173,193,
 * transformer.hpp:27), MPI_Irecv (transform.cpp:55-59), MPI_Isend
 * (transform.cpp:80-84), MPI_Waitany (transform.cpp:102-105), MPI_Waitall
 * (transform.cpp:120), plus Barrier/Wtime for drivers and the datatype
 * constants of mpi_type_wrapper.hpp:9-70.
 *
 * An MPI_Comm here is a per-rank handle: the thread playing rank r passes the
 * handle made for rank r. Sends are eager (the payload is copied into the
 * receiver's mailbox at MPI_Isend), receives complete in MPI_Wait*; messages
 * match on (source, tag) in FIFO order, which keeps MPI's non-overtaking rule.
 * Nothing in the product links this file.
 */
#ifndef G2G_THREAD_MPI_SHIM_H
#define G2G_THREAD_MPI_SHIM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct tmpi_comm_s *MPI_Comm;
typedef struct tmpi_request_s *MPI_Request;
typedef int MPI_Datatype;
typedef struct MPI_Status {
    int MPI_SOURCE;
    int MPI_TAG;
    int MPI_ERROR;
} MPI_Status;

#define MPI_SUCCESS 0
#define MPI_ERR_OTHER 15
#define MPI_REQUEST_NULL ((MPI_Request)0)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_UNDEFINED (-32766)

/* datatype codes; the byte size is tmpi_type_size(code) */
#define MPI_CHAR 1
#define MPI_UNSIGNED_CHAR 2
#define MPI_SHORT 3
#define MPI_INT 4
#define MPI_UINT32_T 5
#define MPI_UNSIGNED_LONG 6
#define MPI_UNSIGNED_LONG_LONG 7
#define MPI_FLOAT 8
#define MPI_DOUBLE 9
#define MPI_CXX_FLOAT_COMPLEX 10
#define MPI_CXX_DOUBLE_COMPLEX 11
#define MPI_CXX_BOOL 12

int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Isend(const void *buf, int count, MPI_Datatype type, int dest, int tag,
              MPI_Comm comm, MPI_Request *req);
int MPI_Irecv(void *buf, int count, MPI_Datatype type, int source, int tag,
              MPI_Comm comm, MPI_Request *req);
int MPI_Wait(MPI_Request *req, MPI_Status *status);
int MPI_Waitany(int count, MPI_Request reqs[], int *index, MPI_Status *status);
int MPI_Waitall(int count, MPI_Request reqs[], MPI_Status statuses[]);
int MPI_Barrier(MPI_Comm comm);
double MPI_Wtime(void);

/* ---- shim control (not MPI) ---- */
typedef struct tmpi_world_s tmpi_world;
/* A world of n_ranks thread-ranks; comm handle of rank r via tmpi_comm(). */
tmpi_world *tmpi_world_create(int n_ranks);
void tmpi_world_destroy(tmpi_world *w);
MPI_Comm tmpi_comm(tmpi_world *w, int rank);
size_t tmpi_type_size(MPI_Datatype type);
/* Bytes still sitting unreceived in all mailboxes (0 after a clean run). */
size_t tmpi_world_pending_bytes(tmpi_world *w);

#ifdef __cplusplus
}
#endif

#endif
