/*
 * Single-rank stand-in for the MPI-1 subset that PAMR/AMRD call.
 *
 * TEST INFRASTRUCTURE (oracle only): used to compile the reference's own C
 * sources (src/pamr.c, src/transfer.c, amrd/util.c, ...) into a CPU checker.
 * With one rank every collective is a copy and point-to-point traffic never
 * happens (transfer() only packs for rank != my_rank, src/transfer.c:1200).
 */
#ifndef ORACLE_SHIM_MPI_H
#define ORACLE_SHIM_MPI_H

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
/* datatype handles are their byte sizes, so sizeof(MPI_DOUBLE) stays legal */
#define MPI_CHAR 1
#define MPI_INT 4
#define MPI_DOUBLE 8
#define MPI_MAX 1
#define MPI_SUM 2
#define MPI_SUCCESS 0

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm);
int MPI_Allreduce(void *sbuf, void *rbuf, int count, MPI_Datatype type, MPI_Op op, MPI_Comm comm);
int MPI_Allgather(void *sbuf, int scount, MPI_Datatype stype, void *rbuf, int rcount,
                  MPI_Datatype rtype, MPI_Comm comm);
int MPI_Allgatherv(void *sbuf, int scount, MPI_Datatype stype, void *rbuf, int *rcounts,
                   int *displs, MPI_Datatype rtype, MPI_Comm comm);
int MPI_Isend(void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm,
              MPI_Request *req);
int MPI_Irecv(void *buf, int count, MPI_Datatype type, int src, int tag, MPI_Comm comm,
              MPI_Request *req);
int MPI_Waitall(int count, MPI_Request *reqs, MPI_Status *stats);

#endif
