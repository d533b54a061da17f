/*
 * mpi.h -- project-written stand-in for the subset of MPI that the reference
 * calls (its collective sites are sanepic.cc:257-259, 485-505, 602-621,
 * 887-894, 1120-1125, 1283-1307, 1404-1407, 1448, 1495, 1544-1552,
 * 1753-1758, 2353-2359).  This image has no MPI; the shim runs the ranks as
 * forked processes of one executable and performs collectives through a
 * shared anonymous mapping, combining contributions in rank order.
 *
 * The number of ranks comes from the environment variable SHIM_MPI_NP
 * (default 2; the reference needs at least 2, sanepic.cc:625).  Only
 * communicators that contain every rank are supported, which is all the
 * reference creates while nsubm == 1 (sanepic.cc:589).
 * TEST INFRASTRUCTURE ONLY.
 */
#ifndef SANEPIC_SHIM_MPI_H
#define SANEPIC_SHIM_MPI_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Group;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct {
  int MPI_SOURCE;
  int MPI_TAG;
  int MPI_ERROR;
} MPI_Status;

#define MPI_SUCCESS 0
#define MPI_COMM_WORLD ((MPI_Comm)0)
#define MPI_COMM_NULL ((MPI_Comm)-1)
#define MPI_GROUP_NULL ((MPI_Group)-1)
#define MPI_INT ((MPI_Datatype)1)
#define MPI_LONG ((MPI_Datatype)2)
#define MPI_DOUBLE ((MPI_Datatype)3)
#define MPI_SUM ((MPI_Op)1)

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Abort(MPI_Comm comm, int errorcode);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Barrier(MPI_Comm comm);
int MPI_Reduce(const void *sendbuf, void *recvbuf, int count,
               MPI_Datatype datatype, MPI_Op op, int root, MPI_Comm comm);
int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count,
                  MPI_Datatype datatype, MPI_Op op, MPI_Comm comm);
int MPI_Bcast(void *buffer, int count, MPI_Datatype datatype, int root,
              MPI_Comm comm);
int MPI_Comm_group(MPI_Comm comm, MPI_Group *group);
int MPI_Group_range_incl(MPI_Group group, int n, int ranges[][3],
                         MPI_Group *newgroup);
int MPI_Comm_create(MPI_Comm comm, MPI_Group group, MPI_Comm *newcomm);
int MPI_Comm_free(MPI_Comm *comm);
int MPI_Group_free(MPI_Group *group);
int MPI_Send(const void *buf, int count, MPI_Datatype datatype, int dest,
             int tag, MPI_Comm comm);
int MPI_Recv(void *buf, int count, MPI_Datatype datatype, int source, int tag,
             MPI_Comm comm, MPI_Status *status);

#ifdef __cplusplus
}
#endif
#endif
