/* Single-rank MPI stand-in used only to compile the unmodified reference
 * solver (aither) as a CPU oracle.  Every communicator has exactly one rank
 * (rank 0), so collectives reduce to local copies and point-to-point
 * messages can never be needed; those entry points abort loudly.
 *
 * This header declares just the subset of MPI-3 that the reference calls
 * (collected with grep over its src/ and include/ trees).  It is test
 * infrastructure: nothing in the product library includes it. */
#ifndef ORACLE_SINGLE_RANK_MPI_H
#define ORACLE_SINGLE_RANK_MPI_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef ptrdiff_t MPI_Aint;
typedef struct {
  int MPI_SOURCE;
  int MPI_TAG;
  int MPI_ERROR;
  int count_bytes;
} MPI_Status;
typedef void MPI_User_function(void *invec, void *inoutvec, int *len,
                               MPI_Datatype *datatype);

#define MPI_SUCCESS 0
#define MPI_COMM_WORLD ((MPI_Comm)1)

/* predefined datatypes: handle values index a size table in the shim */
#define MPI_DATATYPE_NULL ((MPI_Datatype)0)
#define MPI_INT ((MPI_Datatype)1)
#define MPI_DOUBLE ((MPI_Datatype)2)
#define MPI_CHAR ((MPI_Datatype)3)
#define MPI_PACKED ((MPI_Datatype)4)
#define MPI_C_BOOL ((MPI_Datatype)5)
#define MPI_CXX_BOOL ((MPI_Datatype)6)

#define MPI_SUM ((MPI_Op)1)
#define MPI_IN_PLACE ((void *)1)

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Get_version(int *version, int *subversion);
int MPI_Barrier(MPI_Comm comm);
int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm);
int MPI_Reduce(const void *sendbuf, void *recvbuf, int count,
               MPI_Datatype type, MPI_Op op, int root, MPI_Comm comm);
int MPI_Scatter(const void *sendbuf, int sendcount, MPI_Datatype sendtype,
                void *recvbuf, int recvcount, MPI_Datatype recvtype, int root,
                MPI_Comm comm);
int MPI_Pack(const void *inbuf, int incount, MPI_Datatype type, void *outbuf,
             int outsize, int *position, MPI_Comm comm);
int MPI_Unpack(const void *inbuf, int insize, int *position, void *outbuf,
               int outcount, MPI_Datatype type, MPI_Comm comm);
int MPI_Pack_size(int incount, MPI_Datatype type, MPI_Comm comm, int *size);
int MPI_Send(const void *buf, int count, MPI_Datatype type, int dest, int tag,
             MPI_Comm comm);
int MPI_Recv(void *buf, int count, MPI_Datatype type, int source, int tag,
             MPI_Comm comm, MPI_Status *status);
int MPI_Probe(int source, int tag, MPI_Comm comm, MPI_Status *status);
int MPI_Get_count(const MPI_Status *status, MPI_Datatype type, int *count);
int MPI_Sendrecv_replace(void *buf, int count, MPI_Datatype type, int dest,
                         int sendtag, int source, int recvtag, MPI_Comm comm,
                         MPI_Status *status);
int MPI_Get_address(const void *location, MPI_Aint *address);
int MPI_Type_contiguous(int count, MPI_Datatype oldtype, MPI_Datatype *newtype);
int MPI_Type_create_struct(int count, const int blocklengths[],
                           const MPI_Aint displacements[],
                           const MPI_Datatype types[], MPI_Datatype *newtype);
int MPI_Type_create_resized(MPI_Datatype oldtype, MPI_Aint lb, MPI_Aint extent,
                            MPI_Datatype *newtype);
int MPI_Type_get_extent(MPI_Datatype type, MPI_Aint *lb, MPI_Aint *extent);
int MPI_Type_commit(MPI_Datatype *type);
int MPI_Type_free(MPI_Datatype *type);
int MPI_Op_create(MPI_User_function *fn, int commute, MPI_Op *op);
int MPI_Op_free(MPI_Op *op);

#ifdef __cplusplus
}
#endif

#endif
