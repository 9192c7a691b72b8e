/*
 * TEST INFRASTRUCTURE: a minimal MPI for running the reference solver's own MPI build
 * (SIMPLE_TS_MPI.cpp with COMPILE_MPI) on the host cores of one machine, where no MPI is
 * installed.  It provides exactly the calls the reference makes (MPI_Init, Comm_rank/size,
 * Get_version, Barrier, Isend, Irecv, Wait, Send/Ssend, Recv, Reduce, Gather,
 * Type_vector/commit/free, Finalize) between processes started by mpishim_run, with the messages
 * in shared memory.  Used only to time the reference beside the GB300 library; never linked into
 * the library.
 */
#ifndef STS_MPISHIM_MPI_H
#define STS_MPISHIM_MPI_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct {
  int MPI_SOURCE, MPI_TAG, MPI_ERROR;
  int count_bytes;
} MPI_Status;

#define MPI_SUCCESS 0
#define MPI_COMM_WORLD 0
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_CHAR 1
#define MPI_INT 2
#define MPI_UNSIGNED 3
#define MPI_FLOAT 4
#define MPI_DOUBLE 5
#define MPI_LONG 6
#define MPI_UNSIGNED_LONG 7
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3

int MPI_Init(int* argc, char*** argv);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Comm_size(MPI_Comm comm, int* size);
int MPI_Get_version(int* version, int* subversion);
int MPI_Barrier(MPI_Comm comm);
int MPI_Isend(const void* buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm, MPI_Request* req);
int MPI_Irecv(void* buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm comm, MPI_Request* req);
int MPI_Wait(MPI_Request* req, MPI_Status* status);
int MPI_Send(const void* buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm);
int MPI_Ssend(const void* buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm);
int MPI_Recv(void* buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm comm, MPI_Status* status);
int MPI_Reduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype type, MPI_Op op, int root, MPI_Comm comm);
int MPI_Gather(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, int recvcount,
               MPI_Datatype recvtype, int root, MPI_Comm comm);
int MPI_Type_vector(int count, int blocklength, int stride, MPI_Datatype oldtype, MPI_Datatype* newtype);
int MPI_Type_commit(MPI_Datatype* type);
int MPI_Type_free(MPI_Datatype* type);

#ifdef __cplusplus
}
#endif

#endif
