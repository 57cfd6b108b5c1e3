// Single-rank MPI stand-in used only to compile the PV2013 reference sources
// into the CPU checker (oracle/_ref).  TEST INFRASTRUCTURE ONLY.
//
// Every call behaves as MPI would with one rank on MPI_COMM_WORLD:
// broadcasts and halo send/receives are no-ops, Scatterv/Allreduce copy the
// local block, Cartesian topologies are 1x1x1 with MPI_PROC_NULL neighbours.
#pragma once
#include <cstddef>
#include <cstdint>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef std::ptrdiff_t MPI_Aint;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_PROC_NULL (-2)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_SUM 1

// Predefined datatypes; the value indexes a size table in mpi_stub.cpp.
#define MPI_DATATYPE_NULL 0
#define MPI_CHAR 1
#define MPI_SIGNED_CHAR 2
#define MPI_UNSIGNED_CHAR 3
#define MPI_SHORT 4
#define MPI_UNSIGNED_SHORT 5
#define MPI_INT 6
#define MPI_UNSIGNED 7
#define MPI_UINT 7
#define MPI_LONG 8
#define MPI_UNSIGNED_LONG 9
#define MPI_LONG_LONG 10
#define MPI_UNSIGNED_LONG_LONG 11
#define MPI_FLOAT 12
#define MPI_DOUBLE 13
#define MPI_LONG_DOUBLE 14
#define MPI_WCHAR 15
#define MPI_C_BOOL 16
#define MPI_C_COMPLEX 17
#define MPI_C_DOUBLE_COMPLEX 18
#define MPI_C_LONG_DOUBLE_COMPLEX 19

int MPI_Init(int* argc, char*** argv);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Comm_size(MPI_Comm comm, int* size);
int MPI_Comm_free(MPI_Comm* comm);
int MPI_Barrier(MPI_Comm comm);
int MPI_Bcast(void* buf, int count, MPI_Datatype t, int root, MPI_Comm comm);
int MPI_Scatterv(const void* sendbuf, const int* sendcounts, const int* displs, MPI_Datatype st, void* recvbuf,
                 int recvcount, MPI_Datatype rt, int root, MPI_Comm comm);
int MPI_Allreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype t, MPI_Op op, MPI_Comm comm);
int MPI_Send(const void* buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm);
int MPI_Recv(void* buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm comm, MPI_Status* st);
int MPI_Sendrecv(const void* sbuf, int scount, MPI_Datatype stype, int dest, int stag, void* rbuf, int rcount,
                 MPI_Datatype rtype, int src, int rtag, MPI_Comm comm, MPI_Status* st);
int MPI_Type_create_struct(int count, const int* blocklengths, const MPI_Aint* displs, const MPI_Datatype* types,
                           MPI_Datatype* newtype);
int MPI_Type_commit(MPI_Datatype* t);
int MPI_Dims_create(int nnodes, int ndims, int* dims);
int MPI_Cart_create(MPI_Comm old, int ndims, const int* dims, const int* periods, int reorder, MPI_Comm* cart);
int MPI_Cart_shift(MPI_Comm comm, int dir, int disp, int* src, int* dst);
int MPI_Cart_coords(MPI_Comm comm, int rank, int maxdims, int* coords);
int MPI_Cart_get(MPI_Comm comm, int maxdims, int* dims, int* periods, int* coords);
int MPI_Cart_rank(MPI_Comm comm, const int* coords, int* rank);
