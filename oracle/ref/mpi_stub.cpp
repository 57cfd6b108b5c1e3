// Single-rank MPI stand-in for compiling the PV2013 reference sources into the
// CPU checker.  TEST INFRASTRUCTURE ONLY.  See mpi.h.
#include "mpi.h"
#include <cstring>
#include <vector>

namespace {
std::vector<std::size_t>& type_sizes() {
    static std::vector<std::size_t> t = {0, 1, 1, 1, 2, 2, 4, 4, 8, 8, 8, 8, 4, 8, 16, 4, 1, 8, 16, 32};
    return t;
}
std::size_t tsize(MPI_Datatype t) { return type_sizes().at((std::size_t)t); }
}  // namespace

int MPI_Init(int*, char***) { return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm, int* rank) { *rank = 0; return MPI_SUCCESS; }
int MPI_Comm_size(MPI_Comm, int* size) { *size = 1; return MPI_SUCCESS; }
int MPI_Comm_free(MPI_Comm*) { return MPI_SUCCESS; }
int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }

int MPI_Scatterv(const void* sendbuf, const int* sendcounts, const int* displs, MPI_Datatype st, void* recvbuf, int,
                 MPI_Datatype, int, MPI_Comm) {
    std::size_t sz = tsize(st);
    if (sendcounts[0] > 0 && recvbuf != sendbuf)
        std::memcpy(recvbuf, (const char*)sendbuf + (std::size_t)displs[0] * sz, (std::size_t)sendcounts[0] * sz);
    return MPI_SUCCESS;
}

int MPI_Allreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype t, MPI_Op, MPI_Comm) {
    if (recvbuf != sendbuf) std::memcpy(recvbuf, sendbuf, (std::size_t)count * tsize(t));
    return MPI_SUCCESS;
}

int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) { return MPI_SUCCESS; }
int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) { return MPI_SUCCESS; }
int MPI_Sendrecv(const void*, int, MPI_Datatype, int, int, void*, int, MPI_Datatype, int, int, MPI_Comm,
                 MPI_Status*) {
    return MPI_SUCCESS;
}

// A struct type's extent is taken as the end of its last block.
int MPI_Type_create_struct(int count, const int* bl, const MPI_Aint* displs, const MPI_Datatype* types,
                           MPI_Datatype* newtype) {
    std::size_t end = 0;
    for (int i = 0; i < count; ++i) {
        std::size_t e = (std::size_t)displs[i] + (std::size_t)bl[i] * tsize(types[i]);
        if (e > end) end = e;
    }
    type_sizes().push_back(end);
    *newtype = (MPI_Datatype)(type_sizes().size() - 1);
    return MPI_SUCCESS;
}
int MPI_Type_commit(MPI_Datatype*) { return MPI_SUCCESS; }

int MPI_Dims_create(int, int ndims, int* dims) {
    for (int i = 0; i < ndims; ++i) if (dims[i] == 0) dims[i] = 1;
    return MPI_SUCCESS;
}
int MPI_Cart_create(MPI_Comm, int, const int*, const int*, int, MPI_Comm* cart) { *cart = 0; return MPI_SUCCESS; }
int MPI_Cart_shift(MPI_Comm, int, int, int* src, int* dst) {
    *src = MPI_PROC_NULL; *dst = MPI_PROC_NULL;
    return MPI_SUCCESS;
}
int MPI_Cart_coords(MPI_Comm, int, int maxdims, int* coords) {
    for (int i = 0; i < maxdims; ++i) coords[i] = 0;
    return MPI_SUCCESS;
}
int MPI_Cart_get(MPI_Comm, int maxdims, int* dims, int* periods, int* coords) {
    for (int i = 0; i < maxdims; ++i) { dims[i] = 1; periods[i] = 0; coords[i] = 0; }
    return MPI_SUCCESS;
}
int MPI_Cart_rank(MPI_Comm, const int*, int* rank) { *rank = 0; return MPI_SUCCESS; }
