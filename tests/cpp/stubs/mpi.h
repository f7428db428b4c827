/* A single-rank stand-in for the MPI calls the reference's 2D / 3D GPU
 * drivers make (bin/test_nufi_gpu_2d.cpp, bin/test_nufi_gpu_3d.cpp through
 * nufi/mpi.hpp), so that tests/test_cpp_api.py can compile and link them
 * unchanged where MPI is absent: one rank, reductions and gathers copy. */
#ifndef NUFI_TEST_STUB_MPI_H
#define NUFI_TEST_STUB_MPI_H

#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;

#define MPI_SUCCESS 0
#define MPI_MAX_ERROR_STRING 512
#define MPI_COMM_WORLD ((MPI_Comm)0)
#define MPI_FLOAT ((MPI_Datatype)1)
#define MPI_DOUBLE ((MPI_Datatype)2)
#define MPI_SUM ((MPI_Op)1)
#define MPI_IN_PLACE ((void *)1)

static inline size_t nufi_stub_mpi_size(MPI_Datatype t) { return t == MPI_FLOAT ? 4 : 8; }
static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return MPI_SUCCESS; }
static inline int MPI_Finalize(void) { return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm comm, int *size) { (void)comm; *size = 1; return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm comm, int *rank) { (void)comm; *rank = 0; return MPI_SUCCESS; }
static inline int MPI_Error_string(int errorcode, char *string, int *resultlen)
{
    (void)errorcode;
    string[0] = 0;
    *resultlen = 0;
    return MPI_SUCCESS;
}
static inline int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype datatype, MPI_Op op,
                                MPI_Comm comm)
{
    (void)op; (void)comm;
    if (sendbuf != MPI_IN_PLACE) memcpy(recvbuf, sendbuf, (size_t)count * nufi_stub_mpi_size(datatype));
    return MPI_SUCCESS;
}
static inline int MPI_Allgatherv(const void *sendbuf, int sendcount, MPI_Datatype sendtype, void *recvbuf,
                                 const int *recvcounts, const int *displs, MPI_Datatype recvtype, MPI_Comm comm)
{
    (void)recvcounts; (void)comm;
    if (sendbuf != MPI_IN_PLACE)
        memcpy((char *)recvbuf + (size_t)displs[0] * nufi_stub_mpi_size(recvtype), sendbuf,
               (size_t)sendcount * nufi_stub_mpi_size(sendtype));
    return MPI_SUCCESS;
}

#endif
