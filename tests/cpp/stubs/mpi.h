/* Declarations only, for compiling the reference's MPI drivers
 * (bin/test_nufi_gpu_2d.cpp, bin/test_nufi_gpu_3d.cpp through nufi/mpi.hpp)
 * with -fsyntax-only in tests/test_cpp_api.py: the names and signatures of
 * the MPI calls they use.  Nothing is linked or run. */
#ifndef NUFI_TEST_STUB_MPI_H
#define NUFI_TEST_STUB_MPI_H

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

#ifdef __cplusplus
extern "C" {
#endif
int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Error_string(int errorcode, char *string, int *resultlen);
int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype datatype, MPI_Op op, MPI_Comm comm);
int MPI_Allgatherv(const void *sendbuf, int sendcount, MPI_Datatype sendtype, void *recvbuf, const int *recvcounts,
                   const int *displs, MPI_Datatype recvtype, MPI_Comm comm);
#ifdef __cplusplus
}
#endif

#endif
