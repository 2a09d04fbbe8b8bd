// mpi.h.cuh — the __device__ MPI surface of the block-rank runtime.
//
// Drop-in for the reference's gpu_libs/gpu_mpi/mpi.h.cuh (which includes mpi.cuh, mpi_common.cuh,
// group.cuh, communicator.cuh, datatypes.cuh, operators.cuh): same type names, same handle kinds
// (opaque pointers for MPI_Comm / MPI_Group / MPI_Op / MPI_Request, an enum for MPI_Datatype with the
// reference's value order), same constants, same function signatures.  Code converted for the
// reference (every function __device__, main renamed __gpu_main) compiles against this header.
//
// Calling convention: an MPI rank is one thread block; the user program runs on thread 0 of the block
// (scalar code, exactly as in the reference) and MPI calls use the rest of the block internally.
// Call MPI functions from thread 0 of a rank block only.
#pragma once

#include <stdint.h>
#include <stddef.h>

#include "gpumpi_abi.h"

// ---- constants (reference gpu_libs/gpu_mpi/mpi.cuh:4-9, mpi_common.cuh:3-9) ----
#define MPI_MAX_PROCESSOR_NAME 256
#define MPI_ANY_TAG (-1)
#define MPI_ANY_SOURCE (-1)
#define MPI_PROC_NULL (-2)
#define MPI_TAG_UB ((1 << 15) - 1)
#define MPI_SUCCESS 0
#define MPI_FAILURE -1
#define MPI_ERR_OTHER 1
#define MPI_ERR_BUFFER GPUMPI_ERR_BUFFER
#define MPI_ERR_COUNT GPUMPI_ERR_COUNT
#define MPI_ERR_TYPE GPUMPI_ERR_TYPE
#define MPI_ERR_TAG GPUMPI_ERR_TAG
#define MPI_ERR_COMM GPUMPI_ERR_COMM
#define MPI_ERR_RANK GPUMPI_ERR_RANK
#define MPI_ERR_ROOT GPUMPI_ERR_ROOT
#define MPI_ERR_OP GPUMPI_ERR_OP
#define MPI_ERR_ARG GPUMPI_ERR_ARG
#define MPI_ERR_REQUEST GPUMPI_ERR_REQUEST
#define MPI_ERR_TRUNCATE GPUMPI_ERR_TRUNCATE
#define MPI_ERR_NO_MEM GPUMPI_ERR_NO_MEM
#define MPI_ERR_INTERN GPUMPI_ERR_INTERN
#define MPI_UNDEFINED -1
#define MPI_CART 1
#define MPI_MAX_DIMS 8
#define MPI_THREAD_SINGLE 1
#define MPI_THREAD_FUNNELED 2
#define MPI_THREAD_SERIALIZED 3
#define MPI_THREAD_MULTIPLE 4
#define MPI_IN_PLACE ((void*)(intptr_t)1)
#define MPI_BOTTOM ((void*)0)

// ---- datatypes: the reference's enum (gpu_libs/gpu_mpi/datatypes.cuh:12-14) with a fixed
//      underlying type so derived-type handles can share it ----
enum MPI_Datatype : int {
    MPI_CHAR = GPUMPI_CHAR,
    MPI_SHORT = GPUMPI_SHORT,
    MPI_INT = GPUMPI_INT,
    MPI_LONG = GPUMPI_LONG,
    MPI_LONG_LONG_INT = GPUMPI_LONG_LONG_INT,
    MPI_LONG_LONG = GPUMPI_LONG_LONG,
    MPI_SIGNED_CHAR = GPUMPI_SIGNED_CHAR,
    MPI_UNSIGNED_CHAR = GPUMPI_UNSIGNED_CHAR,
    MPI_UNSIGNED_SHORT = GPUMPI_UNSIGNED_SHORT,
    MPI_UNSIGNED = GPUMPI_UNSIGNED,
    MPI_UNSIGNED_LONG = GPUMPI_UNSIGNED_LONG,
    MPI_UNSIGNED_LONG_LONG = GPUMPI_UNSIGNED_LONG_LONG,
    MPI_FLOAT = GPUMPI_FLOAT,
    MPI_DOUBLE = GPUMPI_DOUBLE,
    MPI_LONG_DOUBLE = GPUMPI_LONG_DOUBLE,
    MPI_WCHAR = GPUMPI_WCHAR,
    MPI_C_BOOL = GPUMPI_C_BOOL,
    MPI_INT8_T = GPUMPI_INT8_T,
    MPI_INT16_T = GPUMPI_INT16_T,
    MPI_INT32_T = GPUMPI_INT32_T,
    MPI_INT64_T = GPUMPI_INT64_T,
    MPI_UINT8_T = GPUMPI_UINT8_T,
    MPI_UINT16_T = GPUMPI_UINT16_T,
    MPI_UINT32_T = GPUMPI_UINT32_T,
    MPI_UINT64_T = GPUMPI_UINT64_T,
    MPI_C_COMPLEX = GPUMPI_C_COMPLEX,
    MPI_C_FLOAT_COMPLEX = GPUMPI_C_FLOAT_COMPLEX,
    MPI_C_DOUBLE_COMPLEX = GPUMPI_C_DOUBLE_COMPLEX,
    MPI_C_LONG_DOUBLE_COMPLEX = GPUMPI_C_LONG_DOUBLE_COMPLEX,
    MPI_BYTE = GPUMPI_BYTE,
    MPI_2INT = GPUMPI_2INT,
    MPI_FLOAT_INT = GPUMPI_FLOAT_INT,
    MPI_DOUBLE_INT = GPUMPI_DOUBLE_INT,
    MPI_LONG_INT = GPUMPI_LONG_INT,
    MPI_SHORT_INT = GPUMPI_SHORT_INT,
    MPI_LONG_DOUBLE_INT = GPUMPI_LONG_DOUBLE_INT,
    MPI_DATATYPE_NULL = GPUMPI_DATATYPE_NULL,
};
#define MPI_ORDER_C 56
#define MPI_ORDER_FORTRAN 57

// ---- opaque handles (reference: communicator.cuh:6-8, group.cuh:4-5, operators.cuh:7-8, mpi.cuh:26-29) ----
struct MPI_Comm_impl;
using MPI_Comm = MPI_Comm_impl*;
struct MPI_Group_impl;
typedef MPI_Group_impl* MPI_Group;
struct MPI_Op_impl;
using MPI_Op = MPI_Op_impl*;
struct MPI_Request_impl;
using MPI_Request = MPI_Request_impl*;
#define MPI_REQUEST_NULL nullptr
#define MPI_OP_NULL nullptr

typedef void MPI_User_function(void* invec, void* inoutvec, int* len, MPI_Datatype* datatype);

__device__ extern MPI_Comm MPI_COMM_WORLD;
__device__ extern MPI_Comm MPI_COMM_NULL;
__device__ extern MPI_Comm MPI_COMM_SELF;
__device__ extern MPI_Group MPI_GROUP_WORLD;
__device__ extern MPI_Group MPI_GROUP_NULL;
__device__ extern MPI_Group MPI_GROUP_EMPTY;

__device__ extern MPI_Op MPI_MAX;
__device__ extern MPI_Op MPI_MIN;
__device__ extern MPI_Op MPI_SUM;
__device__ extern MPI_Op MPI_PROD;
__device__ extern MPI_Op MPI_LAND;
__device__ extern MPI_Op MPI_BAND;
__device__ extern MPI_Op MPI_LOR;
__device__ extern MPI_Op MPI_BOR;
__device__ extern MPI_Op MPI_LXOR;
__device__ extern MPI_Op MPI_BXOR;
__device__ extern MPI_Op MPI_MAXLOC;
__device__ extern MPI_Op MPI_MINLOC;

struct MPI_Status {
    int MPI_SOURCE = MPI_ANY_SOURCE;
    int MPI_TAG = MPI_ANY_TAG;
    int MPI_ERROR = MPI_SUCCESS;
    long long count_bytes = 0;
};
#define MPI_STATUSES_IGNORE ((MPI_Status*)nullptr)
#define MPI_STATUS_IGNORE ((MPI_Status*)nullptr)

typedef long long MPI_Aint;
typedef long long MPI_Count;

// ---- environment (reference mpi.cuh:39-46,49,63,66,121) ----
__device__ int MPI_Init(int* argc, char*** argv);
__device__ int MPI_Init_thread(int* argc, char*** argv, int required, int* provided);
__device__ int MPI_Initialized(int* flag);
__device__ int MPI_Finalize(void);
__device__ int MPI_Finalized(int* flag);
__device__ int MPI_Abort(MPI_Comm comm, int errorcode);
__device__ int MPI_Get_processor_name(char* name, int* resultlen);
__device__ double MPI_Wtime(void);
__device__ double MPI_Wtick(void);

// ---- point-to-point (reference mpi.cuh:55-62,113-128) ----
__device__ int MPI_Send(const void* buf, int count, MPI_Datatype datatype, int dest, int tag, MPI_Comm comm);
__device__ int MPI_Ssend(const void* buf, int count, MPI_Datatype datatype, int dest, int tag, MPI_Comm comm);
__device__ int MPI_Recv(void* buf, int count, MPI_Datatype datatype, int source, int tag, MPI_Comm comm,
                        MPI_Status* status);
__device__ int MPI_Sendrecv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, int dest, int sendtag,
                            void* recvbuf, int recvcount, MPI_Datatype recvtype, int source, int recvtag,
                            MPI_Comm comm, MPI_Status* status);
__device__ int MPI_Isend(const void* buf, int count, MPI_Datatype datatype, int dest, int tag, MPI_Comm comm,
                         MPI_Request* request);
__device__ int MPI_Issend(const void* buf, int count, MPI_Datatype datatype, int dest, int tag, MPI_Comm comm,
                          MPI_Request* request);
__device__ int MPI_Irecv(void* buf, int count, MPI_Datatype datatype, int source, int tag, MPI_Comm comm,
                         MPI_Request* request);
__device__ int MPI_Wait(MPI_Request* request, MPI_Status* status);
__device__ int MPI_Waitall(int count, MPI_Request array_of_requests[], MPI_Status* array_of_statuses);
__device__ int MPI_Waitany(int count, MPI_Request array_of_requests[], int* index, MPI_Status* status);
__device__ int MPI_Waitsome(int incount, MPI_Request array_of_requests[], int* outcount, int array_of_indices[],
                            MPI_Status array_of_statuses[]);
__device__ int MPI_Test(MPI_Request* request, int* flag, MPI_Status* status);
__device__ int MPI_Testall(int count, MPI_Request array_of_requests[], int* flag, MPI_Status array_of_statuses[]);
__device__ int MPI_Request_free(MPI_Request* request);
__device__ int MPI_Iprobe(int source, int tag, MPI_Comm comm, int* flag, MPI_Status* status);
__device__ int MPI_Probe(int source, int tag, MPI_Comm comm, MPI_Status* status);
__device__ int MPI_Get_count(const MPI_Status* status, MPI_Datatype datatype, int* count);

// ---- collectives (reference mpi.cuh:47-94) ----
__device__ int MPI_Barrier(MPI_Comm comm);
__device__ int MPI_Bcast(void* buffer, int count, MPI_Datatype datatype, int root, MPI_Comm comm);
__device__ int MPI_Reduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype datatype, MPI_Op op, int root,
                          MPI_Comm comm);
__device__ int MPI_Allreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype datatype, MPI_Op op,
                             MPI_Comm comm);
__device__ int MPI_Gather(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, int recvcount,
                          MPI_Datatype recvtype, int root, MPI_Comm comm);
__device__ int MPI_Gatherv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf,
                           const int recvcounts[], const int displs[], MPI_Datatype recvtype, int root, MPI_Comm comm);
__device__ int MPI_Scatter(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, int recvcount,
                           MPI_Datatype recvtype, int root, MPI_Comm comm);
__device__ int MPI_Scatterv(const void* sendbuf, const int sendcounts[], const int displs[], MPI_Datatype sendtype,
                            void* recvbuf, int recvcount, MPI_Datatype recvtype, int root, MPI_Comm comm);
__device__ int MPI_Allgather(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, int recvcount,
                             MPI_Datatype recvtype, MPI_Comm comm);
__device__ int MPI_Allgatherv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf,
                              const int recvcounts[], const int displs[], MPI_Datatype recvtype, MPI_Comm comm);
__device__ int MPI_Alltoall(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, int recvcount,
                            MPI_Datatype recvtype, MPI_Comm comm);
__device__ int MPI_Alltoallv(const void* sendbuf, const int sendcounts[], const int sdispls[], MPI_Datatype sendtype,
                             void* recvbuf, const int recvcounts[], const int rdispls[], MPI_Datatype recvtype,
                             MPI_Comm comm);

// ---- operators (reference operators.cuh:18-20, mpi.cuh:43-44) ----
__device__ int MPI_Op_create(MPI_User_function* user_fn, int commute, MPI_Op* op);
__device__ int MPI_Op_free(MPI_Op* op);

// ---- datatypes (reference mpi.cuh:53-54,67 are stubs there; implemented here per the MPI standard) ----
__device__ int MPI_Type_size(MPI_Datatype datatype, int* size);
__device__ int MPI_Type_get_extent(MPI_Datatype datatype, MPI_Aint* lb, MPI_Aint* extent);
__device__ int MPI_Type_contiguous(int count, MPI_Datatype oldtype, MPI_Datatype* newtype);
__device__ int MPI_Type_vector(int count, int blocklength, int stride, MPI_Datatype oldtype, MPI_Datatype* newtype);
__device__ int MPI_Type_create_hvector(int count, int blocklength, MPI_Aint stride, MPI_Datatype oldtype,
                                       MPI_Datatype* newtype);
__device__ int MPI_Type_create_subarray(int ndims, const int array_of_sizes[], const int array_of_subsizes[],
                                        const int array_of_starts[], int order, MPI_Datatype oldtype,
                                        MPI_Datatype* newtype);
__device__ int MPI_Type_commit(MPI_Datatype* datatype);
__device__ int MPI_Type_free(MPI_Datatype* datatype);

// ---- communicators and groups (reference communicator.cuh:23-49, group.cuh:21-31) ----
__device__ int MPI_Comm_size(MPI_Comm comm, int* size);
__device__ int MPI_Comm_rank(MPI_Comm comm, int* rank);
__device__ int MPI_Comm_group(MPI_Comm comm, MPI_Group* group);
__device__ int MPI_Comm_create(MPI_Comm comm, MPI_Group group, MPI_Comm* newcomm);
__device__ int MPI_Comm_dup(MPI_Comm comm, MPI_Comm* newcomm);
__device__ int MPI_Comm_split(MPI_Comm comm, int color, int key, MPI_Comm* newcomm);
__device__ int MPI_Comm_free(MPI_Comm* comm);
__device__ int MPI_Group_incl(MPI_Group group, int n, const int ranks[], MPI_Group* newgroup);
__device__ int MPI_Group_range_incl(MPI_Group group, int n, int ranges[][3], MPI_Group* newgroup);
__device__ int MPI_Group_free(MPI_Group* group);
__device__ int MPI_Group_size(MPI_Group group, int* size);
__device__ int MPI_Group_rank(MPI_Group group, int* rank);
__device__ int MPI_Group_translate_ranks(MPI_Group group1, int n, const int ranks1[], MPI_Group group2, int ranks2[]);

// ---- attribute caching on communicators (reference mpi.cuh:95-110 declares the keyval part and
//      traps in every function, mpi.cu:519-536; implemented here per MPI-1.3 section 5.7) ----
// Keyvals and attributes belong to the calling rank.  MPI_Comm_dup calls each attribute's copy
// function and caches the value it returns when it sets *flag; MPI_Comm_free and MPI_Attr_delete call
// the delete function.  MPI_Attr_get(comm, MPI_TAG_UB, ...) returns the tag bound.
typedef int MPI_Copy_function(MPI_Comm oldcomm, int keyval, void* extra_state, void* attribute_val_in,
                              void* attribute_val_out, int* flag);
typedef int MPI_Delete_function(MPI_Comm comm, int keyval, void* attribute_val, void* extra_state);
#define MPI_KEYVAL_INVALID (-1)
#define GPUMPI_MAX_KEYVALS 32          // keyvals a rank can hold at once
#define GPUMPI_MAX_ATTRS 64            // attributes a rank can cache over all its communicators
__device__ int MPI_NULL_COPY_FN(MPI_Comm oldcomm, int keyval, void* extra_state, void* attribute_val_in,
                                void* attribute_val_out, int* flag);
__device__ int MPI_DUP_FN(MPI_Comm oldcomm, int keyval, void* extra_state, void* attribute_val_in,
                          void* attribute_val_out, int* flag);
__device__ int MPI_NULL_DELETE_FN(MPI_Comm comm, int keyval, void* attribute_val, void* extra_state);
__device__ int MPI_Keyval_create(MPI_Copy_function* copy_fn, MPI_Delete_function* delete_fn, int* keyval,
                                 void* extra_state);
__device__ int MPI_Keyval_free(int* keyval);
__device__ int MPI_Attr_put(MPI_Comm comm, int keyval, void* attribute_val);
__device__ int MPI_Attr_get(MPI_Comm comm, int keyval, void* attribute_val, int* flag);
__device__ int MPI_Attr_delete(MPI_Comm comm, int keyval);

// ---- Cartesian topologies (MPI-3.1 section 7.5; not in the reference) ----
// Ranks keep their order (reorder is accepted and ignored); at most MPI_MAX_DIMS dimensions.
__device__ int MPI_Dims_create(int nnodes, int ndims, int dims[]);
__device__ int MPI_Cart_create(MPI_Comm comm_old, int ndims, const int dims[], const int periods[], int reorder,
                               MPI_Comm* comm_cart);
__device__ int MPI_Cart_coords(MPI_Comm comm, int rank, int maxdims, int coords[]);
__device__ int MPI_Cart_rank(MPI_Comm comm, const int coords[], int* rank);
__device__ int MPI_Cart_shift(MPI_Comm comm, int direction, int disp, int* rank_source, int* rank_dest);
__device__ int MPI_Cart_get(MPI_Comm comm, int maxdims, int dims[], int periods[], int coords[]);
__device__ int MPI_Cartdim_get(MPI_Comm comm, int* ndims);
__device__ int MPI_Cart_sub(MPI_Comm comm, const int remain_dims[], MPI_Comm* newcomm);
__device__ int MPI_Topo_test(MPI_Comm comm, int* status);

// ---- MPI-IO (reference gpu_libs/gpu_mpi/io.cuh:13-153; MPI-3.1 chapter 13) ----
// File data and metadata travel over the device -> host request channel; the host process performs the
// file system calls.  MPI_File is an opaque handle here (the reference passes a struct by value), read
// and write calls return MPI_SUCCESS or an error class and report the amount in the status, and file
// pointers count etypes of the current view.
typedef long long MPI_Offset;
struct MPI_Info_impl;
typedef MPI_Info_impl* MPI_Info;
#define MPI_INFO_NULL ((MPI_Info)0)
struct MPI_File_impl;
typedef MPI_File_impl* MPI_File;
#define MPI_FILE_NULL ((MPI_File)0)
#define MPI_MODE_RDONLY 1             // access modes: the reference's values (io.cuh:13-21)
#define MPI_MODE_RDWR 2
#define MPI_MODE_WRONLY 4
#define MPI_MODE_CREATE 8
#define MPI_MODE_EXCL 16
#define MPI_MODE_DELETE_ON_CLOSE 32
#define MPI_MODE_UNIQUE_OPEN 64
#define MPI_MODE_SEQUENTIAL 128
#define MPI_MODE_APPEND 256
#define MPI_SEEK_SET 1                // the reference's values (io.cuh:52-54)
#define MPI_SEEK_CUR 2
#define MPI_SEEK_END 3
#define MPI_DISPLACEMENT_CURRENT (-1)
#define MPI_ERR_FILE GPUMPI_ERR_FILE
#define MPI_ERR_NOT_SAME GPUMPI_ERR_NOT_SAME
#define MPI_ERR_AMODE GPUMPI_ERR_AMODE
#define MPI_ERR_UNSUPPORTED_DATAREP GPUMPI_ERR_UNSUPPORTED_DATAREP
#define MPI_ERR_UNSUPPORTED_OPERATION GPUMPI_ERR_UNSUPPORTED_OPERATION
#define MPI_ERR_NO_SUCH_FILE GPUMPI_ERR_NO_SUCH_FILE
#define MPI_ERR_FILE_EXISTS GPUMPI_ERR_FILE_EXISTS
#define MPI_ERR_BAD_FILE GPUMPI_ERR_BAD_FILE
#define MPI_ERR_ACCESS GPUMPI_ERR_ACCESS
#define MPI_ERR_NO_SPACE GPUMPI_ERR_NO_SPACE
#define MPI_ERR_QUOTA GPUMPI_ERR_QUOTA
#define MPI_ERR_READ_ONLY GPUMPI_ERR_READ_ONLY
#define MPI_ERR_FILE_IN_USE GPUMPI_ERR_FILE_IN_USE
#define MPI_ERR_IO GPUMPI_ERR_IO
__device__ int MPI_File_open(MPI_Comm comm, const char* filename, int amode, MPI_Info info, MPI_File* fh);
__device__ int MPI_File_close(MPI_File* fh);
__device__ int MPI_File_delete(const char* filename, MPI_Info info);
__device__ int MPI_File_get_size(MPI_File fh, MPI_Offset* size);
__device__ int MPI_File_set_size(MPI_File fh, MPI_Offset size);
__device__ int MPI_File_sync(MPI_File fh);
__device__ int MPI_File_get_amode(MPI_File fh, int* amode);
__device__ int MPI_File_set_view(MPI_File fh, MPI_Offset disp, MPI_Datatype etype, MPI_Datatype filetype,
                                 const char* datarep, MPI_Info info);
__device__ int MPI_File_get_view(MPI_File fh, MPI_Offset* disp, MPI_Datatype* etype, MPI_Datatype* filetype,
                                 char* datarep);
__device__ int MPI_File_read(MPI_File fh, void* buf, int count, MPI_Datatype datatype, MPI_Status* status);
__device__ int MPI_File_write(MPI_File fh, const void* buf, int count, MPI_Datatype datatype, MPI_Status* status);
__device__ int MPI_File_read_at(MPI_File fh, MPI_Offset offset, void* buf, int count, MPI_Datatype datatype,
                                MPI_Status* status);
__device__ int MPI_File_write_at(MPI_File fh, MPI_Offset offset, const void* buf, int count, MPI_Datatype datatype,
                                 MPI_Status* status);
__device__ int MPI_File_read_all(MPI_File fh, void* buf, int count, MPI_Datatype datatype, MPI_Status* status);
__device__ int MPI_File_write_all(MPI_File fh, const void* buf, int count, MPI_Datatype datatype, MPI_Status* status);
__device__ int MPI_File_read_at_all(MPI_File fh, MPI_Offset offset, void* buf, int count, MPI_Datatype datatype,
                                    MPI_Status* status);
__device__ int MPI_File_write_at_all(MPI_File fh, MPI_Offset offset, const void* buf, int count,
                                     MPI_Datatype datatype, MPI_Status* status);
__device__ int MPI_File_read_shared(MPI_File fh, void* buf, int count, MPI_Datatype datatype, MPI_Status* status);
__device__ int MPI_File_write_shared(MPI_File fh, const void* buf, int count, MPI_Datatype datatype,
                                     MPI_Status* status);
__device__ int MPI_File_seek(MPI_File fh, MPI_Offset offset, int whence);
__device__ int MPI_File_get_position(MPI_File fh, MPI_Offset* offset);
__device__ int MPI_File_seek_shared(MPI_File fh, MPI_Offset offset, int whence);
__device__ int MPI_File_get_position_shared(MPI_File fh, MPI_Offset* offset);
__device__ int MPI_File_get_byte_offset(MPI_File fh, MPI_Offset offset, MPI_Offset* disp);

// ---- block-rank extensions (no counterpart in the reference) ----
// Rank of the calling block in MPI_COMM_WORLD, usable anywhere in the rank's block.
__device__ int gpumpi_world_rank(void);
// Run fn(arg, tid, nthreads) on every thread of the calling rank's block (called from thread 0);
// gives scalar user code the data-parallel width of its block between MPI calls.
__device__ int gpumpi_block_parallel(void (*fn)(void* arg, int tid, int nthreads), void* arg);
// Inside such a function: a barrier over the block's nthreads threads.
__device__ void gpumpi_block_sync(int nthreads);
// The block's dynamic shared memory (size in *bytes, 0 when the launch has none); free for the rank's
// own block-parallel functions between MPI calls.
__device__ void* gpumpi_block_scratch(size_t* bytes);
// Per-rank copy of a converted program's global variable (reference global_vars.cuh:15 indexes by
// the global thread id; a rank here is a block, so the index is the rank).
#define __gpu_global(var) (var[gpumpi_world_rank()])
