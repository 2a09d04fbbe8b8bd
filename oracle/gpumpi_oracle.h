/*
 * gpumpi_oracle.h — CPU oracle for the intra-GPU MPI hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may call it; the product path never does.
 *
 * It restates, in plain C, what the reference runtime computes for each operation on the path
 * (file:line citations are beside each function in gpumpi_oracle.c).  Parity is pinned by the
 * known-answer vectors of the reference's own tests (tests/golden/*.json, generated by
 * tests/golden/make_golden.py from the formulas in the reference's tests/*.cu).
 */
#ifndef GPUMPI_ORACLE_H
#define GPUMPI_ORACLE_H

#include <stdint.h>
#include "../include/gpumpi_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- datatypes and operators ---- */
int orc_type_size(int dt);                 /* bytes of one element, -1 if unknown */
int orc_op_allowed(int op, int dt);        /* 1 if the reference's legality table allows op on dt */

/* Canonical rank-order fold of the reference: out = x_0; for s = 1..n-1: out = op(x_s, out).
 * inputs[s] points at rank s's count elements.  Returns an MPI error code. */
int orc_reduce(const void* const* inputs, int n, void* out, int64_t count, int dt, int op);

/* Rank-major convenience: rank s's input at sendbufs + s*stride_bytes. */
int orc_reduce_rm(const void* sendbufs, int64_t stride_bytes, int n, void* out, int64_t count,
                  int dt, int op);

/* Allreduce over rank-major buffers: every rank's recv slot receives the canonical fold.
 * threads > 1 splits the element range across POSIX threads (the CPU baseline). */
int orc_allreduce(const void* sendbufs, void* recvbufs, int n, int64_t count, int dt, int op,
                  int threads);

/* Alltoallv over rank-major buffers (elements of size esize):
 *   rank r's send buffer = sendbufs + r*send_stride (bytes), recv buffer = recvbufs + r*recv_stride;
 *   sendcounts/sdispls/recvcounts/rdispls are n*n matrices, row r = rank r's own arrays.
 * Receiver r gets min(sendcounts[s][r], recvcounts[r][s]) elements from sender s.
 * Returns GPUMPI_ERR_TRUNCATE if any sender sends more than the receiver posted. */
int orc_alltoallv(const void* sendbufs, int64_t send_stride, const int* sendcounts, const int* sdispls,
                  void* recvbufs, int64_t recv_stride, const int* recvcounts, const int* rdispls,
                  int n, int esize, int threads);

/* ---- derived datatypes (MPI-standard pack/unpack; the reference has none) ---- */
typedef struct orc_typemap {
    int64_t size;        /* bytes of data in one element of the type */
    int64_t extent;      /* span from lb to ub */
    int64_t lb;
    int64_t block;       /* contiguous bytes at the innermost level */
    int nlev;            /* number of strided levels (0 = contiguous) */
    int64_t cnt[4];      /* level i repeats cnt[i] times ... */
    int64_t stride[4];   /* ... at byte stride stride[i]; level 0 is innermost */
} orc_typemap;

void orc_type_basic(int dt, orc_typemap* out);
int  orc_type_contiguous(int64_t count, const orc_typemap* old, orc_typemap* out);
int  orc_type_vector(int64_t count, int64_t blocklen, int64_t stride_elems, const orc_typemap* old,
                     orc_typemap* out);
int  orc_type_hvector(int64_t count, int64_t blocklen, int64_t stride_bytes, const orc_typemap* old,
                      orc_typemap* out);
/* C-order subarray of up to 3 dims (sizes/subsizes/starts outermost first). */
int  orc_type_subarray(int ndims, const int* sizes, const int* subsizes, const int* starts,
                       const orc_typemap* old, orc_typemap* out);
int64_t orc_pack(const orc_typemap* t, int64_t count, const void* src, void* packed);
int64_t orc_unpack(const orc_typemap* t, int64_t count, const void* packed, void* dst);

/* ---- synthetic inputs: one 64-bit LCG (Knuth MMIX constants) ---- */
uint64_t orc_lcg_next(uint64_t* state);
double   orc_lcg_u01(uint64_t* state);          /* (state >> 11) * 2^-53 after one step */
void     orc_fill_f32(uint64_t seed, int64_t n, float* out);    /* uniform [-1, 1) */
void     orc_fill_f64(uint64_t seed, int64_t n, double* out);   /* uniform [-1, 1) */
void     orc_fill_i32(uint64_t seed, int64_t n, int32_t* out);  /* uniform over all int32 */

/* Monte Carlo pi: pairs (x,y) from the LCG seeded with seed+rank; hit if x*x + y*y < 1. */
int64_t  orc_pi_hits(uint64_t seed, int rank, int64_t pairs);

/* Bucket sort workload: key = floor(2^21 * mean of four U(0,1) draws), LCG seeded seed+rank. */
void     orc_bucket_keys(uint64_t seed, int rank, int64_t nkeys, int32_t* keys);
/* One full iteration of the distributed bucket sort over n ranks (keys_per_rank each, rank-major);
 * writes each rank's sorted received keys rank-major into out (capacity cap_per_rank) and the
 * per-rank counts into out_counts.  Returns 0 or GPUMPI_ERR_COUNT on overflow. */
int      orc_bucket_sort(const int32_t* keys, int n, int64_t keys_per_rank, int32_t* out,
                         int64_t cap_per_rank, int64_t* out_counts);

/* 3D halo exchange check: global grid G^3 (G = P*L), rank (pz,py,px) owns an (L+2)^3 block with
 * 1-cell halos, periodic.  Cell value = orc_halo_value(gz, gy, gx).  Fills rank's expected block. */
double   orc_halo_value(int64_t gz, int64_t gy, int64_t gx);
void     orc_halo_expected(int P, int L, int rank, double* block /* (L+2)^3 */);

/* Comm_split: new rank and size for each of n ranks (colors/keys per rank; color GPUMPI_UNDEFINED
 * gives rank -1, size 0).  Order: key, then parent rank (gpu_libs/gpu_mpi/communicator.cu:164-213). */
void     orc_comm_split(int n, const int* colors, const int* keys, int* newrank, int* newsize);

/* ---- MLP 12 -> 64 -> 64 -> 4 (ReLU), fp64 reference for gradient checks ----
 * params layout (fp64 here, fp32 on the GPU): W1[64][12], b1[64], W2[64][64], b2[64], W3[4][64], b3[4].
 * loss = mean over batch and the 4 outputs of mask * (y - t)^2.  grads same layout as params. */
#define ORC_MLP_IN 12
#define ORC_MLP_H 64
#define ORC_MLP_OUT 4
#define ORC_MLP_NPARAMS (64*12 + 64 + 64*64 + 64 + 4*64 + 4)
double   orc_mlp_loss_grad(const double* params, const double* x, const double* t, const double* mask,
                           int batch, double* grads /* may be NULL */);
void     orc_mlp_forward(const double* params, const double* x, int batch, double* y);

#ifdef __cplusplus
}
#endif
#endif
