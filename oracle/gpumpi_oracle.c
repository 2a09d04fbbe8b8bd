/*
 * gpumpi_oracle.c — CPU oracle (test infrastructure; see gpumpi_oracle.h).
 *
 * Compiled with -ffp-contract=off so that floating-point folds round exactly like the GPU path,
 * which uses explicitly rounded (non-fused) adds and multiplies.
 */
#include "gpumpi_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------------------------ */
/* datatypes: sizes follow gpu_libs/gpu_mpi/mpi_types_list.cuh:3-33 (LP64: long = 8 bytes,
 * wchar_t = 4 bytes, long double stored as double)                                            */
/* ------------------------------------------------------------------------------------------ */
int orc_type_size(int dt) {
    static const int sizes[GPUMPI_NUM_PREDEFINED_TYPES] = {
        1, 2, 4, 8, 8, 8, 1, 1, 2, 4, 8, 8, 4, 8, 8, 4, 1, 1, 2, 4, 8, 1, 2, 4, 8,
        8, 8, 16, 16, 1,
        8, 8, 16, 16, 8, 16};
    if (dt < 0 || dt >= GPUMPI_NUM_PREDEFINED_TYPES) return -1;
    return sizes[dt];
}

enum { C_INT = 1, C_FLOAT = 2, C_LOGICAL = 4, C_COMPLEX = 8, C_BYTE = 16, C_TEXT = 32, C_PAIR = 64 };

/* Type classes of gpu_libs/gpu_mpi/operators.cu:26-73 (IsIntegerType / IsFloatingType /
 * IsLogicalType / IsComplexType / IsByteType / IsTextType).  MPI_CHAR and MPI_WCHAR are text. */
static int type_class(int dt) {
    switch (dt) {
    case GPUMPI_SHORT: case GPUMPI_INT: case GPUMPI_LONG: case GPUMPI_LONG_LONG_INT:
    case GPUMPI_LONG_LONG: case GPUMPI_SIGNED_CHAR: case GPUMPI_UNSIGNED_CHAR:
    case GPUMPI_UNSIGNED_SHORT: case GPUMPI_UNSIGNED: case GPUMPI_UNSIGNED_LONG:
    case GPUMPI_UNSIGNED_LONG_LONG: case GPUMPI_INT8_T: case GPUMPI_INT16_T: case GPUMPI_INT32_T:
    case GPUMPI_INT64_T: case GPUMPI_UINT8_T: case GPUMPI_UINT16_T: case GPUMPI_UINT32_T:
    case GPUMPI_UINT64_T:
        return C_INT;
    case GPUMPI_FLOAT: case GPUMPI_DOUBLE: case GPUMPI_LONG_DOUBLE: return C_FLOAT;
    case GPUMPI_C_BOOL: return C_LOGICAL;
    case GPUMPI_C_COMPLEX: case GPUMPI_C_FLOAT_COMPLEX: case GPUMPI_C_DOUBLE_COMPLEX:
    case GPUMPI_C_LONG_DOUBLE_COMPLEX: return C_COMPLEX;
    case GPUMPI_BYTE: return C_BYTE;
    case GPUMPI_CHAR: case GPUMPI_WCHAR: return C_TEXT;
    case GPUMPI_2INT: case GPUMPI_FLOAT_INT: case GPUMPI_DOUBLE_INT: case GPUMPI_LONG_INT:
    case GPUMPI_SHORT_INT: case GPUMPI_LONG_DOUBLE_INT: return C_PAIR;
    default: return 0;
    }
}

/* Legality table of gpu_libs/gpu_mpi/operators.cu:153-200; MAXLOC/MINLOC on the pair types. */
int orc_op_allowed(int op, int dt) {
    int c = type_class(dt);
    switch (op) {
    case GPUMPI_OP_MAX: case GPUMPI_OP_MIN: return (c & (C_INT | C_FLOAT)) != 0;
    case GPUMPI_OP_SUM: case GPUMPI_OP_PROD: return (c & (C_INT | C_FLOAT | C_COMPLEX)) != 0;
    case GPUMPI_OP_LAND: case GPUMPI_OP_LOR: case GPUMPI_OP_LXOR: return (c & (C_INT | C_LOGICAL)) != 0;
    case GPUMPI_OP_BAND: case GPUMPI_OP_BOR: case GPUMPI_OP_BXOR: return (c & (C_INT | C_BYTE)) != 0;
    case GPUMPI_OP_MAXLOC: case GPUMPI_OP_MINLOC: return c == C_PAIR;
    default: return 0;
    }
}

/* ------------------------------------------------------------------------------------------ */
/* element-wise operator application: inout[i] = op(in[i], inout[i])                            */
/* (gpu_libs/gpu_mpi/operators.cu:73-151 functors, loop at :216-218).  Integer arithmetic wraps */
/* modulo 2^bits (done in unsigned arithmetic here so it is defined behaviour in C).            */
/* ------------------------------------------------------------------------------------------ */
#define INT_OPS(T, U)                                                                             \
    static void apply_##T(int op, const T* in, T* io, int64_t n) {                                \
        int64_t i;                                                                                \
        switch (op) {                                                                             \
        case GPUMPI_OP_MAX: for (i = 0; i < n; i++) io[i] = in[i] > io[i] ? in[i] : io[i]; break; \
        case GPUMPI_OP_MIN: for (i = 0; i < n; i++) io[i] = in[i] > io[i] ? io[i] : in[i]; break; \
        case GPUMPI_OP_SUM: for (i = 0; i < n; i++) io[i] = (T)((U)in[i] + (U)io[i]); break;      \
        case GPUMPI_OP_PROD: for (i = 0; i < n; i++) io[i] = (T)((U)in[i] * (U)io[i]); break;     \
        case GPUMPI_OP_LAND: for (i = 0; i < n; i++) io[i] = (T)(in[i] && io[i]); break;          \
        case GPUMPI_OP_BAND: for (i = 0; i < n; i++) io[i] = (T)(in[i] & io[i]); break;           \
        case GPUMPI_OP_LOR: for (i = 0; i < n; i++) io[i] = (T)(in[i] || io[i]); break;           \
        case GPUMPI_OP_BOR: for (i = 0; i < n; i++) io[i] = (T)(in[i] | io[i]); break;            \
        case GPUMPI_OP_LXOR: for (i = 0; i < n; i++) io[i] = (T)(in[i] != io[i]); break;          \
        case GPUMPI_OP_BXOR: for (i = 0; i < n; i++) io[i] = (T)(in[i] ^ io[i]); break;           \
        }                                                                                         \
    }

typedef signed char s8;
typedef unsigned char u8;
INT_OPS(int8_t, uint8_t)
INT_OPS(int16_t, uint16_t)
INT_OPS(int32_t, uint32_t)
INT_OPS(int64_t, uint64_t)
INT_OPS(uint8_t, uint8_t)
INT_OPS(uint16_t, uint16_t)
INT_OPS(uint32_t, uint32_t)
INT_OPS(uint64_t, uint64_t)

/* uint16 * uint16 promotes to int in C and may overflow; redo PROD for the narrow unsigned types
 * through uint32_t so the wrap is defined. */
static void prod_u16(const uint16_t* in, uint16_t* io, int64_t n) {
    for (int64_t i = 0; i < n; i++) io[i] = (uint16_t)((uint32_t)in[i] * (uint32_t)io[i]);
}
static void prod_i16(const int16_t* in, int16_t* io, int64_t n) {
    for (int64_t i = 0; i < n; i++) io[i] = (int16_t)(uint16_t)((uint32_t)(uint16_t)in[i] * (uint32_t)(uint16_t)io[i]);
}

#define FLT_OPS(T)                                                                                \
    static void apply_##T(int op, const T* in, T* io, int64_t n) {                                \
        int64_t i;                                                                                \
        switch (op) {                                                                             \
        case GPUMPI_OP_MAX: for (i = 0; i < n; i++) io[i] = in[i] > io[i] ? in[i] : io[i]; break; \
        case GPUMPI_OP_MIN: for (i = 0; i < n; i++) io[i] = in[i] > io[i] ? io[i] : in[i]; break; \
        case GPUMPI_OP_SUM: for (i = 0; i < n; i++) io[i] = in[i] + io[i]; break;                 \
        case GPUMPI_OP_PROD: for (i = 0; i < n; i++) io[i] = in[i] * io[i]; break;                \
        }                                                                                         \
    }
FLT_OPS(float)
FLT_OPS(double)

/* complex: (a+bi)(c+di) = (ac - bd) + (ad + bc)i, each product and sum rounded separately */
#define CPX_OPS(T)                                                                                \
    static void apply_c##T(int op, const T* in, T* io, int64_t n) {                               \
        for (int64_t i = 0; i < n; i++) {                                                         \
            T a = in[2 * i], b = in[2 * i + 1], c = io[2 * i], d = io[2 * i + 1];                 \
            if (op == GPUMPI_OP_SUM) { io[2 * i] = a + c; io[2 * i + 1] = b + d; }                \
            else { T ac = a * c, bd = b * d, ad = a * d, bc = b * c; io[2 * i] = ac - bd;         \
                   io[2 * i + 1] = ad + bc; }                                                     \
        }                                                                                         \
    }
CPX_OPS(float)
CPX_OPS(double)

static void apply_bool(int op, const uint8_t* in, uint8_t* io, int64_t n) {
    for (int64_t i = 0; i < n; i++) {
        int a = in[i] != 0, b = io[i] != 0;
        if (op == GPUMPI_OP_LAND) io[i] = (uint8_t)(a && b);
        else if (op == GPUMPI_OP_LOR) io[i] = (uint8_t)(a || b);
        else io[i] = (uint8_t)(a != b);
    }
}

/* MAXLOC / MINLOC with the tie rule of gpu_libs/gpu_mpi/operators.cu:100-151 (lower index wins) */
#define PAIR_OPS(NAME, VT, PAD)                                                                   \
    typedef struct { VT val; PAD int idx; } NAME##_t;                                             \
    static void apply_##NAME(int op, const NAME##_t* in, NAME##_t* io, int64_t n) {               \
        for (int64_t i = 0; i < n; i++) {                                                         \
            NAME##_t a = in[i], b = io[i], c;                                                     \
            if (a.val > b.val) c = (op == GPUMPI_OP_MAXLOC) ? a : b;                              \
            else if (a.val < b.val) c = (op == GPUMPI_OP_MAXLOC) ? b : a;                         \
            else c = a.idx < b.idx ? a : b;                                                       \
            io[i] = c;                                                                            \
        }                                                                                         \
    }
PAIR_OPS(p2int, int32_t, )
PAIR_OPS(pflt, float, )
PAIR_OPS(pdbl, double, )
PAIR_OPS(plong, int64_t, )
PAIR_OPS(pshort, int16_t, )

static int apply(int op, int dt, const void* in, void* io, int64_t n) {
    if (!orc_op_allowed(op, dt)) return GPUMPI_ERR_OP;
    switch (dt) {
    case GPUMPI_SIGNED_CHAR: case GPUMPI_INT8_T: apply_int8_t(op, in, io, n); break;
    case GPUMPI_UNSIGNED_CHAR: case GPUMPI_UINT8_T: apply_uint8_t(op, in, io, n); break;
    case GPUMPI_BYTE: apply_uint8_t(op, in, io, n); break;
    case GPUMPI_SHORT: case GPUMPI_INT16_T:
        if (op == GPUMPI_OP_PROD) prod_i16(in, io, n); else apply_int16_t(op, in, io, n);
        break;
    case GPUMPI_UNSIGNED_SHORT: case GPUMPI_UINT16_T:
        if (op == GPUMPI_OP_PROD) prod_u16(in, io, n); else apply_uint16_t(op, in, io, n);
        break;
    case GPUMPI_INT: case GPUMPI_INT32_T: apply_int32_t(op, in, io, n); break;
    case GPUMPI_UNSIGNED: case GPUMPI_UINT32_T: apply_uint32_t(op, in, io, n); break;
    case GPUMPI_LONG: case GPUMPI_LONG_LONG_INT: case GPUMPI_LONG_LONG: case GPUMPI_INT64_T:
        apply_int64_t(op, in, io, n); break;
    case GPUMPI_UNSIGNED_LONG: case GPUMPI_UNSIGNED_LONG_LONG: case GPUMPI_UINT64_T:
        apply_uint64_t(op, in, io, n); break;
    case GPUMPI_FLOAT: apply_float(op, in, io, n); break;
    case GPUMPI_DOUBLE: case GPUMPI_LONG_DOUBLE: apply_double(op, in, io, n); break;
    case GPUMPI_C_BOOL: apply_bool(op, in, io, n); break;
    case GPUMPI_C_COMPLEX: case GPUMPI_C_FLOAT_COMPLEX: apply_cfloat(op, in, io, n); break;
    case GPUMPI_C_DOUBLE_COMPLEX: case GPUMPI_C_LONG_DOUBLE_COMPLEX: apply_cdouble(op, in, io, n); break;
    case GPUMPI_2INT: apply_p2int(op, in, io, n); break;
    case GPUMPI_FLOAT_INT: apply_pflt(op, in, io, n); break;
    case GPUMPI_DOUBLE_INT: case GPUMPI_LONG_DOUBLE_INT: apply_pdbl(op, in, io, n); break;
    case GPUMPI_LONG_INT: apply_plong(op, in, io, n); break;
    case GPUMPI_SHORT_INT: apply_pshort(op, in, io, n); break;
    default: return GPUMPI_ERR_TYPE;
    }
    return GPUMPI_SUCCESS;
}

/* Canonical fold of MPI_Reduce, gpu_libs/gpu_mpi/mpi.cu:209-225: the result starts as rank 0's
 * data (copied at :218-221), then ranks 1..n-1 are folded in order with invokeOperator(op, x_s, out). */
int orc_reduce(const void* const* inputs, int n, void* out, int64_t count, int dt, int op) {
    int es = orc_type_size(dt);
    if (es <= 0) return GPUMPI_ERR_TYPE;
    if (n <= 0 || count < 0) return GPUMPI_ERR_COUNT;
    if (!orc_op_allowed(op, dt)) return GPUMPI_ERR_OP;
    memcpy(out, inputs[0], (size_t)(count * es));
    for (int s = 1; s < n; s++) {
        int rc = apply(op, dt, inputs[s], out, count);
        if (rc) return rc;
    }
    return GPUMPI_SUCCESS;
}

int orc_reduce_rm(const void* sendbufs, int64_t stride, int n, void* out, int64_t count, int dt, int op) {
    const void** in = (const void**)malloc(sizeof(void*) * (size_t)n);
    if (!in) return GPUMPI_ERR_NO_MEM;
    for (int s = 0; s < n; s++) in[s] = (const char*)sendbufs + (int64_t)s * stride;
    int rc = orc_reduce(in, n, out, count, dt, op);
    free(in);
    return rc;
}

/* ---- multi-threaded allreduce (CPU baseline): element ranges split across threads ---- */
typedef struct {
    const char* send; char* recv; int n; int64_t count, lo, hi; int dt, op, es, rc;
} ar_job;

static void* ar_worker(void* p) {
    ar_job* j = (ar_job*)p;
    int64_t len = j->hi - j->lo;
    if (len <= 0) return NULL;
    int64_t stride = j->count * j->es;
    char* out = j->recv + j->lo * j->es;        /* rank 0's recv slot holds the fold */
    memcpy(out, j->send + j->lo * j->es, (size_t)(len * j->es));
    for (int s = 1; s < j->n && !j->rc; s++)
        j->rc = apply(j->op, j->dt, j->send + (int64_t)s * stride + j->lo * j->es, out, len);
    for (int r = 1; r < j->n; r++)
        memcpy(j->recv + (int64_t)r * stride + j->lo * j->es, out, (size_t)(len * j->es));
    return NULL;
}

int orc_allreduce(const void* sendbufs, void* recvbufs, int n, int64_t count, int dt, int op, int threads) {
    int es = orc_type_size(dt);
    if (es <= 0) return GPUMPI_ERR_TYPE;
    if (!orc_op_allowed(op, dt)) return GPUMPI_ERR_OP;
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    ar_job jobs[256];
    pthread_t tids[256];
    int64_t per = (count + threads - 1) / threads;
    for (int t = 0; t < threads; t++) {
        ar_job* j = &jobs[t];
        j->send = (const char*)sendbufs; j->recv = (char*)recvbufs; j->n = n; j->count = count;
        j->lo = (int64_t)t * per; j->hi = j->lo + per < count ? j->lo + per : count;
        j->dt = dt; j->op = op; j->es = es; j->rc = 0;
    }
    if (threads == 1) { ar_worker(&jobs[0]); return jobs[0].rc; }
    for (int t = 0; t < threads; t++) pthread_create(&tids[t], NULL, ar_worker, &jobs[t]);
    int rc = 0;
    for (int t = 0; t < threads; t++) { pthread_join(tids[t], NULL); if (jobs[t].rc) rc = jobs[t].rc; }
    return rc;
}

/* ---- Alltoallv placement, gpu_libs/gpu_mpi/mpi.cu:363-408: receiver r's recvbuf + rdispls[s]*es
 * gets sender s's sendbuf + sdispls_s[r]*es; the local block is a plain copy (:393-395). ---- */
typedef struct {
    const char* send; int64_t ss; const int *sc, *sd; char* recv; int64_t rs; const int *rc_, *rd;
    int n, es, r0, r1, err;
} a2a_job;

static void* a2a_worker(void* p) {
    a2a_job* j = (a2a_job*)p;
    int n = j->n;
    for (int r = j->r0; r < j->r1; r++) {
        for (int s = 0; s < n; s++) {
            int64_t scount = j->sc[(int64_t)s * n + r], rcount = j->rc_[(int64_t)r * n + s];
            int64_t m = scount < rcount ? scount : rcount;
            if (scount > rcount) j->err = GPUMPI_ERR_TRUNCATE;
            const char* src = j->send + (int64_t)s * j->ss + (int64_t)j->sd[(int64_t)s * n + r] * j->es;
            char* dst = j->recv + (int64_t)r * j->rs + (int64_t)j->rd[(int64_t)r * n + s] * j->es;
            if (m > 0) memcpy(dst, src, (size_t)(m * j->es));
        }
    }
    return NULL;
}

int orc_alltoallv(const void* sendbufs, int64_t send_stride, const int* sendcounts, const int* sdispls,
                  void* recvbufs, int64_t recv_stride, const int* recvcounts, const int* rdispls,
                  int n, int esize, int threads) {
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    if (threads > n) threads = n;
    a2a_job jobs[256];
    pthread_t tids[256];
    int per = (n + threads - 1) / threads;
    for (int t = 0; t < threads; t++) {
        a2a_job* j = &jobs[t];
        j->send = (const char*)sendbufs; j->ss = send_stride; j->sc = sendcounts; j->sd = sdispls;
        j->recv = (char*)recvbufs; j->rs = recv_stride; j->rc_ = recvcounts; j->rd = rdispls;
        j->n = n; j->es = esize; j->r0 = t * per; j->r1 = (t + 1) * per < n ? (t + 1) * per : n;
        j->err = 0;
    }
    if (threads == 1) { a2a_worker(&jobs[0]); return jobs[0].err; }
    for (int t = 0; t < threads; t++) pthread_create(&tids[t], NULL, a2a_worker, &jobs[t]);
    int err = 0;
    for (int t = 0; t < threads; t++) { pthread_join(tids[t], NULL); if (jobs[t].err) err = jobs[t].err; }
    return err;
}

/* ------------------------------------------------------------------------------------------ */
/* derived datatypes, MPI-3.1 ch. 4 (type constructors, pack/unpack).  The reference stubs       */
/* MPI_Type_contiguous / MPI_Type_commit / MPI_Type_size (gpu_libs/gpu_mpi/mpi.cu:237-245,287-290)*/
/* ------------------------------------------------------------------------------------------ */
void orc_type_basic(int dt, orc_typemap* t) {
    memset(t, 0, sizeof(*t));
    int es = orc_type_size(dt);
    t->size = es; t->extent = es; t->lb = 0; t->block = es; t->nlev = 0;
}

static int is_contig(const orc_typemap* t) { return t->nlev == 0 && t->size == t->extent && t->lb == 0; }

static int add_level(const orc_typemap* old, int64_t count, int64_t stride, orc_typemap* out) {
    if (old->nlev >= 4) return GPUMPI_ERR_TYPE;
    *out = *old;
    out->cnt[out->nlev] = count;
    out->stride[out->nlev] = stride;
    out->nlev++;
    return 0;
}

int orc_type_contiguous(int64_t count, const orc_typemap* old, orc_typemap* out) {
    return orc_type_hvector(count, 1, old->extent, old, out);
}

int orc_type_vector(int64_t count, int64_t blocklen, int64_t stride, const orc_typemap* old, orc_typemap* out) {
    return orc_type_hvector(count, blocklen, stride * old->extent, old, out);
}

int orc_type_hvector(int64_t count, int64_t blocklen, int64_t sbytes, const orc_typemap* old, orc_typemap* out) {
    if (count < 0 || blocklen < 0) return GPUMPI_ERR_COUNT;
    orc_typemap blk;
    int rc;
    /* the block of blocklen old elements */
    if (is_contig(old)) {
        blk = *old; blk.size = old->size * blocklen; blk.extent = blk.size; blk.block = blk.size;
    } else {
        if ((rc = add_level(old, blocklen, old->extent, &blk))) return rc;
        blk.size = old->size * blocklen;
        blk.extent = old->extent * blocklen;
    }
    if (count == 1) { *out = blk; out->extent = blk.extent; return 0; }
    if (is_contig(&blk) && sbytes == blk.extent) {
        *out = blk; out->size = blk.size * count; out->extent = out->size; out->block = out->size; return 0;
    }
    if ((rc = add_level(&blk, count, sbytes, out))) return rc;
    out->size = blk.size * count;
    out->lb = 0;
    out->extent = (count - 1) * sbytes + blk.extent;   /* non-negative strides only */
    return 0;
}

int orc_type_subarray(int ndims, const int* sizes, const int* subsizes, const int* starts,
                      const orc_typemap* old, orc_typemap* out) {
    if (ndims < 1 || ndims > 3 || !is_contig(old)) return GPUMPI_ERR_TYPE;
    int64_t es = old->extent;
    /* innermost dimension is contiguous */
    orc_typemap t = *old;
    t.size = es * subsizes[ndims - 1]; t.extent = t.size; t.block = t.size; t.nlev = 0;
    int64_t stride = es * sizes[ndims - 1];
    int64_t offset = es * starts[ndims - 1];
    for (int d = ndims - 2; d >= 0; d--) {
        orc_typemap nt;
        int rc = add_level(&t, subsizes[d], stride, &nt);
        if (rc) return rc;
        nt.size = t.size * subsizes[d];
        t = nt;
        offset += stride * starts[d];
        stride *= sizes[d];
    }
    /* full array extent, data starts at `offset` (encoded as lb) */
    t.lb = offset;
    t.extent = stride;
    *out = t;
    return 0;
}

/* visit contiguous blocks of `count` elements of type t: callback(byte offset, bytes) */
#define VISIT_BLOCKS(t, count, BODY)                                                              \
    do {                                                                                          \
        int64_t c0_, c1_, c2_, c3_;                                                               \
        int64_t n0 = (t)->nlev > 0 ? (t)->cnt[0] : 1, s0 = (t)->nlev > 0 ? (t)->stride[0] : 0;    \
        int64_t n1 = (t)->nlev > 1 ? (t)->cnt[1] : 1, s1 = (t)->nlev > 1 ? (t)->stride[1] : 0;    \
        int64_t n2 = (t)->nlev > 2 ? (t)->cnt[2] : 1, s2 = (t)->nlev > 2 ? (t)->stride[2] : 0;    \
        int64_t n3 = (t)->nlev > 3 ? (t)->cnt[3] : 1, s3 = (t)->nlev > 3 ? (t)->stride[3] : 0;    \
        for (int64_t e_ = 0; e_ < (count); e_++)                                                  \
            for (c3_ = 0; c3_ < n3; c3_++)                                                        \
                for (c2_ = 0; c2_ < n2; c2_++)                                                    \
                    for (c1_ = 0; c1_ < n1; c1_++)                                                \
                        for (c0_ = 0; c0_ < n0; c0_++) {                                          \
                            int64_t off_ = (t)->lb + e_ * (t)->extent + c3_ * s3 + c2_ * s2 +     \
                                           c1_ * s1 + c0_ * s0;                                   \
                            int64_t len_ = (t)->block;                                            \
                            BODY                                                                  \
                        }                                                                         \
    } while (0)

int64_t orc_pack(const orc_typemap* t, int64_t count, const void* src, void* packed) {
    int64_t pos = 0;
    VISIT_BLOCKS(t, count, { memcpy((char*)packed + pos, (const char*)src + off_, (size_t)len_); pos += len_; });
    return pos;
}

int64_t orc_unpack(const orc_typemap* t, int64_t count, const void* packed, void* dst) {
    int64_t pos = 0;
    VISIT_BLOCKS(t, count, { memcpy((char*)dst + off_, (const char*)packed + pos, (size_t)len_); pos += len_; });
    return pos;
}

/* ------------------------------------------------------------------------------------------ */
/* synthetic inputs                                                                             */
/* ------------------------------------------------------------------------------------------ */
uint64_t orc_lcg_next(uint64_t* s) {
    *s = *s * 6364136223846793005ULL + 1442695040888963407ULL;
    return *s;
}

double orc_lcg_u01(uint64_t* s) { return (double)(orc_lcg_next(s) >> 11) * (1.0 / 9007199254740992.0); }

void orc_fill_f32(uint64_t seed, int64_t n, float* out) {
    uint64_t s = seed;
    for (int64_t i = 0; i < n; i++) out[i] = (float)(orc_lcg_u01(&s) * 2.0 - 1.0);
}

void orc_fill_f64(uint64_t seed, int64_t n, double* out) {
    uint64_t s = seed;
    for (int64_t i = 0; i < n; i++) out[i] = orc_lcg_u01(&s) * 2.0 - 1.0;
}

void orc_fill_i32(uint64_t seed, int64_t n, int32_t* out) {
    uint64_t s = seed;
    for (int64_t i = 0; i < n; i++) out[i] = (int32_t)(uint32_t)(orc_lcg_next(&s) >> 32);
}

int64_t orc_pi_hits(uint64_t seed, int rank, int64_t pairs) {
    uint64_t s = seed + (uint64_t)rank;
    int64_t hits = 0;
    for (int64_t i = 0; i < pairs; i++) {
        double x = orc_lcg_u01(&s);
        double y = orc_lcg_u01(&s);
        double xx = x * x;
        double yy = y * y;
        if (xx + yy < 1.0) hits++;
    }
    return hits;
}

void orc_bucket_keys(uint64_t seed, int rank, int64_t nkeys, int32_t* keys) {
    uint64_t s = seed + (uint64_t)rank;
    for (int64_t i = 0; i < nkeys; i++) {
        double a = orc_lcg_u01(&s);
        double b = orc_lcg_u01(&s);
        double c = orc_lcg_u01(&s);
        double d = orc_lcg_u01(&s);
        double sum = ((a + b) + c) + d;
        keys[i] = (int32_t)floor(sum * 524288.0); /* 2^21 * sum / 4 */
    }
}

int orc_bucket_sort(const int32_t* keys, int n, int64_t kpr, int32_t* out, int64_t cap, int64_t* out_counts) {
    /* bucket of key k on n ranks: (k * n) >> 21, so rank r receives exactly the keys in
     * [ceil(r 2^21 / n), ceil((r + 1) 2^21 / n)); its sorted output is that range of the global
     * histogram expanded in increasing key order */
    const int64_t max_key = (int64_t)1 << 21;
    int64_t* hist = (int64_t*)calloc((size_t)max_key, sizeof(int64_t));
    if (!hist) return GPUMPI_ERR_NO_MEM;
    for (int64_t i = 0; i < (int64_t)n * kpr; i++) {
        const int64_t k = keys[i];
        if (k < 0 || k >= max_key) { free(hist); return GPUMPI_ERR_ARG; }
        hist[k]++;
    }
    for (int r = 0; r < n; r++) {
        const int64_t lo = (max_key * r + n - 1) / n, hi = (max_key * (r + 1) + n - 1) / n;
        int64_t cnt = 0;
        for (int64_t k = lo; k < hi; k++) cnt += hist[k];
        out_counts[r] = cnt;
        if (cnt > cap) { free(hist); return GPUMPI_ERR_COUNT; }
        int32_t* o = out + (int64_t)r * cap;
        int64_t pos = 0;
        for (int64_t k = lo; k < hi; k++)
            for (int64_t c = 0; c < hist[k]; c++) o[pos++] = (int32_t)k;
    }
    free(hist);
    return 0;
}

double orc_halo_value(int64_t gz, int64_t gy, int64_t gx) {
    return (double)(gz * 1000003 + gy * 1009 + gx) * 0.125;
}

void orc_halo_expected(int P, int L, int rank, double* block) {
    int64_t G = (int64_t)P * L, W = L + 2;
    int px = rank % P, py = (rank / P) % P, pz = rank / (P * P);
    for (int64_t z = 0; z < W; z++)
        for (int64_t y = 0; y < W; y++)
            for (int64_t x = 0; x < W; x++) {
                int out = (z == 0 || z == W - 1) + (y == 0 || y == W - 1) + (x == 0 || x == W - 1);
                double v;
                if (out > 1) v = -1.0;   /* edges and corners are not exchanged */
                else {
                    int64_t gz = ((int64_t)pz * L + z - 1 + G) % G;
                    int64_t gy = ((int64_t)py * L + y - 1 + G) % G;
                    int64_t gx = ((int64_t)px * L + x - 1 + G) % G;
                    v = orc_halo_value(gz, gy, gx);
                }
                block[(z * W + y) * W + x] = v;
            }
}

void orc_comm_split(int n, const int* colors, const int* keys, int* newrank, int* newsize) {
    for (int r = 0; r < n; r++) {
        if (colors[r] == GPUMPI_UNDEFINED) { newrank[r] = -1; newsize[r] = 0; continue; }
        int rank = 0, size = 0;
        for (int q = 0; q < n; q++) {
            if (colors[q] != colors[r]) continue;
            size++;
            if (keys[q] < keys[r] || (keys[q] == keys[r] && q < r)) rank++;
        }
        newrank[r] = rank; newsize[r] = size;
    }
}

/* ------------------------------------------------------------------------------------------ */
/* MLP 12 -> 64 -> 64 -> 4, ReLU hidden layers, loss = (1/B) sum_b sum_o mask (y - t)^2          */
/* ------------------------------------------------------------------------------------------ */
#define W1_OFF 0
#define B1_OFF (W1_OFF + 64 * 12)
#define W2_OFF (B1_OFF + 64)
#define B2_OFF (W2_OFF + 64 * 64)
#define W3_OFF (B2_OFF + 64)
#define B3_OFF (W3_OFF + 4 * 64)

void orc_mlp_forward(const double* p, const double* x, int batch, double* y) {
    for (int b = 0; b < batch; b++) {
        double h1[64], h2[64];
        const double* xb = x + (int64_t)b * 12;
        for (int j = 0; j < 64; j++) {
            double a = p[B1_OFF + j];
            for (int i = 0; i < 12; i++) a += p[W1_OFF + j * 12 + i] * xb[i];
            h1[j] = a > 0 ? a : 0;
        }
        for (int j = 0; j < 64; j++) {
            double a = p[B2_OFF + j];
            for (int i = 0; i < 64; i++) a += p[W2_OFF + j * 64 + i] * h1[i];
            h2[j] = a > 0 ? a : 0;
        }
        for (int o = 0; o < 4; o++) {
            double a = p[B3_OFF + o];
            for (int i = 0; i < 64; i++) a += p[W3_OFF + o * 64 + i] * h2[i];
            y[(int64_t)b * 4 + o] = a;
        }
    }
}

double orc_mlp_loss_grad(const double* p, const double* x, const double* t, const double* mask,
                         int batch, double* g) {
    if (!t) return 0.0;
    if (g) memset(g, 0, sizeof(double) * ORC_MLP_NPARAMS);
    double loss = 0.0;
    for (int b = 0; b < batch; b++) {
        double z1[64], h1[64], z2[64], h2[64], y[4], dy[4], dh2[64], dz2[64], dh1[64], dz1[64];
        const double* xb = x + (int64_t)b * 12;
        for (int j = 0; j < 64; j++) {
            double a = p[B1_OFF + j];
            for (int i = 0; i < 12; i++) a += p[W1_OFF + j * 12 + i] * xb[i];
            z1[j] = a; h1[j] = a > 0 ? a : 0;
        }
        for (int j = 0; j < 64; j++) {
            double a = p[B2_OFF + j];
            for (int i = 0; i < 64; i++) a += p[W2_OFF + j * 64 + i] * h1[i];
            z2[j] = a; h2[j] = a > 0 ? a : 0;
        }
        for (int o = 0; o < 4; o++) {
            double a = p[B3_OFF + o];
            for (int i = 0; i < 64; i++) a += p[W3_OFF + o * 64 + i] * h2[i];
            y[o] = a;
            double m = mask ? mask[(int64_t)b * 4 + o] : 1.0;
            double d = y[o] - t[(int64_t)b * 4 + o];
            loss += m * d * d;
            dy[o] = 2.0 * m * d / batch;
        }
        if (!g) continue;
        for (int i = 0; i < 64; i++) dh2[i] = 0;
        for (int o = 0; o < 4; o++) {
            g[B3_OFF + o] += dy[o];
            for (int i = 0; i < 64; i++) {
                g[W3_OFF + o * 64 + i] += dy[o] * h2[i];
                dh2[i] += p[W3_OFF + o * 64 + i] * dy[o];
            }
        }
        for (int j = 0; j < 64; j++) dz2[j] = z2[j] > 0 ? dh2[j] : 0;
        for (int i = 0; i < 64; i++) dh1[i] = 0;
        for (int j = 0; j < 64; j++) {
            g[B2_OFF + j] += dz2[j];
            for (int i = 0; i < 64; i++) {
                g[W2_OFF + j * 64 + i] += dz2[j] * h1[i];
                dh1[i] += p[W2_OFF + j * 64 + i] * dz2[j];
            }
        }
        for (int j = 0; j < 64; j++) dz1[j] = z1[j] > 0 ? dh1[j] : 0;
        for (int j = 0; j < 64; j++) {
            g[B1_OFF + j] += dz1[j];
            for (int i = 0; i < 12; i++) g[W1_OFF + j * 12 + i] += dz1[j] * xb[i];
        }
    }
    return loss / batch;
}
