/*
 * gpumpi.h — host C ABI of the block-rank MPI runtime (libgpumpi.so).
 *
 * Plain C: opaque handles, plain pointers and sizes, no CUDA or torch types in the signatures
 * (streams are passed as void*, a cudaStream_t or NULL for the world's own stream; the world's stream is
 * non-blocking, so a caller whose buffers were produced on another stream passes that stream).
 *
 * What each entry point replaces in the reference (lilyyangyn/dphpc-gpu_mpi):
 *   gpumpi_config_init / gpumpi_parse_args  <- parseGPUMPIArgs and its defaults,
 *                                               gpu_libs/gpu_main/main.cu:48-97 (---gpumpi -n -g -b -s -p -e)
 *   gpumpi_world_create / _destroy          <- SharedState::Holder + ThreadPrivateState::Context set-up,
 *                                               gpu_libs/gpu_libc/cuda_mpi.cuh:459-502, main.cu:210-278
 *   gpumpi_run_program                      <- the launch of __gpu_main_caller and the host wait loop,
 *                                               main.cu:280-320 (co-residency check main.cu:188-208)
 *   gpumpi_test_run                         <- TestRunner::run<Kernel>(), tests/test_runner.cuh:26-86
 *   gpumpi_allreduce / _reduce / _bcast /   <- one MPI_Allreduce / MPI_Reduce / MPI_Bcast / MPI_Alltoall /
 *   _alltoall / _alltoallv / _allgather        MPI_Alltoallv / MPI_Allgather call made by every rank of a
 *                                               launch (gpu_libs/gpu_mpi/mpi.cu:276-282,181-235,101-140,
 *                                               333-408,410-419) — the hot path, callable from the host
 *   gpumpi_pingpong / gpumpi_ring           <- MPI_Send/MPI_Recv loops of benchmarks/mpi_communication/
 *                                               mpi_communication.c:10-55 (point-to-point benchmark)
 *   gpumpi_last_error                       <- CudaMPI::printLastError, gpu_libs/gpu_libc/assert.cu:58-71
 *
 * Buffers: every data pointer may be device memory or host memory (pageable or pinned); pageable host
 * memory is staged through device memory inside the call (the host<->device copies are part of the
 * call), page-locked host memory is read and written in place by the kernel; a large Allreduce between
 * host buffers runs as column slices whose copies overlap (GPUMPI_TUNE_HOST_DIRECT).
 * Rank-major layout: rank r's buffer starts at base + r * stride_bytes.
 * Return value: GPUMPI_SUCCESS (0) or an error code from gpumpi_abi.h; never aborts the process.
 */
#ifndef GPUMPI_H
#define GPUMPI_H

#include <stddef.h>
#include <stdint.h>

#include "gpumpi_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gpumpi_world gpumpi_world;

typedef struct gpumpi_config {
    int nranks;               /* -n: MPI ranks = thread blocks */
    int threads_per_block;    /* -b: 0 = pick from occupancy (largest of 256/128/64 that fits) */
    int engine_blocks;        /* copy-engine blocks beside the ranks; -1 = fill the GPU, 0 = none */
    int pending_requests;     /* -e: request slots per rank (reference default 1024) */
    int mailbox_depth;        /* envelope ring slots per rank (power of two) */
    int unexpected_depth;     /* unexpected-message queue depth per rank */
    int eager_bytes;          /* messages up to this size travel inline (multiple of 16) */
    int max_types;            /* derived datatypes per rank */
    int posted_depth;         /* posted receives per rank */
    int device;               /* CUDA device ordinal */
    size_t stack_bytes;       /* -s: per-thread stack limit */
    size_t heap_bytes;        /* -p: device malloc heap (0 = 1 GiB) */
    size_t arena_bytes;       /* communicator objects created at run time */
    long long copy_chunk_bytes;   /* chunk of large point-to-point copies shared with engines */
    long long engine_min_bytes;   /* jobs smaller than this are not offered to engine blocks */
    double timeout_s;         /* bound on every device-side wait */
    int trace_capacity;       /* per-call timing records kept (0 = tracing off) */
    long long host_window_bytes;  /* per-rank payload window of the device -> host channel (file and
                                     stream I/O); 0 = 16 MiB / ranks, 4 KiB .. 1 MiB; -1 = no channel */
} gpumpi_config;

typedef struct gpumpi_world_info {
    int nranks, threads_per_block, engine_blocks, blocks_per_sm, sm_count, device;
    size_t device_bytes;      /* device memory held by the world */
} gpumpi_world_info;

/* generic parameters of a built-in device program */
typedef struct gpumpi_params {
    long long i[16];
    double d[4];
    void* p[16];
} gpumpi_params;

/* built-in device programs (each runs on every rank of a launch) */
enum gpumpi_program {
    /* mirrors of the reference's GPU tests (tests/cuda_mpi_test.cu, collectives_test.cu, communicator_test.cu,
     * sample_test.cu): p[0] = uint8 ok[nranks], p[1] = int64 out[nranks * 64], p[2] = double out[nranks * 64] */
    GPUMPI_T_SINGLE_INT = 1,
    GPUMPI_T_TRANSFER_ARRAY,
    GPUMPI_T_SEND_RECV,
    GPUMPI_T_REPEAT_SEND_RECV,
    GPUMPI_T_NETWORK_FLOOD,
    GPUMPI_T_ALL_TO_ALL,
    GPUMPI_T_REDUCE_INT16_PROD,
    GPUMPI_T_ALLREDUCE_F64,
    GPUMPI_T_ALLGATHER,
    GPUMPI_T_SCATTER,
    GPUMPI_T_SCATTERV,
    GPUMPI_T_COMM_RANK,
    GPUMPI_T_COMM_DUP,
    GPUMPI_T_COMM_SPLIT,
    GPUMPI_T_SAMPLE,
    GPUMPI_T_P2P_MATCHING,     /* wildcards, ordering, probe, sendrecv, proc_null */
    GPUMPI_T_TIMEOUT,          /* a receive nobody sends to: bounded wait returns MPI_ERR_OTHER */
    GPUMPI_T_DATATYPES,        /* vector / subarray / contiguous send-recv round trips */
    GPUMPI_T_SUBCOMM_COLL,     /* collectives on split communicators */
    GPUMPI_T_ERRORS,           /* argument errors return codes, never trap */
    GPUMPI_T_CART,             /* Cartesian topologies: dims, coords, shifts, sub-grids, exchange */
    GPUMPI_T_TINY_STRESS,      /* back-to-back tiny collectives with skewed ranks, every result checked */
    GPUMPI_T_TINY_MIXED,       /* small collectives mixing thread-local/global buffers and datatypes */
    GPUMPI_T_ATTRS,            /* keyvals and cached attributes, MPI_Wtime / MPI_Wtick */
    GPUMPI_T_FILE_IO,          /* MPI-IO and gpumpi stdio over the host channel; p[3] = directory */
    /* hot-path programs */
    GPUMPI_P_COLL = 100,       /* i[0]=kind i[1]=count i[2]=dt i[3]=op i[4]=root i[5]=iters i[6]=send stride
                                  i[7]=recv stride i[8]=variant p[0]=send p[1]=recv p[2..5]=count/displ matrices
                                  p[6]=uint64 iter_ns[iters] p[7]=int rc[nranks] */
    GPUMPI_P_PINGPONG,         /* i[0]=bytes i[1]=iters i[2]=mode(0 blocking,1 nonblocking) i[3]=pairs
                                  p[0]=buffers (rank-major, stride i[4]) p[6]=iter_ns p[7]=rc */
    GPUMPI_P_RING,             /* i[0]=bytes i[1]=iters i[2]=mode i[4]=stride p[0]=send p[1]=recv p[6] p[7] */
    GPUMPI_P_PI,               /* i[0]=seed i[1]=pairs per rank p[0]=int64 hits[nranks] p[1]=int64 total p[7]=rc */
    GPUMPI_P_BUCKET_SORT,      /* see bench / tests */
    GPUMPI_P_HALO,
    GPUMPI_P_BATCH,            /* i[0]=communicators (<= 64) i[1]=iters i[2]=datatype i[3]=op
                                  p[0]=send base p[1]=recv base p[2]=int64 [comms][4] {first world rank,
                                  size, count, element offset} p[5]=int64[2] rank 0's setup ns (group
                                  calls, MPI_Comm_create; may be NULL) p[6]=int64 ns per iteration p[7]=rc */
};

/* collective kinds for GPUMPI_P_COLL */
enum gpumpi_coll_kind {
    GPUMPI_COLL_ALLREDUCE = 0,
    GPUMPI_COLL_REDUCE,
    GPUMPI_COLL_BCAST,
    GPUMPI_COLL_ALLTOALL,
    GPUMPI_COLL_ALLTOALLV,
    GPUMPI_COLL_ALLGATHER,
    GPUMPI_COLL_GATHER,
    GPUMPI_COLL_SCATTER,
    GPUMPI_COLL_BARRIER,
    GPUMPI_COLL_ALLGATHERV,
    GPUMPI_COLL_GATHERV,
    GPUMPI_COLL_SCATTERV,
};

int gpumpi_config_init(gpumpi_config* cfg);
/* Parses the options after "---gpumpi" into cfg; returns the index of "---gpumpi" (= the user's argc)
 * or -1 when it is absent. */
int gpumpi_parse_args(int argc, char** argv, gpumpi_config* cfg);

int gpumpi_world_create(const gpumpi_config* cfg, gpumpi_world** out);
int gpumpi_world_destroy(gpumpi_world* w);
int gpumpi_world_get_info(gpumpi_world* w, gpumpi_world_info* info);
/* Text of the last error of this world (or of the last failed create when w is NULL). */
const char* gpumpi_last_error(gpumpi_world* w);

/* Variant policy for reductions: variant >= 0 forces one, -1 lets the selector decide;
 * mode 0 = plain (DIRECT), 1 = tuned table, 2 = learned MLP. */
int gpumpi_set_policy(gpumpi_world* w, int variant, int mode);
/* Autotuner knobs: GPUMPI_TUNE_VEC (elements per thread of fold chunks, 0 = auto),
 * GPUMPI_TUNE_STAGE_GROUP (ranks per STAGED stage, 0 = auto), GPUMPI_TUNE_ENGINES (copy-engine blocks,
 * -1 = fill the GPU), GPUMPI_TUNE_COPY_CHUNK (bytes), GPUMPI_TUNE_ENGINE_MIN_BYTES (bytes). */
#define GPUMPI_TUNE_VEC 1
#define GPUMPI_TUNE_STAGE_GROUP 2
#define GPUMPI_TUNE_ENGINES 3
#define GPUMPI_TUNE_COPY_CHUNK 4
#define GPUMPI_TUNE_ENGINE_MIN_BYTES 5
/* Learned policy: predicted log-time gain (in 1/1000) the network needs to override the tuned table,
 * for Allreduce / Reduce (MARGIN) and for Alltoall(v) (MARGIN_PULL). */
#define GPUMPI_TUNE_MLP_MARGIN 6
#define GPUMPI_TUNE_MLP_MARGIN_PULL 9
/* Dynamic shared memory per rank block at most, in bytes (default 8192; -1 = all the SM leaves over).
 * It holds the TMA stages of the STAGED variants and block-parallel user scratch; what it does not take
 * stays L1 cache, which the executors' spilled registers and the ranks' private state use. */
#define GPUMPI_TUNE_DYN_SMEM 7
/* GPUMPI_TUNE_HOST_DIRECT: how page-locked host buffers reach the kernel.  1 = read and written in place
 * by the kernel through their device alias (every byte crosses the host link once; the STAGED variants
 * then run as DIRECT); 0 = staged through device memory around the kernel.  2..4 = an Allreduce between
 * host buffers (one call, no per-iteration times, rows 16-byte multiples) runs as column slices, one
 * launch per slice, so inputs of later slices cross the host link while results of earlier ones cross
 * back: 2 = both directions by 2D copies through device staging, 3 (default) = page-locked inputs read in
 * place and results copied back, 4 = inputs copied and page-locked results written in place.  Every
 * element is folded as in one launch.  Other calls treat 2..4 as 1. */
#define GPUMPI_TUNE_HOST_DIRECT 8
/* GPUMPI_TUNE_HOST_SLICE: column slice of the sliced host-buffer Allreduce, bytes per rank (0 = auto:
 * 256 MiB per slice over all ranks, at least 128 KiB per rank; rounded up to 256 bytes, at most 64
 * slices; a call that would take one slice runs as one launch). */
#define GPUMPI_TUNE_HOST_SLICE 10
/* GPUMPI_TUNE_HOST_STREAMS: copy streams per direction of the sliced host-buffer Allreduce (1..4): each
 * slice's 2D copy is split into that many row groups copied concurrently. */
#define GPUMPI_TUNE_HOST_STREAMS 11
/* GPUMPI_TUNE_STATIC_FOLD: an Allreduce / Reduce of more than 64 bytes and at most this many bytes per member,
 * with at most one chunk (a block's threads' elements) per member, runs without a job: the members split
 * the chunks statically between two barriers (0 = always the job path; default 4 KiB). */
#define GPUMPI_TUNE_STATIC_FOLD 13
/* GPUMPI_TUNE_STATIC_BCAST: a Bcast of more than 64 bytes and at most this many runs without a job, every
 * member copying its piece from the root between two barriers (0 = always the job path; default 64 KiB). */
#define GPUMPI_TUNE_STATIC_BCAST 14
/* GPUMPI_TUNE_STATIC_PULL: an Alltoallv among at most 512 members whose members receive about this many bytes
 * or fewer (the estimate of the variant choice, from 8 members' counts) runs without a job: every member
 * pulls its own pieces from the senders between two barriers (0 = always the job path; default 128 KiB). */
#define GPUMPI_TUNE_STATIC_PULL 15
/* GPUMPI_TUNE_PULL_CHUNKS: a pull job (Alltoall(v), Allgather(v), Gather(v), Scatter(v), Bcast) whose pieces
 * are under 64 KiB is cut into about this many chunks per worker block (1..64; default 2). */
#define GPUMPI_TUNE_PULL_CHUNKS 16
int gpumpi_set_tuning(gpumpi_world* w, int key, long long value);
/* Launcher of a converted program (the reference's gpu_main): argv holds the program's arguments, then
 * optionally `---gpumpi` and the run's options (gpumpi_parse_args); creates the world, runs `program` on
 * every rank with the program's arguments copied to the device, and returns the process exit status:
 * 1 when the run failed or any rank returned non-zero (the reason on stderr), else 0. */
int gpumpi_main(int argc, char** argv, int program);
/* Program id of a converted program linked by the program builder (csrc/host/user_main.cu). */
#define GPUMPI_P_USER 200
/* The current value of a GPUMPI_TUNE_* knob. */
int gpumpi_get_tuning(gpumpi_world* w, int key, long long* value);
/* Tuned table: int8 [3][3][2][32][16] (kind: 0 Allreduce, 1 Reduce, 2 Alltoall/Alltoallv; datatype
 * class: 0 MPI_FLOAT, 1 MPI_DOUBLE / MPI_LONG_DOUBLE, 2 every other type; alignment class: 0 when every
 * member's buffers are 16-byte aligned, else 1; log2 bytes per rank; log2 ranks) -> variant or -1, host
 * memory.  A [3][2][32][16] table serves every datatype class, a [3][32][16] one every class of both
 * kinds; a [2][32][16] one leaves Alltoall(v) untuned. */
int gpumpi_set_tuned_table(gpumpi_world* w, const int8_t* table, size_t bytes);
/* Learned selector weights: float[GPUMPI_MLP_NPARAMS] in the layout of the training kernels. */
int gpumpi_set_mlp(gpumpi_world* w, const float* params, size_t count);
/* Timing trace: copies up to `cap` records {log2 bytes, log2 ranks, kind, variant, dt, op, us, aligned}
 * (32 bytes each) into host memory; returns the number of records written in *n. */
int gpumpi_read_trace(gpumpi_world* w, void* host_out, size_t cap, size_t* n);

/* Runs built-in program `program` on all ranks; blocks until it finished when sync != 0. */
int gpumpi_run_program(gpumpi_world* w, int program, const gpumpi_params* params, void* stream, int sync);
/* Recorded launches (no counterpart in the reference, which launches once per process): the reset,
 * runtime install and cooperative launch of `program` with `params`, captured into a CUDA graph once and
 * replayed by gpumpi_graph_launch.  The graph keeps the world's geometry, policy and tuning as they were
 * at creation; replays of one world must not overlap each other or other runs of that world. */
typedef struct gpumpi_graph gpumpi_graph;
int gpumpi_graph_create(gpumpi_world* w, int program, const gpumpi_params* params, gpumpi_graph** out);
/* Replays on `stream` (the world's stream when NULL); with sync != 0 waits and returns like run_program. */
int gpumpi_graph_launch(gpumpi_graph* g, void* stream, int sync);
int gpumpi_graph_destroy(gpumpi_graph* g);
/* Launch-time of the last run in milliseconds (CUDA events around the kernel). */
double gpumpi_last_kernel_ms(gpumpi_world* w);
/* How many kernels the library launched so far (all worlds). */
long long gpumpi_kernel_launches(void);

/* TestRunner equivalent: runs test program `test` on the world's ranks; ok[nranks] (host) receives
 * each rank's flag; outi/outd (host, nranks*64 each, may be NULL) receive the test's values. */
int gpumpi_test_run(gpumpi_world* w, int test, uint8_t* ok, int64_t* outi, double* outd);

/* Hot path from the host: every rank calls the collective `iters` times on its slice of the
 * rank-major buffers.  iter_ns (host, may be NULL) receives rank 0's per-call durations. */
int gpumpi_allreduce(gpumpi_world* w, const void* sendbuf, void* recvbuf, long long count, int datatype,
                     int op, int iters, uint64_t* iter_ns, void* stream);
int gpumpi_reduce(gpumpi_world* w, const void* sendbuf, void* recvbuf, long long count, int datatype, int op,
                  int root, int iters, uint64_t* iter_ns, void* stream);
int gpumpi_bcast(gpumpi_world* w, void* buf, long long count, int datatype, int root, int iters,
                 uint64_t* iter_ns, void* stream);
int gpumpi_alltoall(gpumpi_world* w, const void* sendbuf, void* recvbuf, long long count_per_pair, int datatype,
                    int iters, uint64_t* iter_ns, void* stream);
/* counts/displs: int32 [nranks][nranks] (row r = rank r's array); buffers with strides in bytes */
int gpumpi_alltoallv(gpumpi_world* w, const void* sendbuf, long long send_stride, const int* sendcounts,
                     const int* sdispls, void* recvbuf, long long recv_stride, const int* recvcounts,
                     const int* rdispls, int datatype, int iters, uint64_t* iter_ns, void* stream);
int gpumpi_allgather(gpumpi_world* w, const void* sendbuf, void* recvbuf, long long count, int datatype,
                     int iters, uint64_t* iter_ns, void* stream);
int gpumpi_pingpong(gpumpi_world* w, void* bufs, long long bytes, int pairs, int iters, int nonblocking,
                    uint64_t* iter_ns, void* stream);
int gpumpi_ring(gpumpi_world* w, const void* sendbuf, void* recvbuf, long long bytes, int iters, int nonblocking,
                uint64_t* iter_ns, void* stream);

/* Allocation-free MPI_Allreduce among `nranks` block-ranks (no counterpart in the reference).
 * For callers that cannot allocate device memory when they reduce — code inside an allocator or
 * memory-pool callback that must not re-enter the allocator, processes that reserve a fixed device-memory
 * budget up front, loops that cannot take cudaMalloc's device-wide synchronisation — this call allocates
 * nothing: its scratch (rank table, barrier words, chunk counter, error word) is a fixed static device
 * array of GPUMPI_NOALLOC_SCRATCH_BYTES that every GPU loading the library keeps until exit.
 * sendbuf/recvbuf are rank-major buffers of nranks * count elements in device memory of the current
 * device (else GPUMPI_ERR_BUFFER); nranks <= GPUMPI_NOALLOC_MAX_RANKS (else GPUMPI_ERR_ARG);
 * float/double/int32/int64 with SUM/MAX/MIN/PROD (else GPUMPI_ERR_TYPE).  Asynchronous on `stream`;
 * canonical rank order, bit-identical to gpumpi_allreduce.  All calls share the array: calls that
 * overlap on the GPU race.  The first call on a device looks up the array's address with that device
 * current; make it before any stream capture. */
#define GPUMPI_NOALLOC_MAX_RANKS 4096
#define GPUMPI_NOALLOC_SCRATCH_BYTES (64 * 1024 + 256)
int gpumpi_allreduce_noalloc(const void* sendbuf, void* recvbuf, long long count, int datatype, int op, int nranks,
                             void* stream);
/* Outcome of the most recent gpumpi_allreduce_noalloc on the current device, read from its error word
 * after the caller synchronised that call's stream: GPUMPI_SUCCESS, or GPUMPI_ERR_TIMEOUT when the
 * kernel's bounded grid barrier ran out (the kernel then returned without writing recvbuf). */
int gpumpi_allreduce_noalloc_status(void);
/* Test hook of the allocation-free allreduce's failure path: bounded-wait limit in seconds (0 = the
 * default 20 s) and arrivals its grid barrier waits for beyond the launched blocks (0 = none), so a
 * test can make the barrier run out without faulting the GPU.  (0, 0) restores the defaults. */
int gpumpi_noalloc_test_hook(double timeout_s, int missing_arrivals);

#define GPUMPI_MLP_NPARAMS (64 * 12 + 64 + 64 * 64 + 64 + 4 * 64 + 4)

/* The learned selector's network (12 -> 64 -> 64 -> 4, ReLU), trained on the GPU by these kernels.
 * All pointers are device buffers; params use the layout W1[64][12] b1[64] W2[64][64] b2[64] W3[4][64] b3[4].
 * x: [batch][12] features, t: [batch][4] target log-times, mask: [batch][4] (1 where measured).
 * No counterpart in the reference (it has one algorithm per collective). */
int gpumpi_mlp_forward(const float* params, const float* x, int batch, float* y, void* stream);
int gpumpi_mlp_loss_grad(const float* params, const float* x, const float* t, const float* mask, int batch,
                         float* grads, float* loss, void* stream);
int gpumpi_mlp_adam_step(float* params, const float* grads, float* m, float* v, int step, float lr, float wd,
                         void* stream);

#ifdef __cplusplus
}
#endif
#endif /* GPUMPI_H */
