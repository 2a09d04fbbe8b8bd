// rt_core.cuh — core state and primitives of the block-rank MPI runtime.
//
// Execution model (replaces the reference's one-thread-per-rank model of
// gpu_libs/gpu_main/main.cu:102-130 and its managed-memory SharedState, gpu_libs/gpu_libc/cuda_mpi.cuh:459-533):
//   * one persistent kernel; block b < nranks is MPI rank b, blocks >= nranks are copy-engine blocks;
//   * thread 0 of a rank block runs the (scalar) user program; threads 1..T-1 sleep on a named
//     barrier and wake up to execute bulk "block tasks" (copies, folds, chunks of collectives)
//     that thread 0 dispatches from inside MPI calls;
//   * all runtime state lives in device global memory; cross-block signalling uses gpu-scope
//     acquire/release operations (no managed memory, no system-scope atomics, no locks);
//   * every wait is bounded by a %globaltimer deadline and ends in an error code, never a trap.
#pragma once
#include <cstdint>
#include <cstddef>

#include "gpumpi_abi.h"
#include "mpi.h.cuh"
#include "rt_hostio.cuh"

namespace gpumpi {

// ------------------------------------------------------------------------------------------------
// memory-order primitives (gpu scope, global memory)
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long ld_acquire64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned ld_relaxed(const unsigned* p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long ld_relaxed64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_release64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned atom_add_acqrel(unsigned* p, unsigned v) {
    unsigned old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ unsigned long long atom_add_acqrel64(unsigned long long* p, unsigned long long v) {
    unsigned long long old;
    asm volatile("atom.acq_rel.gpu.global.add.u64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v) : "memory");
    return old;
}
__device__ __forceinline__ unsigned long long atom_add_relaxed64(unsigned long long* p, unsigned long long v) {
    unsigned long long old;
    asm volatile("atom.relaxed.gpu.global.add.u64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v) : "memory");
    return old;
}
// an add whose result nobody waits for (release: the caller's and, through a barrier, its block's earlier
// writes are visible to whoever acquires the new value)
__device__ __forceinline__ void red_add_release64(unsigned long long* p, unsigned long long v) {
    asm volatile("red.release.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long atom_exch_release64(unsigned long long* p, unsigned long long v) {
    unsigned long long old;
    asm volatile("atom.release.gpu.global.exch.b64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v) : "memory");
    return old;
}
// Spin-waits poll with relaxed loads and order what follows with this one fence once the awaited value is
// seen.  An acquire load or fence makes the SM drop its L1 contents, so acquire-polling from any block
// (idle copy engines, a rank waiting for a message) would turn every cached read of the other blocks on
// that SM (runtime tables, descriptors, spilled registers' lines) into an L2 round trip.
__device__ __forceinline__ void fence_acqrel() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

__device__ __forceinline__ unsigned long long now_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Named barrier that divergent threads may reach from different program points (non-.aligned
// form; per-thread arrival on sm_70+).  Id 0 is left to __syncthreads.
__device__ __forceinline__ void bar_sync(int id, int nthreads) {
    asm volatile("barrier.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}
enum { BAR_CMD = 1, BAR_DONE = 2, BAR_TASK = 3 };

__device__ __forceinline__ bool is_global_ptr(const void* p) {
    unsigned r;
    asm("{ .reg .pred q; isspacep.global q, %1; selp.u32 %0, 1, 0, q; }" : "=r"(r) : "l"(p));
    return r != 0;
}
__device__ __forceinline__ bool is_shared_ptr(const void* p) {
    unsigned r;
    asm("{ .reg .pred q; isspacep.shared q, %1; selp.u32 %0, 1, 0, q; }" : "=r"(r) : "l"(p));
    return r != 0;
}

// ------------------------------------------------------------------------------------------------
// datatype descriptors (predefined and derived)
// ------------------------------------------------------------------------------------------------
// What a typed copy reads of a datatype, laid out for six 16-byte loads (filled by desc_prepare in
// rt_types.cuh): the 32-bit mapping of a packed offset to a byte address.
struct alignas(16) TypeImg {
    unsigned d[4];        // divisors: size, block, cnt[0], cnt[1] (1 where unused)
    unsigned m[4];        // their FastDiv multipliers
    unsigned sh[4];       //   and shifts, s1 | s2 << 8
    long long lb, extent;
    long long st[3];      // strides of levels 0..2
    int nlev;
    int fast_unit;        // copy unit when the 32-bit mapping applies (size < 2^31, <= 3 levels), else 0
};

struct TypeDesc {
    long long size;       // bytes of data in one element
    long long extent;     // lb..ub span
    long long lb;         // byte offset of the first data byte
    long long block;      // contiguous bytes at the innermost level
    int nlev;             // strided levels (0 = one contiguous block)
    int base;             // predefined element type all blocks consist of (or -1)
    long long cnt[4];
    long long stride[4];
    int committed;
    int in_use;
    // set when the type is built (desc_prepare in rt_types.cuh):
    int unit;             // largest power of two (<= 16) dividing block, size, extent, lb and the strides
    int fd_ready;         // the 32-bit mapping applies: size < 2^31 and at most 3 levels
    TypeImg img;          // the mapping image (all zero, i.e. not ready, for the predefined types)
};

// ------------------------------------------------------------------------------------------------
// chunked work ("jobs"): a collective instance or a large point-to-point copy, split into chunks
// that any block (rank or engine) may claim with one atomic.
//   next  = (epoch << 32) | next chunk index     (claimed with atomicAdd)
//   limit = (epoch << 32) | number of chunks     (written before next is reset)
//   done  = (epoch << 32) | finished chunks
// ------------------------------------------------------------------------------------------------
enum JobKind {
    JOB_NONE = 0,
    JOB_COPY,         // contiguous bytes src -> dst (point-to-point rendezvous / local copies)
    JOB_ALLREDUCE,    // fold all members' sendbufs, write every member's recvbuf
    JOB_REDUCE,       // fold all members' sendbufs, write root's recvbuf
    JOB_BCAST,        // root's buffer -> every member's buffer
    JOB_ALLTOALLV,    // receiver pulls every sender's block (uniform alltoall included)
    JOB_ALLGATHERV,   // receiver pulls every sender's whole sendbuf (allgather included)
    JOB_GATHERV,      // root pulls every sender's sendbuf
    JOB_SCATTERV,     // every receiver pulls its block from root's sendbuf
    JOB_BARRIER,
};

struct CollSlot;

struct alignas(128) Job {
    unsigned long long next;
    char pad0[120];
    unsigned long long done;
    char pad1[120];
    unsigned long long limit;
    unsigned epoch;
    int kind;
    int variant;
    int dt;          // element type of folds / element size source
    int op;          // predefined op code, or GPUMPI_OP_USER
    int root;
    int esize;
    int vec;         // elements per thread (folds) / tile (pull jobs)
    int tile;        // senders per chunk (pull jobs) / ranks per staged tile
    int aligned16;   // 16: all buffers 16-byte aligned, 8: 8-byte aligned, else 0
    unsigned err;    // MPI error raised while executing chunks (e.g. truncation)
    int nchunks;
    long long count;       // elements (folds) / bytes (copy)
    long long chunk;       // elements or bytes per chunk
    ::MPI_Comm_impl* comm;
    const CollSlot* slots;  // the communicator's slots and size, copied at set-up so that executors
    int csize;              // reach a member's slot without loading the communicator first
    const void* src;       // copy jobs
    void* dst;
    MPI_User_function* ufn;
    unsigned long long t_setup;  // globaltimer at set-up (traces)
    unsigned own_pulls;          // set-up chose the job-free route: every member pulls its own pieces
    long long sel_bytes;         // bytes per rank the variant choice was made for (traces)
};

// ------------------------------------------------------------------------------------------------
// communicators: one object shared by all members (the reference allocates one per rank and
// translates nothing, gpu_libs/gpu_mpi/communicator.cu:16-30; here the comm rank <-> world rank map
// is explicit and used by point-to-point too).
// ------------------------------------------------------------------------------------------------
constexpr int TINY_BYTES = 64;  // reductions of at most this many bytes per rank take the one-barrier path

// What each member publishes when it enters a collective.  The fold executors load every member's buffer
// pointers from these slots once per chunk: 40 more bytes per slot made Allreduce at 1024 ranks x 1 MiB
// 3% slower, so what the pull executors could read here instead of in the datatype descriptors stays out.
struct CollSlot {
    const void* sbuf;
    void* rbuf;
    const int* scounts;
    const int* sdispls;
    const int* rcounts;
    const int* rdispls;
    long long scount, rcount;
    const TypeDesc* sdesc;
    const TypeDesc* rdesc;
    int stype, rtype;
    int op, root;
    long long x0, x1;        // comm creation: colour / key, etc.
    MPI_User_function* ufn;
};

}  // namespace gpumpi

namespace gpumpi {
// The learned policy's final choice for one call shape (network, tuned table and override margin
// applied): kept on a communicator for its later setups, and per rank across launches (data region,
// never zeroed by a launch).  Valid while `epoch` equals the runtime's selector epoch, which the host
// advances whenever the policy, the weights, the table or a margin changes.
struct alignas(16) SelCacheRec {
    long long bytes;
    int kind, n, dt, op, blocks, aligned, variant;
    unsigned epoch;
};

}  // namespace gpumpi

struct alignas(128) MPI_Comm_impl {
    unsigned bar_count;
    char pad0[124];
    unsigned bar_gen;
    char pad1[124];
    gpumpi::Job job;
    int size;
    int ctx;
    int is_world;
    int magic;
    int* members;      // comm rank -> world rank
    int* rank_of;      // world rank -> comm rank (-1 if absent); nullptr for the world
    gpumpi::CollSlot* slots;   // size entries
    unsigned char* tiny;       // size x 2 x TINY_BYTES: inline operands of tiny reductions, by barrier parity
    unsigned misalign[2];               // OR of members' buffer addresses (low bits), per epoch parity
    unsigned long long creation_token;  // comm-creation handshake
    MPI_Comm_impl* created;            // result published by the creating member
    // Cartesian topology (MPI_Cart_create / MPI_Cart_sub); topo_kind 0 = none, 1 = Cartesian
    int topo_kind;
    int topo_ndims;
    int topo_dims[8];
    int topo_periods[8];
    // the learned selector's last choice on this communicator, made by whichever member set the
    // collective up (setups of one communicator are ordered by its barriers)
    gpumpi::SelCacheRec sel;
};
namespace gpumpi {
constexpr int COMM_MAGIC = 0x434f4d4d;

// ------------------------------------------------------------------------------------------------
// point-to-point: per-rank mailbox ring of envelopes (senders claim tickets with atomicAdd; the
// owner drains in ticket order), owner-private unexpected queue and posted-receive list.
// ------------------------------------------------------------------------------------------------
enum EnvFlags { ENV_INLINE = 1, ENV_HEAP = 2, ENV_SYNC = 4 };

struct alignas(64) Envelope {
    unsigned seq;          // ticket + 1 once the envelope is complete (release)
    int src;               // sender's rank in the communicator
    int tag;
    int ctx;
    long long bytes;       // packed message bytes
    const void* data;      // sender's buffer (rendezvous) / heap copy (ENV_HEAP)
    unsigned* done_flag;   // sender request's completion flag (rendezvous)
    const TypeDesc* desc;  // sender's datatype (nullptr = contiguous)
    long long count;       // sender's element count for desc
    int flags;
    int world_src;
};

struct UqEntry {
    Envelope env;
    int slot;              // payload slot index in the unexpected-payload pool (-1 if none)
    int live;              // 0 once matched (the queue keeps arrival order without moving entries)
};

enum ReqKind { REQ_FREE = 0, REQ_SEND = 1, REQ_RECV = 2 };
enum ReqState { RS_IDLE = 0, RS_ACTIVE = 1, RS_DONE = 2 };

}  // namespace gpumpi

struct alignas(64) MPI_Request_impl {
    unsigned done_flag;    // written by the receiver for rendezvous sends
    int kind;
    int state;
    int freed;             // MPI_Request_free on an active request
    int peer;              // send: dest world rank; recv: source comm rank or ANY
    int tag;
    int ctx;
    int index;
    void* buf;
    long long bytes;       // packed bytes
    long long count;
    const gpumpi::TypeDesc* desc;  // nullptr = contiguous
    MPI_Comm_impl* comm;
    void* stage;           // heap staging for buffers other ranks cannot address
    int st_source, st_tag, st_error;
    long long st_bytes;
};


struct MPI_Op_impl {
    int code;                  // predefined op code or GPUMPI_OP_USER
    MPI_User_function* fn;     // user function (GPUMPI_OP_USER)
    int commute;
};

struct MPI_Group_impl {
    int size;
    int* ranks;                // group rank -> world rank
    int refcount;
    int is_static;
};

namespace gpumpi {

// ------------------------------------------------------------------------------------------------
// per-rank and per-block state
// ------------------------------------------------------------------------------------------------
struct alignas(128) RankState {
    unsigned long long mb_tail;     // senders: atomicAdd
    char pad0[120];
    unsigned long long mb_head;     // owner: advances with release; senders read for flow control
    char pad1[120];
    // owner-private below
    int uq_head;                    // unexpected queue: circular, entries [uq_head, uq_tail) in arrival
    int uq_tail;                    // order, matched ones marked dead until the head passes them
    int nposted;                    // posted receives: slots [posted_lo, nposted) of the rank's list in
    int posted_lo;                  // posting order; matched slots hold -1 until trimmed
    int req_free_top;
    int pool_top;                   // scratch pool: bytes in use, and 1 + offset of the last block
    int pool_last1;                 //   (0: none); blocks are released from the top down
    int ntypes;
    int initialized;
    int finalized;
    int exited;
    int uq_free_top;
    int req_hwm;
    int uq_hwm;
    void* attrs;                    // keyvals and cached attributes (device heap, made on first use)
    Job p2p_job;
};

struct Task {                       // block task record, one per block (global memory)
    int kind;
    int i0;
    long long n0, n1;
    const void* p0;
    void* p1;
    const void* p2;
    void* p3;
    const void* p4;
    long long n2, n3;
};
enum TaskKind {
    TASK_EXIT = 0,
    TASK_COPY = 1,         // p1 <- p0, n0 bytes
    TASK_CHUNK = 2,        // p0 = Job*, n0 = chunk index, i0 = epoch
    TASK_TYPED_COPY = 3,   // packed byte range [n0, n1) of (p0, desc p2, count n2) -> (p1, desc p4, count n3)
    TASK_USER = 4,         // p0 = void (*)(void*, int, int), p1 = arg
    TASK_PACK = 5,         // typed -> contiguous: same fields as TYPED_COPY with p4 = nullptr
};

struct ErrorRecord {
    int code;
    int detail;
    int line;
    int rank;
    long long info;
};

struct BoardEntry {
    unsigned seq;          // slot index + 1 once written
    unsigned epoch;
    Job* job;
};

struct alignas(128) Board {
    unsigned long long reserve;
    char pad[120];
    BoardEntry* ring;
    int cap;
};

// Per-call timing record (feeds the autotuner and the learned selector).
struct TraceRec {
    float log2_bytes;
    float log2_ranks;
    int kind;
    int variant;
    int dt;
    int op;
    float us;
    int aligned;   // the call's buffer alignment (16, 8, 4 or 0 bytes): its tuned-table class
};

struct Runtime {
    // configuration
    int nranks, nengines, T;
    int pending, mbox_depth, uq_depth, eager, posted_cap, max_types, uq_payload_slots;
    long long timeout_ns;
    long long copy_chunk_bytes;       // chunk size of point-to-point copy jobs
    long long engine_min_bytes;       // smaller jobs are not posted to the engines
    long long static_fold_bytes;      // reductions of at most this many bytes per member (and at most one
                                      // chunk per member) split their chunks statically, without a job
    long long static_bcast_bytes;     // broadcasts of at most this many bytes copy from the root without a job
    long long static_pull_bytes;      // an Alltoallv whose members receive about this many bytes or fewer
                                      // pulls its pieces without a job
    int pull_chunks;                  // pull jobs of small pieces: chunks per worker block (>= 1)
    int variant_override;             // -1: selector decides
    int selector_mode;                // 0 plain (DIRECT), 1 tuned table, 2 learned MLP, 3 heuristic
    int dyn_smem;                     // dynamic shared memory bytes of this launch (STAGED stages)
    int tune_vec;                     // autotuner override: elements per thread of fold chunks (0 = auto)
    int tune_group;                   // autotuner override: ranks per STAGED stage (0 = auto)
    unsigned char* tree_scratch;      // TREE partials (world communicator)
    long long tree_scratch_bytes;
    unsigned* tree_flags;             // TREE partial-ready flags, tagged with the job epoch
    int tree_flags_cap;
    int trace_enabled;
    int trace_cap;
    // state arrays (device global memory)
    RankState* ranks;
    Envelope* ring;                   // nranks * mbox_depth
    unsigned char* ring_payload;      // nranks * mbox_depth * eager
    UqEntry* uq;                      // nranks * uq_depth
    unsigned char* uq_payload;        // nranks * uq_payload_slots * eager
    int* uq_free;                     // nranks * uq_payload_slots
    MPI_Request_impl* reqs;          // nranks * pending
    int* req_free;                    // nranks * pending
    int* posted;                      // nranks * posted_cap
    TypeDesc* types;                  // nranks * max_types
    Task* tasks;                      // nranks + nengines
    ErrorRecord* errors;              // nranks + nengines
    MPI_Comm_impl* world;
    int* world_members;
    CollSlot* world_slots;
    Board* board;
    unsigned char* scratch_pool;      // nranks * scratch_pool_bytes: each rank's scratch pool (MPI_Group
                                      // objects, staged copies of thread-local buffers)
    long long scratch_pool_bytes;
    unsigned char* arena;             // communicator objects created at run time
    unsigned long long arena_bytes;
    unsigned long long* arena_top;
    unsigned* ctx_counter;
    unsigned* ranks_done;
    unsigned* abort_flag;
    int* exit_codes;                  // nranks
    // selector
    const signed char* tuned_table;   // [kind][datatype class][alignment class][log2 bytes][log2 ranks] -> variant (or nullptr)
    const float* mlp_params;          // learned selector weights (or nullptr)
    SelCacheRec* sel_cache;           // per rank: the last learned choice, across launches
    HostIO hio;                       // the device -> host request channel (files, standard streams)
    unsigned sel_epoch;               // records of another epoch are stale
    float mlp_margin;                 // learned choice overrides the tuned table only if it predicts this
                                      // much lower log-time (Allreduce / Reduce)
    float mlp_margin_pull;            // the same for Alltoall(v)

    TraceRec* trace;
    unsigned long long* trace_count;
    int clock_khz;
};

// The one runtime the current launch works on, copied by the host into constant memory before each
// launch (read-only on the device: its fields are sizes and pointers to the state arrays).  Constant
// memory keeps these reads out of L1, which every acquire on the SM invalidates.
extern __constant__ Runtime c_rt;

__device__ __forceinline__ int nthreads() { return (int)blockDim.x; }

// ------------------------------------------------------------------------------------------------
// errors and bounded waits
// ------------------------------------------------------------------------------------------------
__device__ void record_error(int code, int detail, int line, long long info);

struct Deadline {
    unsigned long long end;
    unsigned spins;
    unsigned ns;
};
__device__ __forceinline__ Deadline make_deadline() {
    Deadline d;
    d.end = now_ns() + (unsigned long long)c_rt.timeout_ns;
    d.spins = 0;
    d.ns = 0;
    return d;
}
// Returns an MPI error code when the wait must stop (timeout or another rank failed), else 0.
// Backs off with nanosleep so idle waiters leave issue slots to working blocks.
__device__ __forceinline__ int wait_tick(Deadline& d, int line, unsigned max_ns = 256) {
    if ((++d.spins & 31u) == 0) {
        if (ld_relaxed(c_rt.abort_flag)) return GPUMPI_ERR_OTHER;
        if (now_ns() > d.end) {
            record_error(GPUMPI_ERR_OTHER, GPUMPI_ERR_TIMEOUT, line, 0);
            return GPUMPI_ERR_OTHER;
        }
    }
    if (d.ns) __nanosleep(d.ns);
    d.ns = d.ns ? (d.ns * 2 > max_ns ? max_ns : d.ns * 2) : 8;
    return 0;
}

// ------------------------------------------------------------------------------------------------
// block tasks (thread 0 -> the whole block)
// ------------------------------------------------------------------------------------------------
__device__ void execute_task(const Task& t, int tid, int nt);
__device__ void dispatch(const Task& t);     // called by thread 0 only
__device__ void helper_loop();               // threads 1..T-1

}  // namespace gpumpi
