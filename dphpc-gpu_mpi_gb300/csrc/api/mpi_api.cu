// mpi_api.cu — the __device__ MPI surface (include/mpi.h.cuh) on top of the block-rank runtime.
//
// One translation unit holds the whole runtime so its internals inline into each MPI call; user
// programs (and the library's own built-in programs) link against these extern __device__ symbols
// with relocatable device code, as converted programs link against the reference's libgpu_mpi.a.
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "../runtime/rt_core.cuh"
#include "../runtime/rt_types.cuh"
#include "../runtime/rt_ops.cuh"
#include "../runtime/rt_copy.cuh"
#include "../runtime/rt_coll.cuh"
#include "../runtime/rt_p2p.cuh"
#include "../runtime/rt_comm.cuh"
#include "../runtime/rt_select.cuh"
#include "gpumpi_stdio.h.cuh"

using namespace gpumpi;

// ------------------------------------------------------------------------------------------------
// globals of the MPI surface
// ------------------------------------------------------------------------------------------------
namespace gpumpi {
__constant__ Runtime c_rt;

#define GPUMPI_PT(sz, dt) {sz, sz, 0, sz, 0, dt, {0, 0, 0, 0}, {0, 0, 0, 0}, 1, 1}
__device__ TypeDesc g_predef_types[GPUMPI_NUM_PREDEFINED_TYPES] = {
    GPUMPI_PT(1, 0),   GPUMPI_PT(2, 1),   GPUMPI_PT(4, 2),   GPUMPI_PT(8, 3),   GPUMPI_PT(8, 4),
    GPUMPI_PT(8, 5),   GPUMPI_PT(1, 6),   GPUMPI_PT(1, 7),   GPUMPI_PT(2, 8),   GPUMPI_PT(4, 9),
    GPUMPI_PT(8, 10),  GPUMPI_PT(8, 11),  GPUMPI_PT(4, 12),  GPUMPI_PT(8, 13),  GPUMPI_PT(8, 14),
    GPUMPI_PT(4, 15),  GPUMPI_PT(1, 16),  GPUMPI_PT(1, 17),  GPUMPI_PT(2, 18),  GPUMPI_PT(4, 19),
    GPUMPI_PT(8, 20),  GPUMPI_PT(1, 21),  GPUMPI_PT(2, 22),  GPUMPI_PT(4, 23),  GPUMPI_PT(8, 24),
    GPUMPI_PT(8, 25),  GPUMPI_PT(8, 26),  GPUMPI_PT(16, 27), GPUMPI_PT(16, 28), GPUMPI_PT(1, 29),
    GPUMPI_PT(8, 30),  GPUMPI_PT(8, 31),  GPUMPI_PT(16, 32), GPUMPI_PT(16, 33), GPUMPI_PT(8, 34),
    GPUMPI_PT(16, 35)};
#undef GPUMPI_PT
}

__device__ MPI_Comm MPI_COMM_WORLD = nullptr;
__device__ MPI_Comm MPI_COMM_NULL = nullptr;
__device__ MPI_Group MPI_GROUP_WORLD = nullptr;
__device__ MPI_Group MPI_GROUP_NULL = nullptr;
__device__ MPI_Group MPI_GROUP_EMPTY = nullptr;

__device__ MPI_Op_impl g_predef_ops[GPUMPI_NUM_PREDEFINED_OPS] = {
    {GPUMPI_OP_MAX, nullptr, 1},  {GPUMPI_OP_MIN, nullptr, 1},  {GPUMPI_OP_SUM, nullptr, 1},
    {GPUMPI_OP_PROD, nullptr, 1}, {GPUMPI_OP_LAND, nullptr, 1}, {GPUMPI_OP_BAND, nullptr, 1},
    {GPUMPI_OP_LOR, nullptr, 1},  {GPUMPI_OP_BOR, nullptr, 1},  {GPUMPI_OP_LXOR, nullptr, 1},
    {GPUMPI_OP_BXOR, nullptr, 1}, {GPUMPI_OP_MAXLOC, nullptr, 1}, {GPUMPI_OP_MINLOC, nullptr, 1}};
__device__ MPI_Op MPI_MAX = &g_predef_ops[GPUMPI_OP_MAX];
__device__ MPI_Op MPI_MIN = &g_predef_ops[GPUMPI_OP_MIN];
__device__ MPI_Op MPI_SUM = &g_predef_ops[GPUMPI_OP_SUM];
__device__ MPI_Op MPI_PROD = &g_predef_ops[GPUMPI_OP_PROD];
__device__ MPI_Op MPI_LAND = &g_predef_ops[GPUMPI_OP_LAND];
__device__ MPI_Op MPI_BAND = &g_predef_ops[GPUMPI_OP_BAND];
__device__ MPI_Op MPI_LOR = &g_predef_ops[GPUMPI_OP_LOR];
__device__ MPI_Op MPI_BOR = &g_predef_ops[GPUMPI_OP_BOR];
__device__ MPI_Op MPI_LXOR = &g_predef_ops[GPUMPI_OP_LXOR];
__device__ MPI_Op MPI_BXOR = &g_predef_ops[GPUMPI_OP_BXOR];
__device__ MPI_Op MPI_MAXLOC = &g_predef_ops[GPUMPI_OP_MAXLOC];
__device__ MPI_Op MPI_MINLOC = &g_predef_ops[GPUMPI_OP_MINLOC];

// ------------------------------------------------------------------------------------------------
// block tasks, errors, block roles
// ------------------------------------------------------------------------------------------------
namespace gpumpi {

__shared__ Task s_task;

__device__ void record_error(int code, int detail, int line, long long info) {
    ErrorRecord* e = &c_rt.errors[blockIdx.x];
    if (e->code == 0) {
        e->code = code;
        e->detail = detail;
        e->line = line;
        e->rank = (int)blockIdx.x;
        e->info = info;
    }
    if (detail == GPUMPI_ERR_TIMEOUT || code == GPUMPI_ERR_INTERN) atomicExch(c_rt.abort_flag, 1u);
}

__device__ __forceinline__ void execute_task(const Task& t, int tid, int nt) {
    switch (t.kind) {
    case TASK_COPY: copy_bytes_inl(t.p1, t.p0, t.n0, tid, nt); break;
    case TASK_CHUNK: exec_chunk((Job*)t.p0, t.n0, tid, nt); break;
    case TASK_TYPED_COPY:
        typed_copy(t.p1, (const TypeDesc*)t.p4, t.p0, (const TypeDesc*)t.p2, t.n0, t.n1, tid, nt);
        break;
    case TASK_USER: ((void (*)(void*, int, int))t.p0)(t.p1, tid, nt); break;
    default: break;
    }
}

__device__ __noinline__ void execute_task_call(const Task& t, int tid, int nt) { execute_task(t, tid, nt); }

// Contiguous copies are latency-bound messages on the rank's critical path: in blocks of two or more
// warps they run on warps 1.. only, so thread 0 waits at the barrier instead of entering the copy (whose
// register saves and restores cost it about as much as a 1 KiB copy).  Typed copies, bound by their
// address arithmetic, keep every warp.
__device__ __forceinline__ bool copy_on_helpers(int kind, int nt) { return nt >= 64 && kind == TASK_COPY; }

// Thread 0: run task t on the whole block and return when every thread has finished it.
__device__ void dispatch(const Task& t) {
    const int nt = nthreads();
    if (nt > 1) {
        s_task = t;
        bar_sync(BAR_CMD, nt);
    }
    if (!copy_on_helpers(t.kind, nt)) execute_task_call(t, 0, nt);
    if (nt > 1) bar_sync(BAR_DONE, nt);
}

// Threads 1..T-1: sleep on the command barrier, execute, report, until EXIT.
__device__ void helper_loop() {
    const int nt = nthreads();
    const int tid = (int)threadIdx.x;
    for (;;) {
        bar_sync(BAR_CMD, nt);
        const int kind = s_task.kind;
        if (kind == TASK_EXIT) return;
        if (copy_on_helpers(kind, nt)) {
            if (tid >= 32) execute_task(s_task, tid - 32, nt - 32);
        } else {
            execute_task(s_task, tid, nt);
        }
        bar_sync(BAR_DONE, nt);
    }
}

__device__ void release_helpers() {
    if (nthreads() == 1) return;
    s_task.kind = TASK_EXIT;
    bar_sync(BAR_CMD, nthreads());
}

// Thread 0 of a rank block after the user program returned.
__device__ void rank_finish(int rc) {
    release_helpers();
    if (c_rt.ranks[blockIdx.x].attrs) {
        free(c_rt.ranks[blockIdx.x].attrs);
        c_rt.ranks[blockIdx.x].attrs = nullptr;
    }
    c_rt.exit_codes[blockIdx.x] = rc;
    c_rt.ranks[blockIdx.x].exited = 1;
    __threadfence();
    atomicAdd(c_rt.ranks_done, 1u);
}

// Thread 0 of a copy-engine block.
__device__ void engine_main() {
    engine_loop();
    release_helpers();
}

__device__ int is_rank_block() { return (int)blockIdx.x < c_rt.nranks; }
__device__ void selector_rank_begin();
__device__ void rank_begin() {
    p2p_rank_begin();
    selector_rank_begin();
}

}  // namespace gpumpi

// ------------------------------------------------------------------------------------------------
// helpers shared by the MPI functions
// ------------------------------------------------------------------------------------------------
namespace {

__device__ __forceinline__ const TypeDesc* tdesc(int dt) { return resolve_type(dt); }

// Stages a buffer other ranks cannot address (thread 0's stack) into the rank's scratch pool (the device
// heap when it is full).
struct Stage {
    void* heap = nullptr;
    void* user = nullptr;
    long long bytes = 0;
};
__device__ __noinline__ void* stage_in(Stage& s, const void* p, long long bytes, bool copy_in) {
    if (p == nullptr || p == MPI_IN_PLACE || is_global_ptr(p) || bytes <= 0) return (void*)p;
    s.heap = scratch_alloc((unsigned long long)bytes);
    s.user = (void*)p;
    s.bytes = bytes;
    if (!s.heap) return nullptr;
    if (copy_in) t0_copy(s.heap, nullptr, p, nullptr, bytes);
    return s.heap;
}
__device__ __noinline__ void stage_out(Stage& s, bool copy_out) {
    if (!s.heap) return;
    if (copy_out) t0_copy(s.user, nullptr, s.heap, nullptr, s.bytes);
    scratch_free(s.heap);
    s.heap = nullptr;
}

struct CollArgs {
    int kind;
    long long count;   // folds: elements
    int dt, op, root, esize;
    MPI_User_function* ufn;
    long long est_piece;   // pulls: estimated bytes per piece
    int variant;
    bool learned = false;  // the learned policy chooses (the setup evaluates the network)
};

__device__ __forceinline__ int learned_choice(MPI_Comm_impl* c, int kind, long long bytes, int n, int dt, int op,
                                              int aligned16);

// Bytes per piece of an Alltoallv, estimated the same way whichever member sets the collective up: the
// mean of 64 counts, 8 entries of the count arrays of 8 members spread over the communicator (a member's
// own estimate differs from another's, and the variant choice and the chunking would then depend on
// which member arrived last).  -1 when a sampled member published no count array.
__device__ __noinline__ long long shared_piece_estimate(const MPI_Comm_impl* c) {
    const int n = c->size;
    const CollSlot* sl = c->slots;
    // two rounds of independent loads, the 8 members' slots and then their counts and type sizes (this
    // runs on the critical path of the collective, in the set-up of the last member to arrive)
    const int* cnt[8];
    const TypeDesc* d[8];
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const int m = (int)(((long long)(2 * q + 1) * n) / 16);
        cnt[q] = (const int*)__ldcg((const unsigned long long*)&sl[m].scounts);
        d[q] = (const TypeDesc*)__ldcg((const unsigned long long*)&sl[m].sdesc);
    }
    bool ok = true;
#pragma unroll
    for (int q = 0; q < 8; q++) ok = ok && cnt[q] != nullptr && d[q] != nullptr;
    if (!ok) return -1;
    long long ssz[8];
#pragma unroll
    for (int q = 0; q < 8; q++) ssz[q] = __ldcg(&d[q]->size);
    long long sum = 0;
#pragma unroll
    for (int q = 0; q < 8; q++) {
        long long part = 0;
#pragma unroll
        for (int i = 0; i < 8; i++) part += __ldcg(cnt[q] + ((long long)(2 * i + 1) * n) / 16);
        sum += part * ssz[q];
    }
    return sum / 64;
}

// Elements per thread for a fold chunk (chunk = T * v elements).  Candidates: one 16-byte vector,
// 8 bytes (4-byte types), one element.  Score = blocks busy per wave x bytes in flight per thread
// (the rank-unrolled loads of fold_fast keep ~128 bytes in flight, at most 16 loads): the canonical
// order makes every element a sequential chain over all ranks, so memory parallelism comes only from
// elements in flight.  When every candidate fits in one wave of blocks the call is latency-bound: the
// time is one thread's chain of ceil(n / U) batches of loads (U ranks per batch, U = min(16, 128 / (v
// es))), so the candidate with the shortest chain wins (measured at 512 ranks x 256 B: one element per
// thread 33 µs, one 16-byte vector 119 µs).  A tuning override (gpumpi_set_tuning) takes precedence
// when it is legal.
__device__ int pick_vec(long long count, int T, int es, long long target, int aligned, int stage_room, int n) {
    int cands[3] = {16 / es, es == 4 ? 2 : 1, 1};
    if (c_rt.tune_vec <= 0) {
        bool one_wave = true;
        int pick = -1;
        long long pick_chain = 0, pick_nch = 0;
        for (int k = 2; k >= 0; k--) {  // narrowest first: on equal chains, more threads keep loads in flight
            const int v = cands[k];
            const int need = v * es >= 16 ? 16 : v * es;
            if ((v > 1 && aligned < need) || stage_room < 2 * T * v * es) continue;
            const long long nch = (count + (long long)T * v - 1) / ((long long)T * v);
            if (nch > target) one_wave = false;
            int u = 128 / (v * es);
            u = u < 1 ? 1 : u > 16 ? 16 : u;
            const long long chain = (n + u - 1) / u;
            if (pick < 0 || chain < pick_chain || (chain == pick_chain && nch > pick_nch)) {
                pick = k;
                pick_chain = chain;
                pick_nch = nch;
            }
        }
        if (one_wave && pick >= 0) return cands[pick];
    }
    double score_of[3] = {-1.0, -1.0, -1.0}, busy_of[3] = {0, 0, 0};
    for (int k = 0; k < 3; k++) {
        const int v = cands[k];
        const int need = v * es >= 16 ? 16 : v * es;
        if (v > 1 && aligned < need) continue;
        if (stage_room < 2 * T * v * es) continue;
        if (c_rt.tune_vec > 0) {
            if (v == c_rt.tune_vec) return v;
            continue;
        }
        const long long nch = (count + (long long)T * v - 1) / ((long long)T * v);
        const long long waves = (nch + target - 1) / (target > 0 ? target : 1);
        busy_of[k] = (double)nch / (double)(waves > 0 ? waves : 1);
        int u = 128 / (v * es);
        u = u < 1 ? 1 : u > 16 ? 16 : u;
        score_of[k] = busy_of[k] * (double)(v * es * u);
    }
    // among candidates within 5% of the best score: most busy blocks, then the widest vector
    double top = -1.0;
    for (int k = 0; k < 3; k++) top = score_of[k] > top ? score_of[k] : top;
    int pick = -1;
    for (int k = 0; k < 3; k++) {
        if (score_of[k] < 0.95 * top || score_of[k] < 0) continue;
        if (pick < 0 || busy_of[k] > busy_of[pick] * 1.01 ||
            (busy_of[k] >= busy_of[pick] * 0.99 && cands[k] > cands[pick]))
            pick = k;
    }
    if (pick >= 0) return cands[pick];
    int best = 1;
    double best_score = -1.0;
    for (int k = 0; k < 3; k++) {
        const int v = cands[k];
        const int need = v * es >= 16 ? 16 : v * es;
        if (v > 1 && aligned < need) continue;
        if (stage_room < 2 * T * v * es) continue;
        if (c_rt.tune_vec > 0) {
            if (v == c_rt.tune_vec) return v;
            continue;
        }
        const long long nch = (count + (long long)T * v - 1) / ((long long)T * v);
        const long long waves = (nch + target - 1) / (target > 0 ? target : 1);
        const double busy = (double)nch / (double)(waves > 0 ? waves : 1);
        int u = 128 / (v * es);
        u = u < 1 ? 1 : u > 16 ? 16 : u;
        const double score = busy * (double)(v * es * u);
        if (score > best_score + 1e-9) {
            best_score = score;
            best = v;
        }
    }
    return best;
}

__device__ __noinline__ void coll_setup(MPI_Comm_impl* c, const CollArgs& a, unsigned e_next) {
    Job* j = &c->job;
    j->own_pulls = 0;
    unsigned mis = ld_relaxed(&c->misalign[e_next & 1]);
    c->misalign[(e_next + 1) & 1] = 0;
    j->kind = a.kind;
    j->comm = c;
    j->slots = c->slots;
    j->csize = c->size;
    j->dt = a.dt;
    j->op = a.op;
    j->root = a.root;
    j->ufn = a.ufn;
    j->esize = a.esize;
    j->err = 0;
    j->aligned16 = (mis & 15) == 0 ? 16 : (mis & 7) == 0 ? 8 : (mis & 3) == 0 ? 4 : 0;
    j->t_setup = now_ns();
    const int T = nthreads();
    const int n = c->size;
    int nchunks = 0;
    long long bytes = 0;
    bool may_post = c_rt.nengines > 0;
    if (a.kind == JOB_ALLREDUCE || a.kind == JOB_REDUCE) {
        j->count = a.count;
        j->sel_bytes = a.count * a.esize;
        bytes = a.count * a.esize * (long long)n;
        int variant = a.learned ? learned_choice(c, a.kind, a.count * a.esize, n, a.dt, a.op, j->aligned16)
                                : select_variant(a.kind, a.count * a.esize, n, a.dt, a.op, a.variant, j->aligned16,
                                                 nullptr);
        may_post = may_post && bytes >= c_rt.engine_min_bytes;
        long long target = n + (may_post ? c_rt.nengines : 0);
        int vec = 1;
        j->tile = 0;
        if (variant == GPUMPI_VARIANT_STAGED) {
            // canonical order through shared-memory stages: needs 16-byte aligned buffers and room for
            // two stages of at least one rank
            const int es = a.esize;
            const int stage_room = c_rt.dyn_smem - 128;
            if (!fold_has_staged(a.dt, a.op, a.ufn) || j->aligned16 < 16 || stage_room < 2 * T * es) {
                variant = GPUMPI_VARIANT_DIRECT;
            } else {
                vec = pick_vec(a.count, T, es, target, 16, stage_room, n);
                int G = stage_room / (2 * T * vec * es);
                if (c_rt.tune_group > 0 && c_rt.tune_group < G) G = c_rt.tune_group;
                j->tile = G < 1 ? 1 : G > 64 ? 64 : G;
            }
        }
        if (variant == GPUMPI_VARIANT_TREE) {
            // two-level rank split on the world communicator: R groups (power of two, >= 8 ranks each)
            // so that chunks x groups covers the blocks; partials and flags must fit the tree scratch
            const int es = a.esize;
            int v = (j->aligned16 >= 16) ? 16 / es : 1;
            if (c_rt.tune_vec > 0) v = c_rt.tune_vec == 16 / es ? v : 1;
            const long long E = (long long)T * v;
            const long long C = (a.count + E - 1) / E;
            int R = 2;
            while (R < 16 && R * 2 <= n / 8 && C * R < target) R *= 2;
            if (c_rt.tune_group > 0) R = c_rt.tune_group;
            const bool ok = fold_has_tree(a.dt, a.op, a.ufn) && c->is_world && n >= 16 && R >= 2 && R <= n &&
                            (long long)R * a.count * es <= c_rt.tree_scratch_bytes && C * R <= c_rt.tree_flags_cap &&
                            c_rt.tree_scratch && c_rt.tree_flags;
            if (ok) {
                vec = v;
                j->tile = R;
            } else {
                variant = GPUMPI_VARIANT_DIRECT;
            }
        }
        j->variant = variant;
        if (variant == GPUMPI_VARIANT_DIRECT && fold_has_fast(a.dt, a.op, a.ufn)) {
            int es = a.esize;
            vec = pick_vec(a.count, T, es, target, j->aligned16, 1 << 30, n);
        }
        j->vec = vec;
        j->chunk = (long long)T * vec;
        nchunks = (int)((a.count + j->chunk - 1) / j->chunk);
        if (variant == GPUMPI_VARIANT_TREE) nchunks *= (j->tile + 1);  // C*R phase-1 + C phase-2 chunks
    } else if (a.kind == JOB_BARRIER) {
        nchunks = 0;
    } else {
        const bool matrix = a.kind == JOB_ALLTOALLV || a.kind == JOB_ALLGATHERV;
        long long P = matrix ? (long long)n * n : (long long)n;
        j->count = P;
        // piece order (DIRECT / TREE / RING, see piece_of) or bulk-copy staging (STAGED)
        long long a_est = a.est_piece;
        if (a.kind == JOB_ALLTOALLV && n >= 16) {
            const long long est = shared_piece_estimate(c);
            if (est >= 0) a_est = est;
        }
        // a small Alltoallv among at most 512 members takes no job (no variant choice either): every member
        // pulls its own pieces (coll_run, own_pulls); with more members one member's n piece resolutions
        // take longer than the job's shared chunks
        if (a.kind == JOB_ALLTOALLV && a.variant < 0 && c_rt.static_pull_bytes > 0 && n <= 512 &&
            a_est * n <= c_rt.static_pull_bytes) {
            j->own_pulls = 1;
            j->variant = GPUMPI_VARIANT_DIRECT;
            j->sel_bytes = a_est * n;
            job_open(j, 0);
            return;
        }
        int variant = a.kind != JOB_ALLTOALLV
                          ? (matrix && a.variant >= 0 && a.variant < GPUMPI_NUM_VARIANTS ? a.variant
                                                                                          : GPUMPI_VARIANT_DIRECT)
                      : a.learned ? learned_choice(c, a.kind, a_est * n, n, a.dt, -1, j->aligned16)
                                  : select_variant(a.kind, a_est * n, n, a.dt, -1, a.variant, j->aligned16, nullptr);
        // STAGED needs shared memory for two bulk-copy stages of at least 512 bytes per warp
        if (variant == GPUMPI_VARIANT_STAGED && (!matrix || staged_pull_stage_bytes(T) < 512))
            variant = GPUMPI_VARIANT_DIRECT;
        j->variant = variant;
        j->sel_bytes = a_est * n;
        bytes = a_est * P;
        may_post = may_post && bytes >= c_rt.engine_min_bytes;
        long long target = n + (may_post ? c_rt.nengines : 0);
        if (a_est >= 65536) {
            int parts = (int)((a_est + 65535) / 65536);
            j->vec = parts;
            j->tile = 1;
            nchunks = (int)(P * parts);
        } else {
            // one piece per thread of the block prepares the chunk; about pull_chunks chunks per worker block
            long long tile = P / ((long long)c_rt.pull_chunks * (target > 0 ? target : 1));
            if (tile < 1) tile = 1;
            if (tile > T) tile = T;
            j->vec = 1;
            j->tile = (int)tile;
            nchunks = (int)((P + tile - 1) / tile);
        }
    }
    unsigned e = job_open(j, nchunks);
    if (may_post && nchunks > n) board_post(j, e);
}

// ---- small Alltoallv without a job: every member pulls its own pieces ----
// When the set-up (the last member to arrive at the collective's barrier) finds the size estimate every
// member would compute from the same 8 members' counts small, it opens no chunks: each member pulls its n
// pieces (senders q = 0..n-1 into its own buffer) with the pull executor's tile copies, and a second
// barrier keeps the senders' buffers valid until every member has read them.
struct OwnPulls {
    JobParams j;
    Job* jg;
    long long p0;
    int n;
};
__shared__ OwnPulls s_own_pulls;

__device__ void own_pulls_task(void* arg, int tid, int nt) {
    OwnPulls* w = (OwnPulls*)arg;
    for (int k = 0; k < w->n; k += nt) pull_tile(&w->j, w->jg, w->p0 + k, min(nt, w->n - k), tid, nt);
}

__device__ __noinline__ int own_pulls(MPI_Comm_impl* c, int cr, int line) {
    const int n = c->size;
    Job* jg = &c_rt.ranks[me()].p2p_job;  // idle during a collective: collects the truncation flag
    jg->err = 0;
    OwnPulls* w = &s_own_pulls;
    JobParams& j = w->j;
    memset(&j, 0, sizeof(j));
    j.kind = JOB_ALLTOALLV;
    j.variant = GPUMPI_VARIANT_DIRECT;  // receiver-major pieces: member cr's are [cr * n, cr * n + n)
    j.comm = c;
    j.slots = c->slots;
    j.csize = n;
    j.vec = 1;
    j.tile = nthreads();
    j.count = (long long)n * n;
    w->jg = jg;
    w->p0 = (long long)cr * n;
    w->n = n;
    Task t;
    t.kind = TASK_USER;
    t.p0 = (const void*)&own_pulls_task;
    t.p1 = w;
    dispatch(t);
    int rc = comm_barrier(c, []() {}, line);
    if (!rc && ld_relaxed(&jg->err)) rc = GPUMPI_ERR_TRUNCATE;
    return rc;
}

__device__ __noinline__ int coll_run(MPI_Comm_impl* c, const CollSlot& mine, const CollArgs& a, int line) {
    const int cr = comm_rank_of(c, me());
    c->slots[cr] = mine;
    const unsigned e_next = c->job.epoch + 1;
    unsigned mis = (unsigned)((size_t)mine.sbuf | (size_t)mine.rbuf) & 15u;
    if (mis) atomicOr(&c->misalign[e_next & 1], mis);
    unsigned long long t0 = c_rt.trace_enabled ? now_ns() : 0;
    int rc = comm_barrier(c, [&]() { coll_setup(c, a, e_next); }, line);
    if (rc) return rc;
    if (a.kind == JOB_BARRIER) return 0;
    if (a.kind == JOB_ALLTOALLV && ld_relaxed(&c->job.own_pulls)) return own_pulls(c, cr, line);
    rc = job_run_and_wait(&c->job, line);
    if (rc) return rc;
    if (c_rt.trace_enabled && cr == 0) trace_record(c, a.kind, c->job.variant, a.dt, a.op, c->job.sel_bytes,
                                                    now_ns() - t0);
    return ld_relaxed(&c->job.err) ? GPUMPI_ERR_TRUNCATE : 0;
}

// ---- small reductions without a job: the members split the chunks statically ----
// Each member publishes its buffers in its slot and enters a barrier; member r then folds chunks r, r + n,
// ... of the result, each over every member in rank order (the canonical order, bit-identical to the job
// path), writes them where they go (every member's receive buffer, or the root's), and a second barrier
// ends the call: the members' reads of the inputs and writes of the results are complete when the
// barrier releases.  At these sizes the job path's set-up by the last arriver, chunk claims and
// completion count cost more than the second barrier.
struct StaticFold {
    JobParams j;
    long long first, step, nch;
};
__shared__ StaticFold s_sfold;

__device__ void static_fold_task(void* arg, int tid, int nt) {
    StaticFold* w = (StaticFold*)arg;
    for (long long k = w->first; k < w->nch; k += w->step) fold_chunk(&w->j, k, tid, nt);
}

// Whether a reduction takes the static split: every member computes the same answer from what all share.
__device__ __forceinline__ bool static_fold_ok(long long count, int es, int n) {
    const long long bytes = count * es;
    return c_rt.static_fold_bytes > 0 && bytes <= c_rt.static_fold_bytes && n >= 2 &&
           count <= (long long)n * nthreads();
}

__device__ __noinline__ int coll_run_static(MPI_Comm_impl* c, const CollSlot& mine, const CollArgs& a, int line) {
    const int cr = comm_rank_of(c, me());
    c->slots[cr] = mine;
    int rc = comm_barrier(c, []() {}, line);
    if (rc) return rc;
    StaticFold* w = &s_sfold;
    JobParams& j = w->j;
    j.kind = a.kind;
    j.dt = a.dt;
    j.op = a.op;
    j.root = a.root;
    j.esize = a.esize;
    j.vec = 1;
    j.tile = 0;
    j.aligned16 = 0;  // element-wide loads: no member's alignment is needed
    j.variant = GPUMPI_VARIANT_DIRECT;
    j.epoch = 0;
    j.count = a.count;
    j.chunk = nthreads();
    j.comm = c;
    j.slots = c->slots;
    j.csize = c->size;
    j.src = nullptr;
    j.dst = nullptr;
    j.ufn = a.ufn;
    w->first = cr;
    w->step = c->size;
    w->nch = (a.count + j.chunk - 1) / j.chunk;
    if (w->first < w->nch) {
        Task t;
        t.kind = TASK_USER;
        t.p0 = (const void*)&static_fold_task;
        t.p1 = w;
        dispatch(t);
    }
    return comm_barrier(c, []() {}, line);
}

__device__ __forceinline__ int op_code_of(MPI_Op op, MPI_User_function** ufn) {
    *ufn = nullptr;
    if (!op) return -1;
    if (op->code == GPUMPI_OP_USER) {
        *ufn = op->fn;
        return GPUMPI_OP_USER;
    }
    return op->code;
}

// ---- learned selector: in-kernel inference of the MLP trained by csrc/selector/mlp.cu ----
// Features (same formula as gpumpi/selector.py, features()): log2 bytes per rank, log2 ranks, datatype
// one-hot (f32, f64, i32, i64), SUM flag, 16-byte and 8-byte alignment flags of the members' buffers,
// rank share of the launch's blocks, kind.  The alignment is known only once every member has arrived, so
// the member that sets the collective up evaluates the network (the table's cell depends on it too).
struct MlpWork {
    float f[12];
    float h1[64];
    float h2[64];
    float y[4];
};
__shared__ MlpWork s_mlp;

__device__ void mlp_infer_task(void* arg, int tid, int nt) {
    MlpWork* w = (MlpWork*)arg;
    const float* p = c_rt.mlp_params;
    constexpr int W1 = 0, B1 = 64 * 12, W2 = B1 + 64, B2 = W2 + 64 * 64, W3 = B2 + 64, B3 = W3 + 4 * 64;
    if (tid < 64) {
        float z = __ldcg(p + B1 + tid);
        for (int i = 0; i < 12; i++) z = fmaf(__ldcg(p + W1 + tid * 12 + i), w->f[i], z);
        w->h1[tid] = z > 0.f ? z : 0.f;
    }
    bar_sync(BAR_TASK, nt);
    if (tid < 64) {
        float z = __ldcg(p + B2 + tid);
        for (int i = 0; i < 64; i++) z = fmaf(__ldcg(p + W2 + tid * 64 + i), w->h1[i], z);
        w->h2[tid] = z > 0.f ? z : 0.f;
    }
    bar_sync(BAR_TASK, nt);
    if (tid < 4) {
        float z = __ldcg(p + B3 + tid);
        for (int i = 0; i < 64; i++) z = fmaf(__ldcg(p + W3 + tid * 64 + i), w->h2[i], z);
        w->y[tid] = z;
    }
}

// The rank's last learned choice, in shared memory: a repeated call of one shape is answered without a
// global-memory round trip.
struct SelCache {
    long long bytes;
    int kind, n, dt, op, blocks, aligned, variant, valid;
};
__shared__ SelCache s_sel;

// Variants the selector chooses among: DIRECT, TREE, RING.  STAGED (bulk-copy staging through shared
// memory) never measured fastest on this GPU: the 8 KiB of dynamic shared memory per rank block leaves it
// stages of a few hundred bytes, and more shared memory takes L1 from the spilled registers of every
// other path (1024 ranks x 1 MiB uneven Alltoallv: DIRECT 3,940 GB/s at 8 KiB, 3,079 at 12-24 KiB,
// STAGED 2,385-2,780); it stays available as an explicit variant.
constexpr int SEL_CHOICES = 3;

__device__ __forceinline__ bool sel_hit(const SelCacheRec& r, int kind, long long bytes, int n, int dt, int op,
                                        int blocks, int al) {
    return r.epoch == c_rt.sel_epoch && r.bytes == bytes && r.kind == kind && r.n == n && r.dt == dt &&
           r.op == op && r.blocks == blocks && r.aligned == al;
}

// The learned policy's choice when the communicator holds none for this shape: the rank's own last
// choice if it matches, else the network (evaluated by this block's threads) weighed against the tuned
// table by the kind's margin (select_variant).  The choice is recorded on the communicator, in shared
// memory and in the rank's record that outlives the launch.
__device__ __noinline__ int learned_decide(MPI_Comm_impl* c, int kind, long long bytes, int n, int dt, int op,
                                           int aligned16, int blocks, int al) {
    SelCache* sc = &s_sel;
    int choice;
    if (sc->valid && sc->bytes == bytes && sc->kind == kind && sc->n == n && sc->dt == dt && sc->op == op &&
        sc->blocks == blocks && sc->aligned == al) {
        choice = sc->variant;
    } else {
        MlpWork* w = &s_mlp;
        for (int i = 0; i < 12; i++) w->f[i] = 0.f;
        w->f[0] = (log2f((float)(bytes > 0 ? bytes : 1)) - 16.f) / 8.f;
        w->f[1] = (log2f((float)n) - 8.f) / 3.f;
        const int dslot = dt == GPUMPI_FLOAT ? 2 : (dt == GPUMPI_DOUBLE || dt == GPUMPI_LONG_DOUBLE) ? 3
                          : (dt == GPUMPI_INT || dt == GPUMPI_INT32_T) ? 4 : 5;
        w->f[dslot] = 1.f;
        w->f[6] = op == GPUMPI_OP_SUM ? 1.f : 0.f;  // pulls have no operator (op < 0)
        w->f[7] = al >= 16 ? 1.f : 0.f;
        w->f[8] = al >= 8 ? 1.f : 0.f;
        w->f[10] = (float)n / (float)blocks;
        w->f[11] = kind == JOB_REDUCE ? 1.f : kind == JOB_ALLTOALLV ? -1.f : 0.f;
        Task t;
        t.kind = TASK_USER;
        t.p0 = (const void*)&mlp_infer_task;
        t.p1 = w;
        dispatch(t);
        int best = 0;
        for (int v = 1; v < SEL_CHOICES; v++)
            if (w->y[v] < w->y[best]) best = v;
        choice = select_variant(kind, bytes, n, dt, op, best, aligned16, w->y);
        sc->kind = kind;
        sc->bytes = bytes;
        sc->n = n;
        sc->dt = dt;
        sc->op = op;
        sc->blocks = blocks;
        sc->aligned = al;
        sc->variant = choice;
        sc->valid = 1;
    }
    SelCacheRec r;
    r.bytes = bytes;
    r.kind = kind;
    r.n = n;
    r.dt = dt;
    r.op = op;
    r.blocks = blocks;
    r.aligned = al;
    r.variant = choice;
    r.epoch = c_rt.sel_epoch;
    c_rt.sel_cache[me()] = r;   // loaded by selector_rank_begin in the rank's later launches
    c->sel = r;
    return choice;
}

// The learned policy's variant for a collective, decided by the member that sets it up.  A setup of the
// shape the communicator last decided reads one record (its loads issue together) and compares: the setup
// runs while every other member waits, so the common path is kept to one global round trip and no call.
__device__ __forceinline__ int learned_choice(MPI_Comm_impl* c, int kind, long long bytes, int n, int dt, int op,
                                              int aligned16) {
    const int blocks = c_rt.nranks + c_rt.nengines;  // the network's occupancy input depends on it
    const int al = aligned16 >= 16 ? 16 : aligned16 >= 8 ? 8 : 0;
    const SelCacheRec cs = c->sel;
    if (sel_hit(cs, kind, bytes, n, dt, op, blocks, al)) return cs.variant;
    return learned_decide(c, kind, bytes, n, dt, op, aligned16, blocks, al);
}

// ---- tiny reductions (at most TINY_BYTES per rank): one barrier, no job ----
// Each member writes its operand into its inline slot of the parity of the barrier it is about to enter,
// enters the barrier, and the members that need the result fold all n operands themselves, in rank order
// (the canonical order: bit-identical to the job path).  The next collective on the communicator writes
// the other parity, and the one after it can only start once every member has passed the barrier in
// between, that is, has finished reading; so no second barrier is needed.  A job would take a barrier,
// a chunk claim and dispatch, completion counting and a wait for the last chunk: about 10 µs more.
struct TinyFold {
    const unsigned char* tiny;
    int n, parity, count, es, dt, op;
    int stride;  // bytes per staged operand in shared memory: the operand's 16-byte vectors only
    alignas(16) unsigned char out[TINY_BYTES];  // the result, also the accumulators (element e at e * es,
                                                // read and written as the element type)
};
static_assert(offsetof(TinyFold, out) % 16 == 0, "the accumulators are accessed as 8- and 16-byte values");
__shared__ TinyFold s_tiny_fold;

// fold of a staged tile of m ranks (the first at r0) into the accumulators, element tid; typed for the
// common (type, op) pairs (the same op_apply as the job path's fast fold), generic otherwise
template <class T, int OP>
__device__ __forceinline__ void tiny_fold_typed(TinyFold* w, const unsigned char* buf, int m, int r0, int tid) {
    T* acc = (T*)w->out + tid;
    const int st = w->stride;
    T a = r0 == 0 ? ((const T*)buf)[tid] : *acc;
    for (int i = r0 == 0 ? 1 : 0; i < m; i++) a = op_apply<OP, T>(((const T*)(buf + (size_t)i * st))[tid], a);
    *acc = a;
}

template <class T>
__device__ __forceinline__ bool tiny_fold_arith(TinyFold* w, const unsigned char* buf, int m, int r0, int tid) {
    switch (w->op) {
    case GPUMPI_OP_SUM: tiny_fold_typed<T, GPUMPI_OP_SUM>(w, buf, m, r0, tid); return true;
    case GPUMPI_OP_MAX: tiny_fold_typed<T, GPUMPI_OP_MAX>(w, buf, m, r0, tid); return true;
    case GPUMPI_OP_MIN: tiny_fold_typed<T, GPUMPI_OP_MIN>(w, buf, m, r0, tid); return true;
    case GPUMPI_OP_PROD: tiny_fold_typed<T, GPUMPI_OP_PROD>(w, buf, m, r0, tid); return true;
    default: return false;
    }
}

__device__ __forceinline__ bool tiny_fold_fast(TinyFold* w, const unsigned char* buf, int m, int r0, int tid) {
    switch (w->dt) {
    case GPUMPI_FLOAT: return tiny_fold_arith<float>(w, buf, m, r0, tid);
    case GPUMPI_DOUBLE: case GPUMPI_LONG_DOUBLE: return tiny_fold_arith<double>(w, buf, m, r0, tid);
    case GPUMPI_INT: case GPUMPI_INT32_T: return tiny_fold_arith<int>(w, buf, m, r0, tid);
    case GPUMPI_LONG: case GPUMPI_LONG_LONG_INT: case GPUMPI_LONG_LONG: case GPUMPI_INT64_T:
        return tiny_fold_arith<long long>(w, buf, m, r0, tid);
    default: return false;
    }
}

__device__ void tiny_fold_task(void* arg, int tid, int nt) {
    TinyFold* w = (TinyFold*)arg;
    unsigned char* buf = (unsigned char*)g_dyn_smem;  // staged operands, w->stride bytes per rank
    const int vecs = (w->count * w->es + 15) / 16;
    // as many operands per tile as the dynamic shared memory holds (8 KiB: 512 operands of 16 bytes)
    const int tile = c_rt.dyn_smem / w->stride;
    unsigned char* acc = w->out + tid * w->es;
    for (int r0 = 0; r0 < w->n; r0 += tile) {
        const int m = min(tile, w->n - r0);
        for (int x = tid; x < m * vecs; x += nt) {
            const int i = x / vecs, k = x % vecs;
            const uint4* src = (const uint4*)(w->tiny + ((size_t)(r0 + i) * 2 + w->parity) * TINY_BYTES) + k;
            ((uint4*)(buf + (size_t)i * w->stride))[k] = __ldcg(src);
        }
        bar_sync(BAR_TASK, nt);
        if (tid < w->count && !tiny_fold_fast(w, buf, m, r0, tid)) {
            for (int i = 0; i < m; i++) {
                const unsigned char* src = buf + (size_t)i * w->stride + tid * w->es;
                if (r0 + i == 0) {
                    for (int b = 0; b < w->es; b++) acc[b] = src[b];
                } else {
                    apply_elem(w->op, w->dt, src, acc);
                }
            }
        }
        bar_sync(BAR_TASK, nt);
    }
}

__device__ __noinline__ int tiny_fold(MPI_Comm_impl* c, int kind, const void* sb, void* recvbuf, int count, int dt,
                                      int op, int root, int es) {
    const int cr = comm_rank_of(c, me());
    const int bytes = count * es;
    const unsigned g = ld_acquire(&c->bar_gen);
    unsigned char* mine = c->tiny + ((size_t)cr * 2 + (g & 1)) * TINY_BYTES;
    small_copy(mine, sb, bytes);
    int rc = comm_barrier_from(c, g, []() {}, __LINE__);
    if (rc || !(kind == JOB_ALLREDUCE || cr == root)) return rc;
    TinyFold* w = &s_tiny_fold;
    w->tiny = c->tiny;
    w->n = c->size;
    w->parity = (int)(g & 1);
    w->count = count;
    w->es = es;
    w->dt = dt;
    w->op = op;
    w->stride = (bytes + 15) / 16 * 16;
    Task t;
    t.kind = TASK_USER;
    t.p0 = (const void*)&tiny_fold_task;
    t.p1 = w;
    dispatch(t);
    small_copy(recvbuf, w->out, bytes);
    return 0;
}

// Route of a reduction of at most TINY_BYTES per member when no variant is forced: ROUTE_TINY = the
// one-barrier path, else the job path with that variant (GPUMPI_VARIANT_AUTO: the selector's choice).  Every member
// computes the same route from what all members share (size, type, op, count).  Measured on GB300
// (Allreduce SUM, p50 of 10 calls): fp64 operands folded by every member in rank order run on the narrow
// FP64 pipes of all members at once, 174.7 us at 1024 ranks x 8 doubles against 83.1 us for the job path
// (55.7 against 45.2 at 512 ranks); a single integer among 2048 ranks takes 64 us on TREE, against
// 100 us for the n^2 inline-slot fold and 102 us for DIRECT.  Integers are exact in any order, floating
// point keeps the canonical order by default.
constexpr int ROUTE_TINY = -2;
__device__ __forceinline__ int small_route(int n, int dt, int opc, int count) {
    const bool fp64 = dt == GPUMPI_DOUBLE || dt == GPUMPI_LONG_DOUBLE || dt == GPUMPI_C_DOUBLE_COMPLEX ||
                      dt == GPUMPI_C_LONG_DOUBLE_COMPLEX;
    if (fp64 && n >= 512) return GPUMPI_VARIANT_AUTO;
    const bool int32_64 = dt == GPUMPI_INT || dt == GPUMPI_INT32_T || dt == GPUMPI_LONG ||
                          dt == GPUMPI_LONG_LONG_INT || dt == GPUMPI_LONG_LONG || dt == GPUMPI_INT64_T;
    const bool assoc = opc == GPUMPI_OP_SUM || opc == GPUMPI_OP_MAX || opc == GPUMPI_OP_MIN || opc == GPUMPI_OP_PROD;
    if (int32_64 && assoc && count == 1 && n >= 2048) return GPUMPI_VARIANT_TREE;
    return ROUTE_TINY;
}

__device__ __noinline__ int fold_collective(int kind, const void* sendbuf, void* recvbuf, int count, MPI_Datatype dt, MPI_Op op,
                               int root, MPI_Comm comm) {
    MPI_Comm_impl* c = check_comm(comm);
    if (!c) return GPUMPI_ERR_COMM;
    if (count < 0) return GPUMPI_ERR_COUNT;
    if (kind == JOB_REDUCE && (root < 0 || root >= c->size)) return GPUMPI_ERR_ROOT;
    if (dt < 0 || dt >= GPUMPI_NUM_PREDEFINED_TYPES) return GPUMPI_ERR_TYPE;
    MPI_User_function* ufn;
    int opc = op_code_of(op, &ufn);
    if (opc < 0) return GPUMPI_ERR_OP;
    if (opc != GPUMPI_OP_USER && !op_allowed(opc, dt)) {
        record_error(GPUMPI_ERR_OP, dt, __LINE__, opc);
        return GPUMPI_ERR_OP;
    }
    if (count == 0) return 0;
    const int es = predefined_size(dt);
    const long long bytes = (long long)count * es;
    const int cr = comm_rank_of(c, me());
    const bool has_out = kind == JOB_ALLREDUCE || cr == root;
    const void* sb = sendbuf == MPI_IN_PLACE ? recvbuf : sendbuf;
    // (a forced variant, as the autotuner and the variant tests set, always takes the job path)
    const int route = opc != GPUMPI_OP_USER && bytes <= TINY_BYTES && c_rt.variant_override < 0
                          ? small_route(c->size, dt, opc, count) : GPUMPI_VARIANT_AUTO;
    if (opc != GPUMPI_OP_USER && bytes <= TINY_BYTES && c->tiny && c_rt.variant_override < 0 && route == ROUTE_TINY &&
        c_rt.dyn_smem >= 32 * TINY_BYTES && nthreads() >= count && sb && (!has_out || recvbuf))
        return tiny_fold(c, kind, sb, recvbuf, count, dt, opc, root, es);
    Stage ss, rs;
    const void* gsb = stage_in(ss, sb, bytes, true);
    void* grb = has_out ? stage_in(rs, recvbuf, bytes, sendbuf == MPI_IN_PLACE) : nullptr;
    if (sendbuf == MPI_IN_PLACE && rs.heap) gsb = rs.heap;
    if ((sb && !gsb) || (has_out && recvbuf && !grb)) return GPUMPI_ERR_NO_MEM;
    CollSlot my{};
    my.sbuf = gsb;
    my.rbuf = grb;
    my.scount = count;
    my.stype = dt;
    my.op = opc;
    my.root = root;
    CollArgs a;
    a.kind = kind;
    a.count = count;
    a.dt = dt;
    a.op = opc;
    a.root = root;
    a.esize = es;
    a.ufn = ufn;
    a.est_piece = 0;
    a.variant = c_rt.variant_override >= 0 ? c_rt.variant_override : route >= 0 ? route : GPUMPI_VARIANT_AUTO;
    a.learned = a.variant < 0 && c_rt.selector_mode == 2 && c_rt.mlp_params;
    // (a forced variant or a route the small-message rules chose keeps the job path)
    const bool stat = c_rt.variant_override < 0 && route == GPUMPI_VARIANT_AUTO && static_fold_ok(count, es, c->size);
    int rc = stat ? coll_run_static(c, my, a, __LINE__) : coll_run(c, my, a, __LINE__);
    stage_out(ss, false);
    stage_out(rs, has_out);
    return rc;
}

// pull collectives; `arrays` that live on thread 0's stack are staged so other ranks can read them
__device__ const int* stage_ints(Stage& s, const int* p, int n) {
    return (const int*)stage_in(s, p, (long long)n * sizeof(int), true);
}

__device__ __noinline__ int pull_collective(int kind, MPI_Comm_impl* c, CollSlot& my, long long sbytes, long long rbytes,
                               long long est_piece, int root) {
    Stage ss, rs;
    const void* gsb = stage_in(ss, my.sbuf, sbytes, true);
    void* grb = stage_in(rs, my.rbuf, rbytes, false);
    if ((my.sbuf && my.sbuf != MPI_IN_PLACE && sbytes > 0 && !gsb) || (my.rbuf && rbytes > 0 && !grb))
        return GPUMPI_ERR_NO_MEM;
    my.sbuf = gsb;
    my.rbuf = grb;
    CollArgs a;
    a.kind = kind;
    a.count = 0;
    a.dt = my.stype;
    a.op = 0;
    a.root = root;
    a.esize = 0;
    a.ufn = nullptr;
    a.est_piece = est_piece;
    a.variant = c_rt.variant_override;
    a.learned = a.variant < 0 && kind == JOB_ALLTOALLV && c_rt.selector_mode == 2 && c_rt.mlp_params;
    int rc = coll_run(c, my, a, __LINE__);
    stage_out(ss, false);
    stage_out(rs, true);
    return rc;
}

__device__ long long sample_counts(const int* counts, int n) {
    if (!counts || n <= 0) return 0;
    long long s = 0;
    int k = n < 16 ? n : 16;
    for (int i = 0; i < k; i++) s += counts[(long long)i * n / k];
    return s / k;
}

}  // namespace

// Shared memory starts undefined in every launch: the cache starts from the rank's record of its last
// choice when that record belongs to the current selector epoch, else empty.
__device__ void gpumpi::selector_rank_begin() {
    s_sel.valid = 0;
    if (c_rt.selector_mode != 2 || !c_rt.sel_cache) return;
    const SelCacheRec g = c_rt.sel_cache[me()];
    if (g.epoch != c_rt.sel_epoch) return;
    s_sel.bytes = g.bytes;
    s_sel.kind = g.kind;
    s_sel.n = g.n;
    s_sel.dt = g.dt;
    s_sel.op = g.op;
    s_sel.blocks = g.blocks;
    s_sel.aligned = g.aligned;
    s_sel.variant = g.variant;
    s_sel.valid = 1;
}

// ------------------------------------------------------------------------------------------------
// environment
// ------------------------------------------------------------------------------------------------
__device__ int MPI_Init(int* argc, char*** argv) {
    (void)argc;
    (void)argv;
    c_rt.ranks[me()].initialized = 1;
    return MPI_SUCCESS;
}
__device__ int MPI_Init_thread(int* argc, char*** argv, int required, int* provided) {
    (void)required;
    if (provided) *provided = MPI_THREAD_SINGLE;
    return MPI_Init(argc, argv);
}
__device__ int MPI_Initialized(int* flag) {
    *flag = c_rt.ranks[me()].initialized;
    return MPI_SUCCESS;
}
__device__ int MPI_Finalize(void) {
    c_rt.ranks[me()].finalized = 1;
    return MPI_Barrier(MPI_COMM_WORLD);
}
__device__ int MPI_Finalized(int* flag) {
    *flag = c_rt.ranks[me()].finalized;
    return MPI_SUCCESS;
}
__device__ int MPI_Abort(MPI_Comm comm, int errorcode) {
    (void)comm;
    record_error(GPUMPI_ERR_OTHER, errorcode, __LINE__, errorcode);
    atomicExch(c_rt.abort_flag, 1u);
    return MPI_SUCCESS;
}
// exit() for converted programs: the calling rank ends as if its program had returned `status` (its block
// releases its helper threads, records the status and leaves; the launcher reports a non-zero status as
// the run's failure) and the call does not return.  Ranks still waiting on it get bounded-wait errors, as
// an MPI job fails when one of its processes exits early.  Only the rank's program thread can leave this
// way; a call from another thread records an error and returns.
__device__ void gpumpi_exit(int status) {
    if (threadIdx.x == 0 && is_rank_block()) {
        rank_finish(status);
        asm volatile("exit;" ::: "memory");
    }
    record_error(GPUMPI_ERR_OTHER, GPUMPI_ERR_ARG, __LINE__, status);
}
__device__ int MPI_Get_processor_name(char* name, int* resultlen) {
    const char n[] = "GB300 block-rank";
    for (int i = 0; i < (int)sizeof(n); i++) name[i] = n[i];
    *resultlen = (int)sizeof(n) - 1;
    return MPI_SUCCESS;
}
// Wall-clock time from the GPU's global nanosecond timer (%globaltimer), which every SM reads alike, so
// times taken by different ranks compare directly (the reference scales clock64 by the peak SM clock,
// mpi.cu:142-146, 271-274, which counts per-SM cycles).
__device__ double MPI_Wtime(void) { return (double)now_ns() * 1e-9; }

namespace {
__device__ unsigned long long g_wtick_ns = 0;
}
// The timer's resolution as observed: the shortest step between consecutive distinct readings, over three
// steps (the first change only ends a partial interval); measured once per process and cached.
__device__ double MPI_Wtick(void) {
    unsigned long long tick = *(volatile unsigned long long*)&g_wtick_ns;
    if (tick) return (double)tick * 1e-9;
    unsigned long long best = ~0ULL, prev = now_ns();
    for (int k = 0; k < 4; k++) {
        unsigned long long t = prev;
        for (int spin = 0; spin < (1 << 20) && t == prev; spin++) t = now_ns();
        if (t == prev) break;  // the timer did not move within the spin bound
        if (k > 0 && t - prev < best) best = t - prev;
        prev = t;
    }
    tick = best == ~0ULL ? 1 : best;
    *(volatile unsigned long long*)&g_wtick_ns = tick;
    return (double)tick * 1e-9;
}
__device__ int gpumpi_world_rank(void) { return (int)blockIdx.x; }
__device__ int gpumpi_block_parallel(void (*fn)(void*, int, int), void* arg) {
    Task t;
    t.kind = TASK_USER;
    t.p0 = (const void*)fn;
    t.p1 = arg;
    dispatch(t);
    return MPI_SUCCESS;
}
__device__ void gpumpi_block_sync(int nthreads) { bar_sync(BAR_TASK, nthreads); }
__device__ void* gpumpi_block_scratch(size_t* bytes) {
    if (bytes) *bytes = (size_t)c_rt.dyn_smem;
    return c_rt.dyn_smem > 0 ? (void*)g_dyn_smem : nullptr;
}

// ------------------------------------------------------------------------------------------------
// point-to-point
// ------------------------------------------------------------------------------------------------
__device__ int MPI_Isend(const void* buf, int count, MPI_Datatype datatype, int dest, int tag, MPI_Comm comm,
                         MPI_Request* request) {
    return p2p_isend(buf, count, datatype, dest, tag, comm, request, false);
}
__device__ int MPI_Issend(const void* buf, int count, MPI_Datatype datatype, int dest, int tag, MPI_Comm comm,
                          MPI_Request* request) {
    return p2p_isend(buf, count, datatype, dest, tag, comm, request, true);
}
__device__ int MPI_Irecv(void* buf, int count, MPI_Datatype datatype, int source, int tag, MPI_Comm comm,
                         MPI_Request* request) {
    return p2p_irecv(buf, count, datatype, source, tag, comm, request);
}
__device__ int MPI_Send(const void* buf, int count, MPI_Datatype datatype, int dest, int tag, MPI_Comm comm) {
    MPI_Request r = nullptr;
    int rc = p2p_isend(buf, count, datatype, dest, tag, comm, &r, false, /*blocking*/ true);
    int rw = r ? req_wait(&r, MPI_STATUS_IGNORE) : 0;
    return rc ? rc : rw;
}
__device__ int MPI_Ssend(const void* buf, int count, MPI_Datatype datatype, int dest, int tag, MPI_Comm comm) {
    MPI_Request r = nullptr;
    int rc = p2p_isend(buf, count, datatype, dest, tag, comm, &r, true);
    int rw = r ? req_wait(&r, MPI_STATUS_IGNORE) : 0;
    return rc ? rc : rw;
}
__device__ int MPI_Recv(void* buf, int count, MPI_Datatype datatype, int source, int tag, MPI_Comm comm,
                        MPI_Status* status) {
    MPI_Request r = nullptr;
    int rc = p2p_irecv(buf, count, datatype, source, tag, comm, &r);
    int rw = r ? req_wait(&r, status) : 0;
    return rc ? rc : rw;
}
__device__ int MPI_Sendrecv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, int dest, int sendtag,
                            void* recvbuf, int recvcount, MPI_Datatype recvtype, int source, int recvtag,
                            MPI_Comm comm, MPI_Status* status) {
    // the reference returns without doing anything (gpu_libs/gpu_mpi/mpi.cu:255-260); this is MPI's
    // definition: a send and a receive executed concurrently
    MPI_Request rq[2] = {nullptr, nullptr};
    int rc = p2p_irecv(recvbuf, recvcount, recvtype, source, recvtag, comm, &rq[0]);
    int rs = p2p_isend(sendbuf, sendcount, sendtype, dest, sendtag, comm, &rq[1], false, /*blocking*/ true);
    int w0 = rq[0] ? req_wait(&rq[0], status) : 0;
    int w1 = rq[1] ? req_wait(&rq[1], MPI_STATUS_IGNORE) : 0;
    return rc ? rc : rs ? rs : w0 ? w0 : w1;
}
__device__ int MPI_Wait(MPI_Request* request, MPI_Status* status) {
    if (!request) return GPUMPI_ERR_REQUEST;
    return req_wait(request, status);
}
__device__ int MPI_Waitall(int count, MPI_Request reqs[], MPI_Status* statuses) {
    // statuses may be MPI_STATUSES_IGNORE (the reference indexes it unconditionally, mpi.cu:579-585)
    int err = 0;
    Deadline dl = make_deadline();
    for (;;) {
        bool all = true;
        for (int i = 0; i < count; i++) {
            if (reqs[i] == MPI_REQUEST_NULL) continue;
            if (req_poll(reqs[i])) {
                int e = req_wait(&reqs[i], statuses ? &statuses[i] : nullptr);
                if (e && !err) err = e;
            } else {
                all = false;
            }
        }
        if (all) return err;
        progress();
        if (int e = wait_tick(dl, __LINE__)) return e;
    }
}
__device__ int MPI_Waitany(int count, MPI_Request reqs[], int* index, MPI_Status* status) {
    Deadline dl = make_deadline();
    for (;;) {
        bool any_active = false;
        for (int i = 0; i < count; i++) {
            if (reqs[i] == MPI_REQUEST_NULL) continue;
            any_active = true;
            if (req_poll(reqs[i])) {
                *index = i;
                return req_wait(&reqs[i], status);
            }
        }
        if (!any_active) {
            *index = MPI_UNDEFINED;
            return MPI_SUCCESS;
        }
        progress();
        if (int e = wait_tick(dl, __LINE__)) return e;
    }
}
__device__ int MPI_Waitsome(int incount, MPI_Request reqs[], int* outcount, int indices[], MPI_Status statuses[]) {
    Deadline dl = make_deadline();
    for (;;) {
        int n = 0;
        bool any_active = false;
        for (int i = 0; i < incount; i++) {
            if (reqs[i] == MPI_REQUEST_NULL) continue;
            any_active = true;
            if (req_poll(reqs[i])) {
                req_wait(&reqs[i], statuses ? &statuses[n] : nullptr);
                indices[n++] = i;
            }
        }
        if (!any_active) {
            *outcount = MPI_UNDEFINED;
            return MPI_SUCCESS;
        }
        if (n > 0) {
            *outcount = n;
            return MPI_SUCCESS;
        }
        progress();
        if (int e = wait_tick(dl, __LINE__)) return e;
    }
}
__device__ int MPI_Test(MPI_Request* request, int* flag, MPI_Status* status) {
    if (!request) return GPUMPI_ERR_REQUEST;
    if (*request == MPI_REQUEST_NULL) {
        *flag = 1;
        if (status) *status = MPI_Status();
        return MPI_SUCCESS;
    }
    progress();
    if (req_poll(*request)) {
        *flag = 1;
        return req_wait(request, status);
    }
    *flag = 0;
    return MPI_SUCCESS;
}
__device__ int MPI_Testall(int count, MPI_Request reqs[], int* flag, MPI_Status statuses[]) {
    progress();
    for (int i = 0; i < count; i++)
        if (reqs[i] != MPI_REQUEST_NULL && !req_poll(reqs[i])) {
            *flag = 0;
            return MPI_SUCCESS;
        }
    *flag = 1;
    int err = 0;
    for (int i = 0; i < count; i++)
        if (reqs[i] != MPI_REQUEST_NULL) {
            int e = req_wait(&reqs[i], statuses ? &statuses[i] : nullptr);
            if (e && !err) err = e;
        }
    return err;
}
__device__ int MPI_Request_free(MPI_Request* request) {
    if (!request || !*request) return MPI_SUCCESS;
    MPI_Request_impl* q = *request;
    if (req_poll(q)) {
        req_release(q);
    } else if (q->kind == REQ_RECV) {
        q->freed = 1;  // recycled when the message arrives
    } else {
        // an active rendezvous send: its completion flag is written by the receiver later, so the
        // request slot is only recycled once that happened (bounded wait)
        req_wait(request, MPI_STATUS_IGNORE);
    }
    *request = MPI_REQUEST_NULL;
    return MPI_SUCCESS;
}
__device__ int MPI_Iprobe(int source, int tag, MPI_Comm comm, int* flag, MPI_Status* status) {
    MPI_Comm_impl* c = check_comm(comm);
    if (!c) return GPUMPI_ERR_COMM;
    progress();
    RankState* R = &c_rt.ranks[me()];
    for (int k = R->uq_head; k < R->uq_tail; k++) {
        if (!uq_at(k)->live) continue;
        const Envelope& e = uq_at(k)->env;
        if (e.ctx == c->ctx && (source == MPI_ANY_SOURCE || source == e.src) && (tag == MPI_ANY_TAG || tag == e.tag)) {
            *flag = 1;
            if (status) {
                status->MPI_SOURCE = e.src;
                status->MPI_TAG = e.tag;
                status->MPI_ERROR = 0;
                status->count_bytes = e.bytes;
            }
            return MPI_SUCCESS;
        }
    }
    *flag = 0;
    return MPI_SUCCESS;
}
__device__ int MPI_Probe(int source, int tag, MPI_Comm comm, MPI_Status* status) {
    Deadline dl = make_deadline();
    for (;;) {
        int flag = 0;
        int rc = MPI_Iprobe(source, tag, comm, &flag, status);
        if (rc || flag) return rc;
        if (int e = wait_tick(dl, __LINE__)) return e;
    }
}
__device__ int MPI_Get_count(const MPI_Status* status, MPI_Datatype datatype, int* count) {
    const TypeDesc* t = tdesc(datatype);
    if (!t) return GPUMPI_ERR_TYPE;
    if (t->size == 0 || status->count_bytes % t->size) {
        *count = MPI_UNDEFINED;
        return MPI_SUCCESS;
    }
    *count = (int)(status->count_bytes / t->size);
    return MPI_SUCCESS;
}

// ------------------------------------------------------------------------------------------------
// collectives
// ------------------------------------------------------------------------------------------------
__device__ int MPI_Barrier(MPI_Comm comm) {
    MPI_Comm_impl* c = check_comm(comm);
    if (!c) return GPUMPI_ERR_COMM;
    // barrier on any communicator (the reference implements only the world, mpi.cu:324-331)
    return comm_barrier(c, []() {}, __LINE__);
}

__device__ int MPI_Allreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype datatype, MPI_Op op,
                             MPI_Comm comm) {
    return fold_collective(JOB_ALLREDUCE, sendbuf, recvbuf, count, datatype, op, 0, comm);
}

__device__ int MPI_Reduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype datatype, MPI_Op op, int root,
                          MPI_Comm comm) {
    return fold_collective(JOB_REDUCE, sendbuf, recvbuf, count, datatype, op, root, comm);
}

__device__ int MPI_Bcast(void* buffer, int count, MPI_Datatype datatype, int root, MPI_Comm comm) {
    MPI_Comm_impl* c = check_comm(comm);
    if (!c) return GPUMPI_ERR_COMM;
    if (root < 0 || root >= c->size) return GPUMPI_ERR_ROOT;
    const TypeDesc* t = tdesc(datatype);
    if (!t) return GPUMPI_ERR_TYPE;
    if (count < 0) return GPUMPI_ERR_COUNT;
    if (count == 0 || c->size == 1) return MPI_SUCCESS;
    long long bytes = (long long)count * t->size;
    long long span = t->lb + (long long)count * t->extent;
    const int cr = comm_rank_of(c, me());
    if (bytes <= TINY_BYTES && c->tiny) {
        // tiny broadcast: the root's packed bytes travel in its inline slot, one barrier (the parity
        // argument of the tiny reductions).  The choice depends on the message size only, which every
        // member shares; each member packs or unpacks its own datatype and buffer.
        const TypeDesc* d = desc_contiguous(t) ? nullptr : t;
        const unsigned g = ld_acquire(&c->bar_gen);
        if (cr == root) t0_copy(c->tiny + ((size_t)cr * 2 + (g & 1)) * TINY_BYTES, nullptr, buffer, d, bytes);
        int rc = comm_barrier_from(c, g, []() {}, __LINE__);
        if (!rc && cr != root) t0_copy(buffer, d, c->tiny + ((size_t)root * 2 + (g & 1)) * TINY_BYTES, nullptr, bytes);
        return rc;
    }
    Stage st;
    void* gb = buffer;
    if (!is_global_ptr(buffer)) {
        if (t->nlev != 0 || t->lb != 0) return GPUMPI_ERR_BUFFER;
        gb = stage_in(st, buffer, span, cr == root);
        if (!gb) return GPUMPI_ERR_NO_MEM;
    }
    CollSlot my{};
    my.sbuf = gb;
    my.rbuf = gb;
    my.scount = count;
    my.rcount = count;
    my.sdesc = t;
    my.rdesc = t;
    my.stype = datatype;
    my.rtype = datatype;
    if (c_rt.variant_override < 0 && bytes <= c_rt.static_bcast_bytes) {
        // small broadcast without a job: every member copies its own piece from the root's buffer between
        // two barriers (the second keeps the root's buffer valid until every member has read it)
        c->slots[cr] = my;
        int rc = comm_barrier(c, []() {}, __LINE__);
        if (!rc && cr != root) {
            const CollSlot* rs = &c->slots[root];
            const void* src = (const void*)__ldcg((const unsigned long long*)&rs->sbuf);
            const TypeDesc* sd = (const TypeDesc*)__ldcg((const unsigned long long*)&rs->sdesc);
            t0_copy(gb, desc_contiguous(t) ? nullptr : t, src, desc_contiguous(sd) ? nullptr : sd, bytes);
        }
        const int rc2 = comm_barrier(c, []() {}, __LINE__);
        stage_out(st, cr != root);
        return rc ? rc : rc2;
    }
    CollArgs a;
    a.kind = JOB_BCAST;
    a.count = 0;
    a.dt = datatype;
    a.op = 0;
    a.root = root;
    a.esize = 0;
    a.ufn = nullptr;
    a.est_piece = bytes;
    a.variant = -1;
    int rc = coll_run(c, my, a, __LINE__);
    stage_out(st, cr != root);
    return rc;
}

__device__ int MPI_Alltoallv(const void* sendbuf, const int sendcounts[], const int sdispls[], MPI_Datatype sendtype,
                             void* recvbuf, const int recvcounts[], const int rdispls[], MPI_Datatype recvtype,
                             MPI_Comm comm) {
    MPI_Comm_impl* c = check_comm(comm);
    if (!c) return GPUMPI_ERR_COMM;
    const TypeDesc* st = tdesc(sendtype);
    const TypeDesc* rt = tdesc(recvtype);
    if (!st || !rt) return GPUMPI_ERR_TYPE;
    const int n = c->size;
    if (sendbuf == MPI_IN_PLACE) return GPUMPI_ERR_ARG;
    // spans of the user buffers (for staging thread-local buffers)
    long long sspan = 0, rspan = 0;
    if (!is_global_ptr(sendbuf) || !is_global_ptr(recvbuf)) {
        for (int i = 0; i < n; i++) {
            long long se = st->lb + ((long long)sdispls[i] + sendcounts[i]) * st->extent;
            long long re = rt->lb + ((long long)rdispls[i] + recvcounts[i]) * rt->extent;
            sspan = se > sspan ? se : sspan;
            rspan = re > rspan ? re : rspan;
        }
    }
    Stage s1, s2, s3, s4;
    CollSlot my{};
    my.sbuf = sendbuf;
    my.rbuf = recvbuf;
    my.scounts = stage_ints(s1, sendcounts, n);
    my.sdispls = stage_ints(s2, sdispls, n);
    my.rcounts = stage_ints(s3, recvcounts, n);
    my.rdispls = stage_ints(s4, rdispls, n);
    my.sdesc = st;
    my.rdesc = rt;
    my.stype = sendtype;
    my.rtype = recvtype;
    // the set-up estimates from 8 members' counts with 16 or more members (shared_piece_estimate)
    long long est = n < 16 ? sample_counts(sendcounts, n) * st->size : 0;
    int rc = pull_collective(JOB_ALLTOALLV, c, my, sspan, rspan, est, 0);
    stage_out(s1, false);
    stage_out(s2, false);
    stage_out(s3, false);
    stage_out(s4, false);
    return rc;
}

namespace {
__device__ int small_alltoall(MPI_Comm_impl* c, const void* sendbuf, int sendcount, const TypeDesc* st, void* recvbuf,
                              int recvcount, const TypeDesc* rt);
}

__device__ int MPI_Alltoall(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, int recvcount,
                            MPI_Datatype recvtype, MPI_Comm comm) {
    // the reference builds four count/displacement arrays with malloc and calls Alltoallv
    // (gpu_libs/gpu_mpi/mpi.cu:333-362); here the uniform layout is described by two scalars
    MPI_Comm_impl* c = check_comm(comm);
    if (!c) return GPUMPI_ERR_COMM;
    const TypeDesc* st = tdesc(sendtype);
    const TypeDesc* rt = tdesc(recvtype);
    if (!st || !rt) return GPUMPI_ERR_TYPE;
    if (sendcount < 0 || recvcount < 0) return GPUMPI_ERR_COUNT;
    const int n = c->size;
    if (int rc = small_alltoall(c, sendbuf, sendcount, st, recvbuf, recvcount, rt); rc != -1) return rc;
    Stage tmp;
    const void* sb = sendbuf;
    if (sendbuf == MPI_IN_PLACE) {  // in place: the send data is the receive buffer's old contents
        sendcount = recvcount;
        sendtype = recvtype;
        st = rt;
        long long span = rt->lb + (long long)n * recvcount * rt->extent;
        tmp.heap = scratch_alloc((unsigned long long)(span > 0 ? span : 1));
        if (!tmp.heap) return GPUMPI_ERR_NO_MEM;
        t0_copy(tmp.heap, nullptr, recvbuf, nullptr, span);
        sb = tmp.heap;
    }
    CollSlot my{};
    my.sbuf = sb;
    my.rbuf = recvbuf;
    my.scount = sendcount;
    my.rcount = recvcount;
    my.sdesc = st;
    my.rdesc = rt;
    my.stype = sendtype;
    my.rtype = recvtype;
    long long sspan = st->lb + (long long)n * sendcount * st->extent;
    long long rspan = rt->lb + (long long)n * recvcount * rt->extent;
    int rc = pull_collective(JOB_ALLTOALLV, c, my, sspan, rspan, (long long)sendcount * st->size, 0);
    scratch_free(tmp.heap);
    return rc;
}

namespace {
// n small pieces into dst + q * bytes, piece q from member q's inline slot of parity p (tiny allgather) or
// from member q's published send buffer at offset cr * bytes (small alltoall); the block copies them in
// 16-byte parts, one part per thread, so that the parts of all pieces are in flight together.
struct PieceGather {
    const unsigned char* tiny;
    const CollSlot* slots;
    unsigned char* dst;
    int n, parity, bytes, cr;
};
__shared__ PieceGather s_piece_gather;
__device__ void piece_gather_task(void* arg, int tid, int nt) {
    const PieceGather* w = (const PieceGather*)arg;
    const int parts = (w->bytes + 15) / 16;
    for (int x = tid; x < w->n * parts; x += nt) {
        const int q = x / parts, k = x % parts;
        const unsigned char* base =
            w->tiny ? w->tiny + ((size_t)q * 2 + w->parity) * TINY_BYTES : (const unsigned char*)slot_in(&w->slots[q]);
        if (!base) continue;  // a member that could not stage its buffer published none
        const unsigned char* src = w->tiny ? base : base + (size_t)w->cr * w->bytes;
        const int len = min(16, w->bytes - 16 * k);
        small_copy(w->dst + (size_t)q * w->bytes + 16 * k, src + 16 * k, len);
    }
}
__device__ __forceinline__ void piece_gather(const unsigned char* tiny, const CollSlot* slots, void* dst, int n,
                                             int parity, int bytes, int cr);

// Small uniform alltoall and allgather (at most SMALL_PIECE bytes per pair or contribution and 64 KiB per
// member, any datatypes and buffers): each member publishes its send buffer, a barrier, every member pulls
// its n pieces straight from the senders' buffers, and a second barrier before any sender may reuse its
// buffer.  Two barriers instead of a job of n^2 (or n) pieces: 1024 ranks x 4 bytes of alltoall took about
// 90 us as a job.  A member whose buffers are thread-local or whose types are not contiguous packs and
// unpacks through its scratch pool.  Returns -1 when the call does not qualify (the choice depends only on
// what every member shares: sizes and the policy).
constexpr long long SMALL_PIECE = 4096;
__device__ int small_pull(MPI_Comm_impl* c, const void* sendbuf, int sendcount, const TypeDesc* st, void* recvbuf,
                          int recvcount, const TypeDesc* rt, bool gather) {
    const long long pb = (long long)sendcount * st->size;
    if (sendbuf == MPI_IN_PLACE || sendcount < 0 || pb != (long long)recvcount * rt->size || pb > SMALL_PIECE ||
        pb * c->size > 65536 || c_rt.variant_override >= 0)
        return -1;
    const int bytes = (int)pb, n = c->size;
    const int cr = comm_rank_of(c, me());
    const long long all = (long long)n * bytes, sall = gather ? bytes : all;
    const bool direct_send = desc_contiguous(st) && is_global_ptr(sendbuf);
    const bool direct_recv = desc_contiguous(rt) && is_global_ptr(recvbuf);
    void* sstage = direct_send || sall == 0 ? nullptr : scratch_alloc((unsigned long long)sall);
    void* rstage = direct_recv || all == 0 ? nullptr : scratch_alloc((unsigned long long)all);
    int rc = 0;
    if ((!direct_send && sall && !sstage) || (!direct_recv && all && !rstage)) rc = GPUMPI_ERR_NO_MEM;
    if (sstage) t0_copy(sstage, nullptr, sendbuf, desc_contiguous(st) ? nullptr : st, sall);
    c->slots[cr].sbuf = direct_send ? sendbuf : sstage;  // nullptr when staging failed: the others skip it
    // (a member that could not stage still takes part in both barriers, so the others do not wait)
    const int rb = comm_barrier(c, []() {}, __LINE__);
    if (!rc) rc = rb;
    // piece q of member cr: member q's send buffer at cr * bytes (alltoall) or at 0 (allgather)
    if (!rc && bytes > 0) piece_gather(nullptr, c->slots, rstage ? rstage : recvbuf, n, 0, bytes, gather ? 0 : cr);
    const int rb2 = comm_barrier(c, []() {}, __LINE__);
    if (!rc) rc = rb2;
    if (!rc && rstage) t0_copy(recvbuf, desc_contiguous(rt) ? nullptr : rt, rstage, nullptr, all);
    scratch_free(rstage);
    scratch_free(sstage);
    return rc;
}
__device__ int small_alltoall(MPI_Comm_impl* c, const void* sendbuf, int sendcount, const TypeDesc* st, void* recvbuf,
                              int recvcount, const TypeDesc* rt) {
    return small_pull(c, sendbuf, sendcount, st, recvbuf, recvcount, rt, false);
}

__device__ __forceinline__ void piece_gather(const unsigned char* tiny, const CollSlot* slots, void* dst, int n,
                                             int parity, int bytes, int cr) {
    PieceGather* w = &s_piece_gather;
    w->tiny = tiny;
    w->slots = slots;
    w->dst = (unsigned char*)dst;
    w->n = n;
    w->parity = parity;
    w->bytes = bytes;
    w->cr = cr;
    Task t;
    t.kind = TASK_USER;
    t.p0 = (const void*)&piece_gather_task;
    t.p1 = w;
    dispatch(t);
}
}  // namespace

__device__ int MPI_Allgather(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, int recvcount,
                             MPI_Datatype recvtype, MPI_Comm comm) {
    MPI_Comm_impl* c = check_comm(comm);
    if (!c) return GPUMPI_ERR_COMM;
    const TypeDesc* st = tdesc(sendtype);
    const TypeDesc* rt = tdesc(recvtype);
    if (!rt || (sendbuf != MPI_IN_PLACE && !st)) return GPUMPI_ERR_TYPE;
    const int n = c->size;
    const int cr = comm_rank_of(c, me());
    if (sendbuf != MPI_IN_PLACE && c->tiny && sendcount >= 0 && recvcount >= 0 &&
        (long long)sendcount * st->size <= TINY_BYTES &&
        (long long)sendcount * st->size == (long long)recvcount * rt->size) {
        // tiny contributions (the choice depends on the contribution size only, which every member
        // shares): packed into the inline slots, one barrier (the parity argument of the tiny
        // reductions), then each member unpacks the n contributions
        const int bytes = (int)((long long)sendcount * st->size);
        const unsigned g = ld_acquire(&c->bar_gen);
        t0_copy(c->tiny + ((size_t)cr * 2 + (g & 1)) * TINY_BYTES, nullptr, sendbuf, desc_contiguous(st) ? nullptr : st,
                bytes);
        const int rc = comm_barrier_from(c, g, []() {}, __LINE__);
        if (rc || bytes == 0) return rc;
        if (desc_contiguous(rt) && is_global_ptr(recvbuf)) {
            piece_gather(c->tiny, nullptr, recvbuf, n, (int)(g & 1), bytes, cr);
        } else {
            for (int q = 0; q < n; q++)
                t0_copy((char*)recvbuf + (long long)q * recvcount * rt->extent, desc_contiguous(rt) ? nullptr : rt,
                        c->tiny + ((size_t)q * 2 + (g & 1)) * TINY_BYTES, nullptr, bytes);
        }
        return MPI_SUCCESS;
    }
    if (sendbuf != MPI_IN_PLACE) {
        if (int rc = small_pull(c, sendbuf, sendcount, st, recvbuf, recvcount, rt, true); rc != -1) return rc;
    }
    CollSlot my{};
    my.rbuf = recvbuf;
    my.rcount = recvcount;
    my.rdesc = rt;
    my.rtype = recvtype;
    long long rspan = rt->lb + (long long)n * recvcount * rt->extent;
    if (sendbuf == MPI_IN_PLACE) {
        my.sbuf = MPI_IN_PLACE;  // resolved after staging below
        my.scount = recvcount;
        my.sdesc = rt;
        my.stype = recvtype;
    } else {
        my.sbuf = sendbuf;
        my.scount = sendcount;
        my.sdesc = st;
        my.stype = sendtype;
    }
    long long sspan = my.sbuf == MPI_IN_PLACE ? 0 : st->lb + (long long)sendcount * st->extent;
    Stage ss, rs;
    const void* gsb = my.sbuf == MPI_IN_PLACE ? MPI_IN_PLACE : stage_in(ss, my.sbuf, sspan, true);
    void* grb = stage_in(rs, recvbuf, rspan, sendbuf == MPI_IN_PLACE);
    if (!grb || !gsb) return GPUMPI_ERR_NO_MEM;
    if (gsb == MPI_IN_PLACE) gsb = (const char*)grb + (long long)cr * recvcount * rt->extent;
    my.sbuf = gsb;
    my.rbuf = grb;
    CollArgs a;
    a.kind = JOB_ALLGATHERV;
    a.count = 0;
    a.dt = recvtype;
    a.op = 0;
    a.root = 0;
    a.esize = 0;
    a.ufn = nullptr;
    a.est_piece = (long long)my.scount * my.sdesc->size;
    a.variant = -1;
    int rc = coll_run(c, my, a, __LINE__);
    stage_out(ss, false);
    stage_out(rs, true);
    return rc;
}

__device__ int MPI_Allgatherv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf,
                              const int recvcounts[], const int displs[], MPI_Datatype recvtype, MPI_Comm comm) {
    MPI_Comm_impl* c = check_comm(comm);
    if (!c) return GPUMPI_ERR_COMM;
    const TypeDesc* st = tdesc(sendtype);
    const TypeDesc* rt = tdesc(recvtype);
    if (!rt || (sendbuf != MPI_IN_PLACE && !st)) return GPUMPI_ERR_TYPE;
    const int n = c->size;
    const int cr = comm_rank_of(c, me());
    long long rspan = 0;
    for (int i = 0; i < n; i++) {
        long long e = rt->lb + ((long long)displs[i] + recvcounts[i]) * rt->extent;
        rspan = e > rspan ? e : rspan;
    }
    Stage ss, rs, s3, s4;
    CollSlot my{};
    my.rcounts = stage_ints(s3, recvcounts, n);
    my.rdispls = stage_ints(s4, displs, n);
    my.rdesc = rt;
    my.rtype = recvtype;
    void* grb = stage_in(rs, recvbuf, rspan, sendbuf == MPI_IN_PLACE);
    if (!grb) return GPUMPI_ERR_NO_MEM;
    if (sendbuf == MPI_IN_PLACE) {
        my.sbuf = (const char*)grb + (long long)displs[cr] * rt->extent;
        my.scount = recvcounts[cr];
        my.sdesc = rt;
        my.stype = recvtype;
    } else {
        my.sbuf = stage_in(ss, sendbuf, st->lb + (long long)sendcount * st->extent, true);
        my.scount = sendcount;
        my.sdesc = st;
        my.stype = sendtype;
    }
    my.rbuf = grb;
    CollArgs a;
    a.kind = JOB_ALLGATHERV;
    a.count = 0;
    a.dt = recvtype;
    a.op = 0;
    a.root = 0;
    a.esize = 0;
    a.ufn = nullptr;
    a.est_piece = (long long)my.scount * my.sdesc->size;
    a.variant = -1;
    int rc = coll_run(c, my, a, __LINE__);
    stage_out(ss, false);
    stage_out(rs, true);
    stage_out(s3, false);
    stage_out(s4, false);
    return rc;
}

__device__ int MPI_Gatherv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf,
                           const int recvcounts[], const int displs[], MPI_Datatype recvtype, int root, MPI_Comm comm) {
    MPI_Comm_impl* c = check_comm(comm);
    if (!c) return GPUMPI_ERR_COMM;
    if (root < 0 || root >= c->size) return GPUMPI_ERR_ROOT;
    const int n = c->size;
    const int cr = comm_rank_of(c, me());
    const TypeDesc* st = sendbuf == MPI_IN_PLACE ? nullptr : tdesc(sendtype);
    const TypeDesc* rt = cr == root ? tdesc(recvtype) : nullptr;
    if ((sendbuf != MPI_IN_PLACE && !st) || (cr == root && !rt)) return GPUMPI_ERR_TYPE;
    Stage s3, s4;
    CollSlot my{};
    my.sbuf = sendbuf;
    my.scount = sendcount;
    my.sdesc = st ? st : rt;
    my.stype = sendtype;
    long long rspan = 0;
    if (cr == root) {
        for (int i = 0; i < n; i++) {
            long long e = rt->lb + ((long long)displs[i] + recvcounts[i]) * rt->extent;
            rspan = e > rspan ? e : rspan;
        }
        my.rbuf = recvbuf;
        my.rcounts = stage_ints(s3, recvcounts, n);
        my.rdispls = stage_ints(s4, displs, n);
        my.rdesc = rt;
        my.rtype = recvtype;
    } else {
        my.rdesc = st;
    }
    long long sspan = st ? st->lb + (long long)sendcount * st->extent : 0;
    int rc = pull_collective(JOB_GATHERV, c, my, sspan, cr == root ? rspan : 0,
                             st ? (long long)sendcount * st->size : 0, root);
    stage_out(s3, false);
    stage_out(s4, false);
    return rc;
}

__device__ int MPI_Gather(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, int recvcount,
                          MPI_Datatype recvtype, int root, MPI_Comm comm) {
    MPI_Comm_impl* c = check_comm(comm);
    if (!c) return GPUMPI_ERR_COMM;
    if (root < 0 || root >= c->size) return GPUMPI_ERR_ROOT;
    const int n = c->size;
    const int cr = comm_rank_of(c, me());
    const TypeDesc* st = sendbuf == MPI_IN_PLACE ? nullptr : tdesc(sendtype);
    const TypeDesc* rt = cr == root ? tdesc(recvtype) : nullptr;
    if ((sendbuf != MPI_IN_PLACE && !st) || (cr == root && !rt)) return GPUMPI_ERR_TYPE;
    CollSlot my{};
    my.sbuf = sendbuf;
    my.scount = sendcount;
    my.sdesc = st ? st : rt;
    my.stype = sendtype;
    long long rspan = 0;
    if (cr == root) {
        my.rbuf = recvbuf;
        my.rcount = recvcount;
        my.rdesc = rt;
        my.rtype = recvtype;
        rspan = rt->lb + (long long)n * recvcount * rt->extent;
    } else {
        my.rdesc = st;
    }
    long long sspan = st ? st->lb + (long long)sendcount * st->extent : 0;
    return pull_collective(JOB_GATHERV, c, my, sspan, rspan, st ? (long long)sendcount * st->size : 0, root);
}

__device__ int MPI_Scatterv(const void* sendbuf, const int sendcounts[], const int displs[], MPI_Datatype sendtype,
                            void* recvbuf, int recvcount, MPI_Datatype recvtype, int root, MPI_Comm comm) {
    MPI_Comm_impl* c = check_comm(comm);
    if (!c) return GPUMPI_ERR_COMM;
    if (root < 0 || root >= c->size) return GPUMPI_ERR_ROOT;
    const int n = c->size;
    const int cr = comm_rank_of(c, me());
    const TypeDesc* st = cr == root ? tdesc(sendtype) : nullptr;
    const TypeDesc* rt = recvbuf == MPI_IN_PLACE ? nullptr : tdesc(recvtype);
    if ((cr == root && !st) || (recvbuf != MPI_IN_PLACE && !rt)) return GPUMPI_ERR_TYPE;
    Stage s1, s2;
    CollSlot my{};
    my.rbuf = recvbuf;
    my.rcount = recvcount;
    my.rdesc = rt ? rt : st;
    my.rtype = recvtype;
    long long sspan = 0;
    if (cr == root) {
        for (int i = 0; i < n; i++) {
            long long e = st->lb + ((long long)displs[i] + sendcounts[i]) * st->extent;
            sspan = e > sspan ? e : sspan;
        }
        my.sbuf = sendbuf;
        my.scounts = stage_ints(s1, sendcounts, n);
        my.sdispls = stage_ints(s2, displs, n);
        my.sdesc = st;
        my.stype = sendtype;
    } else {
        my.sdesc = rt;
    }
    long long rspan = rt ? rt->lb + (long long)recvcount * rt->extent : 0;
    int rc = pull_collective(JOB_SCATTERV, c, my, sspan, rspan, rt ? (long long)recvcount * rt->size : 0, root);
    stage_out(s1, false);
    stage_out(s2, false);
    return rc;
}

__device__ int MPI_Scatter(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, int recvcount,
                           MPI_Datatype recvtype, int root, MPI_Comm comm) {
    MPI_Comm_impl* c = check_comm(comm);
    if (!c) return GPUMPI_ERR_COMM;
    if (root < 0 || root >= c->size) return GPUMPI_ERR_ROOT;
    const int n = c->size;
    const int cr = comm_rank_of(c, me());
    const TypeDesc* st = cr == root ? tdesc(sendtype) : nullptr;
    const TypeDesc* rt = recvbuf == MPI_IN_PLACE ? nullptr : tdesc(recvtype);
    if ((cr == root && !st) || (recvbuf != MPI_IN_PLACE && !rt)) return GPUMPI_ERR_TYPE;
    CollSlot my{};
    my.rbuf = recvbuf;
    my.rcount = recvcount;
    my.rdesc = rt ? rt : st;
    my.rtype = recvtype;
    long long sspan = 0;
    if (cr == root) {
        my.sbuf = sendbuf;
        my.scount = sendcount;
        my.sdesc = st;
        my.stype = sendtype;
        sspan = st->lb + (long long)n * sendcount * st->extent;
    } else {
        my.sdesc = rt;
    }
    long long rspan = rt ? rt->lb + (long long)recvcount * rt->extent : 0;
    return pull_collective(JOB_SCATTERV, c, my, sspan, rspan, rt ? (long long)recvcount * rt->size : 0, root);
}

// ------------------------------------------------------------------------------------------------
// operators
// ------------------------------------------------------------------------------------------------
__device__ int MPI_Op_create(MPI_User_function* user_fn, int commute, MPI_Op* op) {
    MPI_Op o = (MPI_Op)malloc(sizeof(MPI_Op_impl));
    if (!o) return GPUMPI_ERR_NO_MEM;
    o->code = GPUMPI_OP_USER;
    o->fn = user_fn;
    o->commute = commute;
    *op = o;
    return MPI_SUCCESS;
}
__device__ int MPI_Op_free(MPI_Op* op) {
    if (op && *op && (*op)->code == GPUMPI_OP_USER) free(*op);
    if (op) *op = MPI_OP_NULL;
    return MPI_SUCCESS;
}

// ------------------------------------------------------------------------------------------------
// datatypes
// ------------------------------------------------------------------------------------------------
__device__ int MPI_Type_size(MPI_Datatype datatype, int* size) {
    const TypeDesc* t = tdesc(datatype);
    if (!t) return GPUMPI_ERR_TYPE;
    *size = (int)t->size;
    return MPI_SUCCESS;
}
__device__ int MPI_Type_get_extent(MPI_Datatype datatype, MPI_Aint* lb, MPI_Aint* extent) {
    const TypeDesc* t = tdesc(datatype);
    if (!t) return GPUMPI_ERR_TYPE;
    *lb = 0;
    *extent = t->extent;
    return MPI_SUCCESS;
}
namespace {
__device__ int new_type(const TypeDesc& d, MPI_Datatype* out) {
    TypeDesc* slot;
    int h = type_alloc(&slot);
    if (h < 0) return GPUMPI_ERR_NO_MEM;
    *slot = d;
    slot->in_use = 1;
    slot->committed = 0;
    desc_prepare(slot);
    *out = (MPI_Datatype)h;
    return MPI_SUCCESS;
}
}  // namespace
__device__ int MPI_Type_contiguous(int count, MPI_Datatype oldtype, MPI_Datatype* newtype) {
    const TypeDesc* o = tdesc(oldtype);
    if (!o) return GPUMPI_ERR_TYPE;
    TypeDesc d;
    int rc = type_hvector_desc(count, 1, o->extent, o, &d);
    if (rc) return rc;
    d.base = o->base;
    return new_type(d, newtype);
}
__device__ int MPI_Type_vector(int count, int blocklength, int stride, MPI_Datatype oldtype, MPI_Datatype* newtype) {
    const TypeDesc* o = tdesc(oldtype);
    if (!o) return GPUMPI_ERR_TYPE;
    if (stride < 0) return GPUMPI_ERR_ARG;
    TypeDesc d;
    int rc = type_hvector_desc(count, blocklength, (long long)stride * o->extent, o, &d);
    if (rc) return rc;
    d.base = o->base;
    return new_type(d, newtype);
}
__device__ int MPI_Type_create_hvector(int count, int blocklength, MPI_Aint stride, MPI_Datatype oldtype,
                                       MPI_Datatype* newtype) {
    const TypeDesc* o = tdesc(oldtype);
    if (!o) return GPUMPI_ERR_TYPE;
    if (stride < 0) return GPUMPI_ERR_ARG;
    TypeDesc d;
    int rc = type_hvector_desc(count, blocklength, stride, o, &d);
    if (rc) return rc;
    d.base = o->base;
    return new_type(d, newtype);
}
__device__ int MPI_Type_create_subarray(int ndims, const int sizes[], const int subsizes[], const int starts[],
                                        int order, MPI_Datatype oldtype, MPI_Datatype* newtype) {
    const TypeDesc* o = tdesc(oldtype);
    if (!o) return GPUMPI_ERR_TYPE;
    TypeDesc d;
    int rc = type_subarray_desc(ndims, sizes, subsizes, starts, order, o, &d);
    if (rc) return rc;
    d.base = o->base;
    return new_type(d, newtype);
}
__device__ int MPI_Type_commit(MPI_Datatype* datatype) {
    if (!datatype) return GPUMPI_ERR_TYPE;
    if (!is_derived(*datatype)) return MPI_SUCCESS;
    TypeDesc* t = (TypeDesc*)tdesc(*datatype);
    if (!t) return GPUMPI_ERR_TYPE;
    t->committed = 1;
    return MPI_SUCCESS;
}
__device__ int MPI_Type_free(MPI_Datatype* datatype) {
    if (!datatype || !is_derived(*datatype)) return GPUMPI_ERR_TYPE;
    TypeDesc* t = (TypeDesc*)tdesc(*datatype);
    if (t) t->in_use = 0;
    *datatype = MPI_DATATYPE_NULL;
    return MPI_SUCCESS;
}

// ------------------------------------------------------------------------------------------------
// communicators and groups
// ------------------------------------------------------------------------------------------------
__device__ int MPI_Comm_size(MPI_Comm comm, int* size) {
    MPI_Comm_impl* c = check_comm(comm);
    if (!c) return GPUMPI_ERR_COMM;
    *size = c->size;
    return MPI_SUCCESS;
}
__device__ int MPI_Comm_rank(MPI_Comm comm, int* rank) {
    MPI_Comm_impl* c = check_comm(comm);
    if (!c) return GPUMPI_ERR_COMM;
    *rank = comm_rank_of(c, me());
    return MPI_SUCCESS;
}
__device__ int MPI_Comm_split(MPI_Comm comm, int color, int key, MPI_Comm* newcomm) {
    return comm_split_impl(comm, color, key, newcomm);
}
namespace {
// Member 0 of the new communicator o sets its topology, then every member waits for it (a barrier on o).
__device__ int set_topology(MPI_Comm_impl* o, int kind, int ndims, const int* dims, const int* periods) {
    if (comm_rank_of(o, me()) == 0) {
        o->topo_kind = kind;
        o->topo_ndims = ndims;
        for (int i = 0; i < ndims; i++) {
            o->topo_dims[i] = dims[i];
            o->topo_periods[i] = periods[i] ? 1 : 0;
        }
        __threadfence();
    }
    return comm_barrier(o, []() {}, __LINE__);
}
}  // namespace

// ---- attribute caching (MPI-1.3 section 5.7).  The reference declares the keyval functions and traps
// in each (mpi.cu:519-536).  A rank's keyvals and attributes live in one table on the device heap, made
// on first use and released when the rank's program returns; keyval k is slot k - 1. ----
namespace {
struct KeyvalRec {
    MPI_Copy_function* copy;
    MPI_Delete_function* del;
    void* extra;
    int used;
};
struct AttrRec {
    MPI_Comm comm;  // nullptr: free slot
    int keyval;
    void* val;
};
struct AttrState {
    KeyvalRec kv[GPUMPI_MAX_KEYVALS];
    AttrRec at[GPUMPI_MAX_ATTRS];
};
__device__ int g_tag_ub_value = MPI_TAG_UB;

__device__ AttrState* attr_state(bool create) {
    RankState* R = &c_rt.ranks[me()];
    if (!R->attrs && create) {
        AttrState* a = (AttrState*)malloc(sizeof(AttrState));
        if (!a) return nullptr;
        memset(a, 0, sizeof(AttrState));
        R->attrs = a;
    }
    return (AttrState*)R->attrs;
}
__device__ KeyvalRec* keyval_rec(AttrState* a, int keyval) {
    if (!a || keyval < 1 || keyval > GPUMPI_MAX_KEYVALS || !a->kv[keyval - 1].used) return nullptr;
    return &a->kv[keyval - 1];
}
__device__ AttrRec* attr_find(AttrState* a, MPI_Comm comm, int keyval) {
    if (!a) return nullptr;
    for (int i = 0; i < GPUMPI_MAX_ATTRS; i++)
        if (a->at[i].comm == comm && a->at[i].keyval == keyval) return &a->at[i];
    return nullptr;
}
__device__ int attr_set(AttrState* a, MPI_Comm comm, int keyval, void* val) {
    AttrRec* r = attr_find(a, comm, keyval);
    if (!r) r = attr_find(a, nullptr, 0);
    if (!r) return GPUMPI_ERR_NO_MEM;
    r->comm = comm;
    r->keyval = keyval;
    r->val = val;
    return MPI_SUCCESS;
}
// Calls the delete function of the attribute in r and frees the slot.
__device__ int attr_drop(AttrState* a, AttrRec* r) {
    const KeyvalRec* k = keyval_rec(a, r->keyval);
    int rc = MPI_SUCCESS;
    if (k && k->del) rc = k->del(r->comm, r->keyval, r->val, k->extra);
    if (rc == MPI_SUCCESS) {
        r->comm = nullptr;
        r->keyval = 0;
        r->val = nullptr;
    }
    return rc;
}
// MPI_Comm_dup: every attribute of oldc whose copy function sets *flag is cached on newc.
__device__ int attr_copy_all(MPI_Comm oldc, MPI_Comm newc) {
    AttrState* a = attr_state(false);
    if (!a) return MPI_SUCCESS;
    for (int i = 0; i < GPUMPI_MAX_ATTRS; i++) {
        if (a->at[i].comm != oldc) continue;
        const int kv = a->at[i].keyval;
        const KeyvalRec* k = keyval_rec(a, kv);
        if (!k || !k->copy) continue;
        void* out = nullptr;
        int flag = 0;
        const int rc = k->copy(oldc, kv, k->extra, a->at[i].val, &out, &flag);
        if (rc != MPI_SUCCESS) return rc;
        if (flag) {
            const int rs = attr_set(a, newc, kv, out);
            if (rs != MPI_SUCCESS) return rs;
        }
    }
    return MPI_SUCCESS;
}
}  // namespace

__device__ int MPI_NULL_COPY_FN(MPI_Comm, int, void*, void*, void*, int* flag) {
    if (flag) *flag = 0;
    return MPI_SUCCESS;
}
__device__ int MPI_DUP_FN(MPI_Comm, int, void*, void* attribute_val_in, void* attribute_val_out, int* flag) {
    if (attribute_val_out) *(void**)attribute_val_out = attribute_val_in;
    if (flag) *flag = 1;
    return MPI_SUCCESS;
}
__device__ int MPI_NULL_DELETE_FN(MPI_Comm, int, void*, void*) { return MPI_SUCCESS; }

__device__ int MPI_Keyval_create(MPI_Copy_function* copy_fn, MPI_Delete_function* delete_fn, int* keyval,
                                 void* extra_state) {
    if (!keyval) return GPUMPI_ERR_ARG;
    AttrState* a = attr_state(true);
    if (!a) return GPUMPI_ERR_NO_MEM;
    for (int i = 0; i < GPUMPI_MAX_KEYVALS; i++) {
        if (a->kv[i].used) continue;
        a->kv[i].copy = copy_fn;
        a->kv[i].del = delete_fn;
        a->kv[i].extra = extra_state;
        a->kv[i].used = 1;
        *keyval = i + 1;
        return MPI_SUCCESS;
    }
    return GPUMPI_ERR_NO_MEM;
}
__device__ int MPI_Keyval_free(int* keyval) {
    if (!keyval) return GPUMPI_ERR_ARG;
    AttrState* a = attr_state(false);
    KeyvalRec* k = keyval_rec(a, *keyval);
    if (!k) return GPUMPI_ERR_ARG;
    // attributes still cached under the keyval keep their delete function until they are deleted
    bool in_use = false;
    for (int i = 0; i < GPUMPI_MAX_ATTRS; i++) in_use = in_use || (a->at[i].comm && a->at[i].keyval == *keyval);
    if (!in_use) k->used = 0;
    *keyval = MPI_KEYVAL_INVALID;
    return MPI_SUCCESS;
}
__device__ int MPI_Attr_put(MPI_Comm comm, int keyval, void* attribute_val) {
    if (!check_comm(comm)) return GPUMPI_ERR_COMM;
    AttrState* a = attr_state(false);
    if (!keyval_rec(a, keyval)) return GPUMPI_ERR_ARG;
    AttrRec* old = attr_find(a, comm, keyval);
    if (old) {
        const int rc = attr_drop(a, old);  // the standard deletes the old value first
        if (rc != MPI_SUCCESS) return rc;
    }
    return attr_set(a, comm, keyval, attribute_val);
}
__device__ int MPI_Attr_get(MPI_Comm comm, int keyval, void* attribute_val, int* flag) {
    if (!check_comm(comm)) return GPUMPI_ERR_COMM;
    if (!attribute_val || !flag) return GPUMPI_ERR_ARG;
    if (keyval == MPI_TAG_UB) {
        *(void**)attribute_val = &g_tag_ub_value;
        *flag = 1;
        return MPI_SUCCESS;
    }
    AttrState* a = attr_state(false);
    if (!keyval_rec(a, keyval)) return GPUMPI_ERR_ARG;
    const AttrRec* r = attr_find(a, comm, keyval);
    *flag = r != nullptr;
    if (r) *(void**)attribute_val = r->val;
    return MPI_SUCCESS;
}
__device__ int MPI_Attr_delete(MPI_Comm comm, int keyval) {
    if (!check_comm(comm)) return GPUMPI_ERR_COMM;
    AttrState* a = attr_state(false);
    if (!keyval_rec(a, keyval)) return GPUMPI_ERR_ARG;
    AttrRec* r = attr_find(a, comm, keyval);
    return r ? attr_drop(a, r) : GPUMPI_ERR_ARG;
}

__device__ int MPI_Comm_dup(MPI_Comm comm, MPI_Comm* newcomm) {
    MPI_Comm_impl* c = check_comm(comm);
    if (!c) return GPUMPI_FAILURE;  // reference returns MPI_FAILURE for MPI_COMM_NULL (communicator.cu:118-121)
    int rc = comm_split_impl(comm, 0, comm_rank_of(c, me()), newcomm);
    if (rc || *newcomm == MPI_COMM_NULL) return rc;
    rc = attr_copy_all(comm, *newcomm);
    if (rc || !c->topo_kind) return rc;
    // a duplicate keeps the topology
    int dims[MPI_MAX_DIMS], periods[MPI_MAX_DIMS];
    for (int i = 0; i < c->topo_ndims; i++) {
        dims[i] = c->topo_dims[i];
        periods[i] = c->topo_periods[i];
    }
    return set_topology(*newcomm, c->topo_kind, c->topo_ndims, dims, periods);
}
__device__ int MPI_Comm_create(MPI_Comm comm, MPI_Group group, MPI_Comm* newcomm) {
    MPI_Comm_impl* c = check_comm(comm);
    if (!c) return GPUMPI_ERR_COMM;
    int grank = MPI_UNDEFINED;
    if (group) MPI_Group_rank(group, &grank);
    return comm_split_impl(comm, grank == MPI_UNDEFINED ? GPUMPI_UNDEFINED : 0, grank, newcomm);
}
// ---- Cartesian topologies: a Cartesian communicator is a communicator of the first prod(dims) ranks of
// the old one, in their order, that also records the grid; coordinates are row-major (the last
// dimension varies fastest), as the MPI standard specifies. ----
__device__ int MPI_Dims_create(int nnodes, int ndims, int dims[]) {
    if (nnodes < 1 || ndims < 1 || ndims > MPI_MAX_DIMS || !dims) return GPUMPI_ERR_ARG;
    long long fixed = 1;
    int nfree = 0;
    for (int i = 0; i < ndims; i++) {
        if (dims[i] < 0) return GPUMPI_ERR_ARG;
        if (dims[i] > 0) fixed *= dims[i];
        else nfree++;
    }
    if (fixed > nnodes || nnodes % fixed) return GPUMPI_ERR_ARG;
    int rem = (int)(nnodes / fixed);
    if (nfree == 0) return rem == 1 ? MPI_SUCCESS : GPUMPI_ERR_ARG;
    // prime factors of the remainder, each given (largest first) to the smallest free dimension so far,
    // then the free dimensions in non-increasing order
    int primes[32], np = 0;
    for (int p = 2; (long long)p * p <= rem; p++)
        while (rem % p == 0) {
            primes[np++] = p;
            rem /= p;
        }
    if (rem > 1) primes[np++] = rem;
    int f[MPI_MAX_DIMS];
    for (int k = 0; k < nfree; k++) f[k] = 1;
    for (int k = np - 1; k >= 0; k--) {
        int m = 0;
        for (int q = 1; q < nfree; q++)
            if (f[q] < f[m]) m = q;
        f[m] *= primes[k];
    }
    for (int a = 0; a < nfree; a++)  // descending order (at most 8 entries)
        for (int b = a + 1; b < nfree; b++)
            if (f[b] > f[a]) {
                const int t = f[a];
                f[a] = f[b];
                f[b] = t;
            }
    for (int i = 0, k = 0; i < ndims; i++)
        if (dims[i] == 0) dims[i] = f[k++];
    return MPI_SUCCESS;
}

__device__ int MPI_Cart_create(MPI_Comm comm_old, int ndims, const int dims[], const int periods[], int reorder,
                               MPI_Comm* comm_cart) {
    (void)reorder;
    MPI_Comm_impl* c = check_comm(comm_old);
    if (!c) return GPUMPI_ERR_COMM;
    if (ndims < 0 || ndims > MPI_MAX_DIMS || (ndims > 0 && (!dims || !periods)) || !comm_cart) return GPUMPI_ERR_ARG;
    long long prod = 1;
    for (int i = 0; i < ndims; i++) {
        if (dims[i] <= 0) return GPUMPI_ERR_ARG;
        prod *= dims[i];
    }
    if (prod > c->size) return GPUMPI_ERR_ARG;
    const int cr = comm_rank_of(c, me());
    int rc = comm_split_impl(comm_old, cr < prod ? 0 : GPUMPI_UNDEFINED, cr, comm_cart);
    if (rc || *comm_cart == MPI_COMM_NULL) return rc;
    return set_topology(*comm_cart, MPI_CART, ndims, dims, periods);
}

namespace {
__device__ __forceinline__ MPI_Comm_impl* cart_of(MPI_Comm comm) {
    MPI_Comm_impl* c = check_comm(comm);
    return c && c->topo_kind == MPI_CART ? c : nullptr;
}
__device__ void cart_coords_of(const MPI_Comm_impl* c, int rank, int* coords) {
    for (int i = c->topo_ndims - 1; i >= 0; i--) {
        coords[i] = rank % c->topo_dims[i];
        rank /= c->topo_dims[i];
    }
}
// Rank of coords (periodic dimensions wrap); -1 when a non-periodic coordinate is outside the grid.
__device__ int cart_rank_of(const MPI_Comm_impl* c, const int* coords) {
    int r = 0;
    for (int i = 0; i < c->topo_ndims; i++) {
        const int d = c->topo_dims[i];
        int x = coords[i];
        if (x < 0 || x >= d) {
            if (!c->topo_periods[i]) return -1;
            x = ((x % d) + d) % d;
        }
        r = r * d + x;
    }
    return r;
}
}  // namespace

__device__ int MPI_Cart_coords(MPI_Comm comm, int rank, int maxdims, int coords[]) {
    MPI_Comm_impl* c = cart_of(comm);
    if (!c) return GPUMPI_ERR_COMM;
    if (rank < 0 || rank >= c->size) return GPUMPI_ERR_RANK;
    if (maxdims < c->topo_ndims || (c->topo_ndims > 0 && !coords)) return GPUMPI_ERR_ARG;
    cart_coords_of(c, rank, coords);
    return MPI_SUCCESS;
}

__device__ int MPI_Cart_rank(MPI_Comm comm, const int coords[], int* rank) {
    MPI_Comm_impl* c = cart_of(comm);
    if (!c) return GPUMPI_ERR_COMM;
    if (!rank || (c->topo_ndims > 0 && !coords)) return GPUMPI_ERR_ARG;
    const int r = cart_rank_of(c, coords);
    if (r < 0) return GPUMPI_ERR_RANK;
    *rank = r;
    return MPI_SUCCESS;
}

__device__ int MPI_Cart_shift(MPI_Comm comm, int direction, int disp, int* rank_source, int* rank_dest) {
    MPI_Comm_impl* c = cart_of(comm);
    if (!c) return GPUMPI_ERR_COMM;
    if (direction < 0 || direction >= c->topo_ndims || !rank_source || !rank_dest) return GPUMPI_ERR_ARG;
    int coords[MPI_MAX_DIMS];
    cart_coords_of(c, comm_rank_of(c, me()), coords);
    const int x = coords[direction];
    coords[direction] = x + disp;
    int r = cart_rank_of(c, coords);
    *rank_dest = r < 0 ? MPI_PROC_NULL : r;
    coords[direction] = x - disp;
    r = cart_rank_of(c, coords);
    *rank_source = r < 0 ? MPI_PROC_NULL : r;
    return MPI_SUCCESS;
}

__device__ int MPI_Cart_get(MPI_Comm comm, int maxdims, int dims[], int periods[], int coords[]) {
    MPI_Comm_impl* c = cart_of(comm);
    if (!c) return GPUMPI_ERR_COMM;
    if (maxdims < c->topo_ndims) return GPUMPI_ERR_ARG;
    if (c->topo_ndims > 0 && (!dims || !periods || !coords)) return GPUMPI_ERR_ARG;
    for (int i = 0; i < c->topo_ndims; i++) {
        dims[i] = c->topo_dims[i];
        periods[i] = c->topo_periods[i];
    }
    cart_coords_of(c, comm_rank_of(c, me()), coords);
    return MPI_SUCCESS;
}

__device__ int MPI_Cartdim_get(MPI_Comm comm, int* ndims) {
    MPI_Comm_impl* c = cart_of(comm);
    if (!c) return GPUMPI_ERR_COMM;
    if (!ndims) return GPUMPI_ERR_ARG;
    *ndims = c->topo_ndims;
    return MPI_SUCCESS;
}

__device__ int MPI_Cart_sub(MPI_Comm comm, const int remain_dims[], MPI_Comm* newcomm) {
    MPI_Comm_impl* c = cart_of(comm);
    if (!c) return GPUMPI_ERR_COMM;
    if (!newcomm || (c->topo_ndims > 0 && !remain_dims)) return GPUMPI_ERR_ARG;
    int coords[MPI_MAX_DIMS], dims[MPI_MAX_DIMS], periods[MPI_MAX_DIMS];
    cart_coords_of(c, comm_rank_of(c, me()), coords);
    // colour: position in the dropped dimensions; key: position in the kept ones (row-major both)
    int color = 0, key = 0, nd = 0;
    for (int i = 0; i < c->topo_ndims; i++) {
        if (remain_dims[i]) {
            key = key * c->topo_dims[i] + coords[i];
            dims[nd] = c->topo_dims[i];
            periods[nd] = c->topo_periods[i];
            nd++;
        } else {
            color = color * c->topo_dims[i] + coords[i];
        }
    }
    int rc = comm_split_impl(comm, color, key, newcomm);
    if (rc || *newcomm == MPI_COMM_NULL) return rc;
    return set_topology(*newcomm, MPI_CART, nd, dims, periods);
}

__device__ int MPI_Topo_test(MPI_Comm comm, int* status) {
    MPI_Comm_impl* c = check_comm(comm);
    if (!c) return GPUMPI_ERR_COMM;
    if (!status) return GPUMPI_ERR_ARG;
    *status = c->topo_kind == MPI_CART ? MPI_CART : MPI_UNDEFINED;
    return MPI_SUCCESS;
}

__device__ int MPI_Comm_free(MPI_Comm* comm) {
    // communicator objects live in the run's arena and are reclaimed when the launch ends; the
    // attributes the rank cached on the communicator are deleted (their delete functions run)
    if (!comm) return GPUMPI_ERR_ARG;
    if (*comm != MPI_COMM_NULL) {
        AttrState* a = attr_state(false);
        if (a)
            for (int i = 0; i < GPUMPI_MAX_ATTRS; i++)
                if (a->at[i].comm == *comm) {
                    const int rc = attr_drop(a, &a->at[i]);
                    if (rc != MPI_SUCCESS) return rc;
                }
    }
    *comm = MPI_COMM_NULL;
    return MPI_SUCCESS;
}
__device__ int MPI_Comm_group(MPI_Comm comm, MPI_Group* group) {
    MPI_Comm_impl* c = check_comm(comm);
    if (!c) return GPUMPI_ERR_COMM;
    if (c->is_world) {
        *group = MPI_GROUP_WORLD;
        return MPI_SUCCESS;
    }
    MPI_Group g = group_new(c->size);
    if (!g) return GPUMPI_ERR_NO_MEM;
    for (int i = 0; i < c->size; i++) g->ranks[i] = c->members[i];
    *group = g;
    return MPI_SUCCESS;
}
__device__ int MPI_Group_incl(MPI_Group group, int n, const int ranks[], MPI_Group* newgroup) {
    if (!group) return GPUMPI_ERR_ARG;
    MPI_Group g = group_new(n);
    if (!g) return GPUMPI_ERR_NO_MEM;
    for (int i = 0; i < n; i++) {
        if (ranks[i] < 0 || ranks[i] >= group->size) {
            group_delete(g);
            return GPUMPI_ERR_RANK;
        }
        g->ranks[i] = group->ranks[ranks[i]];
    }
    *newgroup = g;
    return MPI_SUCCESS;
}
__device__ int MPI_Group_range_incl(MPI_Group group, int n, int ranges[][3], MPI_Group* newgroup) {
    if (!group) return GPUMPI_ERR_ARG;
    int total = 0;
    for (int i = 0; i < n; i++) {
        int first = ranges[i][0], last = ranges[i][1], stride = ranges[i][2];
        if (stride == 0) return GPUMPI_ERR_ARG;
        int cnt = (last - first) / stride + 1;
        if (cnt < 0) cnt = 0;
        total += cnt;
    }
    MPI_Group g = group_new(total);
    if (!g) return GPUMPI_ERR_NO_MEM;
    int k = 0;
    for (int i = 0; i < n; i++) {
        int first = ranges[i][0], last = ranges[i][1], stride = ranges[i][2];
        for (int r = first; stride > 0 ? r <= last : r >= last; r += stride) {
            if (r < 0 || r >= group->size) {
                group_delete(g);
                return GPUMPI_ERR_RANK;
            }
            g->ranks[k++] = group->ranks[r];
        }
    }
    *newgroup = g;
    return MPI_SUCCESS;
}
__device__ int MPI_Group_free(MPI_Group* group) {
    if (group && *group && !(*group)->is_static) {
        if (--(*group)->refcount <= 0) group_delete(*group);
    }
    if (group) *group = MPI_GROUP_NULL;
    return MPI_SUCCESS;
}
__device__ int MPI_Group_size(MPI_Group group, int* size) {
    if (!group) return GPUMPI_ERR_ARG;
    *size = group->size;
    return MPI_SUCCESS;
}
__device__ int MPI_Group_rank(MPI_Group group, int* rank) {
    // MPI semantics: MPI_UNDEFINED in *rank when the caller is not a member (the reference returns
    // MPI_UNDEFINED as the function result and leaves *rank untouched, group.cu:110-122)
    if (!group) return GPUMPI_ERR_ARG;
    *rank = MPI_UNDEFINED;
    for (int i = 0; i < group->size; i++)
        if (group->ranks[i] == me()) {
            *rank = i;
            break;
        }
    return MPI_SUCCESS;
}
__device__ int MPI_Group_translate_ranks(MPI_Group g1, int n, const int ranks1[], MPI_Group g2, int ranks2[]) {
    if (!g1 || !g2) return GPUMPI_ERR_ARG;
    for (int i = 0; i < n; i++) {
        ranks2[i] = MPI_UNDEFINED;
        if (ranks1[i] < 0 || ranks1[i] >= g1->size) return GPUMPI_ERR_RANK;
        int w = g1->ranks[ranks1[i]];
        for (int k = 0; k < g2->size; k++)
            if (g2->ranks[k] == w) {
                ranks2[i] = k;
                break;
            }
    }
    return MPI_SUCCESS;
}

// ------------------------------------------------------------------------------------------------
// host side of this translation unit: install a runtime before a launch
// ------------------------------------------------------------------------------------------------
extern "C" cudaError_t gpumpi_internal_install(Runtime* d_rt, MPI_Comm world, MPI_Group gworld, MPI_Group gempty,
                                                cudaStream_t stream) {
    cudaError_t e;
    if ((e = cudaMemcpyToSymbolAsync(c_rt, d_rt, sizeof(Runtime), 0, cudaMemcpyDeviceToDevice, stream))) return e;
    if ((e = cudaMemcpyToSymbolAsync(MPI_COMM_WORLD, &world, sizeof(world), 0, cudaMemcpyHostToDevice, stream))) return e;
    if ((e = cudaMemcpyToSymbolAsync(MPI_GROUP_WORLD, &gworld, sizeof(gworld), 0, cudaMemcpyHostToDevice, stream))) return e;
    if ((e = cudaMemcpyToSymbolAsync(MPI_GROUP_EMPTY, &gempty, sizeof(gempty), 0, cudaMemcpyHostToDevice, stream))) return e;
    return cudaSuccess;
}

// The same from device-resident sources (the runtime image and the array {world, group world, group
// empty} at d_vals + 1): device-to-device copies only, so the sequence can be recorded in a CUDA graph
// and replayed later.
extern "C" cudaError_t gpumpi_internal_install_dev(const Runtime* d_rt, const void* const* d_vals, cudaStream_t stream) {
    cudaError_t e;
    if ((e = cudaMemcpyToSymbolAsync(c_rt, d_rt, sizeof(Runtime), 0, cudaMemcpyDeviceToDevice, stream))) return e;
    if ((e = cudaMemcpyToSymbolAsync(MPI_COMM_WORLD, d_vals + 1, sizeof(void*), 0, cudaMemcpyDeviceToDevice, stream)))
        return e;
    if ((e = cudaMemcpyToSymbolAsync(MPI_GROUP_WORLD, d_vals + 2, sizeof(void*), 0, cudaMemcpyDeviceToDevice, stream)))
        return e;
    if ((e = cudaMemcpyToSymbolAsync(MPI_GROUP_EMPTY, d_vals + 3, sizeof(void*), 0, cudaMemcpyDeviceToDevice, stream)))
        return e;
    return cudaSuccess;
}

__device__ MPI_Op gpumpi_predefined_op(int code) {
    return (code >= 0 && code < GPUMPI_NUM_PREDEFINED_OPS) ? &g_predef_ops[code] : nullptr;
}

// file and stream I/O over the device -> host channel
#include "api_io.cuh"
