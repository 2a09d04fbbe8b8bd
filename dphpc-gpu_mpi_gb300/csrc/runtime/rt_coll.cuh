// rt_coll.cuh — collectives as single-pass chunked jobs.
//
// Reference behaviour being replaced:
//   * MPI_Reduce: root gathers n-1 buffers by point-to-point, then one thread folds them in rank
//     order (gpu_libs/gpu_mpi/mpi.cu:181-235); world + MPI_DOUBLE + MPI_SUM uses atomicAdd
//     (mpi.cu:148-179, order non-deterministic);
//   * MPI_Allreduce = Reduce(root 0) + Bcast(root 0) (mpi.cu:276-282);
//   * MPI_Bcast: staging buffer + two grid barriers on the world, n-1 sends otherwise (mpi.cu:86-140);
//   * MPI_Alltoall(v): n-1 Isend + n-1 Irecv + local memcpy + waits (mpi.cu:333-408);
//   * MPI_Gather(v) / Scatter(v) / Allgather: root loops of blocking Send/Recv (mpi.cu:291-322,410-517).
//
// Here every collective is: publish my arguments in the communicator's slot table -> one barrier
// (the last arriver opens a job of N chunks) -> every member block, plus any copy-engine block, claims
// chunks with one atomic each and executes them -> wait until all N chunks are done.  Data moves
// exactly once: folds read every member's input once and write every output once, pulls copy each
// block once.  The canonical reduction order of the reference (result = x_0, then op(x_s, result) for
// s = 1..n-1) is kept per element by the DIRECT and STAGED variants, so results are bit-identical.
#pragma once
#include "rt_core.cuh"
#include "rt_types.cuh"
#include "rt_ops.cuh"
#include "rt_copy.cuh"
#include "rt_tma.cuh"

namespace gpumpi {

// Per-block chunk scratch.  Folds use the pointer tile (member buffers of up to PTILE ranks) and the
// generic path's accumulators; pulls use the piece table of rt_pull.cuh.  A block runs one chunk
// at a time and every chunk starts with a block barrier before it writes here (load_ptile, pull_tile,
// pull_part), so the two views never overlap in time.
constexpr int PTILE = 256;
union ChunkScratch {
    struct {
        unsigned long long ptile[PTILE];
        unsigned char acc[256 * 16];     // generic-path accumulators, one 16-byte element per thread
    } f;
    struct {
        long long d[PTILE];              // destination start of the piece
        long long e[PTILE];              // destination end
        long long delta[PTILE];          // source address - destination address
        long long pref[PTILE / 32][33];  // per warp: exclusive prefix of full 16-byte units, then the total
        unsigned char flag[PTILE];       // PF_* bits
    } p;
};
__shared__ __align__(16) ChunkScratch s_chunk;

__device__ __forceinline__ int comm_rank_of(const MPI_Comm_impl* c, int world) {
    return c->is_world ? world : c->rank_of[world];
}

// ------------------------------------------------------------------------------------------------
// job lifecycle
// ------------------------------------------------------------------------------------------------
// Opens a new epoch of job j with n chunks.  Caller has written the job's parameters already.
__device__ __forceinline__ unsigned job_open(Job* j, int n) {
    unsigned e = j->epoch + 1;
    j->epoch = e;
    j->nchunks = n;
    st_relaxed64(&j->done, (unsigned long long)e << 32);
    st_relaxed64(&j->limit, ((unsigned long long)e << 32) | (unsigned)n);
    atom_exch_release64(&j->next, (unsigned long long)e << 32);
    return e;
}

// Claims one chunk; returns its index or -1 once the current epoch is exhausted.
__device__ __forceinline__ long long job_claim(Job* j) {
    unsigned long long t = atom_add_acqrel64(&j->next, 1ULL);
    unsigned e = (unsigned)(t >> 32);
    unsigned idx = (unsigned)t;
    unsigned long long lim = ld_acquire64(&j->limit);
    if ((unsigned)(lim >> 32) != e || idx >= (unsigned)lim) return -1;
    return idx;
}

// Posts job j (epoch e) on the board so copy-engine blocks help with it.
__device__ __forceinline__ void board_post(Job* j, unsigned e) {
    Board* b = c_rt.board;
    if (!b || c_rt.nengines <= 0) return;
    unsigned long long i = atomicAdd(&b->reserve, 1ULL);
    BoardEntry* en = &b->ring[i % (unsigned long long)b->cap];
    en->job = j;
    en->epoch = e;
    st_release(&en->seq, (unsigned)(i + 1));
}

// Thread 0: executes chunks of j until none is left (one block task claims them in a loop and finishes
// each), then waits for all chunks to finish.
__device__ __noinline__ int job_run_and_wait(Job* j, int line) {
    // the caller opened the job itself or acquired its opening through the communicator barrier, and the
    // epoch cannot end before the caller is done with it: a relaxed claim and a relaxed read of the limit,
    // issued together, cost one round trip
    const unsigned long long tk = atom_add_relaxed64(&j->next, 1ULL);
    const unsigned long long lim = ld_relaxed64(&j->limit);
    const long long idx =
        ((unsigned)(tk >> 32) == (unsigned)(lim >> 32) && (unsigned)tk < (unsigned)lim) ? (long long)(unsigned)tk : -1;
    if (idx >= 0) {
        Task t;
        t.kind = TASK_CHUNK;
        t.p0 = j;
        t.n0 = idx;
        dispatch(t);
    }
    const unsigned long long target = lim;  // (epoch << 32) | nchunks
    if (ld_acquire64(&j->done) == target) return 0;
    Deadline d = make_deadline();
    while (ld_relaxed64(&j->done) != target) {
        if (int e = wait_tick(d, line, 128)) return e;
    }
    fence_acqrel();
    return 0;
}

// ------------------------------------------------------------------------------------------------
// communicator barrier: generation counter; the last arriver runs `setup` before releasing
// ------------------------------------------------------------------------------------------------
// The barrier whose generation word the caller read as g (it cannot change before the caller arrives).
template <class F>
__device__ int comm_barrier_from(MPI_Comm_impl* c, unsigned g, F&& setup, int line) {
    unsigned a = atom_add_acqrel(&c->bar_count, 1u);
    if (a == (unsigned)c->size - 1) {
        c->bar_count = 0;
        setup();
        st_release(&c->bar_gen, g + 1);
        return 0;
    }
    Deadline d = make_deadline();
    while (ld_relaxed(&c->bar_gen) == g) {
        if (int e = wait_tick(d, line, 64)) return e;
    }
    fence_acqrel();
    return 0;
}

template <class F>
__device__ int comm_barrier(MPI_Comm_impl* c, F&& setup, int line) {
    return comm_barrier_from(c, ld_acquire(&c->bar_gen), setup, line);
}

// Parameters of the job epoch being executed, read once per chunk with L2-only loads (the Job
// struct is rewritten by every epoch, so no executing block may keep it in L1).
struct JobParams {
    int kind, dt, op, root, esize, vec, tile, aligned16, variant, nchunks;
    unsigned epoch;
    long long count, chunk;
    const MPI_Comm_impl* comm;
    const CollSlot* slots;
    int csize;
    const void* src;
    void* dst;
    MPI_User_function* ufn;
};

__device__ __forceinline__ void load_params(const Job* j, JobParams& P) {
    P.kind = __ldcg(&j->kind);
    P.variant = __ldcg(&j->variant);
    P.epoch = __ldcg(&j->epoch);
    P.nchunks = __ldcg(&j->nchunks);
    P.dt = __ldcg(&j->dt);
    P.op = __ldcg(&j->op);
    P.root = __ldcg(&j->root);
    P.esize = __ldcg(&j->esize);
    P.vec = __ldcg(&j->vec);
    P.tile = __ldcg(&j->tile);
    P.aligned16 = __ldcg(&j->aligned16);
    P.count = __ldcg(&j->count);
    P.chunk = __ldcg(&j->chunk);
    P.comm = (const MPI_Comm_impl*)__ldcg((const unsigned long long*)&j->comm);
    P.slots = (const CollSlot*)__ldcg((const unsigned long long*)&j->slots);
    P.csize = __ldcg(&j->csize);
    P.src = (const void*)__ldcg((const unsigned long long*)&j->src);
    P.dst = (void*)__ldcg((const unsigned long long*)&j->dst);
    P.ufn = (MPI_User_function*)__ldcg((const unsigned long long*)&j->ufn);
}

// ------------------------------------------------------------------------------------------------
// fold executors (Allreduce / Reduce)
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ const void* slot_in(const CollSlot* s) {
    return (const void*)__ldcg((const unsigned long long*)&s->sbuf);
}
__device__ __forceinline__ void* slot_out(const CollSlot* s) {
    return (void*)__ldcg((const unsigned long long*)&s->rbuf);
}

// loads pointer field `which` (0 = sbuf, 1 = rbuf) of members [r0, r0+m) into s_chunk.f.ptile
// With rot != 0 the tile holds members (r0 + i + rot) mod n: the RING variant's rotated fold order.
__device__ __forceinline__ void load_ptile(const CollSlot* slots, int r0, int m, int which, int tid, int nt,
                                           int rot = 0, int n = 1) {
    bar_sync(BAR_TASK, nt);
    for (int i = tid; i < m; i += nt) {
        const int r = rot ? (r0 + i + rot) % n : r0 + i;
        s_chunk.f.ptile[i] = __ldcg(which == 0 ? (const unsigned long long*)&slots[r].sbuf
                                        : (const unsigned long long*)&slots[r].rbuf);
    }
    bar_sync(BAR_TASK, nt);
}

template <class T, int V>
__device__ __forceinline__ void ld_elems(const T* p, T (&v)[V], int nv, bool vec16) {
    if constexpr ((V * sizeof(T)) % 16 == 0) {
        if (vec16 && nv == V) {
#pragma unroll
            for (int q = 0; q < (int)(V * sizeof(T) / 16); q++) {
                uint4 w = __ldcg((const uint4*)p + q);
                *reinterpret_cast<uint4*>(&v[q * (16 / sizeof(T))]) = w;
            }
            return;
        }
    } else if constexpr ((V * sizeof(T)) == 8 && sizeof(T) < 8) {
        if (vec16 && nv == V) {
            unsigned long long w = __ldcg((const unsigned long long*)p);
            *reinterpret_cast<unsigned long long*>(&v[0]) = w;
            return;
        }
    }
#pragma unroll
    for (int k = 0; k < V; k++)
        if (k < nv) v[k] = __ldcg(p + k);
}

template <class T, int V>
__device__ __forceinline__ void st_elems(T* p, const T (&v)[V], int nv, bool vec16) {
    if constexpr ((V * sizeof(T)) % 16 == 0) {
        if (vec16 && nv == V) {
#pragma unroll
            for (int q = 0; q < (int)(V * sizeof(T) / 16); q++)
                __stcg((uint4*)p + q, *reinterpret_cast<const uint4*>(&v[q * (16 / sizeof(T))]));
            return;
        }
    } else if constexpr ((V * sizeof(T)) == 8 && sizeof(T) < 8) {
        if (vec16 && nv == V) {
            __stcg((unsigned long long*)p, *reinterpret_cast<const unsigned long long*>(&v[0]));
            return;
        }
    }
#pragma unroll
    for (int k = 0; k < V; k++)
        if (k < nv) __stcg(p + k, v[k]);
}

// Member pointers of ranks [r0, r0 + m) of the fold order (sbuf, or rbuf when `out`) copied into dst[0, m)
// of shared memory by asynchronous copies (no registers held while they are in flight); async_ptrs_wait
// returns once this thread's copies have landed.  The slots were published before the collective's
// barrier, whose acquire dropped any older copy of them from this SM's L1, and stay unchanged until the
// job's last chunk is finished.
__device__ __forceinline__ void async_ptrs(unsigned long long* dst, const CollSlot* slots, int r0, int m, bool out,
                                           int rot, int n, int tid, int nt) {
    for (int i = tid; i < m; i += nt) {
        const int r = rot ? (r0 + i + rot) % n : r0 + i;
        const void* src = out ? (const void*)&slots[r].rbuf : (const void*)&slots[r].sbuf;
        unsigned long long g;
        asm("cvta.to.global.u64 %0, %1;" : "=l"(g) : "l"(src));
        const unsigned d = (unsigned)__cvta_generic_to_shared(dst + i);
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(g) : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void async_ptrs_wait() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Canonical-order fold of elements [e0, e0 + nt*V): thread tid owns V consecutive elements.
// order: acc = x_0; acc = op(x_s, acc) for s = 1..n-1 (in comm-rank order).
// The members' pointers come through the two halves of the block's pointer tile: while the ranks of one
// half are folded (or written), the next half's pointers are already being copied into the other half, so
// each group of PTILE / 2 ranks costs one block barrier and no exposed pointer round trip.
template <class T, int OP, int V>
__device__ __noinline__ void fold_fast(const JobParams* j, long long e0, int tid, int nt) {
    constexpr int BYTES = V * (int)sizeof(T);
    // ranks folded per step: ~128 bytes of loads in flight per thread (at most 16 loads)
    constexpr int U = 128 / BYTES > 16 ? 16 : 128 / BYTES < 1 ? 1 : 128 / BYTES;
    constexpr int H = PTILE / 2;
    const CollSlot* slots = j->slots;
    const int n = j->csize;
    const long long count = j->count;
    const long long e = e0 + (long long)tid * V;
    const int nv = e < count ? (int)min((long long)V, count - e) : 0;
    const bool vec16 = j->aligned16 >= (int)((V * sizeof(T)) >= 16 ? 16 : (V * sizeof(T)));
    // RING: chunk k folds members k+1, k+2, ..., k (mod n), the order a ring reduce-scatter produces
    const int rot = j->variant == GPUMPI_VARIANT_RING ? (int)((e0 / j->chunk + 1) % n) : 0;
    T acc[V];
#pragma unroll
    for (int k = 0; k < V; k++) acc[k] = T();
    bar_sync(BAR_TASK, nt);  // the previous chunk's readers are done with the tile
    async_ptrs(s_chunk.f.ptile, slots, 0, min(H, n), false, rot, n, tid, nt);
    async_ptrs_wait();
    bar_sync(BAR_TASK, nt);
    int half = 0;
    for (int r0 = 0; r0 < n; r0 += H) {
        const int m = min(H, n - r0);
        const bool more = r0 + H < n;
        if (more) async_ptrs(s_chunk.f.ptile + (half ^ 1) * H, slots, r0 + H, min(H, n - r0 - H), false, rot, n, tid, nt);
        const unsigned long long* pt = s_chunk.f.ptile + half * H;
        if (nv > 0) {
            int i = 0;
            if (r0 == 0) {
                ld_elems<T, V>((const T*)pt[0] + e, acc, nv, vec16);
                i = 1;
            }
            for (; i + U <= m; i += U) {
                T v[U][V];
#pragma unroll
                for (int u = 0; u < U; u++) ld_elems<T, V>((const T*)pt[i + u] + e, v[u], nv, vec16);
#pragma unroll
                for (int u = 0; u < U; u++)
#pragma unroll
                    for (int k = 0; k < V; k++) acc[k] = op_apply<OP, T>(v[u][k], acc[k]);
            }
            for (; i < m; i++) {
                T v[V];
                ld_elems<T, V>((const T*)pt[i] + e, v, nv, vec16);
#pragma unroll
                for (int k = 0; k < V; k++) acc[k] = op_apply<OP, T>(v[k], acc[k]);
            }
        }
        if (more) async_ptrs_wait();
        bar_sync(BAR_TASK, nt);  // the next half is filled; nobody reads this half any more
        half ^= 1;
    }
    if (j->kind == JOB_REDUCE) {
        if (nv > 0) {
            T* out = (T*)slot_out(&slots[j->root]);
            st_elems<T, V>(out + e, acc, nv, vec16);
        }
        return;
    }
    // every member's result: the same two halves, receive pointers in rank order
    async_ptrs(s_chunk.f.ptile + half * H, slots, 0, min(H, n), true, 0, n, tid, nt);
    async_ptrs_wait();
    bar_sync(BAR_TASK, nt);
    for (int r0 = 0; r0 < n; r0 += H) {
        const int m = min(H, n - r0);
        const bool more = r0 + H < n;
        if (more) async_ptrs(s_chunk.f.ptile + (half ^ 1) * H, slots, r0 + H, min(H, n - r0 - H), true, 0, n, tid, nt);
        const unsigned long long* pt = s_chunk.f.ptile + half * H;
        if (nv > 0)
            for (int i = 0; i < m; i++) st_elems<T, V>((T*)pt[i] + e, acc, nv, vec16);
        if (more) async_ptrs_wait();
        bar_sync(BAR_TASK, nt);
        half ^= 1;
    }
}

}  // namespace gpumpi

#include "rt_staged.cuh"
#include "rt_tree.cuh"

namespace gpumpi {

// Any legal (op, type) and user-defined ops, one element per thread, same canonical order.
__device__ __noinline__ void fold_generic(const JobParams* j, long long e0, int tid, int nt) {
    const CollSlot* slots = j->slots;
    const int n = j->csize;
    const int es = j->esize;
    const long long e = e0 + tid;
    const bool act = e < j->count;
    unsigned char* acc = s_chunk.f.acc + tid * 16;
    MPI_Datatype dtv = (MPI_Datatype)j->dt;
    int one = 1;
    for (int r0 = 0; r0 < n; r0 += PTILE) {
        const int m = min(PTILE, n - r0);
        load_ptile(slots, r0, m, 0, tid, nt);
        if (act) {
            for (int i = 0; i < m; i++) {
                const unsigned char* src = (const unsigned char*)s_chunk.f.ptile[i] + e * es;
                if (r0 == 0 && i == 0) {
                    for (int b = 0; b < es; b++) acc[b] = src[b];
                } else if (j->ufn) {
                    j->ufn((void*)src, acc, &one, &dtv);
                } else {
                    apply_elem(j->op, j->dt, src, acc);
                }
            }
        }
    }
    if (j->kind == JOB_REDUCE) {
        if (act) {
            unsigned char* out = (unsigned char*)slot_out(&slots[j->root]) + e * es;
            for (int b = 0; b < es; b++) out[b] = acc[b];
        }
        return;
    }
    for (int r0 = 0; r0 < n; r0 += PTILE) {
        const int m = min(PTILE, n - r0);
        load_ptile(slots, r0, m, 1, tid, nt);
        if (act)
            for (int i = 0; i < m; i++) {
                unsigned char* out = (unsigned char*)s_chunk.f.ptile[i] + e * es;
                for (int b = 0; b < es; b++) out[b] = acc[b];
            }
    }
}

// storage-type / op dispatch of the fast path; returns false if no fast instantiation exists
// vec choices: 16/sizeof(T) (one 16-byte vector), 8/sizeof(T) (4-byte types), 1
template <class T, int OP>
__device__ __forceinline__ void fold_fast_v(const JobParams* j, long long e0, int tid, int nt) {
    constexpr int VW = 16 / sizeof(T);
    if (j->vec >= VW) fold_fast<T, OP, VW>(j, e0, tid, nt);
    else if constexpr (sizeof(T) == 4) {
        if (j->vec >= 2) fold_fast<T, OP, 2>(j, e0, tid, nt);
        else fold_fast<T, OP, 1>(j, e0, tid, nt);
    } else fold_fast<T, OP, 1>(j, e0, tid, nt);
}

template <class T>
__device__ __forceinline__ bool fold_fast_arith(const JobParams* j, long long e0, int tid, int nt) {
    switch (j->op) {
    case GPUMPI_OP_SUM: fold_fast_v<T, GPUMPI_OP_SUM>(j, e0, tid, nt); return true;
    case GPUMPI_OP_MAX: fold_fast_v<T, GPUMPI_OP_MAX>(j, e0, tid, nt); return true;
    case GPUMPI_OP_MIN: fold_fast_v<T, GPUMPI_OP_MIN>(j, e0, tid, nt); return true;
    case GPUMPI_OP_PROD: fold_fast_v<T, GPUMPI_OP_PROD>(j, e0, tid, nt); return true;
    default: return false;
    }
}

template <class T>
__device__ __forceinline__ bool fold_fast_int(const JobParams* j, long long e0, int tid, int nt) {
    switch (j->op) {
    case GPUMPI_OP_BAND: fold_fast_v<T, GPUMPI_OP_BAND>(j, e0, tid, nt); return true;
    case GPUMPI_OP_BOR: fold_fast_v<T, GPUMPI_OP_BOR>(j, e0, tid, nt); return true;
    case GPUMPI_OP_BXOR: fold_fast_v<T, GPUMPI_OP_BXOR>(j, e0, tid, nt); return true;
    default: return fold_fast_arith<T>(j, e0, tid, nt);
    }
}

// true if the (dt, op) pair has a templated fast path
__device__ __forceinline__ bool fold_has_fast(int dt, int op, MPI_User_function* ufn) {
#ifdef GPUMPI_NO_FAST_FOLD
    return false;
#endif
    if (ufn) return false;
    switch (dt) {
    case GPUMPI_FLOAT: case GPUMPI_DOUBLE: case GPUMPI_LONG_DOUBLE:
        return op == GPUMPI_OP_SUM || op == GPUMPI_OP_MAX || op == GPUMPI_OP_MIN || op == GPUMPI_OP_PROD;
    case GPUMPI_INT: case GPUMPI_INT32_T: case GPUMPI_UNSIGNED: case GPUMPI_UINT32_T: case GPUMPI_LONG:
    case GPUMPI_LONG_LONG_INT: case GPUMPI_LONG_LONG: case GPUMPI_INT64_T: case GPUMPI_UNSIGNED_LONG:
    case GPUMPI_UNSIGNED_LONG_LONG: case GPUMPI_UINT64_T:
        return op == GPUMPI_OP_SUM || op == GPUMPI_OP_MAX || op == GPUMPI_OP_MIN || op == GPUMPI_OP_PROD ||
               op == GPUMPI_OP_BAND || op == GPUMPI_OP_BOR || op == GPUMPI_OP_BXOR;
    default: return false;
    }
}

template <class T, int OP>
__device__ __forceinline__ void fold_staged_v(const JobParams* j, long long idx, int tid, int nt) {
    if (j->vec >= 16 / (int)sizeof(T)) fold_staged<T, OP, 16 / sizeof(T)>(j, idx, tid, nt);
    else if constexpr (sizeof(T) == 4) {
        if (j->vec >= 2) fold_staged<T, OP, 2>(j, idx, tid, nt);
        else fold_staged<T, OP, 1>(j, idx, tid, nt);
    } else fold_staged<T, OP, 1>(j, idx, tid, nt);
}

template <class T>
__device__ __forceinline__ bool fold_staged_t(const JobParams* j, long long idx, int tid, int nt) {
    switch (j->op) {
    case GPUMPI_OP_SUM: fold_staged_v<T, GPUMPI_OP_SUM>(j, idx, tid, nt); return true;
    case GPUMPI_OP_MAX: fold_staged_v<T, GPUMPI_OP_MAX>(j, idx, tid, nt); return true;
    case GPUMPI_OP_MIN: fold_staged_v<T, GPUMPI_OP_MIN>(j, idx, tid, nt); return true;
    default: return false;
    }
}

// true if (dt, op) has a STAGED instantiation
__device__ __forceinline__ bool fold_has_staged(int dt, int op, MPI_User_function* ufn) {
    if (ufn || !(op == GPUMPI_OP_SUM || op == GPUMPI_OP_MAX || op == GPUMPI_OP_MIN)) return false;
    switch (dt) {
    case GPUMPI_FLOAT: case GPUMPI_DOUBLE: case GPUMPI_LONG_DOUBLE: case GPUMPI_INT: case GPUMPI_INT32_T:
    case GPUMPI_LONG: case GPUMPI_LONG_LONG_INT: case GPUMPI_LONG_LONG: case GPUMPI_INT64_T:
        return true;
    default: return false;
    }
}

__device__ __noinline__ void fold_chunk(const JobParams* j, long long idx, int tid, int nt) {
    const long long e0 = idx * j->chunk;
    bool done = false;
#ifndef GPUMPI_NO_FAST_FOLD
    // TREE chunks are numbered by phase (see rt_tree.cuh), not by element range
    if (j->variant == GPUMPI_VARIANT_TREE && j->tile > 0) {
        if (fold_tree_dispatch(j, idx, tid, nt)) return;
    }
    // after an abort no block issues bulk copies: a stage may still hold a copy that never landed
    if (j->variant == GPUMPI_VARIANT_STAGED && j->tile > 0 &&
        ((min(j->chunk, j->count - e0) * j->esize) & 15) == 0 && !ld_relaxed(c_rt.abort_flag)) {
        switch (j->dt) {
        case GPUMPI_FLOAT: done = fold_staged_t<float>(j, idx, tid, nt); break;
        case GPUMPI_DOUBLE: case GPUMPI_LONG_DOUBLE: done = fold_staged_t<double>(j, idx, tid, nt); break;
        case GPUMPI_INT: case GPUMPI_INT32_T: done = fold_staged_t<int>(j, idx, tid, nt); break;
        default: done = fold_staged_t<long long>(j, idx, tid, nt); break;
        }
    }
    if (!done && fold_has_fast(j->dt, j->op, j->ufn)) {
        switch (j->dt) {
        case GPUMPI_FLOAT: done = fold_fast_arith<float>(j, e0, tid, nt); break;
        case GPUMPI_DOUBLE: case GPUMPI_LONG_DOUBLE: done = fold_fast_arith<double>(j, e0, tid, nt); break;
        case GPUMPI_INT: case GPUMPI_INT32_T: done = fold_fast_int<int>(j, e0, tid, nt); break;
        case GPUMPI_UNSIGNED: case GPUMPI_UINT32_T: done = fold_fast_int<unsigned>(j, e0, tid, nt); break;
        case GPUMPI_LONG: case GPUMPI_LONG_LONG_INT: case GPUMPI_LONG_LONG: case GPUMPI_INT64_T:
            done = fold_fast_int<long long>(j, e0, tid, nt); break;
        default: done = fold_fast_int<unsigned long long>(j, e0, tid, nt); break;
        }
    }
#endif
    if (!done) fold_generic(j, e0, tid, nt);
}

// ------------------------------------------------------------------------------------------------
// pull executors (Bcast / Alltoall(v) / Allgather(v) / Gather(v) / Scatter(v))
//   piece p -> (receiver r, sender s); the chunk covers `tile` consecutive pieces (warp per piece),
//   or, when pieces are large, one byte range of one piece (`vec` parts per piece, whole block).
// ------------------------------------------------------------------------------------------------
struct Piece {
    const char* src;
    char* dst;
    const TypeDesc* sdesc;   // nullptr: contiguous
    const TypeDesc* rdesc;
    long long bytes;         // packed bytes to move
    int trunc;
};

__device__ __forceinline__ int ldcg_int(const int* p) { return __ldcg(p); }

__device__ __forceinline__ void piece_of(const JobParams* j, long long p, Piece& pc) {
    const CollSlot* S = j->slots;
    const int n = j->csize;
    int r, s;
    switch (j->kind) {
    case JOB_ALLTOALLV: case JOB_ALLGATHERV:
        // piece order of the variant: DIRECT receiver-major (each chunk fills one receiver's buffer),
        // TREE sender-major (each chunk drains one sender's buffer), RING receiver-major with the
        // senders rotated so receiver r starts at itself (no sender is read by every block at once)
        if (j->variant == GPUMPI_VARIANT_TREE) {
            s = (int)(p / n);
            r = (int)(p % n);
        } else {
            r = (int)(p / n);
            s = (int)(p % n);
            if (j->variant == GPUMPI_VARIANT_RING) s = (s + r) % n;
        }
        break;
    case JOB_GATHERV: r = j->root; s = (int)p; break;
    default: r = (int)p; s = j->root; break;  // SCATTERV, BCAST
    }
    const CollSlot* ss = &S[s];
    const CollSlot* rs = &S[r];
    const char* sbuf = (const char*)__ldcg((const unsigned long long*)&ss->sbuf);
    char* rbuf = (char*)__ldcg((const unsigned long long*)&rs->rbuf);
    const TypeDesc* sd = (const TypeDesc*)__ldcg((const unsigned long long*)&ss->sdesc);
    const TypeDesc* rd = (const TypeDesc*)__ldcg((const unsigned long long*)&rs->rdesc);
    long long sext = __ldcg(&sd->extent), rext = __ldcg(&rd->extent);
    long long ssz = __ldcg(&sd->size), rsz = __ldcg(&rd->size);
    const bool sflat = desc_contiguous(sd), rflat = desc_contiguous(rd);
    long long scount, rcount, soff, roff;
    switch (j->kind) {
    case JOB_ALLTOALLV: {
        const int* sc = (const int*)__ldcg((const unsigned long long*)&ss->scounts);
        const int* sdp = (const int*)__ldcg((const unsigned long long*)&ss->sdispls);
        const int* rc = (const int*)__ldcg((const unsigned long long*)&rs->rcounts);
        const int* rdp = (const int*)__ldcg((const unsigned long long*)&rs->rdispls);
        long long sct = __ldcg(&ss->scount), rct = __ldcg(&rs->rcount);
        scount = sc ? ldcg_int(sc + r) : sct;
        soff = sdp ? (long long)ldcg_int(sdp + r) * sext : (long long)r * sct * sext;
        rcount = rc ? ldcg_int(rc + s) : rct;
        roff = rdp ? (long long)ldcg_int(rdp + s) * rext : (long long)s * rct * rext;
        break;
    }
    case JOB_ALLGATHERV: case JOB_GATHERV: {
        const int* rc = (const int*)__ldcg((const unsigned long long*)&rs->rcounts);
        const int* rdp = (const int*)__ldcg((const unsigned long long*)&rs->rdispls);
        long long rct = __ldcg(&rs->rcount);
        scount = __ldcg(&ss->scount);
        soff = 0;
        rcount = rc ? ldcg_int(rc + s) : rct;
        roff = rdp ? (long long)ldcg_int(rdp + s) * rext : (long long)s * rct * rext;
        break;
    }
    case JOB_SCATTERV: {
        const int* sc = (const int*)__ldcg((const unsigned long long*)&ss->scounts);
        const int* sdp = (const int*)__ldcg((const unsigned long long*)&ss->sdispls);
        long long sct = __ldcg(&ss->scount);
        scount = sc ? ldcg_int(sc + r) : sct;
        soff = sdp ? (long long)ldcg_int(sdp + r) * sext : (long long)r * sct * sext;
        rcount = __ldcg(&rs->rcount);
        roff = 0;
        break;
    }
    default: {  // BCAST: root's buffer (published as sbuf) into every member's buffer (rbuf)
        scount = __ldcg(&ss->scount);
        rcount = __ldcg(&rs->rcount);
        soff = 0;
        roff = 0;
        break;
    }
    }
    long long sbytes = scount * ssz, rbytes = rcount * rsz;
    pc.trunc = sbytes > rbytes;
    pc.bytes = sbytes < rbytes ? sbytes : rbytes;
    // in-place / self pieces move nothing
    if (sbuf == (const char*)MPI_IN_PLACE || rbuf == (char*)MPI_IN_PLACE ||
        (j->kind == JOB_BCAST && r == s) || (sbuf + soff == rbuf + roff && sd == rd))
        pc.bytes = 0;
    pc.src = sbuf + soff;
    pc.dst = rbuf + roff;
    pc.sdesc = sflat ? nullptr : sd;
    pc.rdesc = rflat ? nullptr : rd;
}

__device__ __forceinline__ void piece_copy(const Piece& pc, long long b0, long long b1, int lane, int nl) {
    if (b1 <= b0) return;
    if (!pc.sdesc && !pc.rdesc) copy_bytes(pc.dst + b0, pc.src + b0, b1 - b0, lane, nl);
    else typed_copy(pc.dst, pc.rdesc, pc.src, pc.sdesc, b0, b1, lane, nl);
}

}  // namespace gpumpi

#include "rt_pull.cuh"

namespace gpumpi {

__device__ __noinline__ void copy_chunk(const JobParams* j, long long idx, int tid, int nt) {
    long long off = idx * j->chunk;
    long long len = min(j->chunk, j->count - off);
    copy_bytes((char*)j->dst + off, (const char*)j->src + off, len, tid, nt);
}

// The block's copy of the executing job's parameters: one thread reads them per chunk; every executor
// then reads shared memory instead of a per-thread stack copy (which would live in local memory and,
// with most of the SM's L1 given to shared memory, cost L2 traffic on every access).  Thread 0 starts a
// chunk only after every helper finished the previous task, so no reader of the old values remains.
__shared__ JobParams s_jp;
__shared__ long long s_next_chunk;

// Runs chunk idx of job jg, then keeps claiming and running chunks until none is left; thread 0 marks
// each chunk finished once every thread of the block is done with it (the barrier orders the block's
// writes before thread 0's release).  One task per job and block keeps the call chain (and its saved
// registers) out of the per-chunk path.
// Thread 0 claims the next chunk before it marks this one finished: while this chunk is unfinished the
// epoch cannot end (its owner reopens the job only after every chunk is finished), so the claim returns a
// chunk of the epoch whose parameters are in s_jp, or an index past its end.  The claim is relaxed (the
// block acquired the epoch's parameters and data with its first claim, so no acquire, which would also
// drop the SM's L1 contents, is needed) and the finish is a release add nobody waits for: the two round
// trips overlap.
template <class F>
__device__ __forceinline__ void chunk_loop(Job* jg, long long idx, int tid, int nt, F&& body) {
    for (;;) {
        body(idx);
        bar_sync(BAR_TASK, nt);
        if (tid == 0) {
            const unsigned long long t = atom_add_relaxed64(&jg->next, 1ULL);
            red_add_release64(&jg->done, 1ULL);
            const unsigned i = (unsigned)t;
            s_next_chunk = ((unsigned)(t >> 32) == s_jp.epoch && i < (unsigned)s_jp.nchunks) ? (long long)i : -1;
        }
        bar_sync(BAR_TASK, nt);
        idx = s_next_chunk;
        if (idx < 0) return;
    }
}

__device__ __noinline__ void pull_run(const JobParams* j, Job* jg, long long idx, int tid, int nt) {
    chunk_loop(jg, idx, tid, nt, [&](long long i) { pull_chunk(j, jg, i, tid, nt); });
}
__device__ __noinline__ void fold_run(const JobParams* j, Job* jg, long long idx, int tid, int nt) {
    chunk_loop(jg, idx, tid, nt, [&](long long i) { fold_chunk(j, i, tid, nt); });
}
__device__ __noinline__ void copy_run(const JobParams* j, Job* jg, long long idx, int tid, int nt) {
    chunk_loop(jg, idx, tid, nt, [&](long long i) { copy_chunk(j, i, tid, nt); });
}

__device__ __noinline__ void exec_chunk(Job* jg, long long idx, int tid, int nt) {
    // parameters of the epoch that chunk idx belongs to (the claim that returned it synchronised with
    // the release that opened the epoch, and the epoch cannot end before this chunk is finished)
    if (tid == 0) load_params(jg, s_jp);
    bar_sync(BAR_TASK, nt);
    const JobParams* j = &s_jp;
    switch (j->kind) {
    case JOB_COPY: copy_run(j, jg, idx, tid, nt); break;
    case JOB_ALLREDUCE: case JOB_REDUCE: fold_run(j, jg, idx, tid, nt); break;
    default: pull_run(j, jg, idx, tid, nt); break;
    }
}

// ------------------------------------------------------------------------------------------------
// copy-engine loop (blocks >= nranks): claim chunks of any job posted on the board
// ------------------------------------------------------------------------------------------------
__device__ void engine_loop() {
    Board* b = c_rt.board;
    const unsigned long long cap = (unsigned long long)b->cap;
    unsigned long long cursor = 0;
    unsigned ns = 32;
    for (;;) {
        bool worked = false;
        unsigned long long res = ld_relaxed64(&b->reserve);
        if (res > cap && res - cap > cursor) cursor = res - cap;
        for (unsigned long long i = cursor; i < res; i++) {
            BoardEntry* en = &b->ring[i % cap];
            unsigned seq = ld_relaxed(&en->seq);
            int diff = (int)(seq - (unsigned)(i + 1));
            if (diff < 0) break;             // not written yet
            if (diff == 0) {
                fence_acqrel();
                Job* j = (Job*)__ldcg((const unsigned long long*)&en->job);
                const long long idx = job_claim(j);
                if (idx >= 0) {  // the task claims the job's remaining chunks itself
                    Task t;
                    t.kind = TASK_CHUNK;
                    t.p0 = j;
                    t.n0 = idx;
                    dispatch(t);
                    worked = true;
                }
            }
            if (i == cursor) cursor++;
        }
        if (ld_relaxed(c_rt.ranks_done) >= (unsigned)c_rt.nranks || ld_relaxed(c_rt.abort_flag)) return;
        if (!worked) {
            __nanosleep(ns);
            ns = ns * 2 > 1024 ? 1024 : ns * 2;
        } else {
            ns = 32;
        }
    }
}

}  // namespace gpumpi
