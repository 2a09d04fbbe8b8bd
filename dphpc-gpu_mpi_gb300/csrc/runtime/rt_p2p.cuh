// rt_p2p.cuh — point-to-point engine: lock-free mailboxes, receiver-side matching, eager and
// rendezvous protocols.
//
// Reference being replaced (gpu_libs/gpu_libc/cuda_mpi.{cuh,cu}): per-rank 16-deep circular queues
// in managed memory guarded by an atomicCAS_system spinlock that BOTH sender and receiver take
// (cuda_mpi.cu:136,288), a single-thread memcpy (cu:168,323), and non-synchronous sends that report
// completion before the receiver copied (cu:181-211, hazard H3).
//
// Here:
//   * a sender claims a ticket in the receiver's envelope ring with one atomicAdd and publishes the
//     envelope with a release store of its sequence word; nothing is locked;
//   * only the receiving rank matches: it drains its ring in ticket order into a private
//     unexpected queue (arrival order) and matches posted receives in posting order, so MPI's
//     non-overtaking rule holds per (source, tag, communicator); wildcards work on both sides
//     (the reference honours them only when the receive is posted first, cuda_mpi.cu:300-303);
//   * eager messages (<= `eager` bytes) travel inline in the envelope slot and complete at once;
//     larger messages are pulled by the receiver straight from the sender's buffer (rendezvous)
//     and the send completes only after the copy (fixes H3);
//   * the rank's whole block copies; very large copies become jobs that copy-engine blocks share;
//   * buffers other ranks cannot address (thread-local stack arrays) are staged, as the reference
//     does for non-global buffers (cuda_mpi.cu:183-192,338-349).
#pragma once
#include "rt_core.cuh"
#include "rt_types.cuh"
#include "rt_copy.cuh"
#include "rt_coll.cuh"

namespace gpumpi {

__device__ __forceinline__ int me() { return (int)blockIdx.x; }

__device__ __forceinline__ bool block_addressable(const void* p) { return is_global_ptr(p) || is_shared_ptr(p); }

// The rank's own copies of hot point-to-point state, in shared memory (thread 0 of the rank block is
// their only user): the head of its envelope ring (the global copy is published for senders' flow
// control) and a small cache of other rings' heads.  A cached head is a lower bound (heads only grow),
// so a send re-reads the receiver's head only when the bound does not prove a free slot.
constexpr int HEAD_CACHE = 16;
struct RankFast {
    unsigned long long mb_head;
    unsigned long long hc_head[HEAD_CACHE];
    int hc_rank[HEAD_CACHE];
};
__shared__ RankFast s_rf;

// called by thread 0 of every rank block at the start of a launch (the ring heads are zero then)
__device__ __forceinline__ void p2p_rank_begin() {
    s_rf.mb_head = 0;
    for (int i = 0; i < HEAD_CACHE; i++) {
        s_rf.hc_rank[i] = -1;
        s_rf.hc_head[i] = 0;
    }
}

// Copy of n <= 128 bytes by the calling thread alone, with the widest accesses both addresses allow
// (an out-of-line call would save and restore dozens of registers for a few bytes).  A global source
// is read from L2 (another SM may have written it); local and shared sources with generic loads.
template <class T>
__device__ __forceinline__ void small_copy_t(char* d, const char* s, int n, bool g) {
    if (g)
        for (int i = 0; i < n; i += (int)sizeof(T)) *(T*)(d + i) = __ldcg((const T*)(s + i));
    else
        for (int i = 0; i < n; i += (int)sizeof(T)) *(T*)(d + i) = *(const T*)(s + i);
}
__device__ __forceinline__ void small_copy(void* dst, const void* src, int n) {
    char* d = (char*)dst;
    const char* s = (const char*)src;
    const bool g = is_global_ptr(s);
    const unsigned a = (unsigned)(size_t)d | (unsigned)(size_t)s | (unsigned)n;
    if ((a & 15) == 0) small_copy_t<uint4>(d, s, n, g);
    else if ((a & 7) == 0) small_copy_t<unsigned long long>(d, s, n, g);
    else if ((a & 3) == 0) small_copy_t<unsigned>(d, s, n, g);
    else small_copy_t<unsigned char>(d, s, n, g);
}

// Thread-0 entry to the copy engine: contiguous or typed copy of packed bytes [0, n).
// Uses the whole block when both sides are addressable by it, a shared job for very large
// contiguous global copies, and thread 0 alone for thread-local buffers.
__device__ __noinline__ int t0_copy(void* dst, const TypeDesc* dd, const void* src, const TypeDesc* sd, long long n) {
    if (n <= 0) return 0;
    bool blk = block_addressable(dst) && block_addressable(src);
    if (!blk || n <= 128) {
        if (!dd && !sd) copy_bytes(dst, src, n, 0, 1);
        else typed_copy(dst, dd, src, sd, 0, n, 0, 1);
        return 0;
    }
    if (!dd && !sd && is_global_ptr(dst) && is_global_ptr(src) && c_rt.nengines > 0 &&
        n >= c_rt.engine_min_bytes) {
        Job* j = &c_rt.ranks[me()].p2p_job;
        j->kind = JOB_COPY;
        j->src = src;
        j->dst = dst;
        j->count = n;
        j->chunk = c_rt.copy_chunk_bytes;
        int nch = (int)((n + j->chunk - 1) / j->chunk);
        unsigned e = job_open(j, nch);
        if (nch > 1) board_post(j, e);
        return job_run_and_wait(j, __LINE__);
    }
    Task t;
    if (!dd && !sd) {
        t.kind = TASK_COPY;
        t.p0 = src;
        t.p1 = dst;
        t.n0 = n;
    } else {
        t.kind = TASK_TYPED_COPY;
        t.p0 = src;
        t.p1 = dst;
        t.p2 = sd;
        t.p4 = dd;
        t.n0 = 0;
        t.n1 = n;
    }
    dispatch(t);
    return 0;
}

// ---- request pool ----
__device__ __noinline__ MPI_Request_impl* req_alloc() {
    RankState* R = &c_rt.ranks[me()];
    int* fl = c_rt.req_free + (size_t)me() * c_rt.pending;
    int idx;
    if (R->req_free_top > 0) idx = fl[--R->req_free_top];
    else if (R->req_hwm < c_rt.pending) idx = R->req_hwm++;
    else return nullptr;
    MPI_Request_impl* q = c_rt.reqs + (size_t)me() * c_rt.pending + idx;
    q->index = idx;
    q->done_flag = 0;
    q->freed = 0;
    q->stage = nullptr;
    q->st_source = MPI_ANY_SOURCE;
    q->st_tag = MPI_ANY_TAG;
    q->st_error = 0;
    q->st_bytes = 0;
    return q;
}

__device__ void req_release(MPI_Request_impl* q) {
    RankState* R = &c_rt.ranks[me()];
    q->kind = REQ_FREE;
    q->state = RS_IDLE;
    c_rt.req_free[(size_t)me() * c_rt.pending + R->req_free_top++] = q->index;
}

// (the ring depth is a power of two, so the slot index is a mask, not a 64-bit division)
__device__ __forceinline__ Envelope* ring_slot(int rank, unsigned long long t) {
    return c_rt.ring + (size_t)rank * c_rt.mbox_depth + (size_t)(t & (unsigned long long)(c_rt.mbox_depth - 1));
}
__device__ __forceinline__ unsigned char* ring_payload(int rank, unsigned long long t) {
    return c_rt.ring_payload + ((size_t)rank * c_rt.mbox_depth + (size_t)(t & (unsigned long long)(c_rt.mbox_depth - 1))) *
                                    (size_t)c_rt.eager;
}
// entry k (a monotonic position) of this rank's unexpected queue
__device__ __forceinline__ UqEntry* uq_at(int k) { return c_rt.uq + (size_t)me() * c_rt.uq_depth + (k % c_rt.uq_depth); }

// Makes room by moving the live entries of a full queue to its front, order kept (only when dead entries
// are trapped behind a live one; removal never moves entries).
__device__ __noinline__ void uq_compact(RankState* R) {
    int w = R->uq_head;
    for (int k = R->uq_head; k < R->uq_tail; k++) {
        UqEntry* u = uq_at(k);
        if (!u->live) continue;
        if (w != k) *uq_at(w) = *u;
        w++;
    }
    R->uq_tail = w;
}
__device__ __forceinline__ unsigned char* uq_payload(int slot) {
    return c_rt.uq_payload + ((size_t)me() * c_rt.uq_depth + slot) * (size_t)c_rt.eager;
}

__device__ __forceinline__ bool env_matches(const MPI_Request_impl* q, int src, int tag, int ctx) {
    return q->ctx == ctx && (q->peer == MPI_ANY_SOURCE || q->peer == src) && (q->tag == MPI_ANY_TAG || q->tag == tag);
}

// Completes receive q from envelope e whose inline payload (if any) is at `inl`.
__device__ __noinline__ int complete_recv(MPI_Request_impl* q, const Envelope& e, const unsigned char* inl) {
    long long n = e.bytes < q->bytes ? e.bytes : q->bytes;
    int err = e.bytes > q->bytes ? GPUMPI_ERR_TRUNCATE : 0;
    int rc = 0;
    if (e.flags & ENV_INLINE) {
        if (!q->desc && n <= 128) small_copy(q->buf, inl, (int)n);
        else rc = t0_copy(q->buf, q->desc, inl, nullptr, n);
    } else if (e.flags & ENV_HEAP) {
        rc = t0_copy(q->buf, q->desc, e.data, nullptr, n);
        free((void*)e.data);
    } else {
        rc = t0_copy(q->buf, q->desc, e.data, e.desc, n);
    }
    if (e.done_flag) st_release(e.done_flag, 1u);
    q->st_source = e.src;
    q->st_tag = e.tag;
    q->st_error = err ? err : rc;
    q->st_bytes = n;
    q->state = RS_DONE;
    return rc;
}

// Drains this rank's envelope ring: match posted receives in posting order, else queue as unexpected.
__device__ __noinline__ int progress_drain() {
    RankState* R = &c_rt.ranks[me()];
    unsigned long long head = s_rf.mb_head;
    int* posted = c_rt.posted + (size_t)me() * c_rt.posted_cap;
    int rc = 0;
    for (;;) {
        Envelope* slot = ring_slot(me(), head);
        if (ld_acquire(&slot->seq) != (unsigned)(head + 1)) break;
        Envelope e;
        e.src = __ldcg(&slot->src);
        e.tag = __ldcg(&slot->tag);
        e.ctx = __ldcg(&slot->ctx);
        e.bytes = __ldcg(&slot->bytes);
        e.data = (const void*)__ldcg((const unsigned long long*)&slot->data);
        e.done_flag = (unsigned*)__ldcg((const unsigned long long*)&slot->done_flag);
        e.desc = (const TypeDesc*)__ldcg((const unsigned long long*)&slot->desc);
        e.count = __ldcg(&slot->count);
        e.flags = __ldcg(&slot->flags);
        e.world_src = __ldcg(&slot->world_src);
        int match = -1, qi = -1;
        for (int i = R->posted_lo; i < R->nposted; i++) {
            const int pi = posted[i];
            if (pi < 0) continue;
            MPI_Request_impl* q = c_rt.reqs + (size_t)me() * c_rt.pending + pi;
            if (env_matches(q, e.src, e.tag, e.ctx)) {
                match = i;
                qi = pi;
                break;
            }
        }
        if (match >= 0) {
            MPI_Request_impl* q = c_rt.reqs + (size_t)me() * c_rt.pending + qi;
            // remove without moving the others: a hole, then trim holes at both ends
            posted[match] = -1;
            while (R->posted_lo < R->nposted && posted[R->posted_lo] < 0) R->posted_lo++;
            while (R->nposted > R->posted_lo && posted[R->nposted - 1] < 0) R->nposted--;
            if (R->posted_lo == R->nposted) R->posted_lo = R->nposted = 0;
            int r = complete_recv(q, e, ring_payload(me(), head));
            if (r) rc = r;
            if (q->freed) req_release(q);
        } else {
            if (R->uq_tail - R->uq_head >= c_rt.uq_depth) {
                uq_compact(R);
                if (R->uq_tail - R->uq_head >= c_rt.uq_depth) break;  // full: leave it in the ring
            }
            UqEntry* u = uq_at(R->uq_tail);
            u->env = e;
            u->slot = -1;
            u->live = 1;
            if ((e.flags & ENV_INLINE) && e.bytes > 0) {
                int* fl = c_rt.uq_free + (size_t)me() * c_rt.uq_depth;
                int s = R->uq_free_top > 0 ? fl[--R->uq_free_top] : R->uq_hwm++;
                u->slot = s;
                if (e.bytes <= 128) small_copy(uq_payload(s), ring_payload(me(), head), (int)e.bytes);
                else t0_copy(uq_payload(s), nullptr, ring_payload(me(), head), nullptr, e.bytes);
            }
            R->uq_tail++;
        }
        head++;
        s_rf.mb_head = head;
        st_release64(&R->mb_head, head);
    }
    return rc;
}

// Nothing to do unless the next envelope of this rank's ring has been published (one acquire load).
__device__ __forceinline__ int progress() {
    const unsigned long long h = s_rf.mb_head;
    if (ld_relaxed(&ring_slot(me(), h)->seq) != (unsigned)(h + 1)) return 0;
    return progress_drain();
}

// Removes the entry at position k: it is marked dead, and the head moves past dead entries at the front.
__device__ __forceinline__ void uq_remove(int k) {
    RankState* R = &c_rt.ranks[me()];
    UqEntry* u = uq_at(k);
    if (u->slot >= 0) {
        int* fl = c_rt.uq_free + (size_t)me() * c_rt.uq_depth;
        fl[R->uq_free_top++] = u->slot;
    }
    u->live = 0;
    if (k == R->uq_head) {
        int h = k + 1;
        while (h < R->uq_tail && !uq_at(h)->live) h++;
        R->uq_head = h;
        if (h == R->uq_tail) R->uq_head = R->uq_tail = 0;  // empty: positions restart (no overflow)
    }
}

__device__ __forceinline__ MPI_Comm_impl* check_comm(MPI_Comm c) {
    if (c == nullptr || c->magic != COMM_MAGIC) return nullptr;
    return c;
}

// blocking: the caller waits for completion right away (MPI_Send); an eager send is complete when this
// returns, so it needs no request and *out is set to MPI_REQUEST_NULL.
__device__ __noinline__ int p2p_isend(const void* buf, long long count, int dt, int dest, int tag, MPI_Comm c,
                         MPI_Request* out, bool sync, bool blocking = false) {
    if (out) *out = nullptr;
    if (!check_comm(c)) return GPUMPI_ERR_COMM;
    if (count < 0) return GPUMPI_ERR_COUNT;
    if (tag < 0) return GPUMPI_ERR_TAG;
    const TypeDesc* d = (dest >= 0 && dest < c->size) ? resolve_type(dt) : nullptr;
    const long long bytes = d ? count * d->size : 0;
    const bool eager = d && bytes <= c_rt.eager && !sync;
    MPI_Request_impl* q = nullptr;
    if (!(eager && blocking)) {
        q = req_alloc();
        if (!q) {
            record_error(GPUMPI_ERR_REQUEST, 0, __LINE__, c_rt.pending);
            return GPUMPI_ERR_REQUEST;
        }
        q->kind = REQ_SEND;
        q->comm = c;
        q->tag = tag;
        q->ctx = c->ctx;
        if (out) *out = q;
    }
    if (dest == MPI_PROC_NULL) {
        if (q) {
            q->state = RS_DONE;
            q->st_source = MPI_PROC_NULL;
        }
        return 0;
    }
    if (dest < 0 || dest >= c->size) {
        if (q) q->state = RS_DONE;
        return GPUMPI_ERR_RANK;
    }
    if (!d) {
        if (q) q->state = RS_DONE;
        return GPUMPI_ERR_TYPE;
    }
    const TypeDesc* sdesc = desc_contiguous(d) ? nullptr : d;
    int dw = c->is_world ? dest : c->members[dest];
    int mycr = comm_rank_of(c, me());
    if (q) {
        q->peer = dw;
        q->buf = (void*)buf;
        q->bytes = bytes;
    }
    RankState* RD = &c_rt.ranks[dw];
    unsigned long long t = atomicAdd(&RD->mb_tail, 1ULL);
    // flow control: the receiver's ring must have a free slot for ticket t; a cached head (a lower
    // bound) usually proves it without reading the receiver's head
    const unsigned long long depth = (unsigned long long)c_rt.mbox_depth;
    const int hc = dw & (HEAD_CACHE - 1);
    unsigned long long known = s_rf.hc_rank[hc] == dw ? s_rf.hc_head[hc] : 0;
    if (t - known >= depth) {
        known = ld_acquire64(&RD->mb_head);
        if (t - known >= depth) {
            Deadline dl = make_deadline();
            while (t - (known = ld_acquire64(&RD->mb_head)) >= depth) {
                progress();
                if (int e = wait_tick(dl, __LINE__)) {
                    if (q) q->state = RS_DONE;
                    return e;
                }
            }
        }
        s_rf.hc_rank[hc] = dw;
        s_rf.hc_head[hc] = known;
    }
    Envelope* slot = ring_slot(dw, t);
    int flags = 0;
    const void* data = nullptr;
    unsigned* flag = nullptr;
    const TypeDesc* edesc = nullptr;
    if (eager) {
        if (!sdesc && bytes <= 128) small_copy(ring_payload(dw, t), buf, (int)bytes);
        else t0_copy(ring_payload(dw, t), nullptr, buf, sdesc, bytes);
        flags = ENV_INLINE;
        if (q) q->state = RS_DONE;
    } else if (!is_global_ptr(buf)) {
        void* h = malloc(bytes > 0 ? bytes : 1);
        if (!h) {
            record_error(GPUMPI_ERR_NO_MEM, 0, __LINE__, bytes);
            q->state = RS_DONE;
            return GPUMPI_ERR_NO_MEM;
        }
        t0_copy(h, nullptr, buf, sdesc, bytes);
        flags = ENV_HEAP;
        data = h;
        if (sync) {
            flag = &q->done_flag;
            q->state = RS_ACTIVE;
        } else {
            q->state = RS_DONE;
        }
    } else {
        data = buf;
        edesc = sdesc;
        flag = &q->done_flag;
        q->state = RS_ACTIVE;
    }
    slot->src = mycr;
    slot->tag = tag;
    slot->ctx = c->ctx;
    slot->bytes = bytes;
    slot->data = data;
    slot->done_flag = flag;
    slot->desc = edesc;
    slot->count = count;
    slot->flags = flags;
    slot->world_src = me();
    st_release(&slot->seq, (unsigned)(t + 1));
    progress();
    return 0;
}

__device__ __noinline__ int p2p_irecv(void* buf, long long count, int dt, int src, int tag, MPI_Comm c, MPI_Request* out) {
    if (!check_comm(c)) return GPUMPI_ERR_COMM;
    if (count < 0) return GPUMPI_ERR_COUNT;
    MPI_Request_impl* q = req_alloc();
    if (!q) {
        record_error(GPUMPI_ERR_REQUEST, 0, __LINE__, c_rt.pending);
        return GPUMPI_ERR_REQUEST;
    }
    q->kind = REQ_RECV;
    q->comm = c;
    q->tag = tag;
    q->ctx = c->ctx;
    q->peer = src;
    q->buf = buf;
    if (out) *out = q;
    if (src == MPI_PROC_NULL) {
        q->state = RS_DONE;
        q->st_source = MPI_PROC_NULL;
        q->st_tag = MPI_ANY_TAG;
        return 0;
    }
    if (src != MPI_ANY_SOURCE && (src < 0 || src >= c->size)) {
        q->state = RS_DONE;
        return GPUMPI_ERR_RANK;
    }
    const TypeDesc* d = resolve_type(dt);
    if (!d) {
        q->state = RS_DONE;
        return GPUMPI_ERR_TYPE;
    }
    q->desc = desc_contiguous(d) ? nullptr : d;
    q->bytes = count * d->size;
    q->count = count;
    q->state = RS_ACTIVE;
    RankState* R = &c_rt.ranks[me()];
    // earliest matching unexpected message first
    for (int k = R->uq_head; k < R->uq_tail; k++) {
        UqEntry* u = uq_at(k);
        if (!u->live) continue;
        if (env_matches(q, u->env.src, u->env.tag, u->env.ctx)) {
            Envelope e = u->env;
            int rc = complete_recv(q, e, u->slot >= 0 ? uq_payload(u->slot) : nullptr);
            uq_remove(k);
            return rc;
        }
    }
    if (R->nposted >= c_rt.posted_cap) {  // full: move the live entries to the front, order kept
        int* posted = c_rt.posted + (size_t)me() * c_rt.posted_cap;
        int w = 0;
        for (int i = R->posted_lo; i < R->nposted; i++)
            if (posted[i] >= 0) posted[w++] = posted[i];
        R->posted_lo = 0;
        R->nposted = w;
    }
    if (R->nposted >= c_rt.posted_cap) {
        record_error(GPUMPI_ERR_REQUEST, 1, __LINE__, c_rt.posted_cap);
        q->state = RS_DONE;
        return GPUMPI_ERR_REQUEST;
    }
    c_rt.posted[(size_t)me() * c_rt.posted_cap + R->nposted++] = q->index;
    return progress();
}

// Non-blocking completion check; returns true when q is complete.
__device__ __forceinline__ bool req_poll(MPI_Request_impl* q) {
    if (q->state == RS_DONE) return true;
    if (q->kind == REQ_SEND && ld_relaxed(&q->done_flag)) {
        fence_acqrel();
        q->state = RS_DONE;
        return true;
    }
    return false;
}

__device__ __forceinline__ void fill_status(const MPI_Request_impl* q, MPI_Status* st) {
    if (!st) return;
    st->MPI_SOURCE = q->st_source;
    st->MPI_TAG = q->st_tag;
    st->MPI_ERROR = q->st_error;
    st->count_bytes = q->st_bytes;
}

__device__ __noinline__ int req_wait(MPI_Request* rp, MPI_Status* st) {
    MPI_Request_impl* q = *rp;
    if (!q) {
        if (st) *st = MPI_Status();
        return 0;
    }
    if (!req_poll(q)) {
        progress();
        Deadline dl = make_deadline();
        while (!req_poll(q)) {
            progress();
            if (int e = wait_tick(dl, __LINE__, 32)) return e;
        }
    }
    int err = q->st_error;
    fill_status(q, st);
    req_release(q);
    *rp = MPI_REQUEST_NULL;
    return err;
}

}  // namespace gpumpi
