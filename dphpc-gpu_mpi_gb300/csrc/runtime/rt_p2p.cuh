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
    if (!dd && !sd && is_global_ptr(dst) && is_global_ptr(src) && g_rt->nengines > 0 &&
        n >= g_rt->engine_min_bytes) {
        Job* j = &g_rt->ranks[me()].p2p_job;
        j->kind = JOB_COPY;
        j->src = src;
        j->dst = dst;
        j->count = n;
        j->chunk = g_rt->copy_chunk_bytes;
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
    RankState* R = &g_rt->ranks[me()];
    int* fl = g_rt->req_free + (size_t)me() * g_rt->pending;
    int idx;
    if (R->req_free_top > 0) idx = fl[--R->req_free_top];
    else if (R->req_hwm < g_rt->pending) idx = R->req_hwm++;
    else return nullptr;
    MPI_Request_impl* q = g_rt->reqs + (size_t)me() * g_rt->pending + idx;
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
    RankState* R = &g_rt->ranks[me()];
    q->kind = REQ_FREE;
    q->state = RS_IDLE;
    g_rt->req_free[(size_t)me() * g_rt->pending + R->req_free_top++] = q->index;
}

__device__ __forceinline__ Envelope* ring_slot(int rank, unsigned long long t) {
    return g_rt->ring + (size_t)rank * g_rt->mbox_depth + (t % (unsigned long long)g_rt->mbox_depth);
}
__device__ __forceinline__ unsigned char* ring_payload(int rank, unsigned long long t) {
    return g_rt->ring_payload +
           ((size_t)rank * g_rt->mbox_depth + (t % (unsigned long long)g_rt->mbox_depth)) * (size_t)g_rt->eager;
}
__device__ __forceinline__ UqEntry* uq_at(int i) { return g_rt->uq + (size_t)me() * g_rt->uq_depth + i; }
__device__ __forceinline__ unsigned char* uq_payload(int slot) {
    return g_rt->uq_payload + ((size_t)me() * g_rt->uq_depth + slot) * (size_t)g_rt->eager;
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
        rc = t0_copy(q->buf, q->desc, inl, nullptr, n);
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
__device__ __noinline__ int progress() {
    RankState* R = &g_rt->ranks[me()];
    unsigned long long head = R->mb_head;
    int* posted = g_rt->posted + (size_t)me() * g_rt->posted_cap;
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
        int match = -1;
        for (int i = 0; i < R->nposted; i++) {
            MPI_Request_impl* q = g_rt->reqs + (size_t)me() * g_rt->pending + posted[i];
            if (env_matches(q, e.src, e.tag, e.ctx)) { match = i; break; }
        }
        if (match >= 0) {
            MPI_Request_impl* q = g_rt->reqs + (size_t)me() * g_rt->pending + posted[match];
            for (int i = match; i + 1 < R->nposted; i++) posted[i] = posted[i + 1];
            R->nposted--;
            int r = complete_recv(q, e, ring_payload(me(), head));
            if (r) rc = r;
            if (q->freed) req_release(q);
        } else {
            if (R->uq_count >= g_rt->uq_depth) break;  // unexpected queue full: leave it in the ring
            UqEntry* u = uq_at(R->uq_count);
            u->env = e;
            u->slot = -1;
            if ((e.flags & ENV_INLINE) && e.bytes > 0) {
                int* fl = g_rt->uq_free + (size_t)me() * g_rt->uq_depth;
                int s = R->uq_free_top > 0 ? fl[--R->uq_free_top] : R->uq_hwm++;
                u->slot = s;
                t0_copy(uq_payload(s), nullptr, ring_payload(me(), head), nullptr, e.bytes);
            }
            R->uq_count++;
        }
        head++;
        st_release64(&R->mb_head, head);
    }
    return rc;
}

__device__ __forceinline__ void uq_remove(int i) {
    RankState* R = &g_rt->ranks[me()];
    UqEntry* u = uq_at(i);
    if (u->slot >= 0) {
        int* fl = g_rt->uq_free + (size_t)me() * g_rt->uq_depth;
        fl[R->uq_free_top++] = u->slot;
    }
    for (int k = i; k + 1 < R->uq_count; k++) *uq_at(k) = *uq_at(k + 1);
    R->uq_count--;
}

__device__ __forceinline__ MPI_Comm_impl* check_comm(MPI_Comm c) {
    if (c == nullptr || c->magic != COMM_MAGIC) return nullptr;
    return c;
}

__device__ __noinline__ int p2p_isend(const void* buf, long long count, int dt, int dest, int tag, MPI_Comm c,
                         MPI_Request* out, bool sync) {
    if (!check_comm(c)) return GPUMPI_ERR_COMM;
    if (count < 0) return GPUMPI_ERR_COUNT;
    if (tag < 0) return GPUMPI_ERR_TAG;
    MPI_Request_impl* q = req_alloc();
    if (!q) {
        record_error(GPUMPI_ERR_REQUEST, 0, __LINE__, g_rt->pending);
        return GPUMPI_ERR_REQUEST;
    }
    q->kind = REQ_SEND;
    q->comm = c;
    q->tag = tag;
    q->ctx = c->ctx;
    if (out) *out = q;
    if (dest == MPI_PROC_NULL) {
        q->state = RS_DONE;
        q->st_source = MPI_PROC_NULL;
        return 0;
    }
    if (dest < 0 || dest >= c->size) {
        q->state = RS_DONE;
        return GPUMPI_ERR_RANK;
    }
    const TypeDesc* d = resolve_type(dt);
    if (!d) {
        q->state = RS_DONE;
        return GPUMPI_ERR_TYPE;
    }
    const TypeDesc* sdesc = desc_contiguous(d) ? nullptr : d;
    long long bytes = count * d->size;
    int dw = c->is_world ? dest : c->members[dest];
    int mycr = comm_rank_of(c, me());
    q->peer = dw;
    q->buf = (void*)buf;
    q->bytes = bytes;
    RankState* RD = &g_rt->ranks[dw];
    unsigned long long t = atomicAdd(&RD->mb_tail, 1ULL);
    // flow control: wait for a free slot in the receiver's ring, draining our own meanwhile
    if (t - ld_acquire64(&RD->mb_head) >= (unsigned long long)g_rt->mbox_depth) {
        Deadline dl = make_deadline();
        while (t - ld_acquire64(&RD->mb_head) >= (unsigned long long)g_rt->mbox_depth) {
            progress();
            if (int e = wait_tick(dl, __LINE__)) {
                q->state = RS_DONE;
                return e;
            }
        }
    }
    Envelope* slot = ring_slot(dw, t);
    int flags = 0;
    const void* data = nullptr;
    unsigned* flag = nullptr;
    const TypeDesc* edesc = nullptr;
    if (bytes <= g_rt->eager && !sync) {
        t0_copy(ring_payload(dw, t), nullptr, buf, sdesc, bytes);
        flags = ENV_INLINE;
        q->state = RS_DONE;
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
        record_error(GPUMPI_ERR_REQUEST, 0, __LINE__, g_rt->pending);
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
    RankState* R = &g_rt->ranks[me()];
    // earliest matching unexpected message first
    for (int i = 0; i < R->uq_count; i++) {
        UqEntry* u = uq_at(i);
        if (env_matches(q, u->env.src, u->env.tag, u->env.ctx)) {
            Envelope e = u->env;
            int rc = complete_recv(q, e, u->slot >= 0 ? uq_payload(u->slot) : nullptr);
            uq_remove(i);
            return rc;
        }
    }
    if (R->nposted >= g_rt->posted_cap) {
        record_error(GPUMPI_ERR_REQUEST, 1, __LINE__, g_rt->posted_cap);
        q->state = RS_DONE;
        return GPUMPI_ERR_REQUEST;
    }
    g_rt->posted[(size_t)me() * g_rt->posted_cap + R->nposted++] = q->index;
    return progress();
}

// Non-blocking completion check; returns true when q is complete.
__device__ __forceinline__ bool req_poll(MPI_Request_impl* q) {
    if (q->state == RS_DONE) return true;
    if (q->kind == REQ_SEND && ld_acquire(&q->done_flag)) {
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
            if (int e = wait_tick(dl, __LINE__)) return e;
        }
    }
    int err = q->st_error;
    fill_status(q, st);
    req_release(q);
    *rp = MPI_REQUEST_NULL;
    return err;
}

}  // namespace gpumpi
