// rt_comm.cuh — communicators, groups and derived-type constructors.
//
// Reference: communicators are per-rank heap objects that share nothing but a context id agreed by
// MPI_Allreduce(MAX) (gpu_libs/gpu_mpi/communicator.cu:37-46,164-213), groups are rank vectors with a
// linear-scan rank lookup (gpu_libs/gpu_mpi/group.cu:7-11,110-122), and point-to-point ignores the
// group's rank map (hazard H1: mpi.cu:551,567 pass the communicator rank straight through as a global
// thread index).  Here a communicator is ONE object in device memory shared by its members, created
// collectively: members publish (colour, key), the first member of each colour allocates the object
// from the run's arena, every member writes its own entry of the rank maps, and a barrier on the new
// communicator closes the handshake.  Context ids come from a global counter, so they are unique
// without an agreement round.  The comm-rank <-> world-rank maps are used by every operation.
#pragma once
#include "rt_core.cuh"
#include "rt_coll.cuh"
#include "rt_p2p.cuh"

namespace gpumpi {

__device__ void* arena_alloc(unsigned long long bytes) {
    bytes = (bytes + 127) & ~127ULL;
    unsigned long long off = atomicAdd(c_rt.arena_top, bytes);
    if (off + bytes > c_rt.arena_bytes) return nullptr;
    return c_rt.arena + off;
}

struct SplitScan {
    const CollSlot* slots;
    int n;
    int color, key, cr;
    int newrank, newsize, leader;
    int* fill;            // rank_of array to initialise with -1 (leader only)
    int fill_n;
};
__shared__ SplitScan s_split;

// Block task: position of the calling member among members with the same colour (ordered by key,
// then parent rank — gpu_libs/gpu_mpi/communicator.cu:164-213 sorts by (key, rank) the same way).
__device__ void split_scan_task(void* arg, int tid, int nt) {
    SplitScan* s = (SplitScan*)arg;
    if (s->fill) {
        for (int i = tid; i < s->fill_n; i += nt) s->fill[i] = -1;
        return;
    }
    int rank = 0, size = 0, leader = 0x7fffffff;
    for (int q = tid; q < s->n; q += nt) {
        int cq = (int)__ldcg(&s->slots[q].x0);
        if (cq != s->color) continue;
        int kq = (int)__ldcg(&s->slots[q].x1);
        size++;
        if (kq < s->key || (kq == s->key && q < s->cr)) rank++;
        // leader = member with the smallest (key, rank); encode as key-major ordering index
        if (leader == 0x7fffffff) leader = q;
        else {
            int kl = (int)__ldcg(&s->slots[leader].x1);
            if (kq < kl || (kq == kl && q < leader)) leader = q;
        }
    }
    atomicAdd(&s->newrank, rank);
    atomicAdd(&s->newsize, size);
    // reduce the leader: smallest (key, q)
    if (leader != 0x7fffffff) {
        for (;;) {
            int cur = atomicAdd(&s->leader, 0);
            bool better = cur == 0x7fffffff;
            if (!better) {
                int kc = (int)__ldcg(&s->slots[cur].x1), kl = (int)__ldcg(&s->slots[leader].x1);
                better = kl < kc || (kl == kc && leader < cur);
            }
            if (!better) break;
            if (atomicCAS(&s->leader, cur, leader) == cur) break;
        }
    }
}

__device__ __noinline__ int comm_split_impl(MPI_Comm parent, int color, int key, MPI_Comm* out) {
    MPI_Comm_impl* c = check_comm(parent);
    if (!c) return GPUMPI_ERR_COMM;
    const int cr = comm_rank_of(c, me());
    CollSlot* sl = &c->slots[cr];
    sl->x0 = color;
    sl->x1 = key;
    sl->rbuf = nullptr;
    int rc = comm_barrier(c, []() {}, __LINE__);
    if (rc) return rc;
    MPI_Comm_impl* obj = nullptr;
    int newrank = -1, newsize = 0, leader = -1;
    if (color != GPUMPI_UNDEFINED) {
        s_split.slots = c->slots;
        s_split.n = c->size;
        s_split.color = color;
        s_split.key = key;
        s_split.cr = cr;
        s_split.newrank = 0;
        s_split.newsize = 0;
        s_split.leader = 0x7fffffff;
        s_split.fill = nullptr;
        Task t;
        t.kind = TASK_USER;
        t.p0 = (const void*)&split_scan_task;
        t.p1 = &s_split;
        dispatch(t);
        newrank = s_split.newrank;
        newsize = s_split.newsize;
        leader = s_split.leader;
        if (newrank == 0) {
            obj = (MPI_Comm_impl*)arena_alloc(sizeof(MPI_Comm_impl));
            int* members = (int*)arena_alloc(sizeof(int) * (unsigned long long)newsize);
            int* rank_of = (int*)arena_alloc(sizeof(int) * (unsigned long long)c_rt.nranks);
            CollSlot* slots = (CollSlot*)arena_alloc(sizeof(CollSlot) * (unsigned long long)newsize);
            unsigned char* tiny = (unsigned char*)arena_alloc(2ULL * TINY_BYTES * (unsigned long long)newsize);
            if (!obj || !members || !rank_of || !slots || !tiny) {
                record_error(GPUMPI_ERR_NO_MEM, 0, __LINE__, (long long)c_rt.arena_bytes);
                obj = nullptr;
            } else {
                memset(obj, 0, sizeof(MPI_Comm_impl));
                obj->size = newsize;
                obj->ctx = (int)atomicAdd(c_rt.ctx_counter, 1u);
                obj->is_world = 0;
                obj->members = members;
                obj->rank_of = rank_of;
                obj->slots = slots;
                obj->tiny = tiny;
                obj->magic = COMM_MAGIC;
                s_split.fill = rank_of;
                s_split.fill_n = c_rt.nranks;
                dispatch(t);
            }
            __threadfence();
            sl->rbuf = obj;
        }
    }
    rc = comm_barrier(c, []() {}, __LINE__);
    if (rc) return rc;
    if (color == GPUMPI_UNDEFINED) {
        *out = MPI_COMM_NULL;
        return 0;
    }
    obj = (MPI_Comm_impl*)__ldcg((const unsigned long long*)&c->slots[leader].rbuf);
    if (!obj) {
        *out = MPI_COMM_NULL;
        return GPUMPI_ERR_NO_MEM;
    }
    obj->members[newrank] = me();
    obj->rank_of[me()] = newrank;
    __threadfence();
    rc = comm_barrier(obj, []() {}, __LINE__);
    if (rc) return rc;
    *out = obj;
    return 0;
}

// ---- the rank's scratch pool: a stack in device memory (a freed block is reclaimed once every block above
// it is freed too, the order in which MPI codes free groups and the library releases staging buffers).
// Group objects and staged copies of thread-local buffers come from it; when it is full, from the device
// heap, whose allocator serialises concurrent callers: 512 ranks each building a group per communicator
// spent about 1 ms per communicator in malloc and free. ----
struct PoolBlock {
    int prev1;   // 1 + offset of the block below (0: none)
    int freed;
    int pad[2];
};

__device__ __forceinline__ unsigned char* pool_base() {
    return c_rt.scratch_pool + (long long)me() * c_rt.scratch_pool_bytes;
}

// 16-byte aligned scratch of `bytes` from this rank's pool, or nullptr when it does not fit.
__device__ void* pool_alloc(unsigned long long bytes) {
    const long long need = (long long)((sizeof(PoolBlock) + bytes + 15) & ~15ULL);
    RankState* R = &c_rt.ranks[me()];
    if (!c_rt.scratch_pool || R->pool_top + need > c_rt.scratch_pool_bytes) return nullptr;
    PoolBlock* b = (PoolBlock*)(pool_base() + R->pool_top);
    b->prev1 = R->pool_last1;
    b->freed = 0;
    R->pool_last1 = R->pool_top + 1;
    R->pool_top += (int)need;
    return b + 1;
}

__device__ __forceinline__ bool pool_owns(const void* p) {
    const unsigned char* b = pool_base();
    return c_rt.scratch_pool && (const unsigned char*)p >= b && (const unsigned char*)p < b + c_rt.scratch_pool_bytes;
}

__device__ void pool_free(void* p) {
    ((PoolBlock*)p - 1)->freed = 1;
    RankState* R = &c_rt.ranks[me()];
    unsigned char* base = pool_base();
    while (R->pool_last1 > 0) {
        PoolBlock* top = (PoolBlock*)(base + (R->pool_last1 - 1));
        if (!top->freed) break;
        R->pool_top = R->pool_last1 - 1;
        R->pool_last1 = top->prev1;
    }
}

// Scratch from the pool, else the device heap; release with scratch_free.
__device__ void* scratch_alloc(unsigned long long bytes) {
    void* p = pool_alloc(bytes);
    return p ? p : malloc(bytes ? bytes : 1);
}
__device__ void scratch_free(void* p) {
    if (!p) return;
    if (pool_owns(p)) pool_free(p);
    else free(p);
}

// ---- groups (rank-local objects) ----
__device__ MPI_Group group_new(int n) {
    const unsigned long long body = sizeof(MPI_Group_impl) + sizeof(int) * (unsigned long long)(n > 0 ? n : 1);
    MPI_Group g = (MPI_Group)scratch_alloc(body);
    if (!g) return nullptr;
    g->size = n;
    g->ranks = (int*)(g + 1);
    g->refcount = 1;
    g->is_static = 0;
    return g;
}

// Releases a group object made by group_new.
__device__ void group_delete(MPI_Group g) {
    if (g && !g->is_static) scratch_free(g);
}

// ---- derived datatypes (per-rank table; handle encodes owner rank and slot) ----
__device__ int type_alloc(TypeDesc** out) {
    TypeDesc* tab = c_rt.types + (size_t)me() * c_rt.max_types;
    for (int i = 0; i < c_rt.max_types; i++) {
        if (!tab[i].in_use) {
            tab[i].in_use = 1;
            tab[i].committed = 0;
            *out = &tab[i];
            return GPUMPI_DERIVED_BASE + me() * c_rt.max_types + i;
        }
    }
    return -1;
}

__device__ __forceinline__ bool td_contig(const TypeDesc* t) { return t->nlev == 0 && t->size == t->extent && t->lb == 0; }

// hvector of `count` blocks of `blocklen` old elements at byte stride `sbytes`
__device__ int type_hvector_desc(long long count, long long blocklen, long long sbytes, const TypeDesc* old, TypeDesc* out) {
    if (count < 0 || blocklen < 0) return GPUMPI_ERR_COUNT;
    TypeDesc blk = *old;
    if (td_contig(old)) {
        blk.size = old->size * blocklen;
        blk.extent = blk.size;
        blk.block = blk.size;
    } else {
        if (old->nlev >= 4) return GPUMPI_ERR_TYPE;
        blk.cnt[blk.nlev] = blocklen;
        blk.stride[blk.nlev] = old->extent;
        blk.nlev++;
        blk.size = old->size * blocklen;
        blk.extent = old->extent * blocklen;
    }
    if (count == 1) {
        *out = blk;
        return 0;
    }
    if (td_contig(&blk) && sbytes == blk.extent) {
        *out = blk;
        out->size = blk.size * count;
        out->extent = out->size;
        out->block = out->size;
        return 0;
    }
    if (blk.nlev >= 4) return GPUMPI_ERR_TYPE;
    *out = blk;
    out->cnt[out->nlev] = count;
    out->stride[out->nlev] = sbytes;
    out->nlev++;
    out->size = blk.size * count;
    out->lb = 0;
    out->extent = (count - 1) * sbytes + blk.extent;
    return 0;
}

__device__ int type_subarray_desc(int nd, const int* sizes, const int* subs, const int* starts, int order,
                                  const TypeDesc* old, TypeDesc* out) {
    if (nd < 1 || nd > 3 || !td_contig(old)) return GPUMPI_ERR_TYPE;
    int sz[3], sb[3], st[3];
    for (int d = 0; d < nd; d++) {
        int k = (order == MPI_ORDER_FORTRAN) ? nd - 1 - d : d;  // outermost first
        sz[d] = sizes[k];
        sb[d] = subs[k];
        st[d] = starts[k];
        if (sb[d] < 0 || st[d] < 0 || st[d] + sb[d] > sz[d]) return GPUMPI_ERR_ARG;
    }
    long long es = old->extent;
    TypeDesc t = *old;
    t.size = es * sb[nd - 1];
    t.extent = t.size;
    t.block = t.size;
    t.nlev = 0;
    long long stride = es * sz[nd - 1];
    long long offset = es * st[nd - 1];
    for (int d = nd - 2; d >= 0; d--) {
        t.cnt[t.nlev] = sb[d];
        t.stride[t.nlev] = stride;
        t.nlev++;
        t.size *= sb[d];
        offset += stride * st[d];
        stride *= sz[d];
    }
    t.lb = offset;
    t.extent = stride;
    *out = t;
    return 0;
}

}  // namespace gpumpi
