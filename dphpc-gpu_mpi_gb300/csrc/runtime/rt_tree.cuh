// rt_tree.cuh — TREE variant of the fold (Allreduce / Reduce): a two-level rank split.
//
// The canonical order makes every element one sequential chain over all n ranks, so with few elements
// per rank (many ranks, small messages) there are too few chains to keep HBM busy.  TREE cuts each chain
// into R groups of consecutive ranks: phase-1 chunk (c, g) folds group g of element chunk c in rank order
// and stores the partial in the world's tree scratch, then releases a flag tagged with the job epoch;
// phase-2 chunk c waits for its R flags, folds the partials in group order and writes every member's
// output.  Phase-1 chunks have lower indices than phase-2 chunks, so a phase-2 chunk is only claimed after
// all of its inputs were claimed by running blocks — nothing waits on unclaimed work.  Extra traffic is
// 2*R*b bytes per call against 2*n*b.  The grouping reorders floating-point sums (tolerance-tested against
// an fp64 reference); integer results are exact.
#pragma once
#include "rt_core.cuh"

namespace gpumpi {

__shared__ int s_tree_ok;

// acc (V elements at element e) = canonical fold of members [g0, g1) of the communicator
template <class T, int OP, int V>
__device__ __forceinline__ void tree_fold_range(const CollSlot* slots, int g0, int g1, long long e, int nv, bool vec,
                                                T (&acc)[V], int tid, int nt) {
    constexpr int BYTES = V * (int)sizeof(T);
    constexpr int U = 128 / BYTES > 16 ? 16 : 128 / BYTES < 1 ? 1 : 128 / BYTES;
    for (int r0 = g0; r0 < g1; r0 += PTILE) {
        const int m = min(PTILE, g1 - r0);
        load_ptile(slots, r0, m, 0, tid, nt);
        if (nv == 0) continue;
        int i = 0;
        if (r0 == g0) {
            ld_elems<T, V>((const T*)s_chunk.f.ptile[0] + e, acc, nv, vec);
            i = 1;
        }
        for (; i + U <= m; i += U) {
            T v[U][V];
#pragma unroll
            for (int u = 0; u < U; u++) ld_elems<T, V>((const T*)s_chunk.f.ptile[i + u] + e, v[u], nv, vec);
#pragma unroll
            for (int u = 0; u < U; u++)
#pragma unroll
                for (int q = 0; q < V; q++) acc[q] = op_apply<OP, T>(v[u][q], acc[q]);
        }
        for (; i < m; i++) {
            T v[V];
            ld_elems<T, V>((const T*)s_chunk.f.ptile[i] + e, v, nv, vec);
#pragma unroll
            for (int q = 0; q < V; q++) acc[q] = op_apply<OP, T>(v[q], acc[q]);
        }
    }
}

template <class T, int OP, int V>
__device__ __noinline__ void fold_tree(const JobParams* j, long long idx, int tid, int nt) {
    const CollSlot* slots = j->slots;
    const int n = j->csize;
    const int R = j->tile;
    const long long E = j->chunk;
    const long long count = j->count;
    const long long C = (count + E - 1) / E;
    const bool vec = j->aligned16 >= (int)(V * sizeof(T) >= 16 ? 16 : V * sizeof(T));
    T* partial = (T*)c_rt.tree_scratch;
    unsigned* flags = c_rt.tree_flags;
    T acc[V];
#pragma unroll
    for (int q = 0; q < V; q++) acc[q] = T();
    if (idx < C * R) {
        // phase 1: group g of element chunk cc
        const long long cc = idx / R;
        const int g = (int)(idx % R);
        const long long e = cc * E + (long long)tid * V;
        const int nv = e < count ? (int)min((long long)V, count - e) : 0;
        const int g0 = (int)((long long)g * n / R), g1 = (int)((long long)(g + 1) * n / R);
        tree_fold_range<T, OP, V>(slots, g0, g1, e, nv, vec, acc, tid, nt);
        if (nv > 0) st_elems<T, V>(partial + (long long)g * count + e, acc, nv, vec);
        bar_sync(BAR_TASK, nt);
        if (tid == 0) {
            __threadfence();
            st_release(&flags[cc * R + g], j->epoch);
        }
        return;
    }
    // phase 2: combine the R partials of element chunk cc in group order, write the outputs
    const long long cc = idx - C * R;
    const long long e = cc * E + (long long)tid * V;
    const int nv = e < count ? (int)min((long long)V, count - e) : 0;
    if (tid == 0) {
        s_tree_ok = 1;
        Deadline d = make_deadline();
        for (int g = 0; g < R; g++) {
            while (ld_relaxed(&flags[cc * R + g]) != j->epoch) {
                if (wait_tick(d, __LINE__, 256)) {
                    s_tree_ok = 0;
                    break;
                }
            }
            if (!s_tree_ok) break;
        }
        fence_acqrel();
    }
    bar_sync(BAR_TASK, nt);
    if (!s_tree_ok) return;
    if (nv > 0) {
        ld_elems<T, V>(partial + e, acc, nv, vec);
        for (int g = 1; g < R; g++) {
            T v[V];
            ld_elems<T, V>(partial + (long long)g * count + e, v, nv, vec);
#pragma unroll
            for (int q = 0; q < V; q++) acc[q] = op_apply<OP, T>(v[q], acc[q]);
        }
    }
    if (j->kind == JOB_REDUCE) {
        if (nv > 0) st_elems<T, V>((T*)slot_out(&slots[j->root]) + e, acc, nv, vec);
        return;
    }
    for (int r0 = 0; r0 < n; r0 += PTILE) {
        const int m = min(PTILE, n - r0);
        load_ptile(slots, r0, m, 1, tid, nt);
        if (nv > 0)
            for (int i = 0; i < m; i++) st_elems<T, V>((T*)s_chunk.f.ptile[i] + e, acc, nv, vec);
    }
}

template <class T, int OP>
__device__ __forceinline__ void fold_tree_v(const JobParams* j, long long idx, int tid, int nt) {
    if (j->vec >= 16 / (int)sizeof(T)) fold_tree<T, OP, 16 / sizeof(T)>(j, idx, tid, nt);
    else fold_tree<T, OP, 1>(j, idx, tid, nt);
}

template <class T>
__device__ __forceinline__ bool fold_tree_t(const JobParams* j, long long idx, int tid, int nt) {
    switch (j->op) {
    case GPUMPI_OP_SUM: fold_tree_v<T, GPUMPI_OP_SUM>(j, idx, tid, nt); return true;
    case GPUMPI_OP_MAX: fold_tree_v<T, GPUMPI_OP_MAX>(j, idx, tid, nt); return true;
    case GPUMPI_OP_MIN: fold_tree_v<T, GPUMPI_OP_MIN>(j, idx, tid, nt); return true;
    case GPUMPI_OP_PROD: fold_tree_v<T, GPUMPI_OP_PROD>(j, idx, tid, nt); return true;
    default: return false;
    }
}

// true if (dt, op) has a TREE instantiation
__device__ __forceinline__ bool fold_has_tree(int dt, int op, MPI_User_function* ufn) {
    if (ufn || !(op == GPUMPI_OP_SUM || op == GPUMPI_OP_MAX || op == GPUMPI_OP_MIN || op == GPUMPI_OP_PROD))
        return false;
    switch (dt) {
    case GPUMPI_FLOAT: case GPUMPI_DOUBLE: case GPUMPI_LONG_DOUBLE: case GPUMPI_INT: case GPUMPI_INT32_T:
    case GPUMPI_LONG: case GPUMPI_LONG_LONG_INT: case GPUMPI_LONG_LONG: case GPUMPI_INT64_T:
        return true;
    default: return false;
    }
}

__device__ __forceinline__ bool fold_tree_dispatch(const JobParams* j, long long idx, int tid, int nt) {
    switch (j->dt) {
    case GPUMPI_FLOAT: return fold_tree_t<float>(j, idx, tid, nt);
    case GPUMPI_DOUBLE: case GPUMPI_LONG_DOUBLE: return fold_tree_t<double>(j, idx, tid, nt);
    case GPUMPI_INT: case GPUMPI_INT32_T: return fold_tree_t<int>(j, idx, tid, nt);
    default: return fold_tree_t<long long>(j, idx, tid, nt);
    }
}

}  // namespace gpumpi
