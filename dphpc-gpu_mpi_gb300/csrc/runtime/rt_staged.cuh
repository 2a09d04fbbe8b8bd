// rt_staged.cuh — STAGED variant of the fold (Allreduce / Reduce): canonical rank order, inputs
// streamed through shared memory by TMA bulk copies.
//
// Chunk = nt*V elements.  For each tile of up to 256 ranks the block first stages the tile's input
// pointers in shared memory (so issuing a copy costs no global round trip), then thread 0 keeps S
// stages of G ranks x chunk bytes in flight (one mbarrier per stage, transaction-count completion)
// while every thread folds its V elements of the ready stage in rank order.  The operation order is
// exactly fold_fast's, so results are bit-identical to DIRECT and to the reference's fold
// (gpu_libs/gpu_mpi/mpi.cu:209-225).  Needs 16-byte aligned buffers and a chunk byte count that is a
// multiple of 16 (the caller checks); the output is written with L2-only vector stores.
#pragma once
#include "rt_core.cuh"
#include "rt_tma.cuh"

namespace gpumpi {

__shared__ int s_stage_abort;

// Issues the bulk copies of one group (ranks k0 .. k0+mm-1 of the current pointer tile) into the stage
// at sdst, after checking what the hardware requires of every copy: 16-byte aligned global source,
// 16-byte aligned destination inside this launch's dynamic shared memory, non-zero size that is a
// multiple of 16.  On a violation nothing is issued: the error is recorded, the abort flag is set and
// the stage barrier is completed with a plain arrival so no thread waits for bytes that never come.
template <class T>
__device__ __forceinline__ void stage_issue(unsigned long long* bar, T* sdst, long long E, int k0, int mm, long long e0,
                                            unsigned CB) {
    for (int k = 0; k < mm; k++) {
        const T* src = (const T*)s_chunk.f.ptile[k0 + k] + e0;
        const unsigned long long s_off = (unsigned long long)((const unsigned char*)(sdst + (long long)k * E) - g_dyn_smem);
        const bool ok = (((unsigned long long)(size_t)src | s_off) & 15ull) == 0 && CB > 0 && (CB & 15u) == 0 &&
                        s_off + CB <= (unsigned long long)c_rt.dyn_smem && is_global_ptr(src);
        if (!ok) {
            record_error(GPUMPI_ERR_INTERN, 2, __LINE__, (long long)s_off);
            s_stage_abort = 1;
            mbar_expect_tx(bar, 0);
            return;
        }
    }
    mbar_expect_tx(bar, (unsigned)mm * CB);
    for (int k = 0; k < mm; k++) tma_load_1d(sdst + (long long)k * E, (const T*)s_chunk.f.ptile[k0 + k] + e0, CB, bar);
}

// Thread 0 after an abort: groups gi .. gi+cnt-1 were issued and not consumed, so their bulk copies may
// still be writing into the stages.  Waits (bounded) for every one of them before the stages can be
// reused or the block exits, then retires the barriers.  If a copy still has not landed, the barriers are
// left alone and the error record raises the launch's abort flag, after which no block issues STAGED
// copies again (fold_chunk / copy_units check the flag).
template <int S>
__device__ __noinline__ void drain_stages(unsigned long long* full, unsigned gi, int cnt, long long idx) {
    bool drained = true;
    for (int k = 0; k < cnt; k++) {
        const unsigned gq = gi + (unsigned)k;
        drained = mbar_wait_bounded(&full[gq % S], (gq / S) & 1u) && drained;
    }
    if (!drained) {
        record_error(GPUMPI_ERR_OTHER, GPUMPI_ERR_TIMEOUT, __LINE__, idx);
        return;
    }
    for (int q = 0; q < S; q++) mbar_inval(&full[q]);
}

template <class T, int OP, int V>
__device__ __noinline__ void fold_staged(const JobParams* j, long long idx, int tid, int nt) {
    constexpr int S = 2;
    const CollSlot* slots = j->slots;
    const int n = j->csize;
    const long long E = j->chunk;
    const long long e0 = idx * E;
    const long long ne = min(E, j->count - e0);
    const unsigned CB = (unsigned)(ne * (long long)sizeof(T));
    const int G = j->tile;
    unsigned long long* full = (unsigned long long*)g_dyn_smem;
    T* stage = (T*)(g_dyn_smem + 128);
    const long long stage_elems = (long long)G * E;
    if (tid == 0) {
        for (int q = 0; q < S; q++) mbar_init(&full[q], 1);
        fence_mbar_init();
        s_stage_abort = 0;
    }
    const long long my = (long long)tid * V;
    const int nv = my < ne ? (int)min((long long)V, ne - my) : 0;
    T acc[V];
#pragma unroll
    for (int q = 0; q < V; q++) acc[q] = T();
    unsigned gi = 0;  // groups issued/consumed so far (stage = gi % S, phase parity = (gi / S) & 1)
    bool first = true;
    bool aborted = false;  // only ever read right after a block barrier, so every thread agrees
    for (int r0 = 0; r0 < n && !aborted; r0 += PTILE) {
        const int m = min(PTILE, n - r0);
        load_ptile(slots, r0, m, 0, tid, nt);  // two block barriers; previous stages all consumed
        const int ng = (m + G - 1) / G;
        if (tid == 0) {
            for (int g = 0; g < S && g < ng; g++) {
                const unsigned sidx = (gi + g) % S;
                const int k0 = g * G, mm = min(G, m - k0);
                stage_issue<T>(&full[sidx], stage + (long long)sidx * stage_elems, E, k0, mm, e0, CB);
            }
        }
        for (int g = 0; g < ng; g++, gi++) {
            const unsigned sidx = gi % S;
            const unsigned par = (gi / S) & 1u;
            if (!mbar_wait_bounded(&full[sidx], par)) {
                s_stage_abort = 1;
                if (tid == 0) record_error(GPUMPI_ERR_OTHER, GPUMPI_ERR_TIMEOUT, __LINE__, idx);
            }
            bar_sync(BAR_TASK, nt);  // (a) everyone waited; abort flag visible
            aborted = s_stage_abort != 0;
            if (aborted) {
                // groups g .. min(ng, g + S) - 1 of this tile have been issued and not consumed
                if (tid == 0) drain_stages<S>(full, gi, min(ng, g + S) - g, idx);
                break;
            }
            const int mm = min(G, m - g * G);
            const T* st = stage + (long long)sidx * stage_elems + my;
            if (nv > 0) {
                int k = 0;
                if (first) {
                    for (int q = 0; q < nv; q++) acc[q] = st[q];
                    k = 1;
                }
                if (nv == V) {
                    for (; k < mm; k++) {
                        const T* p = st + (long long)k * E;
#pragma unroll
                        for (int q = 0; q < V; q++) acc[q] = op_apply<OP, T>(p[q], acc[q]);
                    }
                } else {
                    for (; k < mm; k++) {
                        const T* p = st + (long long)k * E;
                        for (int q = 0; q < nv; q++) acc[q] = op_apply<OP, T>(p[q], acc[q]);
                    }
                }
            }
            first = false;
            bar_sync(BAR_TASK, nt);  // (b) stage consumed by every thread
            if (tid == 0 && g + S < ng) {
                const int gg = g + S, k0 = gg * G, m2 = min(G, m - k0);
                stage_issue<T>(&full[sidx], stage + (long long)sidx * stage_elems, E, k0, m2, e0, CB);
            }
        }
    }
    if (aborted) return;
    // every issued copy was waited for: retire the barriers (the next chunk initialises them again)
    if (tid == 0)
        for (int q = 0; q < S; q++) mbar_inval(&full[q]);
    if (j->kind == JOB_REDUCE) {
        if (nv > 0) {
            T* out = (T*)slot_out(&slots[j->root]) + e0 + my;
            for (int q = 0; q < nv; q++) __stcg(out + q, acc[q]);
        }
        return;
    }
    const long long e = e0 + my;
    for (int r0 = 0; r0 < n; r0 += PTILE) {
        const int m = min(PTILE, n - r0);
        load_ptile(slots, r0, m, 1, tid, nt);
        if (nv > 0)
            for (int i = 0; i < m; i++) st_elems<T, V>((T*)s_chunk.f.ptile[i] + e, acc, nv, true);
    }
}

}  // namespace gpumpi
