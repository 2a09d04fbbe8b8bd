// rt_select.cuh — per-call algorithm selection and the timing trace that feeds it.
//
// No counterpart in the reference (it has one algorithm per collective).  The last member to arrive at
// a collective picks the variant: an explicit override, else the tuned table (autotuner output), else
// the learned selector, else DIRECT.  Every timed call can append one record to a device ring buffer;
// the autotuner and the selector's training set are built from these records.
#pragma once
#include "rt_core.cuh"

namespace gpumpi {

__device__ __forceinline__ int clamp_i(int v, int lo, int hi) { return v < lo ? lo : v > hi ? hi : v; }
__device__ __forceinline__ int ilog2_ll(long long v) { return v <= 1 ? 0 : 63 - __clzll(v); }

// tuned table layout: [kind 0..2][datatype class 0..2][alignment class 0..1][log2 bytes-per-rank 0..31]
// [log2 ranks 0..15] -> variant.  Datatype class 0 = float, 1 = double / long double, 2 = every other type
// (integers, bytes, pairs, user types): the fold order's cost depends on the element (at 1024 ranks, 16-byte
// aligned, ~1.2 MiB per rank: fp64 DIRECT 962 us, RING 602; fp32 at 1 MiB DIRECT 368, RING 403), and a
// cell that pooled the types let one type's winner decide for the others.  Alignment class 0 when every
// member's buffers are 16-byte aligned (aligned16 >= 16), else 1; the alignment changes the winner too
// (fp32, 1024 ranks: 1 MiB 16-byte aligned DIRECT 366 us, RING 401; 1.41 MiB 8-byte aligned DIRECT 766,
// RING 721), and only the setup knows it: it ORs every member's buffer addresses.
constexpr int SEL_KINDS = 3, SEL_DCLASSES = 3, SEL_CLASSES = 2, SEL_BYTES = 32, SEL_RANKS = 16;

__device__ __forceinline__ int sel_dclass(int dt) {
    return dt == GPUMPI_FLOAT ? 0 : (dt == GPUMPI_DOUBLE || dt == GPUMPI_LONG_DOUBLE) ? 1 : 2;
}

__device__ __forceinline__ int tuned_cell(int kind, long long bytes_per_rank, int n, int aligned16, int dt) {
    const int k = kind == JOB_ALLREDUCE ? 0 : kind == JOB_REDUCE ? 1 : kind == JOB_ALLTOALLV ? 2 : -1;
    if (k < 0 || !c_rt.tuned_table) return -1;
    const int cls = aligned16 >= 16 ? 0 : 1;
    const int b = clamp_i(ilog2_ll(bytes_per_rank), 0, SEL_BYTES - 1);
    const int r = clamp_i(ilog2_ll(n), 0, SEL_RANKS - 1);
    const int v = c_rt.tuned_table[(((k * SEL_DCLASSES + sel_dclass(dt)) * SEL_CLASSES + cls) * SEL_BYTES + b) *
                                       SEL_RANKS + r];
    return v >= 0 && v < GPUMPI_NUM_VARIANTS ? v : -1;
}

// The setup's choice.  override_v: an explicit variant, or the learned policy's network choice (then
// `pred` holds the network's predicted log-times and the tuned table, now that the alignment is known,
// is the fallback: its choice stands unless the network predicts at least the margin lower time).
__device__ int select_variant(int kind, long long bytes_per_rank, int n, int dt, int op, int override_v,
                              int aligned16, const float* pred) {
    if (override_v >= 0 && override_v < GPUMPI_NUM_VARIANTS) {
        if (pred) {
            const int tv = tuned_cell(kind, bytes_per_rank, n, aligned16, dt);
            const float margin = kind == JOB_ALLTOALLV ? c_rt.mlp_margin_pull : c_rt.mlp_margin;
            if (tv >= 0 && pred[tv] <= pred[override_v] + margin) return tv;
        }
        return override_v;
    }
    if (c_rt.selector_mode == 1) {
        const int tv = tuned_cell(kind, bytes_per_rank, n, aligned16, dt);
        if (tv >= 0) return tv;
    }
    // Heuristic default for small folds whose result does not depend on the order (integers with an
    // associative operator): RING starts chunk k at member k + 1, so the one or two chunks of a small fold
    // do not all read member 0 first.  Measured at 1 KiB int32 SUM per rank (p50 of 10 calls): 15.8 vs
    // 17.8 us at 32 ranks, 20.7 vs 21.9 at 128, 38.1 vs 40.4 at 512, 55.6 vs 57.0 at 1024.  Floating point
    // keeps the canonical order.
    if (c_rt.selector_mode == 3 && (kind == JOB_ALLREDUCE || kind == JOB_REDUCE) && bytes_per_rank <= 4096 &&
        (op == GPUMPI_OP_SUM || op == GPUMPI_OP_MAX || op == GPUMPI_OP_MIN || op == GPUMPI_OP_PROD ||
         op == GPUMPI_OP_BAND || op == GPUMPI_OP_BOR || op == GPUMPI_OP_BXOR) &&
        (dt == GPUMPI_INT || dt == GPUMPI_INT32_T || dt == GPUMPI_UNSIGNED || dt == GPUMPI_UINT32_T ||
         dt == GPUMPI_LONG || dt == GPUMPI_LONG_LONG_INT || dt == GPUMPI_LONG_LONG || dt == GPUMPI_INT64_T ||
         dt == GPUMPI_UNSIGNED_LONG || dt == GPUMPI_UNSIGNED_LONG_LONG || dt == GPUMPI_UINT64_T))
        return GPUMPI_VARIANT_RING;
    return GPUMPI_VARIANT_DIRECT;
}

__device__ __forceinline__ void trace_record(const MPI_Comm_impl* c, int kind, int variant, int dt, int op,
                                             long long bytes, unsigned long long ns) {
    if (!c_rt.trace || !c_rt.trace_count) return;
    unsigned long long i = atomicAdd(c_rt.trace_count, 1ULL);
    if (i >= (unsigned long long)c_rt.trace_cap) return;
    TraceRec* r = &c_rt.trace[i];
    r->log2_bytes = bytes > 0 ? log2f((float)bytes) : 0.f;
    r->log2_ranks = log2f((float)c->size);
    r->kind = kind;
    r->variant = variant;
    r->dt = dt;
    r->op = op;
    r->us = (float)ns * 1e-3f;
    r->aligned = c->job.aligned16;
}

}  // namespace gpumpi
