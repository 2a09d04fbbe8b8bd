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

// tuned table layout: [kind 0..1][log2 bytes-per-rank 0..31][log2 ranks 0..15] -> variant
constexpr int SEL_KINDS = 3, SEL_BYTES = 32, SEL_RANKS = 16;

__device__ int mlp_select(int kind, long long bytes, int n, int dt, int op);

__device__ int select_variant(int kind, long long bytes_per_rank, int n, int dt, int op, int override_v) {
    if (override_v >= 0 && override_v < GPUMPI_NUM_VARIANTS) return override_v;
    const int k = kind == JOB_ALLREDUCE ? 0 : kind == JOB_REDUCE ? 1 : kind == JOB_ALLTOALLV ? 2 : -1;
    if (k < 0) return GPUMPI_VARIANT_DIRECT;
    if (c_rt.selector_mode == 1 && c_rt.tuned_table) {
        int b = clamp_i(ilog2_ll(bytes_per_rank), 0, SEL_BYTES - 1);
        int r = clamp_i(ilog2_ll(n), 0, SEL_RANKS - 1);
        int v = c_rt.tuned_table[(k * SEL_BYTES + b) * SEL_RANKS + r];
        if (v >= 0 && v < GPUMPI_NUM_VARIANTS) return v;
    }
    if (c_rt.selector_mode == 2 && c_rt.mlp_params) return mlp_select(kind, bytes_per_rank, n, dt, op);
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
    r->pad = 0;
}

}  // namespace gpumpi
