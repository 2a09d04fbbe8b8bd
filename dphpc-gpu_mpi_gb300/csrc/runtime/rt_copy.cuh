// rt_copy.cuh — contiguous copy engine used by point-to-point and collective pulls.
//
// Replaces the reference's single-thread byte memcpy (gpu_libs/gpu_libc/cuda_mpi.cu:168,323 and the
// __gpu_memcpy byte loop of gpu_libs/gpu_libc/string.cu:185-192): nl cooperating threads move the
// message with 16-byte vector accesses (8/4/1-byte when the two addresses disagree modulo 16),
// eight independent loads in flight per thread (four left 256 KiB and 1 MiB messages at 1024 ranks 10%
// slower), L2-only loads (ld.global.cg) for global buffers so a
// block never reads a stale L1 line written by another SM (generic accesses for thread-local and
// shared buffers, where the .global forms would be illegal).
#pragma once
#include "rt_core.cuh"

namespace gpumpi {

// CG: both addresses are global, so L2-only accesses (ld/st.global.cg) are legal; otherwise
// (thread-local or shared buffers) plain generic accesses are used.
template <class V, bool CG>
__device__ __forceinline__ V ldv(const V* p) {
    if constexpr (CG) return __ldcg(p);
    else return *p;
}
template <class V, bool CG>
__device__ __forceinline__ void stv(V* p, V v) {
    if constexpr (CG) __stcg(p, v);
    else *p = v;
}

template <class V, bool CG>
__device__ __forceinline__ void copy_vec_body(V* d, const V* s, long long nv, int lane, int nl) {
    constexpr int K = 8;
    long long i = lane;
    for (; i + (K - 1LL) * nl < nv; i += (long long)K * nl) {
        V a[K];
#pragma unroll
        for (int k = 0; k < K; k++) a[k] = ldv<V, CG>(s + i + (long long)k * nl);
#pragma unroll
        for (int k = 0; k < K; k++) stv<V, CG>(d + i + (long long)k * nl, a[k]);
    }
    for (; i < nv; i += nl) stv<V, CG>(d + i, ldv<V, CG>(s + i));
}

__device__ __forceinline__ void copy_bytes_slow(char* d, const char* s, long long n, int lane, int nl) {
    for (long long i = lane; i < n; i += nl) d[i] = s[i];
}

// Cooperative contiguous copy of n bytes; works for global and (same-block) shared addresses.
// Inlined into the block-task loop (an out-of-line call there costs its register saves and restores
// in every helper thread, about as much as a 1 KiB copy); copy_bytes is the out-of-line form.
__device__ __forceinline__ void copy_bytes_inl(void* dst, const void* src, long long n, int lane, int nl) {
    if (n <= 0) return;
    char* d = (char*)dst;
    const char* s = (const char*)src;
    size_t mis = ((size_t)d ^ (size_t)s);
    int w = (mis & 15) == 0 ? 16 : (mis & 7) == 0 ? 8 : (mis & 3) == 0 ? 4 : 1;
    if (w == 1) {
        copy_bytes_slow(d, s, n, lane, nl);
        return;
    }
    // (short copies take the same path: the byte loop's loads cannot move above its possibly aliasing
    // stores, so a 16-byte eager payload would cost 16 dependent memory round trips instead of one)
    long long head = (long long)((w - ((size_t)s & (w - 1))) & (w - 1));
    if (head > n) head = n;
    long long body = (n - head) & ~(long long)(w - 1);
    long long tail = n - head - body;
    for (long long i = lane; i < head; i += nl) d[i] = s[i];
    const bool cg = is_global_ptr(d) && is_global_ptr(s);
    if (cg) {
        if (w == 16) copy_vec_body<uint4, true>((uint4*)(d + head), (const uint4*)(s + head), body / 16, lane, nl);
        else if (w == 8) copy_vec_body<unsigned long long, true>((unsigned long long*)(d + head), (const unsigned long long*)(s + head), body / 8, lane, nl);
        else copy_vec_body<unsigned, true>((unsigned*)(d + head), (const unsigned*)(s + head), body / 4, lane, nl);
    } else {
        if (w == 16) copy_vec_body<uint4, false>((uint4*)(d + head), (const uint4*)(s + head), body / 16, lane, nl);
        else if (w == 8) copy_vec_body<unsigned long long, false>((unsigned long long*)(d + head), (const unsigned long long*)(s + head), body / 8, lane, nl);
        else copy_vec_body<unsigned, false>((unsigned*)(d + head), (const unsigned*)(s + head), body / 4, lane, nl);
    }
    for (long long i = lane; i < tail; i += nl) d[head + body + i] = s[head + body + i];
}

__device__ __noinline__ void copy_bytes(void* dst, const void* src, long long n, int lane, int nl) {
    copy_bytes_inl(dst, src, n, lane, nl);
}

}  // namespace gpumpi
