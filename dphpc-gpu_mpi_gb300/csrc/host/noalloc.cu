// noalloc.cu — MPI_Allreduce among block-ranks without any allocation by the library.
//
// Some callers of this library cannot allocate device memory at the moment they need a reduction:
// code inside an allocator, a scheduler or a memory-pool callback that must not re-enter the allocator,
// processes that reserve every device byte up front and may not grow past that budget, and loops that
// cannot afford cudaMalloc's implicit device-wide synchronisation.  gpumpi_allreduce needs a world
// (cudaMalloc'd runtime state, device-heap staging); this entry point needs nothing but the caller's
// device buffers.
//
// Its scratch memory — the table where every rank publishes its buffer addresses, the grid-barrier
// words and the chunk counter — lives in the file-scope array below, of a fixed maximum size that every
// GPU loading the library keeps until the process exits.  Consequences for callers:
//   * at most GPUMPI_NOALLOC_MAX_RANKS ranks; larger requests are rejected with GPUMPI_ERR_ARG;
//   * every call shares the one array: calls whose kernels overlap on the GPU (different streams,
//     different threads) race and produce wrong results — serialise them;
//   * the first call on a device looks up the array's device address (cudaGetSymbolAddress) with that
//     device current; make that first call before any stream capture begins;
//   * buffers must be device memory of the current device (staging host buffers would allocate);
//   * the grid barrier inside the kernel is bounded: if it runs out, the kernel writes nothing, records
//     the failure in the array's error word and returns; gpumpi_allreduce_noalloc_status reports it
//     once the caller has synchronised the call's stream.
// The reduction is the same canonical rank-order fold as the runtime's DIRECT variant, so results are
// bit-identical to gpumpi_allreduce.
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdio>
#include <mutex>

#include "gpumpi.h"
#include "../runtime/rt_core.cuh"
#include "../runtime/rt_ops.cuh"

namespace {

constexpr int NOALLOC_MAX_RANKS = GPUMPI_NOALLOC_MAX_RANKS;
constexpr int NOALLOC_PTILE = 256;

struct NoallocHeader {
    unsigned arrive;           // grid barrier arrivals
    unsigned gen;              // grid barrier generation
    unsigned long long next;   // next chunk to claim
    unsigned error;            // non-zero: a bounded wait ran out
    unsigned pad[27];
};
struct NoallocTable {
    NoallocHeader h;
    const void* send[NOALLOC_MAX_RANKS];
    void* recv[NOALLOC_MAX_RANKS];
};
static_assert(sizeof(NoallocTable) <= GPUMPI_NOALLOC_SCRATCH_BYTES, "scratch too small");

// The scratch: rank rendezvous table, barrier and chunk counter of the allocation-free allreduce.
static __device__ __align__(256) unsigned char g_noalloc_scratch[GPUMPI_NOALLOC_SCRATCH_BYTES];

__device__ __forceinline__ unsigned ld_acq(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_rel(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long gtime() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

struct NoallocArgs {
    NoallocTable* t;            // device address of g_noalloc_scratch
    const char* send;           // rank-major buffers
    char* recv;
    long long stride;           // bytes per rank
    long long count;            // elements per rank
    int nranks;
    int missing;                // arrivals the barrier waits for beyond the launched blocks (test hook)
    int aligned;                // 16 / 8 / 0: alignment of every rank's buffers
    unsigned long long timeout_ns;
};

template <class T, int OP, int V>
__device__ __forceinline__ void noalloc_fold(const NoallocArgs& a, long long e0, int tid, int nt,
                                             unsigned long long* tile) {
    constexpr int BYTES = V * (int)sizeof(T);
    constexpr int U = 128 / BYTES > 16 ? 16 : 128 / BYTES < 1 ? 1 : 128 / BYTES;
    const int n = a.nranks;
    const long long e = e0 + (long long)tid * V;
    const int nv = e < a.count ? (int)min((long long)V, a.count - e) : 0;
    const bool vec = (BYTES == 16 && a.aligned >= 16) || (BYTES == 8 && a.aligned >= 8);
    T acc[V];
#pragma unroll
    for (int q = 0; q < V; q++) acc[q] = T();
    for (int r0 = 0; r0 < n; r0 += NOALLOC_PTILE) {
        const int m = min(NOALLOC_PTILE, n - r0);
        __syncthreads();
        for (int i = tid; i < m; i += nt) tile[i] = __ldcg((const unsigned long long*)&a.t->send[r0 + i]);
        __syncthreads();
        if (nv == 0) continue;
        int i = 0;
        auto load = [&](int k, T (&v)[V]) {
            const T* p = (const T*)tile[k] + e;
            if constexpr (BYTES == 16) {
                if (vec && nv == V) { *reinterpret_cast<uint4*>(v) = __ldcg((const uint4*)p); return; }
            } else if constexpr (BYTES == 8 && sizeof(T) < 8) {
                if (vec && nv == V) { *reinterpret_cast<unsigned long long*>(v) = __ldcg((const unsigned long long*)p); return; }
            }
#pragma unroll
            for (int q = 0; q < V; q++)
                if (q < nv) v[q] = __ldcg(p + q);
        };
        if (r0 == 0) {
            load(0, acc);
            i = 1;
        }
        for (; i + U <= m; i += U) {
            T v[U][V];
#pragma unroll
            for (int u = 0; u < U; u++) load(i + u, v[u]);
#pragma unroll
            for (int u = 0; u < U; u++)
#pragma unroll
                for (int q = 0; q < V; q++) acc[q] = gpumpi::op_apply<OP, T>(v[u][q], acc[q]);
        }
        for (; i < m; i++) {
            T v[V];
            load(i, v);
#pragma unroll
            for (int q = 0; q < V; q++) acc[q] = gpumpi::op_apply<OP, T>(v[q], acc[q]);
        }
    }
    for (int r0 = 0; r0 < n; r0 += NOALLOC_PTILE) {
        const int m = min(NOALLOC_PTILE, n - r0);
        __syncthreads();
        for (int i = tid; i < m; i += nt) tile[i] = __ldcg((const unsigned long long*)&a.t->recv[r0 + i]);
        __syncthreads();
        if (nv == 0) continue;
        for (int i = 0; i < m; i++) {
            T* p = (T*)tile[i] + e;
            if constexpr (BYTES == 16) {
                if (vec && nv == V) { __stcg((uint4*)p, *reinterpret_cast<const uint4*>(acc)); continue; }
            } else if constexpr (BYTES == 8 && sizeof(T) < 8) {
                if (vec && nv == V) { __stcg((unsigned long long*)p, *reinterpret_cast<const unsigned long long*>(acc)); continue; }
            }
#pragma unroll
            for (int q = 0; q < V; q++)
                if (q < nv) __stcg(p + q, acc[q]);
        }
    }
}

// Block b < nranks is rank b: it publishes its buffers in the scratch table; after a grid barrier
// every block (ranks and the extra blocks that fill the GPU) claims chunks of elements with one
// atomic each and folds them over all ranks in rank order.
template <class T, int OP, int V>
__global__ void __launch_bounds__(256) noalloc_allreduce_kernel(NoallocArgs a) {
    __shared__ unsigned long long tile[NOALLOC_PTILE];
    __shared__ long long s_idx;
    __shared__ int s_fail;
    const int tid = (int)threadIdx.x, nt = (int)blockDim.x;
    NoallocTable* t = a.t;
    if (tid == 0) {
        s_fail = 0;
        if ((int)blockIdx.x < a.nranks) {
            t->send[blockIdx.x] = a.send + (long long)blockIdx.x * a.stride;
            t->recv[blockIdx.x] = a.recv + (long long)blockIdx.x * a.stride;
        }
        // grid barrier (all blocks co-resident: cooperative launch), bounded by the timeout
        const unsigned g = ld_acq(&t->h.gen);
        __threadfence();
        const unsigned arrived = atomicAdd(&t->h.arrive, 1u);
        if (arrived + 1u == gridDim.x + (unsigned)a.missing) {
            t->h.arrive = 0;
            st_rel(&t->h.gen, g + 1);
        } else {
            const unsigned long long end = gtime() + a.timeout_ns;
            unsigned ns = 32;
            while (ld_acq(&t->h.gen) == g) {
                if (gtime() > end) {
                    atomicExch(&t->h.error, 1u);
                    s_fail = 1;
                    break;
                }
                __nanosleep(ns);
                ns = ns < 512 ? ns * 2 : ns;
            }
        }
    }
    __syncthreads();
    if (s_fail) return;
    const long long chunk = (long long)nt * V;
    const long long nchunks = (a.count + chunk - 1) / chunk;
    for (;;) {
        if (tid == 0) s_idx = (long long)atomicAdd(&t->h.next, 1ULL);
        __syncthreads();
        const long long idx = s_idx;
        if (idx >= nchunks) break;
        noalloc_fold<T, OP, V>(a, idx * chunk, tid, nt, tile);
        __syncthreads();
    }
}

template <class T, int OP>
const void* pick_kernel(int v) {
    if (v >= (int)(16 / sizeof(T))) return (const void*)noalloc_allreduce_kernel<T, OP, 16 / sizeof(T)>;
    if constexpr (sizeof(T) == 4) {
        if (v >= 2) return (const void*)noalloc_allreduce_kernel<T, OP, 2>;
    }
    return (const void*)noalloc_allreduce_kernel<T, OP, 1>;
}

template <class T>
const void* pick_op(int op, int v, bool is_int) {
    switch (op) {
    case GPUMPI_OP_SUM: return pick_kernel<T, GPUMPI_OP_SUM>(v);
    case GPUMPI_OP_MAX: return pick_kernel<T, GPUMPI_OP_MAX>(v);
    case GPUMPI_OP_MIN: return pick_kernel<T, GPUMPI_OP_MIN>(v);
    case GPUMPI_OP_PROD: return pick_kernel<T, GPUMPI_OP_PROD>(v);
    default: (void)is_int; return nullptr;
    }
}

const void* select_kernel(int dt, int op, int v) {
    switch (dt) {
    case GPUMPI_FLOAT: return pick_op<float>(op, v, false);
    case GPUMPI_DOUBLE: case GPUMPI_LONG_DOUBLE: return pick_op<double>(op, v, false);
    case GPUMPI_INT: case GPUMPI_INT32_T: return pick_op<int>(op, v, true);
    case GPUMPI_LONG: case GPUMPI_LONG_LONG_INT: case GPUMPI_LONG_LONG: case GPUMPI_INT64_T:
        return pick_op<long long>(op, v, true);
    default: return nullptr;
    }
}

int elem_size(int dt) {
    switch (dt) {
    case GPUMPI_FLOAT: case GPUMPI_INT: case GPUMPI_INT32_T: return 4;
    case GPUMPI_DOUBLE: case GPUMPI_LONG_DOUBLE: case GPUMPI_LONG: case GPUMPI_LONG_LONG_INT: case GPUMPI_LONG_LONG:
    case GPUMPI_INT64_T: return 8;
    default: return 0;
    }
}

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[64] = {};
// test hook: bounded-wait limit and arrivals the barrier pretends are missing (0 / 0 = defaults)
unsigned long long g_noalloc_timeout_ns = 0;
int g_noalloc_missing = 0;
constexpr unsigned long long NOALLOC_DEFAULT_TIMEOUT_NS = 20ull * 1000000000ull;

}  // namespace

extern "C" int gpumpi_allreduce_noalloc(const void* sendbuf, void* recvbuf, long long count, int datatype, int op,
                                        int nranks, void* stream) {
    if (nranks < 1 || nranks > NOALLOC_MAX_RANKS) {
        fprintf(stderr, "gpumpi_allreduce_noalloc: %d ranks requested, at most %d supported\n", nranks,
                NOALLOC_MAX_RANKS);
        return GPUMPI_ERR_ARG;
    }
    const int es = elem_size(datatype);
    if (count < 0 || !sendbuf || !recvbuf) return GPUMPI_ERR_ARG;
    if (!es || !select_kernel(datatype, op, 1)) {
        fprintf(stderr, "gpumpi_allreduce_noalloc: datatype %d with op %d is not supported\n", datatype, op);
        return GPUMPI_ERR_TYPE;
    }
    if (count == 0) return GPUMPI_SUCCESS;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return GPUMPI_ERR_CUDA;
    // host buffers would need a device staging copy (an allocation); a buffer on another GPU would be
    // read through peer access while the kernel and the scratch live on this one
    for (const void* b : {sendbuf, (const void*)recvbuf}) {
        cudaPointerAttributes pa;
        if (cudaPointerGetAttributes(&pa, b) != cudaSuccess || pa.type != cudaMemoryTypeDevice || pa.device != dev) {
            cudaGetLastError();
            return GPUMPI_ERR_BUFFER;
        }
    }
    void* scratch = nullptr;
    {
        // set-up, once per device, with that device current: the array's device address
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        if (!g_noalloc_ptr[dev]) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
                cudaGetLastError();
                return GPUMPI_ERR_CUDA;
            }
            g_noalloc_ptr[dev] = p;
        }
        scratch = g_noalloc_ptr[dev];
    }
    cudaStream_t s = (cudaStream_t)stream;
    const long long stride = count * es;
    unsigned mis = (unsigned)(((size_t)sendbuf | (size_t)recvbuf | (size_t)stride) & 15u);
    const int aligned = (mis & 15u) == 0 ? 16 : (mis & 7u) == 0 ? 8 : 0;
    // geometry: 256/128/64 threads, as many blocks as stay co-resident; elements per thread by the same
    // busy-blocks x bytes-in-flight score as the runtime's DIRECT variant
    int sm = 0;
    cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev);
    int T = 0, bps = 0;
    const int cands[3] = {256, 128, 64};
    for (int k = 0; k < 3 && !T; k++) {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, select_kernel(datatype, op, 1), cands[k], 0) !=
            cudaSuccess)
            return GPUMPI_ERR_CUDA;
        if ((long long)b * sm >= nranks) {
            T = cands[k];
            bps = b;
        }
    }
    if (!T) return GPUMPI_ERR_LAUNCH;
    const long long blocks = (long long)bps * sm;
    int vbest = 1;
    double sbest = -1, bbest = 0;
    const int vc[3] = {16 / es, es == 4 ? 2 : 1, 1};
    for (int k = 0; k < 3; k++) {
        const int v = vc[k];
        const int need = v * es >= 16 ? 16 : v * es;
        if (v > 1 && aligned < need) continue;
        const long long nch = (count + (long long)T * v - 1) / ((long long)T * v);
        const long long waves = (nch + blocks - 1) / blocks;
        const double busy = (double)nch / (double)waves;
        int u = 128 / (v * es);
        u = u < 1 ? 1 : u > 16 ? 16 : u;
        const double sc = busy * v * es * u;
        if (sc > sbest * 1.05 || (sc >= sbest * 0.95 && (busy > bbest * 1.01 || (busy >= bbest * 0.99 && v > vbest)))) {
            if (sc > sbest) sbest = sc;
            bbest = busy;
            vbest = v;
        }
    }
    const void* kern = select_kernel(datatype, op, vbest);
    {
        // the chosen instantiation must co-host the same grid, else fall back to one element per thread
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, T, 0) != cudaSuccess) return GPUMPI_ERR_CUDA;
        if ((long long)b * sm < blocks) {
            vbest = 1;
            kern = select_kernel(datatype, op, 1);
        }
    }
    // the header (barrier words, chunk counter, error word) must start at zero; the tables are rewritten
    if (cudaMemsetAsync(scratch, 0, sizeof(NoallocHeader), s) != cudaSuccess) return GPUMPI_ERR_CUDA;
    NoallocArgs a;
    a.t = (NoallocTable*)scratch;
    a.send = (const char*)sendbuf;
    a.recv = (char*)recvbuf;
    a.stride = stride;
    a.count = count;
    a.nranks = nranks;
    a.aligned = aligned;
    {
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        a.missing = g_noalloc_missing;
        a.timeout_ns = g_noalloc_timeout_ns ? g_noalloc_timeout_ns : NOALLOC_DEFAULT_TIMEOUT_NS;
    }
    void* args[] = {&a};
    cudaError_t e = cudaLaunchCooperativeKernel(kern, dim3((unsigned)blocks), dim3(T), args, 0, s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return GPUMPI_ERR_LAUNCH;
    }
    return GPUMPI_SUCCESS;
}

extern "C" int gpumpi_allreduce_noalloc_status(void) {
    // the error word of the most recent call on the current device; the caller synchronised its stream
    unsigned err = 0;
    if (cudaMemcpyFromSymbol(&err, g_noalloc_scratch, sizeof(err), offsetof(NoallocHeader, error),
                             cudaMemcpyDeviceToHost) != cudaSuccess) {
        cudaGetLastError();
        return GPUMPI_ERR_CUDA;
    }
    return err ? GPUMPI_ERR_TIMEOUT : GPUMPI_SUCCESS;
}

extern "C" int gpumpi_noalloc_test_hook(double timeout_s, int missing_arrivals) {
    if (timeout_s < 0 || missing_arrivals < 0 || missing_arrivals > NOALLOC_MAX_RANKS) return GPUMPI_ERR_ARG;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    g_noalloc_timeout_ns = (unsigned long long)(timeout_s * 1e9);
    g_noalloc_missing = missing_arrivals;
    return GPUMPI_SUCCESS;
}
