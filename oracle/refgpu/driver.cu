// driver.cu — times the REFERENCE gpu_mpi runtime (lilyyangyn/dphpc-gpu_mpi, unmodified, built from its
// own sources) on the GPU: its own MPI_Allreduce (gpu_libs/gpu_mpi/mpi.cu:276-282) and MPI_Alltoallv
// (mpi.cu:363-408) called by every rank of one launch, set up the way the reference's TestRunner does
// (tests/test_runner.cuh:26-86: SharedState holder, ThreadPrivateState context, one thread per block).
//
// COMPARATOR / TEST INFRASTRUCTURE ONLY: built by oracle/refgpu.py into oracle/_ref/, run as a separate
// process by bench.py's reference-runtime leg.  Nothing in the product links or runs it.
//
// Conditions the host enforces before launching, each taken from reading the reference's code:
//  * every count >= 1: a zero-byte MPI_Isend/MPI_Irecv trips a device assert (mpi.cu:548-549,564-565);
//  * ranks * bytes per rank < 2^31: the Reduce root allocates `dataSize * commSize` as an int
//    (mpi.cu:201-202), and the allocation is not checked;
//  * the device heap holds that buffer with room to spare (cudaLimitMallocHeapSize);
//  * pendingBufferSize >= 2 * ranks + 16 and recvListSize >= ranks + 16: a full pending-operation ring
//    spins forever (cuda_mpi.cu:67-71), a full receive list retries only while others progress;
//  * a cooperative launch: the grid barrier needs every block co-resident (main.cu:188-208 checks this
//    by hand); a grid that does not fit is refused by the launch instead of deadlocking.
//
// Usage:
//   ref_gpumpi_bench allreduce RANKS COUNT ITERS SEED OUT      fp32 SUM; inputs fill_f32(SEED, RANKS*COUNT)
//   ref_gpumpi_bench alltoallv RANKS COUNTS_FILE ITERS SEED OUT  int32; counts [RANKS][RANKS] int32 binary,
//                                                                 inputs fill_i32(SEED, RANKS*S)
// Prints one JSON line; OUT receives rank 0's Allreduce result (fp32) or, for Alltoallv, one uint64
// checksum per receiving rank: sum over its received elements e_k of (uint32)e_k * (k + 1), mod 2^64.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "cuda_mpi.cuh"
#include "mpi.h.cuh"

extern "C" {
void orc_fill_f32(uint64_t seed, int64_t n, float* out);
void orc_fill_i32(uint64_t seed, int64_t n, int32_t* out);
}

namespace CudaMPI {
void initError();
void printLastError();
}  // namespace CudaMPI

struct BenchArgs {
    int kind;  // 0 Allreduce fp32 SUM, 1 Alltoallv int32
    int count;
    int iters;
    const char* send;
    char* recv;
    long long sstride, rstride;  // bytes per rank
    const int *sc, *sd, *rc, *rd;
    unsigned long long* t_ns;
};

__device__ __forceinline__ unsigned long long gtimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__global__ void ref_bench_kernel(CudaMPI::SharedState* shared, CudaMPI::ThreadPrivateState::Context tctx,
                                 BenchArgs a) {
    CudaMPI::setSharedState(shared);
    CudaMPI::ThreadPrivateState::Holder holder(tctx);
    MPI_Init(nullptr, nullptr);
    int rank = -1, n = 0;
    MPI_Comm_rank(MPI_COMM_WORLD, &rank);
    MPI_Comm_size(MPI_COMM_WORLD, &n);
    for (int it = 0; it < a.iters; it++) {
        MPI_Barrier(MPI_COMM_WORLD);
        const unsigned long long t0 = gtimer();
        if (a.kind == 0) {
            MPI_Allreduce(a.send + rank * a.sstride, a.recv + rank * a.rstride, a.count, MPI_FLOAT, MPI_SUM,
                          MPI_COMM_WORLD);
        } else {
            MPI_Alltoallv(a.send + rank * a.sstride, a.sc + (long long)rank * n, a.sd + (long long)rank * n, MPI_INT,
                          a.recv + rank * a.rstride, a.rc + (long long)rank * n, a.rd + (long long)rank * n, MPI_INT,
                          MPI_COMM_WORLD);
        }
        MPI_Barrier(MPI_COMM_WORLD);
        const unsigned long long t1 = gtimer();
        if (rank == 0) a.t_ns[it] = t1 - t0;
    }
    MPI_Finalize();
}

static void fail(const char* what, const char* detail) {
    printf("{\"error\": \"%s: %s\"}\n", what, detail);
    fflush(stdout);
    std::exit(2);
}
#define CK(x)                                                          \
    do {                                                               \
        cudaError_t e_ = (x);                                          \
        if (e_ != cudaSuccess) fail(#x, cudaGetErrorString(e_));       \
    } while (0)

int main(int argc, char** argv) {
    if (argc < 7) fail("usage", "allreduce|alltoallv RANKS COUNT|COUNTS_FILE ITERS SEED OUT [LIMIT_S]");
    const bool ar = std::strcmp(argv[1], "allreduce") == 0;
    const int n = std::atoi(argv[2]);
    const int iters = std::atoi(argv[4]);
    const unsigned long long seed = std::strtoull(argv[5], nullptr, 10);
    const char* out_path = argv[6];
    const double limit_s = argc > 7 ? std::atof(argv[7]) : 300.0;
    if (n < 2 || iters < 1) fail("arguments", "RANKS >= 2 and ITERS >= 1 required");

    // inputs
    long long send_elems = 0, recv_elems = 0, moved_bytes = 0;
    int count = 0;
    std::vector<int> sc, sd, rc, rd;
    if (ar) {
        count = std::atoi(argv[3]);
        if (count < 1) fail("arguments", "COUNT >= 1 required (zero-byte messages assert in the reference)");
        if ((long long)n * count * 4 >= (1LL << 31)) fail("arguments", "RANKS * bytes >= 2^31 overflows the reference");
        send_elems = recv_elems = count;
        moved_bytes = 2LL * n * count * 4;
    } else {
        sc.resize((size_t)n * n);
        FILE* f = std::fopen(argv[3], "rb");
        if (!f || std::fread(sc.data(), 4, sc.size(), f) != sc.size()) fail("counts file", argv[3]);
        std::fclose(f);
        rc.resize(sc.size());
        sd.resize(sc.size());
        rd.resize(sc.size());
        long long total = 0;
        for (int r = 0; r < n; r++)
            for (int s = 0; s < n; s++) {
                const int c = sc[(size_t)r * n + s];
                if (c < 1) fail("counts", "every count must be >= 1 (zero-byte messages assert in the reference)");
                rc[(size_t)s * n + r] = c;
                total += c;
            }
        for (int r = 0; r < n; r++) {
            long long so = 0, ro = 0;
            for (int s = 0; s < n; s++) {
                sd[(size_t)r * n + s] = (int)so;
                rd[(size_t)r * n + s] = (int)ro;
                so += sc[(size_t)r * n + s];
                ro += rc[(size_t)r * n + s];
            }
            send_elems = std::max(send_elems, so);
            recv_elems = std::max(recv_elems, ro);
        }
        moved_bytes = 2 * total * 4;
    }
    const long long sbytes = send_elems * 4, rbytes = recv_elems * 4;
    std::vector<char> h_send((size_t)(n * sbytes));
    if (ar) orc_fill_f32(seed, (int64_t)n * send_elems, (float*)h_send.data());
    else orc_fill_i32(seed, (int64_t)n * send_elems, (int32_t*)h_send.data());

    // runtime limits before any kernel: the Reduce root's n * bytes buffer, pending rings, groups
    const size_t heap = (size_t)(ar ? (long long)n * count * 4 : 0) * 2 + ((size_t)1 << 30);
    CK(cudaDeviceSetLimit(cudaLimitMallocHeapSize, heap));
    CK(cudaDeviceSetLimit(cudaLimitStackSize, 8192));
    CudaMPI::initError();

    int dev = 0, sms = 0, bps = 0, clock_khz = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CK(cudaDeviceGetAttribute(&clock_khz, cudaDevAttrClockRate, dev));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, ref_bench_kernel, 1, 0));
    if ((long long)bps * sms < n) fail("co-residency", "the grid does not fit on the GPU at once");

    char *d_send = nullptr, *d_recv = nullptr;
    int* d_cnt = nullptr;
    unsigned long long* d_t = nullptr;
    CK(cudaMalloc(&d_send, (size_t)(n * sbytes)));
    CK(cudaMalloc(&d_recv, (size_t)(n * rbytes)));
    CK(cudaMalloc(&d_t, sizeof(unsigned long long) * iters));
    CK(cudaMemcpy(d_send, h_send.data(), (size_t)(n * sbytes), cudaMemcpyHostToDevice));
    CK(cudaMemset(d_recv, 0, (size_t)(n * rbytes)));
    BenchArgs a{};
    a.kind = ar ? 0 : 1;
    a.count = count;
    a.iters = iters;
    a.send = d_send;
    a.recv = d_recv;
    a.sstride = sbytes;
    a.rstride = rbytes;
    a.t_ns = d_t;
    if (!ar) {
        const size_t mb = sizeof(int) * (size_t)n * n;
        CK(cudaMalloc(&d_cnt, 4 * mb));
        CK(cudaMemcpy(d_cnt, sc.data(), mb, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(d_cnt + (size_t)n * n, sd.data(), mb, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(d_cnt + 2 * (size_t)n * n, rc.data(), mb, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(d_cnt + 3 * (size_t)n * n, rd.data(), mb, cudaMemcpyHostToDevice));
        a.sc = d_cnt;
        a.sd = d_cnt + (size_t)n * n;
        a.rc = d_cnt + 2 * (size_t)n * n;
        a.rd = d_cnt + 3 * (size_t)n * n;
    }

    // the reference's runtime state, as its TestRunner sets it up, with queues sized for n ranks
    CudaMPI::SharedState::Context sctx;
    sctx.numThreads = n;
    sctx.recvListSize = n + 16;
    CudaMPI::SharedState::Holder holder(sctx);
    CudaMPI::SharedState* shared = holder.get();
    CudaMPI::ThreadPrivateState::Context tctx;
    tctx.pendingBufferSize = 2 * n + 16;
    tctx.peakClockKHz = clock_khz;

    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    void* params[] = {(void*)&shared, (void*)&tctx, (void*)&a};
    CK(cudaEventRecord(e0));
    CK(cudaLaunchCooperativeKernel((const void*)ref_bench_kernel, dim3(n), dim3(1), params, 0, nullptr));
    CK(cudaEventRecord(e1));
    const auto t_start = std::chrono::steady_clock::now();
    for (;;) {
        const cudaError_t q = cudaEventQuery(e1);
        if (q == cudaSuccess) break;
        if (q != cudaErrorNotReady) fail("kernel", cudaGetErrorString(q));
        const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
        if (el > limit_s) {
            printf("{\"error\": \"still running after %.0f s: stopped by the host\"}\n", el);
            fflush(stdout);
            std::_Exit(3);
        }
        std::this_thread::sleep_for(std::chrono::milliseconds(2));
    }
    float kernel_ms = 0;
    CK(cudaEventElapsedTime(&kernel_ms, e0, e1));
    std::vector<unsigned long long> t(iters);
    CK(cudaMemcpy(t.data(), d_t, sizeof(unsigned long long) * iters, cudaMemcpyDeviceToHost));
    std::vector<char> h_recv((size_t)(n * rbytes));
    CK(cudaMemcpy(h_recv.data(), d_recv, h_recv.size(), cudaMemcpyDeviceToHost));

    bool rows_identical = true;
    FILE* fo = std::fopen(out_path, "wb");
    if (!fo) fail("output file", out_path);
    if (ar) {
        for (int r = 1; r < n && rows_identical; r++)
            rows_identical = std::memcmp(h_recv.data(), h_recv.data() + (size_t)r * rbytes, (size_t)rbytes) == 0;
        std::fwrite(h_recv.data(), 1, (size_t)rbytes, fo);
    } else {
        std::vector<unsigned long long> sums(n, 0);
        for (int r = 0; r < n; r++) {
            const unsigned* e = (const unsigned*)(h_recv.data() + (size_t)r * rbytes);
            unsigned long long s = 0;
            for (long long k = 0; k < recv_elems; k++) s += (unsigned long long)e[k] * (unsigned long long)(k + 1);
            sums[r] = s;
        }
        std::fwrite(sums.data(), 8, sums.size(), fo);
    }
    std::fclose(fo);
    printf("{\"kind\": \"%s\", \"ranks\": %d, \"iters\": %d, \"moved_bytes_per_call\": %lld, \"kernel_ms\": %.3f, "
           "\"rows_identical\": %s, \"blocks_per_sm\": %d, \"heap_bytes\": %zu, \"t_ns\": [",
           ar ? "allreduce" : "alltoallv", n, iters, moved_bytes, kernel_ms, rows_identical ? "true" : "false", bps,
           heap);
    for (int i = 0; i < iters; i++) printf("%s%llu", i ? ", " : "", t[i]);
    printf("]}\n");
    fflush(stdout);
    return 0;
}
