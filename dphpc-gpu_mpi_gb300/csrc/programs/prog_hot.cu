// prog_hot.cu — device programs for the hot path: one collective (or point-to-point pattern) called
// `iters` times by every rank on its slice of rank-major buffers.  These back the host C-ABI entry
// points gpumpi_allreduce / _alltoallv / ... and the benchmark; rank 0 records each call's duration
// from %globaltimer (entry to completion).
#include "rt_kernel.cuh"

namespace {

__device__ __forceinline__ unsigned long long gtime() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

struct Coll {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        int rank = -1, n = 0;
        MPI_Comm_rank(MPI_COMM_WORLD, &rank);
        MPI_Comm_size(MPI_COMM_WORLD, &n);
        const int kind = (int)p.i[0];
        const long long count = p.i[1];
        const MPI_Datatype dt = (MPI_Datatype)p.i[2];
        const MPI_Op op = gpumpi_predefined_op((int)p.i[3]);
        const int root = (int)p.i[4];
        const int iters = (int)p.i[5];
        char* sb = (char*)p.p[0] + (long long)rank * p.i[6];
        char* rb = (char*)p.p[1] + (long long)rank * p.i[7];
        const int* sc = p.p[2] ? (const int*)p.p[2] + (long long)rank * n : nullptr;
        const int* sd = p.p[3] ? (const int*)p.p[3] + (long long)rank * n : nullptr;
        const int* rc_ = p.p[4] ? (const int*)p.p[4] + (long long)rank * n : nullptr;
        const int* rd = p.p[5] ? (const int*)p.p[5] + (long long)rank * n : nullptr;
        unsigned long long* iter_ns = (unsigned long long*)p.p[6];
        int rc = 0;
        for (int it = 0; it < iters && rc == 0; it++) {
            unsigned long long t0 = gtime();
            switch (kind) {
            case GPUMPI_COLL_ALLREDUCE: rc = MPI_Allreduce(sb, rb, (int)count, dt, op, MPI_COMM_WORLD); break;
            case GPUMPI_COLL_REDUCE: rc = MPI_Reduce(sb, rb, (int)count, dt, op, root, MPI_COMM_WORLD); break;
            case GPUMPI_COLL_BCAST: rc = MPI_Bcast(rb, (int)count, dt, root, MPI_COMM_WORLD); break;
            case GPUMPI_COLL_ALLTOALL: rc = MPI_Alltoall(sb, (int)count, dt, rb, (int)count, dt, MPI_COMM_WORLD); break;
            case GPUMPI_COLL_ALLTOALLV: rc = MPI_Alltoallv(sb, sc, sd, dt, rb, rc_, rd, dt, MPI_COMM_WORLD); break;
            case GPUMPI_COLL_ALLGATHER: rc = MPI_Allgather(sb, (int)count, dt, rb, (int)count, dt, MPI_COMM_WORLD); break;
            case GPUMPI_COLL_GATHER: rc = MPI_Gather(sb, (int)count, dt, rb, (int)count, dt, root, MPI_COMM_WORLD); break;
            case GPUMPI_COLL_SCATTER: rc = MPI_Scatter(sb, (int)count, dt, rb, (int)count, dt, root, MPI_COMM_WORLD); break;
            case GPUMPI_COLL_BARRIER: rc = MPI_Barrier(MPI_COMM_WORLD); break;
            case GPUMPI_COLL_ALLGATHERV: rc = MPI_Allgatherv(sb, (int)count, dt, rb, rc_, rd, dt, MPI_COMM_WORLD); break;
            case GPUMPI_COLL_GATHERV: rc = MPI_Gatherv(sb, (int)count, dt, rb, rc_, rd, dt, root, MPI_COMM_WORLD); break;
            case GPUMPI_COLL_SCATTERV: rc = MPI_Scatterv(sb, sc, sd, dt, rb, (int)count, dt, root, MPI_COMM_WORLD); break;
            default: rc = MPI_ERR_ARG;
            }
            if (rank == 0 && iter_ns) iter_ns[it] = gtime() - t0;
        }
        if (p.p[7]) ((int*)p.p[7])[rank] = rc;
        return rc;
    }
};

// Pairs (2k, 2k+1), k < pairs: ping-pong of `bytes` bytes, `iters` round trips.  The layout of
// benchmarks/mpi_communication/mpi_communication.c:10-55 (even rank sends first).
struct PingPong {
    static __device__ int run(const gpumpi_params& p) {
        int rank = -1;
        MPI_Comm_rank(MPI_COMM_WORLD, &rank);
        const long long bytes = p.i[0];
        const int iters = (int)p.i[1];
        const int nb = (int)p.i[2];
        const int pairs = (int)p.i[3];
        char* buf = (char*)p.p[0] + (long long)rank * p.i[4];
        unsigned long long* iter_ns = (unsigned long long*)p.p[6];
        int rc = 0;
        if (rank / 2 < pairs) {
            int peer = rank ^ 1;
            for (int it = 0; it < iters && rc == 0; it++) {
                unsigned long long t0 = gtime();
                if (!nb) {
                    if ((rank & 1) == 0) {
                        rc = MPI_Send(buf, (int)bytes, MPI_BYTE, peer, 10, MPI_COMM_WORLD);
                        if (!rc) rc = MPI_Recv(buf, (int)bytes, MPI_BYTE, peer, 10, MPI_COMM_WORLD, MPI_STATUS_IGNORE);
                    } else {
                        rc = MPI_Recv(buf, (int)bytes, MPI_BYTE, peer, 10, MPI_COMM_WORLD, MPI_STATUS_IGNORE);
                        if (!rc) rc = MPI_Send(buf, (int)bytes, MPI_BYTE, peer, 10, MPI_COMM_WORLD);
                    }
                } else {
                    MPI_Request rq;
                    if ((rank & 1) == 0) {
                        rc = MPI_Isend(buf, (int)bytes, MPI_BYTE, peer, 10, MPI_COMM_WORLD, &rq);
                        if (!rc) rc = MPI_Wait(&rq, MPI_STATUS_IGNORE);
                        if (!rc) rc = MPI_Irecv(buf, (int)bytes, MPI_BYTE, peer, 10, MPI_COMM_WORLD, &rq);
                        if (!rc) rc = MPI_Wait(&rq, MPI_STATUS_IGNORE);
                    } else {
                        rc = MPI_Irecv(buf, (int)bytes, MPI_BYTE, peer, 10, MPI_COMM_WORLD, &rq);
                        if (!rc) rc = MPI_Wait(&rq, MPI_STATUS_IGNORE);
                        if (!rc) rc = MPI_Isend(buf, (int)bytes, MPI_BYTE, peer, 10, MPI_COMM_WORLD, &rq);
                        if (!rc) rc = MPI_Wait(&rq, MPI_STATUS_IGNORE);
                    }
                }
                if (rank == 0 && iter_ns) iter_ns[it] = gtime() - t0;
            }
        }
        if (p.p[7]) ((int*)p.p[7])[rank] = rc;
        return rc;
    }
};

// Ring: every rank sends `bytes` to rank+1 and receives from rank-1, `iters` times.  Blocking mode
// orders even/odd ranks so standard-mode sends cannot deadlock; nonblocking mode is Irecv+Isend+Waitall.
struct Ring {
    static __device__ int run(const gpumpi_params& p) {
        int rank = -1, n = 0;
        MPI_Comm_rank(MPI_COMM_WORLD, &rank);
        MPI_Comm_size(MPI_COMM_WORLD, &n);
        const long long bytes = p.i[0];
        const int iters = (int)p.i[1];
        const int nb = (int)p.i[2];
        const char* sb = (const char*)p.p[0] + (long long)rank * p.i[4];
        char* rb = (char*)p.p[1] + (long long)rank * p.i[4];
        unsigned long long* iter_ns = (unsigned long long*)p.p[6];
        const int next = (rank + 1) % n, prev = (rank + n - 1) % n;
        int rc = 0;
        for (int it = 0; it < iters && rc == 0; it++) {
            unsigned long long t0 = gtime();
            if (nb || (n & 1)) {
                MPI_Request rq[2];
                rc = MPI_Irecv(rb, (int)bytes, MPI_BYTE, prev, 11, MPI_COMM_WORLD, &rq[0]);
                if (!rc) rc = MPI_Isend(sb, (int)bytes, MPI_BYTE, next, 11, MPI_COMM_WORLD, &rq[1]);
                if (!rc) rc = MPI_Waitall(2, rq, MPI_STATUSES_IGNORE);
            } else if ((rank & 1) == 0) {
                rc = MPI_Send(sb, (int)bytes, MPI_BYTE, next, 11, MPI_COMM_WORLD);
                if (!rc) rc = MPI_Recv(rb, (int)bytes, MPI_BYTE, prev, 11, MPI_COMM_WORLD, MPI_STATUS_IGNORE);
            } else {
                rc = MPI_Recv(rb, (int)bytes, MPI_BYTE, prev, 11, MPI_COMM_WORLD, MPI_STATUS_IGNORE);
                if (!rc) rc = MPI_Send(sb, (int)bytes, MPI_BYTE, next, 11, MPI_COMM_WORLD);
            }
            if (rank == 0 && iter_ns) iter_ns[it] = gtime() - t0;
        }
        if (p.p[7]) ((int*)p.p[7])[rank] = rc;
        return rc;
    }
};

// Monte Carlo pi (stands in for the reference's cpi example, which integrates instead): each rank
// draws pairs from the 64-bit LCG seeded seed+rank, counts x*x + y*y < 1 with explicitly rounded
// double operations, and the counts are combined with MPI_Reduce(SUM, root 0).
struct PiWork {
    unsigned long long seed;
    long long pairs;
    int rank;
    unsigned long long hits;
};
__shared__ PiWork s_pi;

__device__ void pi_task(void* arg, int tid, int nt) {
    PiWork* w = (PiWork*)arg;
    // thread tid takes the contiguous sub-range [lo, hi) of the rank's pair sequence and jumps the
    // LCG ahead to it (affine composition by repeated squaring)
    long long per = (w->pairs + nt - 1) / nt;
    long long lo = per * tid, hi = lo + per < w->pairs ? lo + per : w->pairs;
    unsigned long long a = 6364136223846793005ULL, c = 1442695040888963407ULL;
    unsigned long long s = w->seed + (unsigned long long)w->rank;
    // advance by 2*lo steps: s <- A*s + C with (A, C) = (a, c)^(2*lo)
    unsigned long long A = 1, C = 0, ak = a, ck = c;
    unsigned long long k = 2ULL * (unsigned long long)(lo > 0 ? lo : 0);
    while (k) {
        if (k & 1) {
            A = ak * A;
            C = ak * C + ck;
        }
        ck = ak * ck + ck;
        ak = ak * ak;
        k >>= 1;
    }
    s = A * s + C;
    unsigned long long hits = 0;
    for (long long i = lo; i < hi; i++) {
        s = s * a + c;
        double x = (double)(s >> 11) * (1.0 / 9007199254740992.0);
        s = s * a + c;
        double y = (double)(s >> 11) * (1.0 / 9007199254740992.0);
        double r2 = __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y));
        hits += r2 < 1.0;
    }
    atomicAdd(&w->hits, hits);
}

struct Pi {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        int rank = -1;
        MPI_Comm_rank(MPI_COMM_WORLD, &rank);
        s_pi.seed = (unsigned long long)p.i[0];
        s_pi.pairs = p.i[1];
        s_pi.rank = rank;
        s_pi.hits = 0;
        gpumpi_block_parallel(&pi_task, &s_pi);
        long long hits = (long long)s_pi.hits, total = 0;
        ((long long*)p.p[0])[rank] = hits;
        int rc = MPI_Reduce(&hits, &total, 1, MPI_INT64_T, MPI_SUM, 0, MPI_COMM_WORLD);
        if (rank == 0) *(long long*)p.p[1] = total;
        if (p.p[7]) ((int*)p.p[7])[rank] = rc;
        return rc ? rc : MPI_Finalize();
    }
};

}  // namespace

extern const gpumpi_prog_entry g_hot_programs[] = {
    GPUMPI_PROGRAM(GPUMPI_P_COLL, "coll", Coll),
    GPUMPI_PROGRAM(GPUMPI_P_PINGPONG, "pingpong", PingPong),
    GPUMPI_PROGRAM(GPUMPI_P_RING, "ring", Ring),
    GPUMPI_PROGRAM(GPUMPI_P_PI, "pi", Pi),
};
extern const int g_num_hot_programs = sizeof(g_hot_programs) / sizeof(g_hot_programs[0]);
