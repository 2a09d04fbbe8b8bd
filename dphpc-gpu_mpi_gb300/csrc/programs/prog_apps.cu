// prog_apps.cu — application programs on the MPI surface: the distributed bucket sort of integer keys,
// the 3D halo exchange with derived-datatype faces, and a batch of communicators of uneven sizes.
//
// Scalar per-rank logic runs on each rank block's thread 0, like converted MPI code; the data-parallel
// loops between MPI calls use the block's threads through gpumpi_block_parallel.
#include "rt_kernel.cuh"

namespace {

__device__ __forceinline__ unsigned long long gtime() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

constexpr unsigned long long LCG_A = 6364136223846793005ULL, LCG_C = 1442695040888963407ULL;

// LCG state after k steps from s (affine map (A, C) raised to the k-th power by repeated squaring)
__device__ unsigned long long lcg_jump(unsigned long long s, unsigned long long k) {
    unsigned long long A = 1, C = 0, ak = LCG_A, ck = LCG_C;
    while (k) {
        if (k & 1) {
            A = ak * A;
            C = ak * C + ck;
        }
        ck = ak * ck + ck;
        ak = ak * ak;
        k >>= 1;
    }
    return A * s + C;
}

__device__ __forceinline__ double lcg_u01(unsigned long long& s) {
    s = s * LCG_A + LCG_C;
    return (double)(s >> 11) * (1.0 / 9007199254740992.0);
}

__shared__ int s_scan[257];

// Exclusive prefix of the nt per-thread sums in s_scan; s_scan[nt] = total.
__device__ void scan_thread_sums(int tid, int nt) {
    gpumpi_block_sync(nt);
    if (tid == 0) {
        int run = 0;
        for (int t = 0; t < nt; t++) {
            const int v = s_scan[t];
            s_scan[t] = run;
            run += v;
        }
        s_scan[nt] = run;
    }
    gpumpi_block_sync(nt);
}

// exclusive prefix sum of a[0..m) in place (a may be shared or global); returns the total to every thread
__device__ int block_exclusive_scan(int* a, int m, int tid, int nt) {
    const int seg = (m + nt - 1) / nt;
    const int lo = min(m, tid * seg), hi = min(m, lo + seg);
    int s = 0;
    for (int i = lo; i < hi; i++) s += a[i];
    s_scan[tid] = s;
    scan_thread_sums(tid, nt);
    int acc = s_scan[tid];
    for (int i = lo; i < hi; i++) {
        const int v = a[i];
        a[i] = acc;
        acc += v;
    }
    const int total = s_scan[nt];
    gpumpi_block_sync(nt);
    return total;
}

// ------------------------------------------------------------------------------------------------
// Distributed bucket sort (the call pattern of an integer sort benchmark: bucket counts by
// MPI_Alltoall, keys by MPI_Alltoallv, then a local counting sort).  Keys: key = floor(2^21 * mean of
// four U(0,1) draws) from the 64-bit LCG seeded seed + rank; bucket of key k on n ranks: (k * n) >> 21,
// so rank r receives exactly the keys in [ceil(r 2^21 / n), ceil((r + 1) 2^21 / n)).
//   i[0] seed  i[1] keys per rank  i[2] iterations  i[3] receive capacity per rank (keys)
//   i[4] 1: generate the keys on the device  i[5] per-rank stride of the global histogram scratch
//   p[0] keys [n][kpr]  p[1] send buffer [n][kpr]  p[2] receive buffer [n][cap]  p[3] sorted [n][cap]
//   p[4] int64 received count [n]  p[5] int32 scratch [n][4n]  p[6] int32 histogram scratch [n][i[5]]
//   p[7] int rc [n]  p[8] int64 per-iteration ns (rank 0)
// ------------------------------------------------------------------------------------------------
constexpr int KEY_BITS = 21;

struct SortWork {
    unsigned long long seed;
    long long kpr;
    int rank, n;
    int* keys;
    int* send;
    int* recv;
    int* out;
    int* sc;  // send counts [n], then send displacements, receive counts, receive displacements
    int* hist_global;
    long long nrecv;
    int lo, range;
    int err;
};
__shared__ SortWork s_sort;

__device__ void sort_gen_task(void* arg, int tid, int nt) {
    SortWork* w = (SortWork*)arg;
    const long long per = (w->kpr + nt - 1) / nt;
    const long long lo = min(w->kpr, per * tid), hi = min(w->kpr, lo + per);
    unsigned long long s = lcg_jump(w->seed + (unsigned long long)w->rank, 4ULL * (unsigned long long)lo);
    for (long long i = lo; i < hi; i++) {
        const double a = lcg_u01(s), b = lcg_u01(s), c = lcg_u01(s), d = lcg_u01(s);
        const double sum = __dadd_rn(__dadd_rn(__dadd_rn(a, b), c), d);
        w->keys[i] = (int)floor(__dmul_rn(sum, 524288.0));  // 2^21 * sum / 4
    }
}

// Calls f(key) for every key of keys[0, count), in no particular order.  The 16-byte-aligned body is read
// as uint4 vectors, NV of them per thread before any key is handled (the handler's atomics and stores may
// alias the keys as far as the compiler knows, so one load at a time would cost a full memory round trip
// each): one block alone reads a rank's keys, so the bytes it keeps in flight set the speed.
template <int NV, class F>
__device__ __forceinline__ void for_keys(const int* keys, long long count, int tid, int nt, F&& f) {
    if (count <= 0) return;
    const long long head = min(count, (long long)(((16 - ((unsigned long long)keys & 15)) & 15) >> 2));
    if (tid < head) f(__ldcg(keys + tid));
    const uint4* v = (const uint4*)(keys + head);
    const long long nv = (count - head) >> 2;
    long long i = tid;
    for (; i + (long long)(NV - 1) * nt < nv; i += (long long)NV * nt) {
        uint4 k[NV];
#pragma unroll
        for (int j = 0; j < NV; j++) k[j] = __ldcg(v + i + (long long)j * nt);
#pragma unroll
        for (int j = 0; j < NV; j++) {
            f((int)k[j].x);
            f((int)k[j].y);
            f((int)k[j].z);
            f((int)k[j].w);
        }
    }
    for (; i < nv; i += nt) {
        const uint4 k = __ldcg(v + i);
        f((int)k.x);
        f((int)k.y);
        f((int)k.z);
        f((int)k.w);
    }
    const long long t = head + nv * 4 + tid;
    if (t < count) f(__ldcg(keys + t));
}

// bucket counts, send displacements and the packed send buffer (keys grouped by destination rank)
__device__ void sort_pack_task(void* arg, int tid, int nt) {
    SortWork* w = (SortWork*)arg;
    const int n = w->n;
    size_t sbytes = 0;
    int* bins = (int*)gpumpi_block_scratch(&sbytes);
    const bool in_smem = bins && sbytes >= (size_t)n * sizeof(int);
    if (!in_smem) bins = w->sc;
    for (int d = tid; d < n; d += nt) bins[d] = 0;
    gpumpi_block_sync(nt);
    for_keys<8>(w->keys, w->kpr, tid, nt, [&](int k) { atomicAdd(&bins[((long long)k * n) >> KEY_BITS], 1); });
    gpumpi_block_sync(nt);
    int* sd = w->sc + n;
    for (int d = tid; d < n; d += nt) {
        const int c = bins[d];
        w->sc[d] = c;
        sd[d] = c;
    }
    gpumpi_block_sync(nt);
    block_exclusive_scan(sd, n, tid, nt);
    // cursors start at the displacements; the order inside a bucket does not matter (sorted later)
    int* cur = in_smem ? bins : w->sc + 3 * n;  // spare n ints of the scratch row when not in shared memory
    for (int d = tid; d < n; d += nt) cur[d] = sd[d];
    gpumpi_block_sync(nt);
    int* send = w->send;
    // each key takes a slot of its bucket with a cursor atomic and is stored there; the keys come in uint4
    // vectors, sixteen keys per thread at a time: their loads, then their cursor atomics, then their stores
    // (a store between two atomics would keep the second from issuing before the first returned)
    const int* keys = w->keys;
    const long long kpr = w->kpr;
    auto slot = [&](int k) { return atomicAdd(&cur[((long long)k * n) >> KEY_BITS], 1); };
    const long long head = min(kpr, (long long)(((16 - ((unsigned long long)keys & 15)) & 15) >> 2));
    if (tid < head) {
        const int k = __ldcg(keys + tid);
        send[slot(k)] = k;
    }
    const uint4* v = (const uint4*)(keys + head);
    const long long nv = (kpr - head) >> 2;
    long long i = tid;
    for (; i + 3LL * nt < nv; i += 4LL * nt) {
        uint4 a[4];
#pragma unroll
        for (int u = 0; u < 4; u++) a[u] = __ldcg(v + i + (long long)u * nt);
        int k[16], pos[16];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            k[4 * u] = (int)a[u].x;
            k[4 * u + 1] = (int)a[u].y;
            k[4 * u + 2] = (int)a[u].z;
            k[4 * u + 3] = (int)a[u].w;
        }
#pragma unroll
        for (int j = 0; j < 16; j++) pos[j] = slot(k[j]);
#pragma unroll
        for (int j = 0; j < 16; j++) send[pos[j]] = k[j];
    }
    for (; i < nv; i += nt) {
        const uint4 a = __ldcg(v + i);
        const int k[4] = {(int)a.x, (int)a.y, (int)a.z, (int)a.w};
        int pos[4];
#pragma unroll
        for (int j = 0; j < 4; j++) pos[j] = slot(k[j]);
#pragma unroll
        for (int j = 0; j < 4; j++) send[pos[j]] = k[j];
    }
    const long long t = head + nv * 4 + tid;
    if (t < kpr) {
        const int k = __ldcg(keys + t);
        send[slot(k)] = k;
    }
}

__device__ void sort_rdispl_task(void* arg, int tid, int nt) {
    SortWork* w = (SortWork*)arg;
    const int n = w->n;
    const int* rc = w->sc + 2 * n;
    int* rd = w->sc + 3 * n;
    for (int d = tid; d < n; d += nt) rd[d] = rc[d];
    gpumpi_block_sync(nt);
    const int total = block_exclusive_scan(rd, n, tid, nt);
    if (tid == 0) w->nrecv = total;
}

// counting sort of the received keys (all in [lo, lo + range))
__device__ void sort_local_task(void* arg, int tid, int nt) {
    SortWork* w = (SortWork*)arg;
    size_t sbytes = 0;
    int* hist = (int*)gpumpi_block_scratch(&sbytes);
    if (!hist || sbytes < (size_t)w->range * sizeof(int)) hist = w->hist_global;
    for (int k = tid; k < w->range; k += nt) hist[k] = 0;
    gpumpi_block_sync(nt);
    const int lo = w->lo, range = w->range;
    bool bad = false;
    for_keys<4>(w->recv, w->nrecv, tid, nt, [&](int key) {
        const int k = key - lo;
        if (k >= 0 && k < range) atomicAdd(&hist[k], 1);
        else bad = true;
    });
    if (bad) w->err = 1;
    gpumpi_block_sync(nt);
    // start of every value's run in the output; then a warp takes 32 consecutive values at a time, whose
    // runs fill one contiguous range of the output, and its lanes store 32 consecutive positions per step
    // (coalesced), each finding its value by a binary search over the 32 starts held in the warp's lanes.
    // Four steps are interleaved so that their shuffles overlap; a range without keys costs nothing.
    const int total = block_exclusive_scan(hist, range, tid, nt);
    gpumpi_block_sync(nt);
    const int lane = tid & 31, wi = tid >> 5, nw = nt >> 5;
    int* out = w->out;
    for (int k0 = wi * 32; k0 < range; k0 += nw * 32) {
        const int st = k0 + lane < range ? hist[k0 + lane] : total;  // values past the range start at the end
        const int s0 = __shfl_sync(0xffffffffu, st, 0);
        const int s1 = k0 + 32 < range ? hist[k0 + 32] : total;
        for (int base = s0; base < s1; base += 128) {
            int q[4], v[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                q[u] = base + 32 * u + lane;
                v[u] = 0;
            }
#pragma unroll
            for (int b = 16; b; b >>= 1)
#pragma unroll
                for (int u = 0; u < 4; u++)
                    if (__shfl_sync(0xffffffffu, st, v[u] + b) <= q[u]) v[u] += b;
#pragma unroll
            for (int u = 0; u < 4; u++)
                if (q[u] < s1) out[q[u]] = lo + k0 + v[u];
        }
    }
}

struct BucketSort {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        int rank = -1, n = 0;
        MPI_Comm_rank(MPI_COMM_WORLD, &rank);
        MPI_Comm_size(MPI_COMM_WORLD, &n);
        const long long kpr = p.i[1], cap = p.i[3];
        const int iters = (int)p.i[2];
        SortWork* w = &s_sort;
        w->seed = (unsigned long long)p.i[0];
        w->kpr = kpr;
        w->rank = rank;
        w->n = n;
        w->keys = (int*)p.p[0] + (long long)rank * kpr;
        w->send = (int*)p.p[1] + (long long)rank * kpr;
        w->recv = (int*)p.p[2] + (long long)rank * cap;
        w->out = (int*)p.p[3] + (long long)rank * cap;
        w->sc = (int*)p.p[5] + (long long)rank * 4 * n;
        w->hist_global = (int*)p.p[6] + (long long)rank * p.i[5];
        const long long max_key = 1LL << KEY_BITS;
        w->lo = (int)((max_key * rank + n - 1) / n);
        w->range = (int)((max_key * (rank + 1) + n - 1) / n) - w->lo;
        w->err = 0;
        w->nrecv = 0;
        long long* iter_ns = (long long*)p.p[8];
        int rc = (w->range > p.i[5]) ? MPI_ERR_COUNT : MPI_SUCCESS;
        if (p.i[4]) gpumpi_block_parallel(&sort_gen_task, w);
        int brc = MPI_Barrier(MPI_COMM_WORLD);
        if (!rc) rc = brc;
        int* sc = w->sc;
        for (int it = 0; it < iters && rc == 0; it++) {
            const unsigned long long t0 = gtime();
            gpumpi_block_parallel(&sort_pack_task, w);
            rc = MPI_Alltoall(sc, 1, MPI_INT, sc + 2 * n, 1, MPI_INT, MPI_COMM_WORLD);
            if (rc) break;
            gpumpi_block_parallel(&sort_rdispl_task, w);
            int overflow = 0;
            if (w->nrecv > cap) {
                // the receive buffer cannot hold this rank's bucket: receive nothing (the senders' pieces
                // are reported truncated) and fail after the collective every rank takes part in
                for (int d = 0; d < n; d++) sc[2 * n + d] = 0;
                w->nrecv = 0;
                overflow = 1;
            }
            rc = MPI_Alltoallv(w->send, sc, sc + n, MPI_INT, w->recv, sc + 2 * n, sc + 3 * n, MPI_INT,
                               MPI_COMM_WORLD);
            if (overflow) rc = MPI_ERR_COUNT;
            if (rc) break;
            gpumpi_block_parallel(&sort_local_task, w);
            if (w->err) rc = MPI_ERR_OTHER;
            if (rank == 0 && iter_ns) iter_ns[it] = (long long)(gtime() - t0);
        }
        ((long long*)p.p[4])[rank] = w->nrecv;
        if (p.p[7]) ((int*)p.p[7])[rank] = rc;
        return rc ? rc : MPI_Finalize();
    }
};

// ------------------------------------------------------------------------------------------------
// 3D halo exchange: global grid G^3, G = P * L, periodic, on P^3 ranks (rank = (pz * P + py) * P + px);
// each rank holds an (L + 2)^3 block of doubles whose interior is its L^3 sub-grid and whose one-cell
// faces are filled from the six neighbours every iteration (edges and corners are not exchanged).  The
// faces are derived datatypes: z faces MPI_Type_vector(L, L, W), y faces MPI_Type_vector(L, L, W * W),
// x faces an hvector over z of the columns MPI_Type_vector(L, 1, W) (mode 0), or all twelve face
// positions as MPI_Type_create_subarray of the block (mode 1).  Isend/Irecv + Waitall, 12 requests.
//   i[0] P  i[1] L  i[2] iterations  i[3] face type mode  p[0] blocks [P^3][(L + 2)^3]
//   p[6] int64 per-iteration ns (rank 0)  p[7] int rc [n]
// Cell value: (gz * 1000003 + gy * 1009 + gx) * 0.125 (exact in double); halos start at -1.
// ------------------------------------------------------------------------------------------------
struct HaloWork {
    double* blk;
    int L, P, px, py, pz;
};
__shared__ HaloWork s_halo;

__device__ void halo_fill_task(void* arg, int tid, int nt) {
    HaloWork* w = (HaloWork*)arg;
    const long long W = w->L + 2;
    const long long cells = W * W * W;
    for (long long c = tid; c < cells; c += nt) {
        const long long z = c / (W * W), y = (c / W) % W, x = c % W;
        const bool halo = z == 0 || z == W - 1 || y == 0 || y == W - 1 || x == 0 || x == W - 1;
        double v = -1.0;
        if (!halo) {  // interior cell: global coordinates are inside [0, G)
            const long long gz = (long long)w->pz * w->L + z - 1, gy = (long long)w->py * w->L + y - 1,
                            gx = (long long)w->px * w->L + x - 1;
            v = (double)(gz * 1000003 + gy * 1009 + gx) * 0.125;
        }
        w->blk[c] = v;
    }
}

struct Halo {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        int rank = -1, n = 0;
        MPI_Comm_rank(MPI_COMM_WORLD, &rank);
        MPI_Comm_size(MPI_COMM_WORLD, &n);
        const int P = (int)p.i[0], L = (int)p.i[1], iters = (int)p.i[2], mode = (int)p.i[3];
        const int W = L + 2;
        if (P * P * P != n || L < 1) {
            if (p.p[7]) ((int*)p.p[7])[rank] = MPI_ERR_ARG;
            return MPI_ERR_ARG;
        }
        HaloWork* w = &s_halo;
        w->L = L;
        w->P = P;
        w->px = rank % P;
        w->py = (rank / P) % P;
        w->pz = rank / (P * P);
        w->blk = (double*)p.p[0] + (long long)rank * W * W * W;
        gpumpi_block_parallel(&halo_fill_task, w);

        // mode 0: face[d] is one face normal to dimension d (0 = x, 1 = y, 2 = z), placed by its address;
        // mode 1: sub[d][k] is the face at position k (send low, send high, recv low, recv high) of the block
        MPI_Datatype face[3] = {MPI_DATATYPE_NULL, MPI_DATATYPE_NULL, MPI_DATATYPE_NULL};
        MPI_Datatype sub[3][4];
        int rc = MPI_SUCCESS;
        if (mode == 0) {
            MPI_Datatype col;
            rc |= MPI_Type_vector(L, 1, W, MPI_DOUBLE, &col);
            rc |= MPI_Type_create_hvector(L, 1, (MPI_Aint)W * W * (MPI_Aint)sizeof(double), col, &face[0]);
            rc |= MPI_Type_vector(L, L, W * W, MPI_DOUBLE, &face[1]);
            rc |= MPI_Type_vector(L, L, W, MPI_DOUBLE, &face[2]);
            for (int d = 0; d < 3; d++) rc |= MPI_Type_commit(&face[d]);
            rc |= MPI_Type_free(&col);
        } else {
            const int sizes[3] = {W, W, W};  // C order: z, y, x
            for (int d = 0; d < 3; d++) {
                const int axis = 2 - d;  // array axis of dimension d
                int sub_sizes[3] = {L, L, L};
                sub_sizes[axis] = 1;
                const int pos[4] = {1, L, 0, L + 1};
                for (int k = 0; k < 4; k++) {
                    int starts[3] = {1, 1, 1};
                    starts[axis] = pos[k];
                    rc |= MPI_Type_create_subarray(3, sizes, sub_sizes, starts, MPI_ORDER_C, MPI_DOUBLE, &sub[d][k]);
                    rc |= MPI_Type_commit(&sub[d][k]);
                }
            }
        }
        const int brc = MPI_Barrier(MPI_COMM_WORLD);
        if (!rc) rc = brc;
        const int pc[3] = {w->px, w->py, w->pz};
        long long* iter_ns = (long long*)p.p[6];
        for (int it = 0; it < iters && rc == 0; it++) {
            const unsigned long long t0 = gtime();
            MPI_Request rq[12];
            int nr = 0;
            for (int d = 0; d < 3 && !rc; d++) {
                const long long stride = d == 0 ? 1 : d == 1 ? W : (long long)W * W;
                int up[3] = {pc[0], pc[1], pc[2]}, dn[3] = {pc[0], pc[1], pc[2]};
                up[d] = (pc[d] + 1) % P;
                dn[d] = (pc[d] + P - 1) % P;
                const int rup = (up[2] * P + up[1]) * P + up[0], rdn = (dn[2] * P + dn[1]) * P + dn[0];
                double* b = w->blk;
                // tag 2d: a high face travelling up; tag 2d+1: a low face travelling down
                if (mode == 0) {
                    // address of the face at coordinate 0 of dimension d; coordinate c adds c * stride
                    const long long base = d == 0 ? (long long)W * W + W : d == 1 ? (long long)W * W + 1 : W + 1;
                    rc |= MPI_Irecv(b + base, 1, face[d], rdn, 2 * d, MPI_COMM_WORLD, &rq[nr++]);
                    rc |= MPI_Irecv(b + base + (L + 1) * stride, 1, face[d], rup, 2 * d + 1, MPI_COMM_WORLD, &rq[nr++]);
                    rc |= MPI_Isend(b + base + L * stride, 1, face[d], rup, 2 * d, MPI_COMM_WORLD, &rq[nr++]);
                    rc |= MPI_Isend(b + base + stride, 1, face[d], rdn, 2 * d + 1, MPI_COMM_WORLD, &rq[nr++]);
                } else {
                    rc |= MPI_Irecv(b, 1, sub[d][2], rdn, 2 * d, MPI_COMM_WORLD, &rq[nr++]);
                    rc |= MPI_Irecv(b, 1, sub[d][3], rup, 2 * d + 1, MPI_COMM_WORLD, &rq[nr++]);
                    rc |= MPI_Isend(b, 1, sub[d][1], rup, 2 * d, MPI_COMM_WORLD, &rq[nr++]);
                    rc |= MPI_Isend(b, 1, sub[d][0], rdn, 2 * d + 1, MPI_COMM_WORLD, &rq[nr++]);
                }
            }
            if (nr) {
                const int wrc = MPI_Waitall(nr, rq, MPI_STATUSES_IGNORE);
                if (!rc) rc = wrc;
            }
            if (rank == 0 && iter_ns) iter_ns[it] = (long long)(gtime() - t0);
        }
        if (mode == 0) {
            for (int d = 0; d < 3; d++)
                if (face[d] != MPI_DATATYPE_NULL) MPI_Type_free(&face[d]);
        } else {
            for (int d = 0; d < 3; d++)
                for (int k = 0; k < 4; k++) MPI_Type_free(&sub[d][k]);
        }
        if (p.p[7]) ((int*)p.p[7])[rank] = rc;
        return rc ? rc : MPI_Finalize();
    }
};

// ------------------------------------------------------------------------------------------------
// Batched communicators: up to 64 communicators, each a contiguous range of world ranks made with
// MPI_Comm_create, each running its own MPI_Allreduce every iteration in this one persistent launch.  A
// rank in several communicators runs their collectives in communicator order (the same order on every
// rank, so no cycle of waits can form); communicators on disjoint ranks progress at the same time and
// each call's variant comes from the world's selection policy.  A world barrier ends each iteration, so
// rank 0's time is the whole batch.
//   i[0] communicators  i[1] iterations  i[2] datatype  i[3] op
//   p[0] send base  p[1] recv base  p[2] int64 [comms][4] = {first world rank, size, count, element offset}
//   p[6] int64 per-iteration ns (rank 0)  p[7] int rc [n]
// Member i of communicator c sends from send + (offset_c + i * count_c) elements and receives likewise.
// ------------------------------------------------------------------------------------------------
constexpr int MAX_BATCH_COMMS = 64;

struct Batch {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        int rank = -1, n = 0;
        MPI_Comm_rank(MPI_COMM_WORLD, &rank);
        MPI_Comm_size(MPI_COMM_WORLD, &n);
        const int ncomms = (int)p.i[0] < MAX_BATCH_COMMS ? (int)p.i[0] : MAX_BATCH_COMMS;
        const int iters = (int)p.i[1];
        const MPI_Datatype dt = (MPI_Datatype)p.i[2];
        const MPI_Op op = gpumpi_predefined_op((int)p.i[3]);
        const long long* tab = (const long long*)p.p[2];
        int es = 0;
        int rc = MPI_Type_size(dt, &es);
        MPI_Group gw;
        if (!rc) rc = MPI_Comm_group(MPI_COMM_WORLD, &gw);
        MPI_Comm comms[MAX_BATCH_COMMS];
        // setup_ns (optional): rank 0's time in the group calls and in MPI_Comm_create, summed
        long long* setup_ns = (long long*)p.p[5];
        long long t_group = 0, t_create = 0;
        for (int c = 0; c < ncomms; c++) {
            comms[c] = MPI_COMM_NULL;
            if (rc) continue;
            const int first = (int)tab[4 * c], size = (int)tab[4 * c + 1];
            int range[1][3] = {{first, first + size - 1, 1}};
            MPI_Group g;
            const unsigned long long ta = gtime();
            rc = MPI_Group_range_incl(gw, 1, range, &g);
            const unsigned long long tb = gtime();
            if (!rc) rc = MPI_Comm_create(MPI_COMM_WORLD, g, &comms[c]);
            const unsigned long long tc = gtime();
            if (!rc) rc = MPI_Group_free(&g);
            t_group += (long long)(tb - ta + gtime() - tc);
            t_create += (long long)(tc - tb);
        }
        if (!rc) rc = MPI_Group_free(&gw);
        if (rank == 0 && setup_ns) {
            setup_ns[0] = t_group;
            setup_ns[1] = t_create;
        }
        long long* iter_ns = (long long*)p.p[6];
        for (int it = 0; it < iters && rc == 0; it++) {
            const unsigned long long t0 = gtime();
            for (int c = 0; c < ncomms && rc == 0; c++) {
                if (comms[c] == MPI_COMM_NULL) continue;
                const long long count = tab[4 * c + 2];
                const long long off = (tab[4 * c + 3] + (long long)(rank - (int)tab[4 * c]) * count) * es;
                rc = MPI_Allreduce((const char*)p.p[0] + off, (char*)p.p[1] + off, (int)count, dt, op, comms[c]);
            }
            if (!rc) rc = MPI_Barrier(MPI_COMM_WORLD);
            if (rank == 0 && iter_ns) iter_ns[it] = (long long)(gtime() - t0);
        }
        for (int c = 0; c < ncomms; c++)
            if (comms[c] != MPI_COMM_NULL) MPI_Comm_free(&comms[c]);
        if (p.p[7]) ((int*)p.p[7])[rank] = rc;
        return rc ? rc : MPI_Finalize();
    }
};

}  // namespace

extern const gpumpi_prog_entry g_app_programs[] = {
    GPUMPI_PROGRAM(GPUMPI_P_BUCKET_SORT, "bucket_sort", BucketSort),
    GPUMPI_PROGRAM(GPUMPI_P_HALO, "halo", Halo),
    GPUMPI_PROGRAM(GPUMPI_P_BATCH, "batch", Batch),
};
extern const int g_num_app_programs = sizeof(g_app_programs) / sizeof(g_app_programs[0]);
