// prog_tests.cu — device programs that mirror the reference's GPU tests.
//
// Each program does what the corresponding reference test does (same ranks, same buffers on the
// rank's stack or device heap, same values), written against the MPI surface instead of the
// reference's CudaMPI:: internals, and reports per rank: ok flag (the reference's REQUIRE(ok[i])),
// plus the received values so the host can compare them with the golden vectors.
//   p[0] = uint8 ok[nranks], p[1] = int64 outi[nranks*64], p[2] = double outd[nranks*64]
#include "rt_kernel.cuh"
#include "gpumpi_stdio.h.cuh"

namespace {

__device__ __forceinline__ int wrank() {
    int r = -1;
    MPI_Comm_rank(MPI_COMM_WORLD, &r);
    return r;
}
__device__ __forceinline__ unsigned char* okp(const gpumpi_params& p) { return (unsigned char*)p.p[0]; }
__device__ __forceinline__ long long* outi(const gpumpi_params& p, int r) { return (long long*)p.p[1] + (long long)r * 64; }
__device__ __forceinline__ double* outd(const gpumpi_params& p, int r) { return (double*)p.p[2] + (long long)r * 64; }

// tests/cuda_mpi_test.cu:5-36
struct SingleInt {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        int rank = wrank();
        bool ok = true;
        if (rank == 0) {
            int x = 3456;
            MPI_Request r;
            ok = MPI_Isend(&x, 1, MPI_INT, 1, 15, MPI_COMM_WORLD, &r) == MPI_SUCCESS;
            ok = ok && MPI_Wait(&r, MPI_STATUS_IGNORE) == MPI_SUCCESS;
        } else if (rank == 1) {
            int x = 0;
            MPI_Request r;
            MPI_Irecv(&x, 1, MPI_INT, 0, 15, MPI_COMM_WORLD, &r);
            MPI_Wait(&r, MPI_STATUS_IGNORE);
            ok = x == 3456;
            outi(p, rank)[0] = x;
        }
        okp(p)[rank] = ok;
        return MPI_Finalize();
    }
};

// tests/cuda_mpi_test.cu:38-73
struct TransferArray {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        int rank = wrank();
        bool ok = true;
        if (rank == 0) {
            int x[16];
            for (int i = 0; i < 16; i++) x[i] = i;
            MPI_Send(x, 16, MPI_INT, 1, 15, MPI_COMM_WORLD);
        } else if (rank == 1) {
            int x[16] = {};
            MPI_Recv(x, 16, MPI_INT, 0, 15, MPI_COMM_WORLD, MPI_STATUS_IGNORE);
            for (int i = 0; i < 16; i++) {
                ok = ok && x[i] == i;
                outi(p, rank)[i] = x[i];
            }
        }
        okp(p)[rank] = ok;
        return MPI_Finalize();
    }
};

// tests/cuda_mpi_test.cu:75-127 — both ranks post the receive, then the send
struct SendRecv {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        int rank = wrank();
        int other = 1 - rank;
        int x[16], y[16] = {};
        for (int i = 0; i < 16; i++) x[i] = rank == 0 ? i : -i;
        MPI_Request rq[2];
        MPI_Irecv(y, 16, MPI_INT, other, 15, MPI_COMM_WORLD, &rq[0]);
        MPI_Isend(x, 16, MPI_INT, other, 15, MPI_COMM_WORLD, &rq[1]);
        MPI_Wait(&rq[0], MPI_STATUS_IGNORE);
        bool ok = true;
        for (int i = 0; i < 16; i++) {
            ok = ok && y[i] == (rank == 0 ? -i : i);
            outi(p, rank)[i] = y[i];
        }
        MPI_Wait(&rq[1], MPI_STATUS_IGNORE);
        okp(p)[rank] = ok;
        return MPI_Finalize();
    }
};

// tests/cuda_mpi_test.cu:129-174 — five messages of 1,2,4,8,16 ints, tags 10..14, one buffer
struct RepeatSendRecv {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        int rank = wrank();
        int other = (rank + 1) % 2;
        int local[16], remote[16] = {};
        for (int i = 0; i < 16; i++) local[i] = (rank + 1) * i;
        MPI_Request s[5], r[5];
        for (int i = 0; i < 5; i++) {
            MPI_Isend(local, 1 << i, MPI_INT, other, 10 + i, MPI_COMM_WORLD, &s[i]);
            MPI_Irecv(remote, 1 << i, MPI_INT, other, 10 + i, MPI_COMM_WORLD, &r[i]);
        }
        for (int i = 0; i < 5; i++) {
            MPI_Wait(&s[i], MPI_STATUS_IGNORE);
            MPI_Wait(&r[i], MPI_STATUS_IGNORE);
        }
        bool ok = true;
        for (int i = 0; i < 16; i++) {
            ok = ok && remote[i] == (other + 1) * i;
            outi(p, rank)[i] = remote[i];
        }
        okp(p)[rank] = ok;
        return MPI_Finalize();
    }
};

// tests/cuda_mpi_test.cu:177-233 — 3-rank ring, both directions, 5 sizes
struct NetworkFlood {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        int rank = wrank();
        const int n = 3;
        int next = (rank + 1) % n, prev = (rank + n - 1) % n;
        int local[16], prevd[16] = {}, nextd[16] = {};
        for (int i = 0; i < 16; i++) local[i] = (rank + 1) * i;
        MPI_Request sn[5], rn[5], sp[5], rp[5];
        for (int i = 0; i < 5; i++) {
            int tag = 10 + i;
            MPI_Isend(local, 1 << i, MPI_INT, next, tag, MPI_COMM_WORLD, &sn[i]);
            MPI_Irecv(nextd, 1 << i, MPI_INT, next, tag, MPI_COMM_WORLD, &rn[i]);
            MPI_Isend(local, 1 << i, MPI_INT, prev, tag, MPI_COMM_WORLD, &sp[i]);
            MPI_Irecv(prevd, 1 << i, MPI_INT, prev, tag, MPI_COMM_WORLD, &rp[i]);
        }
        for (int i = 0; i < 5; i++) {
            MPI_Wait(&rp[i], MPI_STATUS_IGNORE);
            MPI_Wait(&sn[i], MPI_STATUS_IGNORE);
            MPI_Wait(&sp[i], MPI_STATUS_IGNORE);
            MPI_Wait(&rn[i], MPI_STATUS_IGNORE);
        }
        bool ok = true;
        for (int i = 0; i < 16; i++) {
            ok = ok && prevd[i] == (prev + 1) * i && nextd[i] == (next + 1) * i;
            outi(p, rank)[i] = prevd[i];
            outi(p, rank)[16 + i] = nextd[i];
        }
        okp(p)[rank] = ok;
        return MPI_Finalize();
    }
};

// tests/cuda_mpi_test.cu:235-317 — 10 ranks x 20 repeats x 16 ints to every other rank, heap buffers
struct AllToAll {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        int rank = wrank();
        int n = 0;
        MPI_Comm_size(MPI_COMM_WORLD, &n);
        const int reps = 20, ds = 16;
        int* local = (int*)malloc(sizeof(int) * ds * reps * n);
        int* remote = (int*)malloc(sizeof(int) * ds * reps * n);
        MPI_Request* sreq = (MPI_Request*)malloc(sizeof(MPI_Request) * reps * n);
        MPI_Request* rreq = (MPI_Request*)malloc(sizeof(MPI_Request) * reps * n);
        bool ok = local && remote && sreq && rreq;
        if (!ok) {
            okp(p)[rank] = 0;
            return MPI_ERR_NO_MEM;
        }
        for (int r = 0; r < n; r++)
            for (int k = 0; k < reps; k++)
                for (int i = 0; i < ds; i++) {
                    int idx = i + k * ds + r * ds * reps;
                    local[idx] = i * k * r;
                    remote[idx] = 0;
                }
        for (int k = 0; k < reps; k++)
            for (int r = 0; r < n; r++)
                if (r != rank) {
                    int idx = k * ds + r * ds * reps;
                    MPI_Isend(local + idx, ds, MPI_INT, r, 15, MPI_COMM_WORLD, &sreq[r + k * n]);
                    MPI_Irecv(remote + idx, ds, MPI_INT, r, 15, MPI_COMM_WORLD, &rreq[r + k * n]);
                }
        for (int k = 0; k < reps; k++)
            for (int r = 0; r < n; r++)
                if (r != rank) {
                    MPI_Wait(&sreq[r + k * n], MPI_STATUS_IGNORE);
                    MPI_Wait(&rreq[r + k * n], MPI_STATUS_IGNORE);
                }
        long long bad = 0, sum = 0;
        for (int k = 0; k < reps; k++)
            for (int r = 0; r < n; r++)
                if (r != rank)
                    for (int i = 0; i < ds; i++) {
                        int v = remote[i + k * ds + r * ds * reps];
                        sum += v;
                        if (v != i * k * rank) bad++;
                    }
        outi(p, rank)[0] = bad;
        outi(p, rank)[1] = sum;
        okp(p)[rank] = bad == 0;
        free(local);
        free(remote);
        free(sreq);
        free(rreq);
        return MPI_Finalize();
    }
};

// tests/collectives_test.cu:6-54 — MPI_Reduce int16 PROD on 5 ranks, 14 stack elements
struct ReduceInt16Prod {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        int rank = wrank(), n = 0;
        MPI_Comm_size(MPI_COMM_WORLD, &n);
        short buf[14], rb[14] = {};
        for (int i = 0; i < 14; i++) buf[i] = (short)((rank + 1) * (i + 1));
        int rc = MPI_Reduce(buf, rb, 14, MPI_INT16_T, MPI_PROD, 0, MPI_COMM_WORLD);
        bool ok = rc == MPI_SUCCESS;
        if (rank == 0) {
            for (int i = 0; i < 14; i++) {
                short e = 1;
                for (int r = 0; r < n; r++) e = (short)(e * (short)((r + 1) * (i + 1)));
                ok = ok && rb[i] == e;
                outi(p, rank)[i] = rb[i];
            }
        }
        okp(p)[rank] = ok;
        return MPI_Finalize();
    }
};

// tests/collectives_test.cu:57-98 — MPI_Allreduce fp64 SUM on 7 ranks, 17 stack elements
struct AllreduceF64 {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        int rank = wrank(), n = 0;
        MPI_Comm_size(MPI_COMM_WORLD, &n);
        double buf[17], rb[17] = {};
        for (int i = 0; i < 17; i++) buf[i] = (double)((rank + 1) * (i + 1));
        int rc = MPI_Allreduce(buf, rb, 17, MPI_DOUBLE, MPI_SUM, MPI_COMM_WORLD);
        bool ok = rc == MPI_SUCCESS;
        for (int i = 0; i < 17; i++) {
            double e = 0;
            for (int r = 0; r < n; r++) e += (double)((r + 1) * (i + 1));
            ok = ok && fabs(rb[i] - e) <= 1e-5;
            outd(p, rank)[i] = rb[i];
        }
        okp(p)[rank] = ok;
        return MPI_Finalize();
    }
};

// tests/collectives_test.cu:100-141 — MPI_Allgather 7 ranks x 7 ints (device-heap vectors there)
struct Allgather {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        int rank = wrank(), n = 0;
        MPI_Comm_size(MPI_COMM_WORLD, &n);
        const int bs = 7;
        int* buf = (int*)malloc(sizeof(int) * bs);
        int* rb = (int*)malloc(sizeof(int) * bs * n);
        for (int i = 0; i < bs; i++) buf[i] = (rank + 1) * (i + 1);
        for (int i = 0; i < bs * n; i++) rb[i] = 0;
        int rc = MPI_Allgather(buf, bs, MPI_INT, rb, bs, MPI_INT, MPI_COMM_WORLD);
        bool ok = rc == MPI_SUCCESS;
        for (int r = 0; r < n; r++)
            for (int i = 0; i < bs; i++) {
                ok = ok && rb[r * bs + i] == (r + 1) * (i + 1);
                if (r * bs + i < 64) outi(p, rank)[r * bs + i] = rb[r * bs + i];
            }
        okp(p)[rank] = ok;
        free(buf);
        free(rb);
        return MPI_Finalize();
    }
};

// tests/collectives_test.cu:144-196 — MPI_Scatter root 2, 4 ints per rank
struct Scatter {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        int rank = wrank(), n = 0;
        MPI_Comm_size(MPI_COMM_WORLD, &n);
        const int root = 2, bs = 4;
        int* sb = (int*)malloc(sizeof(int) * bs * n);
        int* rb = (int*)malloc(sizeof(int) * bs);
        for (int j = 0; j < n; j++)
            for (int i = 0; i < bs; i++) sb[i + j * bs] = rank == root ? j : -2;
        for (int i = 0; i < bs; i++) rb[i] = -1;
        int rc = MPI_Scatter(sb, bs, MPI_INT, rb, bs, MPI_INT, root, MPI_COMM_WORLD);
        bool ok = rc == MPI_SUCCESS;
        for (int i = 0; i < bs; i++) {
            ok = ok && rb[i] == rank;
            outi(p, rank)[i] = rb[i];
        }
        okp(p)[rank] = ok;
        free(sb);
        free(rb);
        return MPI_Finalize();
    }
};

// tests/collectives_test.cu:199-288 — MPI_Scatterv root 2, sizes i+1, packed displacements
struct Scatterv {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        int rank = wrank(), n = 0;
        MPI_Comm_size(MPI_COMM_WORLD, &n);
        const int root = 2;
        int* sizes = (int*)malloc(sizeof(int) * n);
        int* displs = (int*)malloc(sizeof(int) * n);
        for (int i = 0; i < n; i++) {
            sizes[i] = i + 1;
            displs[i] = i == 0 ? 0 : displs[i - 1] + sizes[i - 1];
        }
        int total = displs[n - 1] + sizes[n - 1];
        int* sb = (int*)malloc(sizeof(int) * total);
        int* rb = (int*)malloc(sizeof(int) * sizes[rank]);
        for (int j = 0; j < n; j++)
            for (int i = 0; i < sizes[j]; i++) sb[displs[j] + i] = rank == root ? j : -2;
        for (int i = 0; i < sizes[rank]; i++) rb[i] = -1;
        int rc = MPI_Scatterv(sb, sizes, displs, MPI_INT, rb, sizes[rank], MPI_INT, root, MPI_COMM_WORLD);
        MPI_Barrier(MPI_COMM_WORLD);
        bool ok = rc == MPI_SUCCESS;
        for (int i = 0; i < sizes[rank]; i++) {
            ok = ok && rb[i] == rank;
            outi(p, rank)[i] = rb[i];
        }
        okp(p)[rank] = ok;
        free(sizes);
        free(displs);
        free(sb);
        free(rb);
        return MPI_Finalize();
    }
};

// tests/communicator_test.cu:5-25
struct CommRank {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        int rank = wrank();
        okp(p)[rank] = rank == gpumpi_world_rank();
        outi(p, rank)[0] = rank;
        return MPI_Finalize();
    }
};

// tests/communicator_test.cu:27-90 — three dup'ed communicators, same tag, crossing order
struct CommDup {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        int rank = wrank();
        MPI_Comm c1, c2, c3;
        MPI_Comm_dup(MPI_COMM_WORLD, &c1);
        MPI_Comm_dup(MPI_COMM_WORLD, &c2);
        MPI_Comm_dup(c2, &c3);
        MPI_Request rq[3] = {nullptr, nullptr, nullptr};
        short data[30] = {};
        if (rank == 0) {
            for (int i = 0; i < 30; i++) data[i] = (short)(i + 1);
            MPI_Isend(data + 0, 10, MPI_INT16_T, 1, 17, c1, &rq[0]);
            MPI_Irecv(data + 10, 10, MPI_INT16_T, 1, 17, c2, &rq[1]);
            MPI_Isend(data + 20, 10, MPI_INT16_T, 1, 17, c3, &rq[2]);
        } else if (rank == 1) {
            for (int i = 0; i < 30; i++) data[i] = (short)-(i + 1);
            MPI_Irecv(data + 20, 10, MPI_INT16_T, 0, 17, c3, &rq[2]);
            MPI_Irecv(data + 0, 10, MPI_INT16_T, 0, 17, c1, &rq[0]);
            MPI_Isend(data + 10, 10, MPI_INT16_T, 0, 17, c2, &rq[1]);
        }
        MPI_Status st[3];
        MPI_Waitall(3, rq, st);
        bool ok = true;
        if (rank == 0) {
            for (int i = 10; i < 20; i++) ok = ok && data[i] == -(i + 1);
        } else if (rank == 1) {
            for (int i = 0; i < 10; i++) ok = ok && data[i] == i + 1;
            for (int i = 20; i < 30; i++) ok = ok && data[i] == i + 1;
        }
        for (int i = 0; i < 30; i++) outi(p, rank)[i] = data[i];
        MPI_Comm_free(&c1);
        MPI_Comm_free(&c2);
        MPI_Comm_free(&c3);
        okp(p)[rank] = ok;
        return MPI_Finalize();
    }
};

// tests/communicator_test.cu:93-152 — Comm_split colours/keys over 10 ranks
struct CommSplit {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        int rank = wrank();
        int color, key;
        if (rank < 3) { color = 0; key = rank; }
        else if (rank < 6) { color = 1; key = 6 - rank; }
        else if (rank < 9) { color = 2; key = 1; }
        else { color = 2; key = 0; }
        MPI_Comm c;
        int rc = MPI_Comm_split(MPI_COMM_WORLD, color, key, &c);
        int nr = -1, ns = -1;
        MPI_Comm_rank(c, &nr);
        MPI_Comm_size(c, &ns);
        bool ok = rc == MPI_SUCCESS;
        if (rank < 3) ok = ok && nr == rank && ns == 3;
        else if (rank < 6) ok = ok && nr == 5 - rank && ns == 3;
        else if (rank < 9) ok = ok && nr == rank - 5 && ns == 4;
        else ok = ok && nr == 0 && ns == 4;
        // traffic on the new communicator uses its ranks (the reference sends to global indices, H1)
        int token = rank, got = -1;
        int next = (nr + 1) % ns, prev = (nr + ns - 1) % ns;
        MPI_Sendrecv(&token, 1, MPI_INT, next, 5, &got, 1, MPI_INT, prev, 5, c, MPI_STATUS_IGNORE);
        int expect_prev_world = -1;
        // world rank of my predecessor in the new communicator
        MPI_Group g, wg;
        MPI_Comm_group(c, &g);
        MPI_Comm_group(MPI_COMM_WORLD, &wg);
        MPI_Group_translate_ranks(g, 1, &prev, wg, &expect_prev_world);
        ok = ok && got == expect_prev_world;
        MPI_Group_free(&g);
        MPI_Group_free(&wg);
        outi(p, rank)[0] = nr;
        outi(p, rank)[1] = ns;
        outi(p, rank)[2] = got;
        MPI_Comm_free(&c);
        okp(p)[rank] = ok;
        return MPI_Finalize();
    }
};

// tests/sample_test.cu
struct Sample {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        okp(p)[wrank()] = 1;
        return MPI_Finalize();
    }
};

// ---- beyond the reference's tests ----

// wildcard receives posted after the send (the reference matches them only when posted first,
// cuda_mpi.cu:300-303), non-overtaking order, Iprobe/Probe/Get_count, Sendrecv, MPI_PROC_NULL,
// Ssend, truncation error.  Ranks: >= 3.
struct P2PMatching {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        int rank = wrank(), n = 0;
        MPI_Comm_size(MPI_COMM_WORLD, &n);
        bool ok = true;
        long long* o = outi(p, rank);
        if (rank == 1 || rank == 2) {
            // 4 messages each, alternating tags; payload encodes (sender, sequence)
            for (int k = 0; k < 4; k++) {
                int v = rank * 100 + k;
                MPI_Send(&v, 1, MPI_INT, 0, 7 + (k & 1), MPI_COMM_WORLD);
            }
        }
        MPI_Barrier(MPI_COMM_WORLD);  // all small sends are now queued at rank 0
        if (rank == 1 || rank == 2) {
            int* big = (int*)malloc(sizeof(int) * 300);
            for (int i = 0; i < 300; i++) big[i] = rank * 1000 + i;
            int rc = MPI_Ssend(big, 300, MPI_INT, 0, 99, MPI_COMM_WORLD);
            ok = ok && rc == 0;
            free(big);
        } else if (rank == 0) {
            // probe then receive with wildcards: per sender, values must arrive in send order
            int last[3] = {-1, -1, -1};
            for (int m = 0; m < 8; m++) {
                MPI_Status st;
                int rc = MPI_Probe(MPI_ANY_SOURCE, MPI_ANY_TAG, MPI_COMM_WORLD, &st);
                int cnt = -1;
                MPI_Get_count(&st, MPI_INT, &cnt);
                ok = ok && rc == 0 && cnt == 1;
                int v = -1;
                MPI_Status st2;
                MPI_Recv(&v, 1, MPI_INT, st.MPI_SOURCE, st.MPI_TAG, MPI_COMM_WORLD, &st2);
                int s = v / 100, k = v % 100;
                ok = ok && s == st2.MPI_SOURCE && (s == 1 || s == 2) && k > last[s] && st2.MPI_TAG == 7 + (k & 1);
                if (s == 1 || s == 2) last[s] = k;
                o[m] = v;
            }
            ok = ok && last[1] == 3 && last[2] == 3;
            // synchronous (rendezvous) sends; the second one is truncated on purpose
            int* big = (int*)malloc(sizeof(int) * 300);
            MPI_Status st;
            int rc = MPI_Recv(big, 300, MPI_INT, 1, 99, MPI_COMM_WORLD, &st);
            ok = ok && rc == 0 && big[0] == 1000 && big[299] == 1299;
            rc = MPI_Recv(big, 10, MPI_INT, 2, 99, MPI_COMM_WORLD, &st);
            ok = ok && rc == MPI_ERR_TRUNCATE && big[9] == 2009 && big[10] == 1010;
            o[8] = rc;
            free(big);
        }
        // Sendrecv ring + PROC_NULL
        int tok = rank * 7, got = -1;
        MPI_Sendrecv(&tok, 1, MPI_INT, (rank + 1) % n, 3, &got, 1, MPI_INT, (rank + n - 1) % n, 3, MPI_COMM_WORLD,
                     MPI_STATUS_IGNORE);
        ok = ok && got == ((rank + n - 1) % n) * 7;
        MPI_Status stn;
        int dummy = 5;
        int rc = MPI_Recv(&dummy, 1, MPI_INT, MPI_PROC_NULL, 0, MPI_COMM_WORLD, &stn);
        ok = ok && rc == 0 && dummy == 5 && stn.MPI_SOURCE == MPI_PROC_NULL;
        rc = MPI_Send(&dummy, 1, MPI_INT, MPI_PROC_NULL, 0, MPI_COMM_WORLD);
        ok = ok && rc == 0;
        okp(p)[rank] = ok;
        return MPI_Finalize();
    }
};

// Failure detection without a GPU fault: rank 0 waits for a message nobody sends.  The bounded wait
// must end with MPI_ERR_OTHER; the other ranks skip the final barrier so the kernel ends.
struct Timeout {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        int rank = wrank();
        if (rank == 0) {
            int x = 0;
            int rc = MPI_Recv(&x, 1, MPI_INT, 1, 1234, MPI_COMM_WORLD, MPI_STATUS_IGNORE);
            outi(p, rank)[0] = rc;
            okp(p)[rank] = rc == MPI_ERR_OTHER;
        } else {
            okp(p)[rank] = 1;
        }
        return 0;
    }
};

// Derived datatypes: vector columns, subarray faces and contiguous blocks sent between ranks 0 and 1,
// checked element by element (results also copied out for a host-side check).
struct Datatypes {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        int rank = wrank();
        bool ok = true;
        double* grid = (double*)malloc(sizeof(double) * 6 * 6 * 6);
        double* recv = (double*)malloc(sizeof(double) * 64);
        for (int i = 0; i < 216; i++) grid[i] = rank * 1000.0 + i;
        for (int i = 0; i < 64; i++) recv[i] = -1;
        // column of a 6x6 matrix: vector(6, 1, 6)
        MPI_Datatype col, face, blk;
        MPI_Type_vector(6, 1, 6, MPI_DOUBLE, &col);
        MPI_Type_commit(&col);
        int sizes[3] = {6, 6, 6}, subs[3] = {4, 4, 1}, starts[3] = {1, 1, 4};
        MPI_Type_create_subarray(3, sizes, subs, starts, MPI_ORDER_C, MPI_DOUBLE, &face);
        MPI_Type_commit(&face);
        MPI_Type_contiguous(5, MPI_DOUBLE, &blk);
        MPI_Type_commit(&blk);
        int sz = 0;
        MPI_Type_size(face, &sz);
        ok = ok && sz == 16 * 8;
        if (rank == 0) {
            MPI_Send(grid + 2, 1, col, 1, 1, MPI_COMM_WORLD);     // column 2 of the first 6x6 plane
            MPI_Send(grid, 1, face, 1, 2, MPI_COMM_WORLD);        // x = 4 face of the interior
            MPI_Send(grid + 100, 2, blk, 1, 3, MPI_COMM_WORLD);   // 10 contiguous doubles
            // typed receive side: 16 contiguous doubles scattered into a face of my grid
            double packed[16];
            for (int i = 0; i < 16; i++) packed[i] = 5000.0 + i;
            MPI_Send(packed, 16, MPI_DOUBLE, 1, 4, MPI_COMM_WORLD);
        } else if (rank == 1) {
            MPI_Status st;
            MPI_Recv(recv, 6, MPI_DOUBLE, 0, 1, MPI_COMM_WORLD, &st);
            for (int i = 0; i < 6; i++) ok = ok && recv[i] == 2 + 6 * i;
            MPI_Recv(recv + 6, 16, MPI_DOUBLE, 0, 2, MPI_COMM_WORLD, &st);
            for (int z = 0; z < 4; z++)
                for (int y = 0; y < 4; y++) ok = ok && recv[6 + z * 4 + y] == (z + 1) * 36 + (y + 1) * 6 + 4;
            MPI_Recv(recv + 22, 10, MPI_DOUBLE, 0, 3, MPI_COMM_WORLD, &st);
            for (int i = 0; i < 10; i++) ok = ok && recv[22 + i] == 100 + i;
            MPI_Recv(grid, 1, face, 0, 4, MPI_COMM_WORLD, &st);
            for (int z = 0; z < 4; z++)
                for (int y = 0; y < 4; y++) ok = ok && grid[(z + 1) * 36 + (y + 1) * 6 + 4] == 5000.0 + z * 4 + y;
            ok = ok && grid[0] == 1000.0 && grid[4] == 1004.0;
            for (int i = 0; i < 32; i++) outd(p, rank)[i] = recv[i];
        }
        MPI_Type_free(&col);
        MPI_Type_free(&face);
        MPI_Type_free(&blk);
        free(grid);
        free(recv);
        okp(p)[rank] = ok;
        return MPI_Finalize();
    }
};

// Collectives on split communicators of uneven sizes (the reference has Bcast via p2p with wrong
// rank translation there, H1, and no sub-communicator Barrier).
struct SubcommColl {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        int rank = wrank(), n = 0;
        MPI_Comm_size(MPI_COMM_WORLD, &n);
        int color = rank % 3;
        MPI_Comm c;
        MPI_Comm_split(MPI_COMM_WORLD, color, -rank, &c);
        int cr = -1, cs = -1;
        MPI_Comm_rank(c, &cr);
        MPI_Comm_size(c, &cs);
        long long v[5], s[5];
        for (int i = 0; i < 5; i++) v[i] = rank * 10 + i;
        int rc = MPI_Allreduce(v, s, 5, MPI_LONG_LONG, MPI_SUM, c);
        bool ok = rc == 0;
        for (int i = 0; i < 5; i++) {
            long long e = 0;
            for (int q = color; q < n; q += 3) e += q * 10 + i;
            ok = ok && s[i] == e;
        }
        int b[4] = {0, 0, 0, 0};
        if (cr == cs - 1)
            for (int i = 0; i < 4; i++) b[i] = rank + i;
        rc = MPI_Bcast(b, 4, MPI_INT, cs - 1, c);
        int root_world = color;  // highest key -rank -> comm rank cs-1 is the smallest world rank
        ok = ok && rc == 0 && b[0] == root_world && b[3] == root_world + 3;
        rc = MPI_Barrier(c);
        ok = ok && rc == 0;
        int* g = (int*)malloc(sizeof(int) * cs);
        rc = MPI_Allgather(&rank, 1, MPI_INT, g, 1, MPI_INT, c);
        for (int i = 0; i < cs; i++) ok = ok && g[i] == color + 3 * (cs - 1 - i);
        free(g);
        outi(p, rank)[0] = cr;
        outi(p, rank)[1] = cs;
        outi(p, rank)[2] = s[0];
        okp(p)[rank] = ok;
        return MPI_Finalize();
    }
};

// Argument errors come back as MPI error codes; nothing traps.
struct Errors {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        int rank = wrank(), n = 0;
        MPI_Comm_size(MPI_COMM_WORLD, &n);
        bool ok = true;
        int x = 0;
        ok = ok && MPI_Send(&x, 1, MPI_INT, n + 5, 0, MPI_COMM_WORLD) == MPI_ERR_RANK;
        ok = ok && MPI_Send(&x, 1, (MPI_Datatype)999, 0, 0, MPI_COMM_WORLD) == MPI_ERR_TYPE;
        ok = ok && MPI_Send(&x, -1, MPI_INT, 0, 0, MPI_COMM_WORLD) == MPI_ERR_COUNT;
        ok = ok && MPI_Send(&x, 1, MPI_INT, 0, 0, (MPI_Comm)nullptr) == MPI_ERR_COMM;
        float f = 1.f, g = 0.f;
        // BAND is not defined on float (operators.cu IsTypeOpAllowed)
        ok = ok && MPI_Allreduce(&f, &g, 1, MPI_FLOAT, MPI_BAND, MPI_COMM_WORLD) == MPI_ERR_OP;
        ok = ok && MPI_Reduce(&f, &g, 1, MPI_FLOAT, MPI_SUM, n + 1, MPI_COMM_WORLD) == MPI_ERR_ROOT;
        okp(p)[rank] = ok;
        return MPI_Finalize();
    }
};

// Cartesian topologies: MPI_Dims_create on fixed cases (rank 0), a periodic/non-periodic 3D grid over
// the world, coordinates, ranks, shifts, MPI_Cart_sub and a neighbour exchange along each dimension.
// Values go to outi for the host to check against the restatement of the same rules.
//   outi[0..2] dims of the world grid   [3..5] coords   [6] Cart_rank(coords)   [7..12] shift (src, dst)
//   for dims 0..2 with disp 1   [13..14] Cart_sub({1,0,1}) size, rank   [15] Cartdim_get   [16] Topo_test
//   cart   [17] Topo_test world   [18..20] value received along dims 0..2 (-7 from MPI_PROC_NULL)
//   [21] Cart_rank of out-of-grid coords on the non-periodic dimension (error code)
//   rank 0 only: [24..] Dims_create cases, 4 entries each
struct Cart {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        int rank = wrank(), n = 0;
        MPI_Comm_size(MPI_COMM_WORLD, &n);
        long long* o = outi(p, rank);
        bool ok = true;
        int dims[3] = {0, 0, 0};
        ok = ok && MPI_Dims_create(n, 3, dims) == MPI_SUCCESS;
        const int periods[3] = {1, 0, 1};
        MPI_Comm cart = MPI_COMM_NULL;
        ok = ok && MPI_Cart_create(MPI_COMM_WORLD, 3, dims, periods, 1, &cart) == MPI_SUCCESS;
        int crank = -1;
        MPI_Comm_rank(cart, &crank);
        int coords[3] = {-1, -1, -1}, back = -1;
        ok = ok && MPI_Cart_coords(cart, crank, 3, coords) == MPI_SUCCESS;
        ok = ok && MPI_Cart_rank(cart, coords, &back) == MPI_SUCCESS;
        for (int i = 0; i < 3; i++) {
            o[i] = dims[i];
            o[3 + i] = coords[i];
        }
        o[6] = back;
        int src[3], dst[3];
        for (int d = 0; d < 3; d++) {
            ok = ok && MPI_Cart_shift(cart, d, 1, &src[d], &dst[d]) == MPI_SUCCESS;
            o[7 + 2 * d] = src[d];
            o[8 + 2 * d] = dst[d];
        }
        MPI_Comm sub = MPI_COMM_NULL;
        const int remain[3] = {1, 0, 1};
        ok = ok && MPI_Cart_sub(cart, remain, &sub) == MPI_SUCCESS;
        int ssize = -1, srank = -1;
        MPI_Comm_size(sub, &ssize);
        MPI_Comm_rank(sub, &srank);
        o[13] = ssize;
        o[14] = srank;
        int nd = -1, tc = -1, tw = -1;
        MPI_Cartdim_get(cart, &nd);
        MPI_Topo_test(cart, &tc);
        MPI_Topo_test(MPI_COMM_WORLD, &tw);
        o[15] = nd;
        o[16] = tc;
        o[17] = tw;
        for (int d = 0; d < 3; d++) {  // send my rank up dimension d, receive from below
            int got = -7;
            ok = ok && MPI_Sendrecv(&crank, 1, MPI_INT, dst[d], 30 + d, &got, 1, MPI_INT, src[d], 30 + d, cart,
                                    MPI_STATUS_IGNORE) == MPI_SUCCESS;
            o[18 + d] = got;
        }
        int far[3] = {coords[0], dims[1], coords[2]}, r2 = -1;
        o[21] = MPI_Cart_rank(cart, far, &r2);
        if (rank == 0) {
            const int cases[6][4] = {{12, 2, 0, 0}, {30, 3, 0, 0}, {16, 4, 0, 0}, {7, 2, 0, 0}, {24, 3, 3, 0}, {360, 3, 0, 0}};
            for (int k = 0; k < 6; k++) {
                int dd[4] = {0, 0, 0, 0};
                dd[1] = cases[k][2];  // a fixed second dimension where given
                const int rc = MPI_Dims_create(cases[k][0], cases[k][1], dd);
                o[24 + 4 * k] = rc;
                for (int i = 0; i < 3; i++) o[25 + 4 * k + i] = i < cases[k][1] ? dd[i] : 0;
            }
        }
        okp(p)[rank] = ok;
        return MPI_Finalize();
    }
};

// Back-to-back tiny collectives (one-barrier path, inline operands alternating between two slots by
// barrier parity) with per-iteration values and deliberately skewed ranks: every result is checked, so a
// slot overwritten while a slower rank still reads it would show.  Also on a split communicator.
//   outi[0] = first failing iteration (-1 if none)
struct TinyStress {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        int rank = wrank(), n = 0;
        MPI_Comm_size(MPI_COMM_WORLD, &n);
        MPI_Comm half;
        MPI_Comm_split(MPI_COMM_WORLD, rank & 1, rank, &half);
        int hn = 0, hr = 0;
        MPI_Comm_size(half, &hn);
        MPI_Comm_rank(half, &hr);
        long long bad = -1;
        int* all = (int*)p.p[3];  // optional int[n][n]: allgather rows
        for (int it = 0; it < 200 && bad < 0; it++) {
            if ((rank + it) % 7 == 0) {  // skew: some ranks arrive late
                const long long t0 = clock64();
                while (clock64() - t0 < 20000) {
                }
            }
            long long v[3] = {rank * 1000LL + it, -rank - it, (long long)it * rank}, s[3] = {0, 0, 0};
            MPI_Allreduce(v, s, 3, MPI_LONG_LONG, MPI_SUM, MPI_COMM_WORLD);
            const long long tri = (long long)n * (n - 1) / 2;
            if (s[0] != tri * 1000 + (long long)n * it || s[1] != -tri - (long long)n * it || s[2] != (long long)it * tri)
                bad = it;
            double d = rank + 0.25 * it, mx = 0;
            MPI_Allreduce(&d, &mx, 1, MPI_DOUBLE, MPI_MAX, half);
            const int top = (rank & 1) + 2 * (hn - 1);  // the half's highest world rank
            if (mx != top + 0.25 * it) bad = it;
            int root = it % n, b = rank == root ? it * 7 + root : -1;
            MPI_Bcast(&b, 1, MPI_INT, root, MPI_COMM_WORLD);
            if (b != it * 7 + root) bad = it;
            int mine = rank + it, red = -1;
            MPI_Reduce(&mine, &red, 1, MPI_INT, MPI_SUM, root, MPI_COMM_WORLD);
            if (rank == root && red != (int)(tri + (long long)n * it)) bad = it;
            if (all) {  // tiny allgather into a global buffer
                int* row = all + (size_t)rank * n;
                MPI_Allgather(&mine, 1, MPI_INT, row, 1, MPI_INT, MPI_COMM_WORLD);
                for (int q = 0; q < n; q++)
                    if (row[q] != q + it) bad = it;
            }
        }
        outi(p, rank)[0] = bad;
        okp(p)[rank] = bad < 0;
        (void)hr;
        return MPI_Finalize();
    }
};

// The small-message paths choose by message size only, so members may mix thread-local and global
// buffers and different (same-signature) datatypes: odd ranks use stack arrays and a strided type, even
// ranks global memory and contiguous types.  Ranks: 2..64.  p[3]: int scratch [n][288] (global): bcast
// [0, 4), allgather row [8, 138), alltoall send [140, 204), receive [208, 272).
struct TinyMixed {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        int rank = wrank(), n = 0;
        MPI_Comm_size(MPI_COMM_WORLD, &n);
        if (n > 64) {  // the local arrays hold 64 ranks (every member returns here alike)
            okp(p)[rank] = 0;
            return MPI_Finalize();
        }
        bool ok = true;
        int* g = (int*)p.p[3] + (size_t)rank * 288;
        const bool odd = rank & 1;
        MPI_Datatype vec;
        MPI_Type_vector(4, 1, 2, MPI_INT, &vec);
        MPI_Type_commit(&vec);
        int loc[8];
        for (int i = 0; i < 8; i++) loc[i] = -1;
        int vals[4] = {11, 22, 33, 44};
        // broadcast of 16 bytes: root contiguous, odd ranks into a strided local array
        if (rank == 0) MPI_Bcast(vals, 4, MPI_INT, 0, MPI_COMM_WORLD);
        else if (odd) MPI_Bcast(loc, 1, vec, 0, MPI_COMM_WORLD);
        else MPI_Bcast(g, 4, MPI_INT, 0, MPI_COMM_WORLD);
        for (int i = 0; i < 4 && rank != 0; i++) ok = ok && (odd ? loc[2 * i] == vals[i] && loc[2 * i + 1] == -1 : g[i] == vals[i]);
        // allgather of 2 ints per member
        int mine[2] = {rank, rank * 3}, lrow[128];
        int* grow = g + 8;
        if (odd) MPI_Allgather(mine, 2, MPI_INT, lrow, 2, MPI_INT, MPI_COMM_WORLD);
        else {
            grow[0] = mine[0];
            grow[1] = mine[1];
            MPI_Allgather(grow, 2, MPI_INT, grow + 2, 2, MPI_INT, MPI_COMM_WORLD);
        }
        for (int q = 0; q < n && ok; q++) {
            const int* r = odd ? lrow : grow + 2;
            ok = r[2 * q] == q && r[2 * q + 1] == 3 * q;
        }
        // alltoall of one int per pair: send q gets rank * 100 + q
        int ls[64], lr[64];
        int* gs = g + 140;
        int* gr = g + 208;
        for (int q = 0; q < n && q < 64; q++) (odd ? ls : gs)[q] = rank * 100 + q;
        if (odd) MPI_Alltoall(ls, 1, MPI_INT, lr, 1, MPI_INT, MPI_COMM_WORLD);
        else MPI_Alltoall(gs, 1, MPI_INT, gr, 1, MPI_INT, MPI_COMM_WORLD);
        for (int q = 0; q < n && ok; q++) ok = (odd ? lr : gr)[q] == q * 100 + rank;
        MPI_Type_free(&vec);
        okp(p)[rank] = ok;
        return MPI_Finalize();
    }
};

// Attribute caching (MPI-1.3 section 5.7; the reference declares MPI_Keyval_create, MPI_NULL_COPY_FN,
// MPI_NULL_DELETE_FN, mpi.cuh:95-110, and MPI_Attr_get/put, communicator.cuh:44-47, and does nothing or
// traps in them) and the timer (MPI_Wtime, MPI_Wtick).  outi[r][0] = copy/delete counter,
// outd[r][0..2] = Wtime before and after a world barrier, Wtick.
__device__ int attrs_copy(MPI_Comm, int, void* extra, void* in, void* out, int* flag) {
    (*(int*)extra) += 1;
    *(void**)out = in;
    *flag = 1;
    return MPI_SUCCESS;
}
__device__ int attrs_delete(MPI_Comm, int, void*, void* extra) {
    (*(int*)extra) += 100;
    return MPI_SUCCESS;
}
struct Attrs {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        const int rank = wrank();
        int n = 0;
        MPI_Comm_size(MPI_COMM_WORLD, &n);
        long long* oi = outi(p, rank);
        double* od = outd(p, rank);
        bool ok = true;
        const double wt = MPI_Wtick();
        ok = ok && wt > 0 && wt <= 1e-5;
        double prev = MPI_Wtime();
        for (int i = 0; i < 100; i++) {
            const double t = MPI_Wtime();
            ok = ok && t >= prev;
            prev = t;
        }
        od[0] = MPI_Wtime();
        MPI_Barrier(MPI_COMM_WORLD);
        od[1] = MPI_Wtime();
        od[2] = wt;
        int counter = 0;  // copies + 100 x deletes
        int value = 1000 + rank;
        int kv = MPI_KEYVAL_INVALID, kv_null = MPI_KEYVAL_INVALID, flag = -1;
        int* got = nullptr;
        ok = ok && MPI_Keyval_create(attrs_copy, attrs_delete, &kv, &counter) == MPI_SUCCESS;
        ok = ok && MPI_Keyval_create(MPI_NULL_COPY_FN, MPI_NULL_DELETE_FN, &kv_null, nullptr) == MPI_SUCCESS;
        ok = ok && kv != MPI_KEYVAL_INVALID && kv_null != MPI_KEYVAL_INVALID && kv != kv_null;
        MPI_Comm c1 = MPI_COMM_NULL, c2 = MPI_COMM_NULL;
        ok = ok && MPI_Comm_dup(MPI_COMM_WORLD, &c1) == MPI_SUCCESS;
        ok = ok && MPI_Attr_put(c1, kv, &value) == MPI_SUCCESS && MPI_Attr_put(c1, kv_null, &value) == MPI_SUCCESS;
        ok = ok && MPI_Attr_get(c1, kv, &got, &flag) == MPI_SUCCESS && flag == 1 && got == &value;
        ok = ok && MPI_Attr_get(MPI_COMM_WORLD, kv, &got, &flag) == MPI_SUCCESS && flag == 0;
        ok = ok && MPI_Comm_dup(c1, &c2) == MPI_SUCCESS && counter == 1;   // kv's copy function ran once
        got = nullptr;
        ok = ok && MPI_Attr_get(c2, kv, &got, &flag) == MPI_SUCCESS && flag == 1 && got == &value;
        ok = ok && MPI_Attr_get(c2, kv_null, &got, &flag) == MPI_SUCCESS && flag == 0;  // not copied
        int sum = 0;
        ok = ok && MPI_Allreduce(&value, &sum, 1, MPI_INT, MPI_SUM, c2) == MPI_SUCCESS;
        ok = ok && sum == 1000 * n + n * (n - 1) / 2;
        ok = ok && MPI_Attr_delete(c2, kv) == MPI_SUCCESS && counter == 101;
        ok = ok && MPI_Attr_get(c2, kv, &got, &flag) == MPI_SUCCESS && flag == 0;
        ok = ok && MPI_Attr_put(c1, kv, &value) == MPI_SUCCESS && counter == 201;  // replacing deletes first
        ok = ok && MPI_Comm_free(&c1) == MPI_SUCCESS && c1 == MPI_COMM_NULL && counter == 301;
        ok = ok && MPI_Comm_free(&c2) == MPI_SUCCESS && counter == 301;
        int* ub = nullptr;
        ok = ok && MPI_Attr_get(MPI_COMM_WORLD, MPI_TAG_UB, &ub, &flag) == MPI_SUCCESS && flag == 1 && ub &&
             *ub == MPI_TAG_UB;
        ok = ok && MPI_Keyval_free(&kv) == MPI_SUCCESS && kv == MPI_KEYVAL_INVALID;
        ok = ok && MPI_Attr_put(MPI_COMM_WORLD, GPUMPI_MAX_KEYVALS + 5, &value) == MPI_ERR_ARG;
        ok = ok && MPI_Keyval_free(&kv_null) == MPI_SUCCESS;
        oi[0] = counter;
        okp(p)[rank] = ok;
        return MPI_Finalize();
    }
};


// File and stream I/O over the device -> host channel (MPI-IO, MPI-3.1 chapter 13; the reference's
// tests/test_io_file_open.cu, test_io_file_access.cu, test_io_file_write.cu and
// toolchain_tests/basicIO cover open modes, size, read-back and views with its own semantics).
// p[3] = device string: a directory the program may create files in.  Files left for the host to check:
//   io_block.bin   rank r's ints r * 1000 + i, i < K, at ints [r K, (r + 1) K) (explicit offsets)
//   io_view.bin    view of 2 blocks of NW ints NW * n apart at disp r NW ints: rank r's ints r * 100 + i
//   io_shared.bin  one int per rank through the shared file pointer (a permutation of the ranks)
//   io_stdio.txt   rank 0's formatted line (gpumpi_fprintf)
// outi[r][0] = the first failed check (0 = all passed), outi[r][1..] = error codes seen.
__device__ void io_path(char* dst, const char* dir, const char* name) {
    int k = 0;
    for (; dir[k] && k < 200; k++) dst[k] = dir[k];
    dst[k++] = '/';
    for (int j = 0; name[j]; j++) dst[k++] = name[j];
    dst[k] = 0;
}
struct FileIO {
    static __device__ int run(const gpumpi_params& p) {
        MPI_Init(nullptr, nullptr);
        const int rank = wrank();
        int n = 0;
        MPI_Comm_size(MPI_COMM_WORLD, &n);
        long long* oi = outi(p, rank);
        const char* dir = (const char*)p.p[3];
        char path[256];
        int fail = 0, check = 0;
#define IO_CHECK(c)                      \
    do {                                 \
        check++;                         \
        if (!(c) && !fail) fail = check; \
    } while (0)
        constexpr int K = 300, NW = 50;
        MPI_File fh = MPI_FILE_NULL;
        MPI_Status st;
        // explicit offsets, read-back of the neighbour's block, size
        io_path(path, dir, "io_block.bin");
        IO_CHECK(MPI_File_open(MPI_COMM_WORLD, path, MPI_MODE_CREATE | MPI_MODE_RDWR, MPI_INFO_NULL, &fh) ==
                 MPI_SUCCESS);
        int* buf = (int*)malloc(sizeof(int) * 2 * K);
        for (int i = 0; i < K; i++) buf[i] = rank * 1000 + i;
        IO_CHECK(MPI_File_write_at(fh, (MPI_Offset)rank * K * 4, buf, K, MPI_INT, &st) == MPI_SUCCESS);
        int cnt = -1;
        MPI_Get_count(&st, MPI_INT, &cnt);
        IO_CHECK(cnt == K);
        MPI_Barrier(MPI_COMM_WORLD);
        const int nb = (rank + 1) % n;
        IO_CHECK(MPI_File_read_at(fh, (MPI_Offset)nb * K * 4, buf + K, K, MPI_INT, &st) == MPI_SUCCESS);
        bool same = true;
        for (int i = 0; i < K; i++) same = same && buf[K + i] == nb * 1000 + i;
        IO_CHECK(same);
        MPI_Offset size = -1;
        IO_CHECK(MPI_File_get_size(fh, &size) == MPI_SUCCESS && size == (MPI_Offset)n * K * 4);
        // individual pointer with an int view from this rank's block
        IO_CHECK(MPI_File_set_view(fh, (MPI_Offset)rank * K * 4, MPI_INT, MPI_INT, "native", MPI_INFO_NULL) ==
                 MPI_SUCCESS);
        IO_CHECK(MPI_File_seek(fh, 10, MPI_SEEK_SET) == MPI_SUCCESS);
        int two[2] = {-1, -1};
        IO_CHECK(MPI_File_read(fh, two, 2, MPI_INT, &st) == MPI_SUCCESS && two[0] == rank * 1000 + 10 &&
                 two[1] == rank * 1000 + 11);
        MPI_Offset pos = -1, byte = -1;
        IO_CHECK(MPI_File_get_position(fh, &pos) == MPI_SUCCESS && pos == 12);
        IO_CHECK(MPI_File_get_byte_offset(fh, pos, &byte) == MPI_SUCCESS && byte == (MPI_Offset)rank * K * 4 + 48);
        IO_CHECK(MPI_File_close(&fh) == MPI_SUCCESS && fh == MPI_FILE_NULL);
        // a non-contiguous view: 2 blocks of NW ints, NW * n ints apart, starting at this rank's slot
        io_path(path, dir, "io_view.bin");
        MPI_Datatype fileblk;
        MPI_Type_vector(2, NW, NW * n, MPI_INT, &fileblk);
        MPI_Type_commit(&fileblk);
        IO_CHECK(MPI_File_open(MPI_COMM_WORLD, path, MPI_MODE_CREATE | MPI_MODE_WRONLY, MPI_INFO_NULL, &fh) ==
                 MPI_SUCCESS);
        IO_CHECK(MPI_File_set_view(fh, (MPI_Offset)rank * NW * 4, MPI_INT, fileblk, "native", MPI_INFO_NULL) ==
                 MPI_SUCCESS);
        MPI_Datatype got_e, got_f;
        MPI_Offset got_d = -1;
        char rep[16];
        IO_CHECK(MPI_File_get_view(fh, &got_d, &got_e, &got_f, rep) == MPI_SUCCESS &&
                 got_d == (MPI_Offset)rank * NW * 4 && got_e == MPI_INT && got_f == fileblk && rep[0] == 'n');
        for (int i = 0; i < 2 * NW; i++) buf[i] = rank * 100 + i;
        IO_CHECK(MPI_File_write_all(fh, buf, 2 * NW, MPI_INT, &st) == MPI_SUCCESS);
        int dummy = 0;
        oi[1] = MPI_File_read(fh, &dummy, 1, MPI_INT, &st);  // write-only: MPI_ERR_AMODE
        IO_CHECK(oi[1] == MPI_ERR_AMODE);
        IO_CHECK(MPI_File_close(&fh) == MPI_SUCCESS);
        MPI_Type_free(&fileblk);
        // the shared file pointer: one int per rank, in the order the ranks arrive
        io_path(path, dir, "io_shared.bin");
        IO_CHECK(MPI_File_open(MPI_COMM_WORLD, path, MPI_MODE_CREATE | MPI_MODE_RDWR, MPI_INFO_NULL, &fh) ==
                 MPI_SUCCESS);
        IO_CHECK(MPI_File_set_view(fh, 0, MPI_INT, MPI_INT, "native", MPI_INFO_NULL) == MPI_SUCCESS);
        IO_CHECK(MPI_File_write_shared(fh, &rank, 1, MPI_INT, &st) == MPI_SUCCESS);
        MPI_Barrier(MPI_COMM_WORLD);
        MPI_Offset sp = -1;
        IO_CHECK(MPI_File_get_position_shared(fh, &sp) == MPI_SUCCESS && sp == n);
        IO_CHECK(MPI_File_seek_shared(fh, 0, MPI_SEEK_SET) == MPI_SUCCESS);
        int first = -1;
        if (rank == 0) IO_CHECK(MPI_File_read_shared(fh, &first, 1, MPI_INT, &st) == MPI_SUCCESS && first >= 0 && first < n);
        IO_CHECK(MPI_File_close(&fh) == MPI_SUCCESS);
        // errors: bad access modes, a missing file, writing a read-only file
        oi[2] = MPI_File_open(MPI_COMM_WORLD, path, MPI_MODE_RDONLY | MPI_MODE_RDWR, MPI_INFO_NULL, &fh);
        IO_CHECK(oi[2] == MPI_ERR_AMODE && fh == MPI_FILE_NULL);
        oi[3] = MPI_File_open(MPI_COMM_WORLD, path, MPI_MODE_CREATE | MPI_MODE_RDONLY, MPI_INFO_NULL, &fh);
        IO_CHECK(oi[3] == MPI_ERR_AMODE);
        io_path(path, dir, "io_missing.bin");
        oi[4] = MPI_File_open(MPI_COMM_WORLD, path, MPI_MODE_RDONLY, MPI_INFO_NULL, &fh);
        IO_CHECK(oi[4] == MPI_ERR_NO_SUCH_FILE);
        io_path(path, dir, "io_block.bin");
        IO_CHECK(MPI_File_open(MPI_COMM_WORLD, path, MPI_MODE_RDONLY, MPI_INFO_NULL, &fh) == MPI_SUCCESS);
        oi[5] = MPI_File_write(fh, buf, 1, MPI_INT, &st);
        IO_CHECK(oi[5] == MPI_ERR_READ_ONLY);
        IO_CHECK(MPI_File_close(&fh) == MPI_SUCCESS);
        // delete on close, and delete of a missing file
        io_path(path, dir, "io_tmp.bin");
        IO_CHECK(MPI_File_open(MPI_COMM_WORLD, path, MPI_MODE_CREATE | MPI_MODE_WRONLY | MPI_MODE_DELETE_ON_CLOSE,
                               MPI_INFO_NULL, &fh) == MPI_SUCCESS);
        IO_CHECK(MPI_File_close(&fh) == MPI_SUCCESS);
        if (rank == 0) {
            oi[6] = MPI_File_delete(path, MPI_INFO_NULL);
            IO_CHECK(oi[6] == MPI_ERR_NO_SUCH_FILE);
            // stdio through the host
            io_path(path, dir, "io_stdio.txt");
            gpumpi_FILE* f = gpumpi_fopen(path, "w");
            IO_CHECK(f != nullptr);
            IO_CHECK(gpumpi_fprintf(f, "rank %d of %d pi %.6f name %s hex %#x pad [%5d] [%-4s] %c%%\n", rank, n,
                                    3.14159265358979, "gb300", 255, 42, "ab", 'z') > 0);
            IO_CHECK(gpumpi_fputs("second line\n", f) == 0);
            IO_CHECK(gpumpi_fclose(f) == 0);
            f = gpumpi_fopen(path, "r");
            char line[8] = {};
            IO_CHECK(f && gpumpi_fread(line, 1, 4, f) == 4 && line[0] == 'r' && line[3] == 'k');
            IO_CHECK(gpumpi_fclose(f) == 0);
            IO_CHECK(gpumpi_printf("gpumpi_printf from rank %d of %d: %s %.3e\n", rank, n, "ok", 1234.5) > 0);
        }
        free(buf);
#undef IO_CHECK
        oi[0] = fail;
        okp(p)[rank] = fail == 0;
        return MPI_Finalize();
    }
};

}  // namespace

extern const gpumpi_prog_entry g_test_programs[] = {
    GPUMPI_PROGRAM(GPUMPI_T_SINGLE_INT, "single_int", SingleInt),
    GPUMPI_PROGRAM(GPUMPI_T_TRANSFER_ARRAY, "transfer_array", TransferArray),
    GPUMPI_PROGRAM(GPUMPI_T_SEND_RECV, "send_recv", SendRecv),
    GPUMPI_PROGRAM(GPUMPI_T_REPEAT_SEND_RECV, "repeat_send_recv", RepeatSendRecv),
    GPUMPI_PROGRAM(GPUMPI_T_NETWORK_FLOOD, "network_flood", NetworkFlood),
    GPUMPI_PROGRAM(GPUMPI_T_ALL_TO_ALL, "all_to_all", AllToAll),
    GPUMPI_PROGRAM(GPUMPI_T_REDUCE_INT16_PROD, "reduce_int16_prod", ReduceInt16Prod),
    GPUMPI_PROGRAM(GPUMPI_T_ALLREDUCE_F64, "allreduce_f64_sum", AllreduceF64),
    GPUMPI_PROGRAM(GPUMPI_T_ALLGATHER, "allgather_int", Allgather),
    GPUMPI_PROGRAM(GPUMPI_T_SCATTER, "scatter_int", Scatter),
    GPUMPI_PROGRAM(GPUMPI_T_SCATTERV, "scatterv_int", Scatterv),
    GPUMPI_PROGRAM(GPUMPI_T_COMM_RANK, "comm_rank", CommRank),
    GPUMPI_PROGRAM(GPUMPI_T_COMM_DUP, "comm_dup_isolation", CommDup),
    GPUMPI_PROGRAM(GPUMPI_T_COMM_SPLIT, "comm_split", CommSplit),
    GPUMPI_PROGRAM(GPUMPI_T_SAMPLE, "sample", Sample),
    GPUMPI_PROGRAM(GPUMPI_T_P2P_MATCHING, "p2p_matching", P2PMatching),
    GPUMPI_PROGRAM(GPUMPI_T_TIMEOUT, "timeout", Timeout),
    GPUMPI_PROGRAM(GPUMPI_T_DATATYPES, "datatypes", Datatypes),
    GPUMPI_PROGRAM(GPUMPI_T_SUBCOMM_COLL, "subcomm_coll", SubcommColl),
    GPUMPI_PROGRAM(GPUMPI_T_ERRORS, "errors", Errors),
    GPUMPI_PROGRAM(GPUMPI_T_CART, "cart", Cart),
    GPUMPI_PROGRAM(GPUMPI_T_TINY_STRESS, "tiny_stress", TinyStress),
    GPUMPI_PROGRAM(GPUMPI_T_TINY_MIXED, "tiny_mixed", TinyMixed),
    GPUMPI_PROGRAM(GPUMPI_T_ATTRS, "attrs", Attrs),
    GPUMPI_PROGRAM(GPUMPI_T_FILE_IO, "file_io", FileIO),
};
extern const int g_num_test_programs = sizeof(g_test_programs) / sizeof(g_test_programs[0]);
