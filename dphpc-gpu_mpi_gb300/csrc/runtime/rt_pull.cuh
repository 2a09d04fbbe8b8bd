// rt_pull.cuh — chunk executors of the pull collectives (Alltoall(v), Allgather(v), Gather(v),
// Scatter(v), Bcast): one chunk = up to one piece per thread of the block (tile mode) or one byte range
// of one large piece (parts mode).
//
// Replaces the reference's per-pair point-to-point transfers, each a one-thread byte memcpy
// (gpu_libs/gpu_mpi/mpi.cu:363-408 -> gpu_libs/gpu_libc/cuda_mpi.cu:168,323).
//
// Destination runs.  Consecutive pieces of a chunk whose destination ranges touch (receiver-major order
// with packed displacements, the Alltoallv of bucketed keys) form one run; a run's destination is cut
// into 16-byte blocks and each block is written once, whole, by one thread.  A block inside one piece is
// a "full" unit: its source is one or two aligned 16-byte loads, realigned with funnel shifts when source
// and destination disagree modulo 16.  A block straddling pieces is written by the thread of the piece
// holding its first byte inside the run (the run's first piece also writes the block holding the run's
// start), assembled from every piece of the run that covers it.  Only a run's two end blocks are written
// partially (byte-masked, as 1/2/4/8-byte stores), so no destination sector receives two partial writes
// from different pieces.
//
// Tile mode works per warp: each warp resolves 32 pieces (one per lane, warp shuffles for the run links
// and the prefix of full units), keeps their table in shared memory and copies their full units in tiles
// of 32*K consecutive units (K = 3) (lane l moves units l, l+32, ... so each access is contiguous and a lane's
// piece cursor only moves forward).  Warps never wait for one another inside a chunk.  STAGED moves the
// full units through shared-memory stages filled by bulk asynchronous copies instead of registers.
//
// Included by rt_coll.cuh after Piece, piece_of, piece_copy and the chunk scratch are defined.
#pragma once

namespace gpumpi {

enum : unsigned { PF_SLOW = 1, PF_EMPTY = 2, PF_CONTIG = 4 };

// A piece table: slots [base, base + cnt) of the chunk scratch with their prefix of full units `pr`
// (pr[k] = first unit of slot base + k, pr[cnt] = total).
struct PTab {
    int base, cnt;
    const long long* pr;
};

__device__ __forceinline__ unsigned long long full_base(int i) {
    return ((unsigned long long)s_chunk.p.d[i] + 15) & ~15ULL;
}

// bytes sh .. sh+15 of the 32-byte concatenation a:b (little endian), sh in 1..15
__device__ __forceinline__ uint4 realign16(const uint4& a, const uint4& b, int sh) {
    const int q = sh >> 2, r = (sh & 3) * 8;
    unsigned c0, c1, c2, c3, c4;
    switch (q) {
    case 0: c0 = a.x; c1 = a.y; c2 = a.z; c3 = a.w; c4 = b.x; break;
    case 1: c0 = a.y; c1 = a.z; c2 = a.w; c3 = b.x; c4 = b.y; break;
    case 2: c0 = a.z; c1 = a.w; c2 = b.x; c3 = b.y; c4 = b.z; break;
    default: c0 = a.w; c1 = b.x; c2 = b.y; c3 = b.z; c4 = b.w; break;
    }
    uint4 o;
    o.x = __funnelshift_r(c0, c1, r);
    o.y = __funnelshift_r(c1, c2, r);
    o.z = __funnelshift_r(c2, c3, r);
    o.w = __funnelshift_r(c3, c4, r);
    return o;
}

// n <= 16 source bytes starting at s (any alignment), returned from byte 0; only the aligned vectors that
// hold some of them are read (the rest of the result is unspecified)
__device__ __forceinline__ uint4 load_bytes16(unsigned long long s, int n) {
    const int h = (int)(s & 15);
    const uint4* sa = (const uint4*)(s - (unsigned long long)h);
    const uint4 a = __ldcg(sa);
    if (!h) return a;
    const uint4 b = h + n > 16 ? __ldcg(sa + 1) : make_uint4(0, 0, 0, 0);
    return realign16(a, b, h);
}

// word q of v (selects, no indexed array: an indexed array would live in local memory)
__device__ __forceinline__ unsigned word_of(const uint4& v, int q) {
    return q == 0 ? v.x : q == 1 ? v.y : q == 2 ? v.z : v.w;
}

// Stores bytes [lo, hi) of v to the 16-byte block at B with naturally aligned 1/2/4/8/16-byte stores.
__device__ __forceinline__ void store16_masked(unsigned long long B, const uint4& v, int lo, int hi) {
    if (lo == 0 && hi == 16) {
        __stcg((uint4*)B, v);
        return;
    }
    int x = lo;
    while (x < hi) {
        const int left = hi - x;
        const unsigned w = word_of(v, x >> 2);
        if ((x & 1) || left < 2) {
            __stcg((unsigned char*)(B + x), (unsigned char)(w >> ((x & 3) * 8)));
            x += 1;
        } else if ((x & 2) || left < 4) {
            __stcg((unsigned short*)(B + x), (unsigned short)(w >> ((x & 3) * 8)));
            x += 2;
        } else if ((x & 4) || left < 8) {
            __stcg((unsigned*)(B + x), w);
            x += 4;
        } else {
            __stcg((unsigned long long*)(B + x),
                   (unsigned long long)w | ((unsigned long long)word_of(v, (x >> 2) + 1) << 32));
            x += 8;
        }
    }
}

// Writes the block at B that piece i writes but that is not inside piece i: assembles the bytes of every
// piece of the run that covers it (piece i and its contiguous successors before slot `end`), then
// stores the covered part.
__device__ __forceinline__ void mixed_block(int i, unsigned long long B, int end) {
    uint4 out = make_uint4(0, 0, 0, 0);
    int lo = 16, hi = 0;
    const uint4 zero = make_uint4(0, 0, 0, 0);
    for (int p = i; p < end; p++) {
        const unsigned f = s_chunk.p.flag[p];
        if (f & PF_SLOW) break;
        if (f & PF_EMPTY) continue;
        if (p > i && !(f & PF_CONTIG)) break;
        const long long d = s_chunk.p.d[p], e = s_chunk.p.e[p];
        if ((unsigned long long)d >= B + 16) break;
        const int a = (int)(max((unsigned long long)d, B) - B);
        const int b = (int)(min((unsigned long long)e, B + 16) - B);
        if (b > a) {
            // source of block byte a, loaded as 16 bytes and shifted to position a
            const unsigned long long s = B + (unsigned long long)a + (unsigned long long)s_chunk.p.delta[p];
            uint4 v = load_bytes16(s, b - a);
            if (a) v = realign16(zero, v, 16 - a);
            unsigned mk[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                // bytes [a, b) of word q
                const int w0 = max(a, 4 * q), w1 = min(b, 4 * q + 4);
                mk[q] = w1 > w0 ? (unsigned)(((1ULL << (8 * (w1 - w0))) - 1) << (8 * (w0 - 4 * q))) : 0u;
            }
            out.x = (out.x & ~mk[0]) | (v.x & mk[0]);
            out.y = (out.y & ~mk[1]) | (v.y & mk[1]);
            out.z = (out.z & ~mk[2]) | (v.z & mk[2]);
            out.w = (out.w & ~mk[3]) | (v.w & mk[3]);
            lo = min(lo, a);
            hi = max(hi, b);
        }
        if ((unsigned long long)e >= B + 16) break;
    }
    if (hi > lo) store16_masked(B, out, lo, hi);
}

// The partial blocks piece t writes (at most two): the block holding its start when it starts a run,
// and the block holding its end when that block starts inside it.
__device__ __forceinline__ void piece_edges(int t, int end) {
    const unsigned f = s_chunk.p.flag[t];
    if (f & (PF_SLOW | PF_EMPTY)) return;
    const unsigned long long d = (unsigned long long)s_chunk.p.d[t], e = (unsigned long long)s_chunk.p.e[t];
    const unsigned long long bt = e & ~15ULL;
    const bool head = (d & 15) && !(f & PF_CONTIG);
    const bool tail = (e & 15) && bt >= d;
    for (int k = 0; k < 2; k++) {  // one inlined copy of the assembly for both blocks
        if (k == 0 ? !head : !tail) continue;
        mixed_block(t, k == 0 ? (d & ~15ULL) : bt, end);
    }
}

__device__ __forceinline__ long long full_units(long long d, long long e) {
    const long long f0 = (d + 15) & ~15LL, f1 = e & ~15LL;
    return f1 > f0 ? (f1 - f0) >> 4 : 0;
}

// local index of the piece holding unit u, from a cursor that only moves forward
__device__ __forceinline__ int unit_piece(const PTab& t, long long u, int cur) {
    if (t.pr[cur + 1] > u) return cur;
    if (cur + 2 <= t.cnt && t.pr[cur + 2] > u) return cur + 1;
    int lo = cur + 1, hi = t.cnt;  // pr[lo] <= u < pr[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (t.pr[mid] <= u) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Copies full units [u0, u1) of table t: tiles of 32*K units, tile k taken by worker warp k mod nwk;
// MIS: some source disagrees with its destination modulo 16 (two loads per unit, fewer units in flight).
template <int K, bool MIS>
__device__ __forceinline__ void flat_copy_t(const PTab& t, long long u0, long long u1, int lane, int wi, int nwk) {
    int cur = 0;
    for (long long tb = u0 + (long long)wi * 32 * K; tb < u1; tb += (long long)nwk * 32 * K) {
        uint4 a[K], b[K];
        unsigned long long dst[K];
        int sh[K];
#pragma unroll
        for (int k = 0; k < K; k++) {
            const long long u = tb + 32 * k + lane;
            sh[k] = -1;
            if (u < u1) {
                cur = unit_piece(t, u, cur);
                const int i = t.base + cur;
                const unsigned long long d = full_base(i) + 16ULL * (unsigned long long)(u - t.pr[cur]);
                const unsigned long long s = d + (unsigned long long)s_chunk.p.delta[i];
                const int h = MIS ? (int)(s & 15) : 0;
                const uint4* sa = (const uint4*)(s - (unsigned long long)h);
                // realigned units read two neighbouring vectors and lane l's second vector is lane l+1's
                // first: allocating them in L1 serves the second read there instead of from L2
                a[k] = MIS ? __ldca(sa) : __ldcg(sa);
                if (MIS && h) b[k] = __ldca(sa + 1);
                dst[k] = d;
                sh[k] = h;
            }
        }
#pragma unroll
        for (int k = 0; k < K; k++) {
            if (sh[k] < 0) continue;
            if (MIS && sh[k]) __stcg((uint4*)dst[k], realign16(a[k], b[k], sh[k]));
            else __stcg((uint4*)dst[k], a[k]);
        }
    }
}

// Three units in flight per lane on both paths.  Measured at 1024 ranks (GB/s of algorithmic bytes,
// same box): uniform 1 KiB pieces (aligned) K=3 5,154, K=4 4,888, K=6 4,780; uneven pieces of U[0,512]
// int32 (misaligned) K=3 4,095, K=2 3,935, K=4 3,613 (more units spill under the 64-register cap);
// K=3 is also the fastest on U[0,128] pieces and on the bucket-sort shape.
// Cache operators, same box and shapes (uneven 1 MiB / uniform 1 MiB / bucket-sort shape): L2-only
// loads and stores everywhere 4,068-4,078 / 5,073-5,080 / 2,484-2,498; misaligned loads through L1
// 4,167-4,177 / 5,059-5,072 / 2,461-2,510; streaming (evict-first) loads on the misaligned path
// 3,897-3,911 / - / 2,429-2,452; an L2 evict-first policy on every access 3,979-3,994 / 5,013-5,030 /
// 2,656; evict-first loads and stores everywhere 4,097-4,109 / 5,032-5,039 / 2,650-2,658, whose gain on
// the bucket-sort shape (2 x 128 MiB per call, about twice the L2) depends on how much of the previous
// call's data the L2 still holds.
__device__ __noinline__ void flat_copy_aligned(PTab t, long long u0, long long u1, int lane, int wi, int nwk) {
    flat_copy_t<3, false>(t, u0, u1, lane, wi, nwk);
}
__device__ __noinline__ void flat_copy_mis(PTab t, long long u0, long long u1, int lane, int wi, int nwk) {
    flat_copy_t<3, true>(t, u0, u1, lane, wi, nwk);
}

// ---- STAGED: a warp moves its share of the full units through two shared-memory stages filled by bulk
// asynchronous copies (cp.async.bulk global -> shared, completion counted in bytes on one mbarrier per
// stage).  Lanes issue one bulk copy per piece segment (the aligned source vectors of the segment, one
// more when source and destination disagree modulo 16), so a warp keeps two stages of several KiB in
// flight without registers; the lanes then write the 16-byte blocks from shared memory, realigned where
// needed.  While one stage drains the other is in flight.
struct SegRec {
    long long lo;  // first unit of the segment
    int off;       // byte offset of its first source vector in the stage
    int piece;     // local index in the table
};
constexpr int SP_HDR = 128 + 2 * 32 * (int)sizeof(SegRec);  // 2 mbarriers (padded) + 2 segment tables

__device__ __forceinline__ int staged_pull_stage_bytes(int nt) {
    const int q = (c_rt.dyn_smem / (nt >> 5)) & ~127;
    const int h = ((q - SP_HDR) / 2) & ~127;
    return h;
}

// `warp` selects this warp's shared-memory region; the warp moves share wi of nwk of [u0, u1)
__device__ __noinline__ bool staged_copy(PTab t, long long u0, long long u1, int lane, int warp, int nw, int wi,
                                         int nwk) {
    const int q = (c_rt.dyn_smem / nw) & ~127;
    const int H = ((q - SP_HDR) / 2) & ~127;
    const long long per = (u1 - u0 + nwk - 1) / nwk;
    const long long wb = min(u1, u0 + per * wi), we = min(u1, wb + per);
    if (wb >= we) return true;
    unsigned char* base = g_dyn_smem + (size_t)warp * q;
    unsigned long long* bar = (unsigned long long*)base;
    SegRec* seg = (SegRec*)(base + 128);
    unsigned char* stages = base + SP_HDR;
    if (lane == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
    }
    fence_proxy_async_global();
    __syncwarp();
    long long x = wb;  // next unit to issue (warp-uniform, like everything below but the per-lane segment)
    int cur = 0;       // local piece holding x
    long long slo[2] = {0, 0}, shi[2] = {0, 0};
    int nseg[2] = {0, 0};
    unsigned par[2] = {0, 0};
    bool busy[2] = {false, false};

    auto issue = [&](int st) {
        slo[st] = shi[st] = x;
        nseg[st] = 0;
        if (x >= we) return;
        cur = unit_piece(t, x, cur);
        const int li = cur + lane;
        const int i = t.base + li;
        long long lo = x, hi = x;
        int h = 0, nvec = 0;
        if (li < t.cnt) {
            lo = max(x, t.pr[li]);
            hi = min(we, t.pr[li + 1]);
            if (hi > lo) {
                h = (int)(s_chunk.p.delta[i] & 15);
                if (hi - lo > (long long)(H >> 4)) hi = lo + (H >> 4);
                nvec = (int)(hi - lo) + (h ? 1 : 0);
            } else {
                hi = lo;
            }
        }
        int end = nvec * 16;  // inclusive scan of the stage bytes over the lanes
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, end, o);
            if (lane >= o) end += y;
        }
        const int off = end - nvec * 16;
        if (nvec > 0 && off + nvec * 16 > H) {  // cut at the stage boundary; later lanes take nothing
            const int room = (H - off) / 16 - (h ? 1 : 0);
            if (off >= H || room <= 0) {
                nvec = 0;
                hi = lo;
            } else {
                hi = lo + room;
                nvec = room + (h ? 1 : 0);
            }
        }
        const unsigned ball = __ballot_sync(0xffffffffu, nvec > 0);
        const int last = 31 - __clz((int)ball);  // lane 0 always keeps a unit: ball != 0
        const int total = __shfl_sync(0xffffffffu, off + nvec * 16, last);
        const long long xn = __shfl_sync(0xffffffffu, hi, last);
        if (lane <= last) {
            SegRec r;
            r.lo = lo;
            r.off = off;
            r.piece = li;
            seg[st * 32 + lane] = r;
        }
        if (lane == 0) mbar_expect_tx(&bar[st], (unsigned)total);
        __syncwarp();
        if (nvec > 0) {
            const unsigned long long src = full_base(i) + 16ULL * (unsigned long long)(lo - t.pr[li]) +
                                           (unsigned long long)s_chunk.p.delta[i];
            tma_load_1d(stages + st * H + off, (const void*)(src & ~15ULL), (unsigned)(nvec * 16), &bar[st]);
        }
        __syncwarp();
        shi[st] = xn;
        nseg[st] = last + 1;
        busy[st] = true;
        x = xn;
    };

    bool ok = true;
    issue(0);
    issue(1);
    int st = 0;
    while (shi[st] > slo[st]) {
        const bool landed = mbar_wait_bounded(&bar[st], par[st]);
        if (!__all_sync(0xffffffffu, landed)) {  // warp-uniform outcome: the lanes shuffle together below
            ok = false;
            break;
        }
        par[st] ^= 1u;
        busy[st] = false;
        const SegRec* sg = seg + st * 32;
        const unsigned char* sb = stages + st * H;
        const long long m1 = shi[st];
        const int ns = nseg[st];
        int jx = 0;
        for (long long m = slo[st] + lane; m < m1; m += 32) {
            while (jx + 1 < ns && sg[jx + 1].lo <= m) jx++;
            const int li = sg[jx].piece;
            const int i = t.base + li;
            const int h = (int)(s_chunk.p.delta[i] & 15);
            const uint4* sp = (const uint4*)(sb + sg[jx].off + 16 * (m - sg[jx].lo));
            const uint4 a = sp[0];
            uint4* d = (uint4*)(full_base(i) + 16ULL * (unsigned long long)(m - t.pr[li]));
            __stcg(d, h ? realign16(a, sp[1], h) : a);
        }
        __syncwarp();  // the stage is drained before it is refilled
        issue(st);
        st ^= 1;
    }
    bool drained = true;
    if (!ok) {
        // a stage did not complete in time: let any copy still in flight land before the shared memory is
        // reused (bounded), and report.  The error record raises the launch's abort flag, after which no
        // block issues STAGED copies again, so barriers whose copies never landed are left as they are.
        if (lane == 0) record_error(GPUMPI_ERR_OTHER, GPUMPI_ERR_TIMEOUT, __LINE__, wb);
        for (int k = 0; k < 2; k++)
            if (busy[k]) drained = mbar_wait_bounded(&bar[k], par[k]) && drained;
        drained = __all_sync(0xffffffffu, drained);
    }
    __syncwarp();
    if (lane == 0 && drained) {
        mbar_inval(&bar[0]);
        mbar_inval(&bar[1]);
    }
    return ok;
}

__device__ __forceinline__ void copy_units(const JobParams* j, const PTab& t, long long u0, long long u1, bool mis,
                                           int lane, int warp, int nw, int wi, int nwk) {
    if (j->variant == GPUMPI_VARIANT_STAGED && !ld_relaxed(c_rt.abort_flag))
        staged_copy(t, u0, u1, lane, warp, nw, wi, nwk);
    else if (mis) flat_copy_mis(t, u0, u1, lane, wi, nwk);
    else flat_copy_aligned(t, u0, u1, lane, wi, nwk);
}

// Resolves piece p: destination range, source offset and flags (PF_SLOW / PF_EMPTY).
__device__ __forceinline__ unsigned resolve_piece(const JobParams* j, Job* jg, long long p, bool report,
                                                  long long& d, long long& e, long long& delta) {
    Piece pc;
    piece_of(j, p, pc);
    if (report && pc.trunc) atomicOr(&jg->err, 1u);
    const bool fast = !pc.sdesc && !pc.rdesc && is_global_ptr(pc.src) && is_global_ptr(pc.dst);
    d = (long long)(unsigned long long)pc.dst;
    e = d + (pc.bytes > 0 ? pc.bytes : 0);
    delta = (long long)((unsigned long long)pc.src - (unsigned long long)pc.dst);
    return pc.bytes <= 0 ? PF_EMPTY : (fast ? 0u : PF_SLOW);
}

// tile mode: pieces [p0, p0 + np), np <= 32 * warps; warp w handles pieces [w * pw, (w + 1) * pw) on its
// own, pw = ceil(np / warps), so every warp has work even when the chunk holds few pieces
__device__ __forceinline__ void pull_tile(const JobParams* j, Job* jg, long long p0, int np, int tid, int nt) {
    const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
    const int pw = (np + nw - 1) / nw;
    const int base = warp * 32;          // this warp's slots in the table
    const int first = warp * pw;         // its first piece in the chunk
    const int cnt = min(pw, np - first);
    if (cnt <= 0) return;
    long long d = 0, e = 0, delta = 0;
    unsigned f = PF_EMPTY;
    if (lane < cnt) f = resolve_piece(j, jg, p0 + first + lane, true, d, e, delta);
    // run link: the nearest previous non-empty lane must be a fast piece ending where this one starts
    int key = (lane < cnt && !(f & PF_EMPTY)) ? lane : -1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, key, o);
        if (lane >= o) key = max(key, y);
    }
    int prev = __shfl_up_sync(0xffffffffu, key, 1);
    if (lane == 0) prev = -1;
    const long long pe = __shfl_sync(0xffffffffu, e, prev < 0 ? 0 : prev);
    const unsigned pfl = __shfl_sync(0xffffffffu, f, prev < 0 ? 0 : prev);
    if (!(f & (PF_SLOW | PF_EMPTY)) && prev >= 0 && !(pfl & PF_SLOW) && pe == d) f |= PF_CONTIG;
    // prefix of full units over the warp's pieces
    const long long fc = (f & (PF_SLOW | PF_EMPTY)) ? 0 : full_units(d, e);
    long long x = fc;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    const long long total = __shfl_sync(0xffffffffu, x, 31);
    const bool mis = __any_sync(0xffffffffu, fc > 0 && (delta & 15) != 0);
    const unsigned slow = __ballot_sync(0xffffffffu, (f & PF_SLOW) != 0);
    long long* pr = s_chunk.p.pref[warp];
    s_chunk.p.d[base + lane] = d;
    s_chunk.p.e[base + lane] = e;
    s_chunk.p.delta[base + lane] = delta;
    s_chunk.p.flag[base + lane] = (unsigned char)f;
    pr[lane] = x - fc;
    if (lane == 31) pr[32] = total;
    __syncwarp();
    if (lane < cnt) piece_edges(base + lane, base + cnt);
    PTab t;
    t.base = base;
    t.cnt = cnt;
    t.pr = pr;
    copy_units(j, t, 0, total, mis, lane, warp, nw, 0, 1);
    for (unsigned m = slow; m; m &= m - 1) {  // derived datatypes / non-global buffers: whole warp per piece
        Piece pc;
        piece_of(j, p0 + first + (__ffs(m) - 1), pc);
        piece_copy(pc, 0, pc.bytes, lane, 32);
    }
    __syncwarp();  // this warp's table is free for its next chunk
}

// parts mode: unit range `part` of `parts` of piece p, whole block
__device__ __forceinline__ void pull_part(const JobParams* j, Job* jg, long long p, int part, int parts, int tid,
                                          int nt) {
    const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
    if (tid == 0) {
        long long d, e, delta;
        const unsigned f = resolve_piece(j, jg, p, part == 0, d, e, delta);
        s_chunk.p.d[0] = d;
        s_chunk.p.e[0] = e;
        s_chunk.p.delta[0] = delta;
        s_chunk.p.flag[0] = (unsigned char)f;
        s_chunk.p.pref[0][0] = 0;
        s_chunk.p.pref[0][1] = (f & (PF_SLOW | PF_EMPTY)) ? 0 : full_units(d, e);
        if (part == 0) piece_edges(0, 1);
    }
    bar_sync(BAR_TASK, nt);
    if (s_chunk.p.flag[0] & PF_SLOW) {
        Piece pc;
        piece_of(j, p, pc);
        const long long per = ((pc.bytes + parts - 1) / parts + 15) & ~15LL;
        const long long b0 = per * part, b1 = min(pc.bytes, b0 + per);
        piece_copy(pc, b0, b1, tid, nt);
        return;
    }
    const long long units = s_chunk.p.pref[0][1];
    const long long per = (units + parts - 1) / parts;
    const long long u0 = min(units, per * part), u1 = min(units, u0 + per);
    PTab t;
    t.base = 0;
    t.cnt = 1;
    t.pr = s_chunk.p.pref[0];
    copy_units(j, t, u0, u1, units > 0 && (s_chunk.p.delta[0] & 15) != 0, lane, warp, nw, warp, nw);
}

__device__ __forceinline__ void pull_chunk(const JobParams* j, Job* jg, long long idx, int tid, int nt) {
    if (j->vec > 1) {
        pull_part(j, jg, idx / j->vec, (int)(idx % j->vec), j->vec, tid, nt);
        return;
    }
    const long long p0 = idx * j->tile;
    const long long np = min(j->count - p0, (long long)j->tile);
    pull_tile(j, jg, p0, (int)np, tid, nt);
}

}  // namespace gpumpi
