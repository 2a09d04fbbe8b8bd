// rt_types.cuh — predefined and derived datatypes, and the typed (pack/unpack-fused) copy.
//
// The reference knows only the 30 predefined types (gpu_libs/gpu_mpi/mpi_types_list.cuh:3-33,
// plainTypeSize at gpu_libs/gpu_mpi/datatypes.cu:10-15) and stubs MPI_Type_contiguous /
// MPI_Type_commit / MPI_Type_size (gpu_libs/gpu_mpi/mpi.cu:237-245,287-290).  Derived types here follow
// the MPI standard: a type is "block bytes repeated over up to 4 strided levels", which covers
// contiguous, vector, hvector and C-order subarray of up to 3 dimensions (the halo-exchange faces).
// A message is moved in ONE pass: each thread maps its packed-stream offset to a source address
// (sender's type map) and a destination address (receiver's type map); nothing is packed first.
#pragma once
#include "rt_core.cuh"

namespace gpumpi {

// element sizes, same table as include/gpumpi_abi.h numbering (LP64, long double stored as double)
__device__ __forceinline__ int predefined_size(int dt) {
    switch (dt) {
    case GPUMPI_CHAR: case GPUMPI_SIGNED_CHAR: case GPUMPI_UNSIGNED_CHAR: case GPUMPI_C_BOOL:
    case GPUMPI_INT8_T: case GPUMPI_UINT8_T: case GPUMPI_BYTE: return 1;
    case GPUMPI_SHORT: case GPUMPI_UNSIGNED_SHORT: case GPUMPI_INT16_T: case GPUMPI_UINT16_T: return 2;
    case GPUMPI_INT: case GPUMPI_UNSIGNED: case GPUMPI_FLOAT: case GPUMPI_WCHAR: case GPUMPI_INT32_T:
    case GPUMPI_UINT32_T: return 4;
    case GPUMPI_LONG: case GPUMPI_LONG_LONG_INT: case GPUMPI_LONG_LONG: case GPUMPI_UNSIGNED_LONG:
    case GPUMPI_UNSIGNED_LONG_LONG: case GPUMPI_DOUBLE: case GPUMPI_LONG_DOUBLE: case GPUMPI_INT64_T:
    case GPUMPI_UINT64_T: case GPUMPI_C_COMPLEX: case GPUMPI_C_FLOAT_COMPLEX: case GPUMPI_2INT:
    case GPUMPI_FLOAT_INT: case GPUMPI_SHORT_INT: return 8;
    case GPUMPI_C_DOUBLE_COMPLEX: case GPUMPI_C_LONG_DOUBLE_COMPLEX: case GPUMPI_DOUBLE_INT:
    case GPUMPI_LONG_INT: case GPUMPI_LONG_DOUBLE_INT: return 16;
    default: return -1;
    }
}

__device__ __forceinline__ bool is_derived(int dt) { return dt >= GPUMPI_DERIVED_BASE; }

// Descriptors of the predefined types (defined in the runtime translation unit), so that every
// handle resolves to an address any rank can read.
extern __device__ TypeDesc g_predef_types[GPUMPI_NUM_PREDEFINED_TYPES];

// Descriptor of datatype handle dt; derived handles encode their owner rank and table slot.
__device__ __forceinline__ const TypeDesc* resolve_type(int dt) {
    if (dt >= 0 && dt < GPUMPI_NUM_PREDEFINED_TYPES) return &g_predef_types[dt];
    if (is_derived(dt)) {
        long long idx = (long long)dt - GPUMPI_DERIVED_BASE;
        long long total = (long long)c_rt.nranks * c_rt.max_types;
        if (idx < total) {
            const TypeDesc* t = &c_rt.types[idx];
            if (t->in_use) return t;
        }
    }
    return nullptr;
}

__device__ __forceinline__ bool desc_contiguous(const TypeDesc* t) {
    return t->nlev == 0 && t->size == t->extent && t->lb == 0;
}

// byte address of packed offset `off` inside `count` elements of type t starting at base
__device__ __forceinline__ long long desc_map(const TypeDesc* t, long long off) {
    long long e = off / t->size;
    long long q = off - e * t->size;
    long long blk = q / t->block;
    long long w = q - blk * t->block;
    long long addr = t->lb + e * t->extent + w;
    for (int l = 0; l < t->nlev; l++) {
        long long c = t->cnt[l];
        long long i = blk % c;
        blk /= c;
        addr += i * t->stride[l];
    }
    return addr;
}

// Unsigned 32-bit division by a divisor fixed for the life of a datatype, as a multiply-high and two
// shifts (division by invariant integers, Granlund & Montgomery 1994): with l = ceil(log2 d) and
// m = floor(2^32 (2^l - d) / d) + 1, n / d = (t + ((n - t) >> min(l, 1))) >> max(l - 1, 0), t = mulhi(m, n),
// exact for every 32-bit n.
struct FastDiv {
    unsigned m, s1, s2;
    __device__ __forceinline__ void init(unsigned d) {
        if (d == 0) d = 1;
        const unsigned l = d > 1 ? 32u - (unsigned)__clz((int)(d - 1)) : 0u;
        m = (unsigned)((((unsigned long long)1 << 32) * (((unsigned long long)1 << l) - d)) / d + 1);
        s1 = l < 1 ? l : 1;
        s2 = l > 1 ? l - 1 : 0;
    }
};

__device__ __forceinline__ long long pow2_div(long long v) {  // largest power of two dividing v (<= 16)
    if (v == 0) return 16;
    long long a = v & -v;
    return a > 16 ? 16 : a;
}

// Completes a descriptor once its shape is final: the copy unit it allows and the image of its 32-bit
// mapping with the division constants, so that no copy divides by a variable and a copying warp reads the
// whole mapping with one 16-byte load per lane.
__device__ __forceinline__ void desc_prepare(TypeDesc* t) {
    long long u = 16;
    u = min(u, pow2_div(t->block));
    u = min(u, pow2_div(t->size));
    u = min(u, pow2_div(t->extent));
    u = min(u, pow2_div(t->lb));
    for (int l = 0; l < t->nlev; l++) u = min(u, pow2_div(t->stride[l]));
    t->unit = (int)u;
    TypeImg& g = t->img;
    const long long v[4] = {t->size, t->block, t->cnt[0], t->cnt[1]};
    for (int k = 0; k < 4; k++) {
        const unsigned dv = v[k] > 0 && v[k] <= 0x7fffffffLL ? (unsigned)v[k] : 1u;
        FastDiv f;
        f.init(dv);
        g.d[k] = dv;
        g.m[k] = f.m;
        g.sh[k] = f.s1 | (f.s2 << 8);
    }
    g.lb = t->lb;
    g.extent = t->extent;
    for (int l = 0; l < 3; l++) g.st[l] = t->stride[l];
    g.nlev = t->nlev;
    t->fd_ready = t->size >= 0 && t->size <= 0x7fffffffLL && t->nlev <= 3;
    g.fast_unit = t->fd_ready ? t->unit : 0;
}

// Unit (1..16 bytes) that divides every block, stride, extent, offset and base address involved.
__device__ __forceinline__ int typed_unit(const TypeDesc* s, const void* sb, const TypeDesc* d, const void* db) {
    long long u = 16;
    const TypeDesc* ts[2] = {s, d};
    for (int k = 0; k < 2; k++) {
        const TypeDesc* t = ts[k];
        if (!t) continue;
        if (t->fd_ready) {
            u = min(u, (long long)t->unit);
            continue;
        }
        u = min(u, pow2_div(t->block));
        u = min(u, pow2_div(t->size));
        u = min(u, pow2_div(t->extent));
        u = min(u, pow2_div(t->lb));
        for (int l = 0; l < t->nlev; l++) u = min(u, pow2_div(t->stride[l]));
    }
    u = min(u, pow2_div((long long)(size_t)sb));
    u = min(u, pow2_div((long long)(size_t)db));
    return (int)u;
}

template <int U> struct UnitType;
template <> struct UnitType<16> { using T = uint4; };
template <> struct UnitType<8> { using T = unsigned long long; };
template <> struct UnitType<4> { using T = unsigned; };
template <> struct UnitType<2> { using T = unsigned short; };
template <> struct UnitType<1> { using T = unsigned char; };

template <int U, bool CG>
__device__ __forceinline__ typename UnitType<U>::T load_unit(const char* s) {
    using T = typename UnitType<U>::T;
    if constexpr (U >= 4) {
        if constexpr (CG) return __ldcg((const T*)s);
        else return *(const T*)s;
    } else {
        return *(const volatile T*)s;
    }
}

template <int U, bool CG>
__device__ __forceinline__ void store_unit(char* d, typename UnitType<U>::T v) {
    using T = typename UnitType<U>::T;
    if constexpr (U >= 4 && CG) __stcg((T*)d, v);
    else *(T*)d = v;
}

// ---- 32-bit mapping through a per-warp copy of the descriptor in shared memory ----
// A copy group is one thread or whole warps, so each warp owns one slot pair.  Reading the fields from
// shared memory at every use (volatile) keeps the loop's registers for the data in flight: with both
// descriptors in registers the loop spills, and a spilled load serialises the memory round trips.
struct DescS {
    TypeImg t;
    int same;                    // (destination slot) both sides have the same mapping, lb aside
    int pad;
    long long shift;             // (destination slot) destination lb - source lb, when same
};
constexpr int kMaxWarps = 8;
constexpr int kImgVecs = (int)(sizeof(TypeImg) / 16);
static_assert(sizeof(TypeImg) % 16 == 0 && kImgVecs <= 8, "a mapping image is at most eight 16-byte vectors");
__shared__ DescS s_tdesc[kMaxWarps][2];

// Lane l < kImgVecs copies vector l of the source image, lane 8 + l that of the destination image
// (a null descriptor's slot is left alone): the whole mapping in one memory round trip per warp.
__device__ __forceinline__ void img_load_lane(DescS* slot, const TypeDesc* st_, const TypeDesc* dt_, int l32) {
    const int k = l32 & 7;
    const TypeDesc* t = l32 < 8 ? st_ : l32 < 16 ? dt_ : nullptr;
    if (t && k < kImgVecs) ((uint4*)&slot[l32 >> 3].t)[k] = ((const uint4*)&t->img)[k];
}

// Both images map every packed offset to the same address up to lb: equal divisors, levels, extent and
// the strides of the levels in use (the multipliers follow from the divisors).
__device__ __forceinline__ bool same_mapping(const volatile TypeImg* a, const volatile TypeImg* b) {
    bool eq = a->nlev == b->nlev && a->extent == b->extent;
    for (int k = 0; k < 4; k++) eq = eq && a->d[k] == b->d[k];
    for (int l = 0; l < 3; l++) eq = eq && (l >= a->nlev || a->st[l] == b->st[l]);
    return eq;
}

__device__ __forceinline__ unsigned fdiv_s(const volatile TypeImg* t, int k, unsigned n) {
    const unsigned th = __umulhi(t->m[k], n);
    const unsigned sh = t->sh[k];
    return (th + ((n - th) >> (sh & 255u))) >> (sh >> 8);
}

// Byte address of packed offset off.  q < size = block * cnt[0] * ... * cnt[nlev-1], so the outermost
// level's index is the last quotient and needs no division.
__device__ __forceinline__ long long map_s(const volatile TypeImg* t, unsigned off) {
    const unsigned e = fdiv_s(t, 0, off);
    const unsigned q = off - e * t->d[0];
    const unsigned blk = fdiv_s(t, 1, q);
    long long a = t->lb + (long long)e * t->extent + (q - blk * t->d[1]);
    const int nl = t->nlev;
    if (nl == 1) {
        a += (long long)blk * t->st[0];
    } else if (nl == 2) {
        const unsigned b1 = fdiv_s(t, 2, blk);
        a += (long long)(blk - b1 * t->d[2]) * t->st[0] + (long long)b1 * t->st[1];
    } else if (nl == 3) {
        const unsigned b1 = fdiv_s(t, 2, blk);
        const unsigned b2 = fdiv_s(t, 3, b1);
        a += (long long)(blk - b1 * t->d[2]) * t->st[0] + (long long)(b1 - b2 * t->d[3]) * t->st[1] +
             (long long)b2 * t->st[2];
    }
    return a;
}

// CG selects L2-only accesses; legal only when both buffers are in global memory.
template <int U, bool CG>
__device__ __forceinline__ void typed_copy_fast(char* db, bool dmap, const char* sb, bool smap, unsigned b0, unsigned b1,
                                             int lane, int nl) {
    const volatile DescS* ss_ = &s_tdesc[threadIdx.x >> 5][0];
    const volatile DescS* ds_ = &s_tdesc[threadIdx.x >> 5][1];
    const volatile TypeImg* ss = &ss_->t;
    const volatile TypeImg* ds = &ds_->t;
    const bool same = smap && dmap && ds_->same;
    if (same) db += ds_->shift;
    const unsigned step = (unsigned)nl * U;
    unsigned off = b0 + (unsigned)lane * U;
    // K loads issued before the K stores: a strided unit is its own memory round trip, and a store
    // followed by the next load would serialise them (the compiler cannot move a load above a store it
    // cannot prove disjoint).
    constexpr int K = 4;
    using T = typename UnitType<U>::T;
    for (; (unsigned long long)off + (K - 1) * (unsigned long long)step < b1; off += K * step) {
        T v[K];
        long long sa[K];
#pragma unroll
        for (int k = 0; k < K; k++) {
            const unsigned o = off + k * step;
            sa[k] = smap ? map_s(ss, o) : (long long)o;
            v[k] = load_unit<U, CG>(sb + sa[k]);
        }
#pragma unroll
        for (int k = 0; k < K; k++) {
            const unsigned o = off + k * step;
            const long long da = same ? sa[k] : (dmap ? map_s(ds, o) : (long long)o);
            store_unit<U, CG>(db + da, v[k]);
        }
    }
    for (; off < b1; off += step) {
        const long long sa = smap ? map_s(ss, off) : (long long)off;
        const long long da = same ? sa : (dmap ? map_s(ds, off) : (long long)off);
        store_unit<U, CG>(db + da, load_unit<U, CG>(sb + sa));
    }
}

// The general form: 64-bit offsets, up to 4 levels, descriptors read through the pointers.
template <int U, bool CG>
__device__ __noinline__ void typed_copy_u(char* db, const TypeDesc* dt_, const char* sb, const TypeDesc* st_,
                                          long long b0, long long b1, int lane, int nl) {
    for (long long off = b0 + (long long)lane * U; off < b1; off += (long long)nl * U) {
        long long sa = st_ ? desc_map(st_, off) : off;
        long long da = dt_ ? desc_map(dt_, off) : off;
        store_unit<U, CG>(db + da, load_unit<U, CG>(sb + sa));
    }
}

#define GPUMPI_TYPED_SWITCH(F, CG, ...)                  \
    switch (u) {                                         \
    case 16: F<16, CG>(__VA_ARGS__); break;              \
    case 8: F<8, CG>(__VA_ARGS__); break;                \
    case 4: F<4, CG>(__VA_ARGS__); break;                \
    case 2: F<2, CG>(__VA_ARGS__); break;                \
    default: F<1, CG>(__VA_ARGS__); break;               \
    }

// Copy packed-stream bytes [b0, b1) from (sb, st) to (db, dt); a null descriptor means contiguous.
// Executed by nl cooperating threads, this one being `lane`: one thread, or whole warps.
__device__ __noinline__ void typed_copy(void* db, const TypeDesc* dt_, const void* sb, const TypeDesc* st_,
                                        long long b0, long long b1, int lane, int nl) {
    char* d = (char*)db;
    const char* s = (const char*)sb;
    const bool cg = is_global_ptr(db) && is_global_ptr(sb);
    int u;
    if (b1 <= 0x7fffffffLL && b0 >= 0 && (nl == 1 || (nl & 31) == 0) && (threadIdx.x >> 5) < kMaxWarps) {
        // the mapping images into this warp's slots (one round trip), then every decision from shared memory
        DescS* slot = s_tdesc[threadIdx.x >> 5];
        if (nl > 1) {
            __syncwarp();
            img_load_lane(slot, st_, dt_, (int)(threadIdx.x & 31));
            __syncwarp();
        } else {
#pragma unroll
            for (int l = 0; l < 16; l++) img_load_lane(slot, st_, dt_, l);
        }
        const volatile DescS* vs = slot;
        const int us = st_ ? vs[0].t.fast_unit : 16, ud = dt_ ? vs[1].t.fast_unit : 16;
        if (us && ud) {
            if (nl == 1 || (threadIdx.x & 31) == 0) {
                const bool same = st_ && dt_ && same_mapping(&vs[0].t, &vs[1].t);
                slot[1].same = same;
                slot[1].shift = same ? vs[1].t.lb - vs[0].t.lb : 0;
            }
            if (nl > 1) __syncwarp();
            u = min(us, ud);
            u = min(u, (int)pow2_div((long long)(size_t)sb));
            u = min(u, (int)pow2_div((long long)(size_t)db));
            u = min(u, (int)pow2_div(b0));
            u = min(u, (int)pow2_div(b1));
            const unsigned c0 = (unsigned)b0, c1 = (unsigned)b1;
            if (cg) {
                GPUMPI_TYPED_SWITCH(typed_copy_fast, true, d, dt_ != nullptr, s, st_ != nullptr, c0, c1, lane, nl)
            } else {
                GPUMPI_TYPED_SWITCH(typed_copy_fast, false, d, dt_ != nullptr, s, st_ != nullptr, c0, c1, lane, nl)
            }
            return;
        }
    }
    u = typed_unit(st_, sb, dt_, db);
    u = min(u, (int)pow2_div(b0));
    u = min(u, (int)pow2_div(b1));
    if (cg) {
        GPUMPI_TYPED_SWITCH(typed_copy_u, true, d, dt_, s, st_, b0, b1, lane, nl)
    } else {
        GPUMPI_TYPED_SWITCH(typed_copy_u, false, d, dt_, s, st_, b0, b1, lane, nl)
    }
}
#undef GPUMPI_TYPED_SWITCH

}  // namespace gpumpi
