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
        long long total = (long long)g_rt->nranks * g_rt->max_types;
        if (idx < total) {
            const TypeDesc* t = &g_rt->types[idx];
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

__device__ __forceinline__ long long pow2_div(long long v) {  // largest power of two dividing v (<= 16)
    if (v == 0) return 16;
    long long a = v & -v;
    return a > 16 ? 16 : a;
}

// Unit (1..16 bytes) that divides every block, stride, extent, offset and base address involved.
__device__ __forceinline__ int typed_unit(const TypeDesc* s, const void* sb, const TypeDesc* d, const void* db) {
    long long u = 16;
    const TypeDesc* ts[2] = {s, d};
    for (int k = 0; k < 2; k++) {
        const TypeDesc* t = ts[k];
        if (!t) continue;
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

template <int U, bool CG>
__device__ __forceinline__ void copy_unit(char* d, const char* s) {
    if constexpr (U == 16) {
        if constexpr (CG) __stcg((uint4*)d, __ldcg((const uint4*)s));
        else *(uint4*)d = *(const uint4*)s;
    } else if constexpr (U == 8) {
        if constexpr (CG) __stcg((unsigned long long*)d, __ldcg((const unsigned long long*)s));
        else *(unsigned long long*)d = *(const unsigned long long*)s;
    } else if constexpr (U == 4) {
        if constexpr (CG) __stcg((unsigned*)d, __ldcg((const unsigned*)s));
        else *(unsigned*)d = *(const unsigned*)s;
    } else if constexpr (U == 2) {
        *(unsigned short*)d = *(const volatile unsigned short*)s;
    } else {
        *d = *(const volatile char*)s;
    }
}

// CG selects L2-only accesses; legal only when both buffers are in global memory.
template <int U, bool CG>
__device__ __noinline__ void typed_copy_u(char* db, const TypeDesc* dt_, const char* sb, const TypeDesc* st_,
                                          long long b0, long long b1, int lane, int nl) {
    for (long long off = b0 + (long long)lane * U; off < b1; off += (long long)nl * U) {
        long long sa = st_ ? desc_map(st_, off) : off;
        long long da = dt_ ? desc_map(dt_, off) : off;
        copy_unit<U, CG>(db + da, sb + sa);
    }
}

// Copy packed-stream bytes [b0, b1) from (sb, st) to (db, dt); a null descriptor means contiguous.
// Executed by nl cooperating threads, this one being `lane`.
__device__ __noinline__ void typed_copy(void* db, const TypeDesc* dt_, const void* sb, const TypeDesc* st_,
                                           long long b0, long long b1, int lane, int nl) {
    int u = typed_unit(st_, sb, dt_, db);
    u = min(u, (int)pow2_div(b0));
    u = min(u, (int)pow2_div(b1));
    char* d = (char*)db;
    const char* s = (const char*)sb;
    if (is_global_ptr(db) && is_global_ptr(sb)) {
        switch (u) {
        case 16: typed_copy_u<16, true>(d, dt_, s, st_, b0, b1, lane, nl); break;
        case 8: typed_copy_u<8, true>(d, dt_, s, st_, b0, b1, lane, nl); break;
        case 4: typed_copy_u<4, true>(d, dt_, s, st_, b0, b1, lane, nl); break;
        case 2: typed_copy_u<2, true>(d, dt_, s, st_, b0, b1, lane, nl); break;
        default: typed_copy_u<1, true>(d, dt_, s, st_, b0, b1, lane, nl); break;
        }
    } else {
        switch (u) {
        case 16: typed_copy_u<16, false>(d, dt_, s, st_, b0, b1, lane, nl); break;
        case 8: typed_copy_u<8, false>(d, dt_, s, st_, b0, b1, lane, nl); break;
        case 4: typed_copy_u<4, false>(d, dt_, s, st_, b0, b1, lane, nl); break;
        default: typed_copy_u<1, false>(d, dt_, s, st_, b0, b1, lane, nl); break;
        }
    }
}

}  // namespace gpumpi
