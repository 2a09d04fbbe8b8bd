// rt_ops.cuh — reduction operators.
//
// Semantics follow the reference functors exactly (gpu_libs/gpu_mpi/operators.cu:73-151), applied as
// inout = op(in, inout) (operators.cu:216-218) with in = the next rank's value and inout = the running
// result.  Notable reference behaviours kept for bit-exact parity:
//   * MAX: in > acc ? in : acc;  MIN: in > acc ? acc : in  (NaN and signed-zero outcomes follow);
//   * LXOR is (in != acc) on the raw values, not a truthiness xor;
//   * integer arithmetic wraps modulo 2^bits.
// Legality follows the reference's IsTypeOpAllowed table (operators.cu:153-200); MAXLOC / MINLOC are
// defined on the pair types (value, int index), lower index winning ties.
// Floating-point products and sums are single IEEE operations (no contraction possible: each step is
// one add or one multiply), complex products use explicitly rounded __fmul_rn / __fadd_rn steps.
#pragma once
#include <type_traits>
#include "rt_core.cuh"

namespace gpumpi {

enum TypeClass { TC_INT = 1, TC_FLOAT = 2, TC_LOGICAL = 4, TC_COMPLEX = 8, TC_BYTE = 16, TC_TEXT = 32, TC_PAIR = 64 };

__device__ __forceinline__ int type_class(int dt) {
    switch (dt) {
    case GPUMPI_SHORT: case GPUMPI_INT: case GPUMPI_LONG: case GPUMPI_LONG_LONG_INT: case GPUMPI_LONG_LONG:
    case GPUMPI_SIGNED_CHAR: case GPUMPI_UNSIGNED_CHAR: case GPUMPI_UNSIGNED_SHORT: case GPUMPI_UNSIGNED:
    case GPUMPI_UNSIGNED_LONG: case GPUMPI_UNSIGNED_LONG_LONG: case GPUMPI_INT8_T: case GPUMPI_INT16_T:
    case GPUMPI_INT32_T: case GPUMPI_INT64_T: case GPUMPI_UINT8_T: case GPUMPI_UINT16_T: case GPUMPI_UINT32_T:
    case GPUMPI_UINT64_T:
        return TC_INT;
    case GPUMPI_FLOAT: case GPUMPI_DOUBLE: case GPUMPI_LONG_DOUBLE: return TC_FLOAT;
    case GPUMPI_C_BOOL: return TC_LOGICAL;
    case GPUMPI_C_COMPLEX: case GPUMPI_C_FLOAT_COMPLEX: case GPUMPI_C_DOUBLE_COMPLEX:
    case GPUMPI_C_LONG_DOUBLE_COMPLEX: return TC_COMPLEX;
    case GPUMPI_BYTE: return TC_BYTE;
    case GPUMPI_CHAR: case GPUMPI_WCHAR: return TC_TEXT;
    case GPUMPI_2INT: case GPUMPI_FLOAT_INT: case GPUMPI_DOUBLE_INT: case GPUMPI_LONG_INT: case GPUMPI_SHORT_INT:
    case GPUMPI_LONG_DOUBLE_INT: return TC_PAIR;
    default: return 0;
    }
}

__device__ __forceinline__ bool op_allowed(int op, int dt) {
    int c = type_class(dt);
    switch (op) {
    case GPUMPI_OP_MAX: case GPUMPI_OP_MIN: return (c & (TC_INT | TC_FLOAT)) != 0;
    case GPUMPI_OP_SUM: case GPUMPI_OP_PROD: return (c & (TC_INT | TC_FLOAT | TC_COMPLEX)) != 0;
    case GPUMPI_OP_LAND: case GPUMPI_OP_LOR: case GPUMPI_OP_LXOR: return (c & (TC_INT | TC_LOGICAL)) != 0;
    case GPUMPI_OP_BAND: case GPUMPI_OP_BOR: case GPUMPI_OP_BXOR: return (c & (TC_INT | TC_BYTE)) != 0;
    case GPUMPI_OP_MAXLOC: case GPUMPI_OP_MINLOC: return c == TC_PAIR;
    default: return false;
    }
}

// ---- typed scalar op for the fast (templated) fold path ----
template <int OP, class T>
__device__ __forceinline__ T op_apply(T in, T acc) {
    if constexpr (OP == GPUMPI_OP_MAX) return in > acc ? in : acc;
    else if constexpr (OP == GPUMPI_OP_MIN) return in > acc ? acc : in;
    else if constexpr (OP == GPUMPI_OP_SUM) {
        if constexpr (std::is_same_v<T, float>) return __fadd_rn(in, acc);
        else if constexpr (std::is_same_v<T, double>) return __dadd_rn(in, acc);
        else { using U = std::make_unsigned_t<T>; return (T)(U)((U)in + (U)acc); }
    } else if constexpr (OP == GPUMPI_OP_PROD) {
        if constexpr (std::is_same_v<T, float>) return __fmul_rn(in, acc);
        else if constexpr (std::is_same_v<T, double>) return __dmul_rn(in, acc);
        else { using U = std::make_unsigned_t<T>; return (T)(U)((unsigned long long)(U)in * (unsigned long long)(U)acc); }
    } else if constexpr (OP == GPUMPI_OP_BAND) return (T)(in & acc);
    else if constexpr (OP == GPUMPI_OP_BOR) return (T)(in | acc);
    else if constexpr (OP == GPUMPI_OP_BXOR) return (T)(in ^ acc);
    else if constexpr (OP == GPUMPI_OP_LAND) return (T)(in && acc);
    else if constexpr (OP == GPUMPI_OP_LOR) return (T)(in || acc);
    else return (T)(in != acc);  // LXOR
}

// ---- generic element-wise application: *acc = op(*in, *acc) for any legal (op, dt) ----
template <class T>
__device__ __forceinline__ void gen_int(int op, const void* in, void* acc) {
    T a = *(const T*)in, b = *(T*)acc, r;
    switch (op) {
    case GPUMPI_OP_MAX: r = op_apply<GPUMPI_OP_MAX>(a, b); break;
    case GPUMPI_OP_MIN: r = op_apply<GPUMPI_OP_MIN>(a, b); break;
    case GPUMPI_OP_SUM: r = (T)(a + b); break;
    case GPUMPI_OP_PROD: r = (T)((unsigned long long)a * (unsigned long long)b); break;
    case GPUMPI_OP_LAND: r = (T)(a && b); break;
    case GPUMPI_OP_BAND: r = (T)(a & b); break;
    case GPUMPI_OP_LOR: r = (T)(a || b); break;
    case GPUMPI_OP_BOR: r = (T)(a | b); break;
    case GPUMPI_OP_LXOR: r = (T)(a != b); break;
    default: r = (T)(a ^ b); break;
    }
    *(T*)acc = r;
}

template <class T>
__device__ __forceinline__ void gen_flt(int op, const void* in, void* acc) {
    T a = *(const T*)in, b = *(T*)acc, r;
    switch (op) {
    case GPUMPI_OP_MAX: r = op_apply<GPUMPI_OP_MAX>(a, b); break;
    case GPUMPI_OP_MIN: r = op_apply<GPUMPI_OP_MIN>(a, b); break;
    case GPUMPI_OP_SUM: r = op_apply<GPUMPI_OP_SUM>(a, b); break;
    default: r = op_apply<GPUMPI_OP_PROD>(a, b); break;
    }
    *(T*)acc = r;
}

__device__ __forceinline__ void gen_cpx_f(int op, const void* in, void* acc) {
    const float* a = (const float*)in;
    float* c = (float*)acc;
    float ar = a[0], ai = a[1], cr = c[0], ci = c[1];
    if (op == GPUMPI_OP_SUM) { c[0] = __fadd_rn(ar, cr); c[1] = __fadd_rn(ai, ci); }
    else { c[0] = __fsub_rn(__fmul_rn(ar, cr), __fmul_rn(ai, ci)); c[1] = __fadd_rn(__fmul_rn(ar, ci), __fmul_rn(ai, cr)); }
}
__device__ __forceinline__ void gen_cpx_d(int op, const void* in, void* acc) {
    const double* a = (const double*)in;
    double* c = (double*)acc;
    double ar = a[0], ai = a[1], cr = c[0], ci = c[1];
    if (op == GPUMPI_OP_SUM) { c[0] = __dadd_rn(ar, cr); c[1] = __dadd_rn(ai, ci); }
    else { c[0] = __dsub_rn(__dmul_rn(ar, cr), __dmul_rn(ai, ci)); c[1] = __dadd_rn(__dmul_rn(ar, ci), __dmul_rn(ai, cr)); }
}

template <class V>
__device__ __forceinline__ void gen_pair(int op, const void* in, void* acc) {
    struct P { V val; int idx; };
    P a = *(const P*)in, b = *(P*)acc, c;
    if (a.val > b.val) c = (op == GPUMPI_OP_MAXLOC) ? a : b;
    else if (a.val < b.val) c = (op == GPUMPI_OP_MAXLOC) ? b : a;
    else c = a.idx < b.idx ? a : b;
    *(P*)acc = c;
}

__device__ __forceinline__ void apply_elem(int op, int dt, const void* in, void* acc) {
    switch (dt) {
    case GPUMPI_SIGNED_CHAR: case GPUMPI_INT8_T: gen_int<signed char>(op, in, acc); break;
    case GPUMPI_UNSIGNED_CHAR: case GPUMPI_UINT8_T: case GPUMPI_BYTE: gen_int<unsigned char>(op, in, acc); break;
    case GPUMPI_SHORT: case GPUMPI_INT16_T: gen_int<short>(op, in, acc); break;
    case GPUMPI_UNSIGNED_SHORT: case GPUMPI_UINT16_T: gen_int<unsigned short>(op, in, acc); break;
    case GPUMPI_INT: case GPUMPI_INT32_T: gen_int<int>(op, in, acc); break;
    case GPUMPI_UNSIGNED: case GPUMPI_UINT32_T: gen_int<unsigned>(op, in, acc); break;
    case GPUMPI_LONG: case GPUMPI_LONG_LONG_INT: case GPUMPI_LONG_LONG: case GPUMPI_INT64_T:
        gen_int<long long>(op, in, acc); break;
    case GPUMPI_UNSIGNED_LONG: case GPUMPI_UNSIGNED_LONG_LONG: case GPUMPI_UINT64_T:
        gen_int<unsigned long long>(op, in, acc); break;
    case GPUMPI_FLOAT: gen_flt<float>(op, in, acc); break;
    case GPUMPI_DOUBLE: case GPUMPI_LONG_DOUBLE: gen_flt<double>(op, in, acc); break;
    case GPUMPI_C_BOOL: {
        bool a = *(const unsigned char*)in != 0, b = *(unsigned char*)acc != 0;
        *(unsigned char*)acc = (unsigned char)(op == GPUMPI_OP_LAND ? (a && b) : op == GPUMPI_OP_LOR ? (a || b) : (a != b));
        break;
    }
    case GPUMPI_C_COMPLEX: case GPUMPI_C_FLOAT_COMPLEX: gen_cpx_f(op, in, acc); break;
    case GPUMPI_C_DOUBLE_COMPLEX: case GPUMPI_C_LONG_DOUBLE_COMPLEX: gen_cpx_d(op, in, acc); break;
    case GPUMPI_2INT: gen_pair<int>(op, in, acc); break;
    case GPUMPI_FLOAT_INT: gen_pair<float>(op, in, acc); break;
    case GPUMPI_DOUBLE_INT: case GPUMPI_LONG_DOUBLE_INT: gen_pair<double>(op, in, acc); break;
    case GPUMPI_LONG_INT: gen_pair<long long>(op, in, acc); break;
    case GPUMPI_SHORT_INT: gen_pair<short>(op, in, acc); break;
    default: break;
    }
}

}  // namespace gpumpi
