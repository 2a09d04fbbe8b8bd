/*
 * gpumpi_abi.h — numeric constants shared by the device MPI surface, the host C ABI
 * and the CPU oracle.  Plain C, no CUDA, no torch.
 *
 * Datatype numbering keeps the reference's enum order exactly
 * (gpu_libs/gpu_mpi/mpi_types_list.cuh:3-33, enum built at gpu_libs/gpu_mpi/datatypes.cuh:12-14),
 * so an MPI_Datatype value means the same element type on both sides.  Values 30..35 are the
 * pair types that MPI_MAXLOC / MPI_MINLOC need; the reference declares those ops
 * (gpu_libs/gpu_mpi/mpi_operators_list.cuh:14-15) but has no type they can be applied to.
 * Derived datatypes get handles >= GPUMPI_DERIVED_BASE.
 *
 * Operator numbering keeps the reference's list order (gpu_libs/gpu_mpi/mpi_operators_list.cuh:4-16).
 */
#ifndef GPUMPI_ABI_H
#define GPUMPI_ABI_H

/* ---- datatypes (reference order) ---- */
#define GPUMPI_CHAR                   0
#define GPUMPI_SHORT                  1
#define GPUMPI_INT                    2
#define GPUMPI_LONG                   3
#define GPUMPI_LONG_LONG_INT          4
#define GPUMPI_LONG_LONG              5
#define GPUMPI_SIGNED_CHAR            6
#define GPUMPI_UNSIGNED_CHAR          7
#define GPUMPI_UNSIGNED_SHORT         8
#define GPUMPI_UNSIGNED               9
#define GPUMPI_UNSIGNED_LONG         10
#define GPUMPI_UNSIGNED_LONG_LONG    11
#define GPUMPI_FLOAT                 12
#define GPUMPI_DOUBLE                13
#define GPUMPI_LONG_DOUBLE           14  /* stored as double, as in the reference */
#define GPUMPI_WCHAR                 15
#define GPUMPI_C_BOOL                16
#define GPUMPI_INT8_T                17
#define GPUMPI_INT16_T               18
#define GPUMPI_INT32_T               19
#define GPUMPI_INT64_T               20
#define GPUMPI_UINT8_T               21
#define GPUMPI_UINT16_T              22
#define GPUMPI_UINT32_T              23
#define GPUMPI_UINT64_T              24
#define GPUMPI_C_COMPLEX             25
#define GPUMPI_C_FLOAT_COMPLEX       26
#define GPUMPI_C_DOUBLE_COMPLEX      27
#define GPUMPI_C_LONG_DOUBLE_COMPLEX 28  /* stored as double complex, as in the reference */
#define GPUMPI_BYTE                  29
/* pair types for MAXLOC / MINLOC (value first, then int index) */
#define GPUMPI_2INT                  30
#define GPUMPI_FLOAT_INT             31
#define GPUMPI_DOUBLE_INT            32
#define GPUMPI_LONG_INT              33
#define GPUMPI_SHORT_INT             34
#define GPUMPI_LONG_DOUBLE_INT       35
#define GPUMPI_NUM_PREDEFINED_TYPES  36
#define GPUMPI_DATATYPE_NULL         (-1)
#define GPUMPI_DERIVED_BASE          1024

/* ---- reduction operators (reference order) ---- */
#define GPUMPI_OP_MAX     0
#define GPUMPI_OP_MIN     1
#define GPUMPI_OP_SUM     2
#define GPUMPI_OP_PROD    3
#define GPUMPI_OP_LAND    4
#define GPUMPI_OP_BAND    5
#define GPUMPI_OP_LOR     6
#define GPUMPI_OP_BOR     7
#define GPUMPI_OP_LXOR    8
#define GPUMPI_OP_BXOR    9
#define GPUMPI_OP_MAXLOC 10
#define GPUMPI_OP_MINLOC 11
#define GPUMPI_NUM_PREDEFINED_OPS 12
#define GPUMPI_OP_USER   64   /* MPI_Op_create handles */

/* ---- error codes.  MPI_SUCCESS / MPI_FAILURE / MPI_ERR_OTHER keep the reference values
 *      (gpu_libs/gpu_mpi/mpi_common.cuh:3-9); the rest are new and distinct. ---- */
#define GPUMPI_SUCCESS         0
#define GPUMPI_FAILURE        (-1)
#define GPUMPI_ERR_OTHER       1   /* also: a bounded wait ran out (see GPUMPI_ERR_TIMEOUT detail) */
#define GPUMPI_ERR_BUFFER      2
#define GPUMPI_ERR_COUNT       3
#define GPUMPI_ERR_TYPE        4
#define GPUMPI_ERR_TAG         5
#define GPUMPI_ERR_COMM        6
#define GPUMPI_ERR_RANK        7
#define GPUMPI_ERR_ROOT        8
#define GPUMPI_ERR_OP          9
#define GPUMPI_ERR_ARG        10
#define GPUMPI_ERR_REQUEST    11
#define GPUMPI_ERR_TRUNCATE   12
#define GPUMPI_ERR_NO_MEM     13
#define GPUMPI_ERR_INTERN     14
#define GPUMPI_ERR_TIMEOUT    15   /* detail code recorded beside MPI_ERR_OTHER */
#define GPUMPI_ERR_ABORTED    16   /* another rank failed first; this rank gave up */
#define GPUMPI_ERR_NOT_IMPL   17
#define GPUMPI_ERR_LAUNCH     18   /* host side: launch / co-residency failure */
#define GPUMPI_ERR_CUDA       19   /* host side: a CUDA runtime call failed */
/* MPI-IO error classes (MPI-3.1 table 13.4).  The reference numbers its I/O classes 1..16 in a space of
 * their own (gpu_libs/gpu_mpi/io.cuh:28-45), which overlaps MPI_ERR_OTHER..; here they are distinct. */
#define GPUMPI_ERR_FILE                  20
#define GPUMPI_ERR_NOT_SAME              21
#define GPUMPI_ERR_AMODE                 22
#define GPUMPI_ERR_UNSUPPORTED_DATAREP   23
#define GPUMPI_ERR_UNSUPPORTED_OPERATION 24
#define GPUMPI_ERR_NO_SUCH_FILE          25
#define GPUMPI_ERR_FILE_EXISTS           26
#define GPUMPI_ERR_BAD_FILE              27
#define GPUMPI_ERR_ACCESS                28
#define GPUMPI_ERR_NO_SPACE              29
#define GPUMPI_ERR_QUOTA                 30
#define GPUMPI_ERR_READ_ONLY             31
#define GPUMPI_ERR_FILE_IN_USE           32
#define GPUMPI_ERR_IO                    33

/* ---- collective algorithm variants (what the tuned table and the learned selector pick) ---- */
#define GPUMPI_VARIANT_AUTO     (-1)
#define GPUMPI_VARIANT_DIRECT     0   /* canonical rank order, one pass, element chunks */
#define GPUMPI_VARIANT_TREE       1   /* pairwise tree over ranks (reordered: tolerance) */
#define GPUMPI_VARIANT_RING       2   /* ring-chunked reduce-scatter + allgather (reordered) */
#define GPUMPI_VARIANT_STAGED     3   /* canonical order, inputs staged through shared memory by TMA bulk copies */
#define GPUMPI_NUM_VARIANTS       4

/* ---- wildcards ---- */
#define GPUMPI_ANY_SOURCE (-1)
#define GPUMPI_ANY_TAG    (-1)
#define GPUMPI_PROC_NULL  (-2)
#define GPUMPI_UNDEFINED  (-1)

#endif /* GPUMPI_ABI_H */
