"""ctypes binding of the CPU oracle (oracle/gpumpi_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as the checker, and by the
cpu_baseline / reference legs of bench.py.  Nothing in the product package imports this module.

`build()` compiles the C restatement with gcc into oracle/_build/liboracle.so (plain gcc, no CUDA).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"
SRC = HERE / "gpumpi_oracle.c"

_lib = None


def build(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    if force or not LIB.exists() or LIB.stat().st_mtime < max(SRC.stat().st_mtime,
                                                              (HERE / "gpumpi_oracle.h").stat().st_mtime):
        cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
               "-pthread", str(SRC), "-o", str(LIB), "-lm"]
        subprocess.run(cmd, check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB))
        c_i64, c_int, c_vp, c_u64 = ctypes.c_int64, ctypes.c_int, ctypes.c_void_p, ctypes.c_uint64
        L.orc_type_size.argtypes = [c_int]
        L.orc_op_allowed.argtypes = [c_int, c_int]
        L.orc_reduce_rm.argtypes = [c_vp, c_i64, c_int, c_vp, c_i64, c_int, c_int]
        L.orc_allreduce.argtypes = [c_vp, c_vp, c_int, c_i64, c_int, c_int, c_int]
        L.orc_alltoallv.argtypes = [c_vp, c_i64, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp, c_int, c_int, c_int]
        L.orc_lcg_next.argtypes = [ctypes.POINTER(c_u64)]
        L.orc_lcg_next.restype = c_u64
        L.orc_fill_f32.argtypes = [c_u64, c_i64, c_vp]
        L.orc_fill_f64.argtypes = [c_u64, c_i64, c_vp]
        L.orc_fill_i32.argtypes = [c_u64, c_i64, c_vp]
        L.orc_pi_hits.argtypes = [c_u64, c_int, c_i64]
        L.orc_pi_hits.restype = c_i64
        L.orc_bucket_keys.argtypes = [c_u64, c_int, c_i64, c_vp]
        L.orc_bucket_sort.argtypes = [c_vp, c_int, c_i64, c_vp, c_i64, c_vp]
        L.orc_halo_value.argtypes = [c_i64, c_i64, c_i64]
        L.orc_halo_value.restype = ctypes.c_double
        L.orc_halo_expected.argtypes = [c_int, c_int, c_int, c_vp]
        L.orc_comm_split.argtypes = [c_int, c_vp, c_vp, c_vp, c_vp]
        L.orc_mlp_loss_grad.argtypes = [c_vp, c_vp, c_vp, c_vp, c_int, c_vp]
        L.orc_mlp_loss_grad.restype = ctypes.c_double
        L.orc_mlp_forward.argtypes = [c_vp, c_vp, c_int, c_vp]
        L.orc_pack.argtypes = [c_vp, c_i64, c_vp, c_vp]
        L.orc_pack.restype = c_i64
        L.orc_unpack.argtypes = [c_vp, c_i64, c_vp, c_vp]
        L.orc_unpack.restype = c_i64
        for name in ("orc_type_basic",):
            getattr(L, name).argtypes = [c_int, c_vp]
        L.orc_type_contiguous.argtypes = [c_i64, c_vp, c_vp]
        L.orc_type_vector.argtypes = [c_i64, c_i64, c_i64, c_vp, c_vp]
        L.orc_type_hvector.argtypes = [c_i64, c_i64, c_i64, c_vp, c_vp]
        L.orc_type_subarray.argtypes = [c_int, c_vp, c_vp, c_vp, c_vp, c_vp]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


# numpy dtypes of the predefined MPI datatypes (same numbering as include/gpumpi_abi.h)
NP_DTYPES = {
    0: np.int8, 1: np.int16, 2: np.int32, 3: np.int64, 4: np.int64, 5: np.int64, 6: np.int8,
    7: np.uint8, 8: np.uint16, 9: np.uint32, 10: np.uint64, 11: np.uint64, 12: np.float32,
    13: np.float64, 14: np.float64, 15: np.int32, 16: np.uint8, 17: np.int8, 18: np.int16,
    19: np.int32, 20: np.int64, 21: np.uint8, 22: np.uint16, 23: np.uint32, 24: np.uint64,
    25: np.complex64, 26: np.complex64, 27: np.complex128, 28: np.complex128, 29: np.uint8,
}


def type_size(dt: int) -> int:
    return lib().orc_type_size(dt)


def op_allowed(op: int, dt: int) -> bool:
    return bool(lib().orc_op_allowed(op, dt))


def reduce(sendbufs: np.ndarray, dt: int, op: int) -> np.ndarray:
    """Canonical fold over axis 0 of a [n, count] array (rank-major)."""
    sendbufs = np.ascontiguousarray(sendbufs)
    n = sendbufs.shape[0]
    out = np.empty_like(sendbufs[0])
    count = out.size if dt < 30 else out.nbytes // type_size(dt)
    rc = lib().orc_reduce_rm(_p(sendbufs), sendbufs[0].nbytes, n, _p(out), count, dt, op)
    if rc:
        raise ValueError(f"oracle reduce failed with MPI error {rc}")
    return out


def allreduce(sendbufs: np.ndarray, dt: int, op: int, threads: int = 1) -> np.ndarray:
    sendbufs = np.ascontiguousarray(sendbufs)
    recv = np.empty_like(sendbufs)
    n = sendbufs.shape[0]
    count = sendbufs[0].size if dt < 30 else sendbufs[0].nbytes // type_size(dt)
    rc = lib().orc_allreduce(_p(sendbufs), _p(recv), n, count, dt, op, threads)
    if rc:
        raise ValueError(f"oracle allreduce failed with MPI error {rc}")
    return recv


def alltoallv(sendbufs: np.ndarray, sendcounts: np.ndarray, sdispls: np.ndarray, recv_elems: int,
              recvcounts: np.ndarray, rdispls: np.ndarray, threads: int = 1, recvbufs=None) -> np.ndarray:
    """sendbufs: [n, send_elems] rank-major; counts/displs: [n, n] int32 (row = that rank's array)."""
    sendbufs = np.ascontiguousarray(sendbufs)
    n = sendbufs.shape[0]
    es = sendbufs.itemsize
    if recvbufs is None:
        recvbufs = np.zeros((n, recv_elems), dtype=sendbufs.dtype)
    arrs = [np.ascontiguousarray(a, dtype=np.int32) for a in (sendcounts, sdispls, recvcounts, rdispls)]
    rc = lib().orc_alltoallv(_p(sendbufs), sendbufs[0].nbytes, _p(arrs[0]), _p(arrs[1]), _p(recvbufs),
                             recvbufs[0].nbytes, _p(arrs[2]), _p(arrs[3]), n, es, threads)
    if rc:
        raise ValueError(f"oracle alltoallv failed with MPI error {rc}")
    return recvbufs


def fill_f32(seed: int, n: int) -> np.ndarray:
    out = np.empty(n, dtype=np.float32)
    lib().orc_fill_f32(seed, n, _p(out))
    return out


def fill_f64(seed: int, n: int) -> np.ndarray:
    out = np.empty(n, dtype=np.float64)
    lib().orc_fill_f64(seed, n, _p(out))
    return out


def fill_i32(seed: int, n: int) -> np.ndarray:
    out = np.empty(n, dtype=np.int32)
    lib().orc_fill_i32(seed, n, _p(out))
    return out


def lcg_sequence(seed: int, n: int) -> np.ndarray:
    s = ctypes.c_uint64(seed)
    return np.array([lib().orc_lcg_next(ctypes.byref(s)) for _ in range(n)], dtype=np.uint64)


def pi_hits(seed: int, rank: int, pairs: int) -> int:
    return int(lib().orc_pi_hits(seed, rank, pairs))


def bucket_keys(seed: int, rank: int, nkeys: int) -> np.ndarray:
    out = np.empty(nkeys, dtype=np.int32)
    lib().orc_bucket_keys(seed, rank, nkeys, _p(out))
    return out


def bucket_sort(keys: np.ndarray, n: int, cap: int):
    keys = np.ascontiguousarray(keys, dtype=np.int32)
    kpr = keys.size // n
    out = np.zeros((n, cap), dtype=np.int32)
    counts = np.zeros(n, dtype=np.int64)
    rc = lib().orc_bucket_sort(_p(keys), n, kpr, _p(out), cap, _p(counts))
    if rc:
        raise ValueError(f"oracle bucket sort failed with MPI error {rc}")
    return out, counts


def halo_expected(P: int, L: int, rank: int) -> np.ndarray:
    W = L + 2
    out = np.empty((W, W, W), dtype=np.float64)
    lib().orc_halo_expected(P, L, rank, _p(out))
    return out


def comm_split(colors, keys):
    colors = np.ascontiguousarray(colors, dtype=np.int32)
    keys = np.ascontiguousarray(keys, dtype=np.int32)
    n = colors.size
    nr = np.empty(n, dtype=np.int32)
    ns = np.empty(n, dtype=np.int32)
    lib().orc_comm_split(n, _p(colors), _p(keys), _p(nr), _p(ns))
    return nr, ns


MLP_NPARAMS = 64 * 12 + 64 + 64 * 64 + 64 + 4 * 64 + 4


def mlp_loss_grad(params, x, t, mask):
    params = np.ascontiguousarray(params, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64)
    t = np.ascontiguousarray(t, dtype=np.float64)
    mask = np.ascontiguousarray(mask, dtype=np.float64)
    g = np.zeros(MLP_NPARAMS, dtype=np.float64)
    loss = lib().orc_mlp_loss_grad(_p(params), _p(x), _p(t), _p(mask), x.shape[0], _p(g))
    return loss, g


def mlp_forward(params, x):
    params = np.ascontiguousarray(params, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty((x.shape[0], 4), dtype=np.float64)
    lib().orc_mlp_forward(_p(params), _p(x), x.shape[0], _p(y))
    return y


class TypeMap(ctypes.Structure):
    _fields_ = [("size", ctypes.c_int64), ("extent", ctypes.c_int64), ("lb", ctypes.c_int64),
                ("block", ctypes.c_int64), ("nlev", ctypes.c_int), ("cnt", ctypes.c_int64 * 4),
                ("stride", ctypes.c_int64 * 4)]


def type_basic(dt: int) -> TypeMap:
    t = TypeMap()
    lib().orc_type_basic(dt, ctypes.byref(t))
    return t


def type_vector(count, blocklen, stride, old: TypeMap) -> TypeMap:
    t = TypeMap()
    rc = lib().orc_type_vector(count, blocklen, stride, ctypes.byref(old), ctypes.byref(t))
    if rc:
        raise ValueError(rc)
    return t


def type_hvector(count, blocklen, stride_bytes, old: TypeMap) -> TypeMap:
    t = TypeMap()
    rc = lib().orc_type_hvector(count, blocklen, stride_bytes, ctypes.byref(old), ctypes.byref(t))
    if rc:
        raise ValueError(rc)
    return t


def type_contiguous(count, old: TypeMap) -> TypeMap:
    t = TypeMap()
    rc = lib().orc_type_contiguous(count, ctypes.byref(old), ctypes.byref(t))
    if rc:
        raise ValueError(rc)
    return t


def type_subarray(sizes, subsizes, starts, old: TypeMap) -> TypeMap:
    nd = len(sizes)
    arr = [np.ascontiguousarray(v, dtype=np.int32) for v in (sizes, subsizes, starts)]
    t = TypeMap()
    rc = lib().orc_type_subarray(nd, _p(arr[0]), _p(arr[1]), _p(arr[2]), ctypes.byref(old), ctypes.byref(t))
    if rc:
        raise ValueError(rc)
    return t


def pack(t: TypeMap, count: int, src: np.ndarray) -> np.ndarray:
    out = np.zeros(t.size * count, dtype=np.uint8)
    lib().orc_pack(ctypes.byref(t), count, _p(src), _p(out))
    return out


def unpack(t: TypeMap, count: int, packed: np.ndarray, dst: np.ndarray) -> np.ndarray:
    lib().orc_unpack(ctypes.byref(t), count, _p(np.ascontiguousarray(packed)), _p(dst))
    return dst


# ---- Cartesian topologies (MPI-3.1 section 7.5; the reference has no topology functions) ----
PROC_NULL = -2


def dims_create(nnodes: int, dims):
    """MPI_Dims_create: the zero entries of dims filled so that the product is nnodes, as balanced as the
    greedy rule makes them (prime factors of the remainder, largest first, each to the smallest free
    dimension so far; the free dimensions then in non-increasing order).  Returns None when impossible."""
    dims = list(dims)
    fixed = 1
    for d in dims:
        if d < 0:
            return None
        if d > 0:
            fixed *= d
    nfree = dims.count(0)
    if fixed > nnodes or nnodes % fixed:
        return None
    rem = nnodes // fixed
    if nfree == 0:
        return dims if rem == 1 else None
    primes, r, q = [], rem, 2
    while q * q <= r:
        while r % q == 0:
            primes.append(q)
            r //= q
        q += 1
    if r > 1:
        primes.append(r)
    f = [1] * nfree
    for pr in reversed(primes):
        m = min(range(nfree), key=lambda k: (f[k], k))
        f[m] *= pr
    f.sort(reverse=True)
    it = iter(f)
    return [d if d > 0 else next(it) for d in dims]


def cart_coords(dims, rank: int):
    """Row-major coordinates (the last dimension varies fastest)."""
    c = [0] * len(dims)
    for i in range(len(dims) - 1, -1, -1):
        c[i] = rank % dims[i]
        rank //= dims[i]
    return c


def cart_rank(dims, periods, coords):
    """Rank of coords; periodic dimensions wrap, None outside a non-periodic one."""
    r = 0
    for d, p, x in zip(dims, periods, coords):
        if not 0 <= x < d:
            if not p:
                return None
            x %= d
        r = r * d + x
    return r


def cart_shift(dims, periods, rank: int, direction: int, disp: int):
    """(source, dest) of MPI_Cart_shift; PROC_NULL off a non-periodic edge."""
    c = cart_coords(dims, rank)
    out = []
    for s in (-disp, disp):
        cc = list(c)
        cc[direction] += s
        r = cart_rank(dims, periods, cc)
        out.append(PROC_NULL if r is None else r)
    return out[0], out[1]


if __name__ == "__main__":
    print(build(force=bool(os.environ.get("FORCE"))))
