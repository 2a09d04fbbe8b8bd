"""Python host mirror of the block-rank MPI runtime (ctypes over libgpumpi.so's C ABI).

`World(nranks)` plays the role of the reference's TestRunner / gpu_main launcher
(tests/test_runner.cuh:26-86, gpu_libs/gpu_main/main.cu:133-320): it owns the device state of one
MPI world whose ranks are thread blocks of one persistent kernel.  The hot-path calls
(`allreduce`, `alltoallv`, ...) make every rank call the MPI collective on its slice of rank-major
buffers.  Buffers may be numpy arrays (host memory, staged by the library) or torch CUDA tensors.

There is no CPU fallback: if libgpumpi.so is missing or no GPU is present, calls raise.
"""
from __future__ import annotations

import ctypes
import sys
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent.parent
LIB_PATH = PKG / "_build" / "libgpumpi.so"

# ---- constants (include/gpumpi_abi.h, include/gpumpi.h) ----
CHAR, SHORT, INT, LONG, LONG_LONG_INT, LONG_LONG = 0, 1, 2, 3, 4, 5
SIGNED_CHAR, UNSIGNED_CHAR, UNSIGNED_SHORT, UNSIGNED, UNSIGNED_LONG, UNSIGNED_LONG_LONG = 6, 7, 8, 9, 10, 11
FLOAT, DOUBLE, LONG_DOUBLE, WCHAR, C_BOOL = 12, 13, 14, 15, 16
INT8_T, INT16_T, INT32_T, INT64_T, UINT8_T, UINT16_T, UINT32_T, UINT64_T = 17, 18, 19, 20, 21, 22, 23, 24
C_COMPLEX, C_FLOAT_COMPLEX, C_DOUBLE_COMPLEX, C_LONG_DOUBLE_COMPLEX, BYTE = 25, 26, 27, 28, 29
OP_MAX, OP_MIN, OP_SUM, OP_PROD, OP_LAND, OP_BAND, OP_LOR, OP_BOR, OP_LXOR, OP_BXOR = range(10)
OP_MAXLOC, OP_MINLOC = 10, 11
VARIANT_AUTO, VARIANT_DIRECT, VARIANT_TREE, VARIANT_RING, VARIANT_STAGED = -1, 0, 1, 2, 3
VARIANT_NAMES = ["direct", "tree", "ring", "staged"]

ERR_OTHER, ERR_RANK, ERR_TRUNCATE, ERR_TIMEOUT = 1, 7, 12, 15
MPI_CART = 1
(TUNE_VEC, TUNE_STAGE_GROUP, TUNE_ENGINES, TUNE_COPY_CHUNK, TUNE_ENGINE_MIN_BYTES, TUNE_MLP_MARGIN, TUNE_DYN_SMEM,
 TUNE_HOST_DIRECT, TUNE_MLP_MARGIN_PULL, TUNE_HOST_SLICE, TUNE_HOST_STREAMS) = 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11
TUNE_STATIC_FOLD, TUNE_STATIC_BCAST, TUNE_STATIC_PULL, TUNE_PULL_CHUNKS = 13, 14, 15, 16

TESTS = {
    "single_int": 1, "transfer_array": 2, "send_recv": 3, "repeat_send_recv": 4, "network_flood": 5,
    "all_to_all": 6, "reduce_int16_prod": 7, "allreduce_f64_sum": 8, "allgather_int": 9, "scatter_int": 10,
    "scatterv_int": 11, "comm_rank": 12, "comm_dup_isolation": 13, "comm_split": 14, "sample": 15,
    "p2p_matching": 16, "timeout": 17, "datatypes": 18, "subcomm_coll": 19, "errors": 20, "cart": 21, "tiny_stress": 22, "tiny_mixed": 23, "attrs": 24, "file_io": 25,
}
P_COLL, P_PINGPONG, P_RING, P_PI, P_BUCKET_SORT, P_HALO, P_BATCH = 100, 101, 102, 103, 104, 105, 106
COLL = {"allreduce": 0, "reduce": 1, "bcast": 2, "alltoall": 3, "alltoallv": 4, "allgather": 5, "gather": 6,
        "scatter": 7, "barrier": 8, "allgatherv": 9, "gatherv": 10, "scatterv": 11}

NP_OF = {INT: np.int32, INT32_T: np.int32, FLOAT: np.float32, DOUBLE: np.float64, INT64_T: np.int64,
         LONG_LONG: np.int64, LONG: np.int64, UNSIGNED: np.uint32, UINT64_T: np.uint64, SHORT: np.int16,
         INT16_T: np.int16, BYTE: np.uint8, CHAR: np.int8, UNSIGNED_CHAR: np.uint8, UINT8_T: np.uint8,
         INT8_T: np.int8, UINT32_T: np.uint32, UNSIGNED_LONG_LONG: np.uint64, UNSIGNED_LONG: np.uint64,
         SIGNED_CHAR: np.int8, UNSIGNED_SHORT: np.uint16, UINT16_T: np.uint16, LONG_LONG_INT: np.int64,
         LONG_DOUBLE: np.float64, C_BOOL: np.uint8}

MLP_NPARAMS = 64 * 12 + 64 + 64 * 64 + 64 + 4 * 64 + 4

# symbols include/gpumpi.h declares (checked by the CPU test suite)
EXPORTS = [
    "gpumpi_config_init", "gpumpi_parse_args", "gpumpi_world_create", "gpumpi_world_destroy",
    "gpumpi_world_get_info", "gpumpi_last_error", "gpumpi_set_policy", "gpumpi_set_tuning", "gpumpi_get_tuning", "gpumpi_set_tuned_table",
    "gpumpi_set_mlp", "gpumpi_read_trace", "gpumpi_run_program", "gpumpi_last_kernel_ms",
    "gpumpi_kernel_launches", "gpumpi_test_run", "gpumpi_allreduce", "gpumpi_reduce", "gpumpi_bcast",
    "gpumpi_alltoall", "gpumpi_alltoallv", "gpumpi_allgather", "gpumpi_pingpong", "gpumpi_ring",
    "gpumpi_allreduce_noalloc", "gpumpi_allreduce_noalloc_status", "gpumpi_noalloc_test_hook", "gpumpi_mlp_forward", "gpumpi_mlp_loss_grad", "gpumpi_mlp_adam_step",
    "gpumpi_graph_create", "gpumpi_graph_launch", "gpumpi_graph_destroy", "gpumpi_main",
]


class GpumpiError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"gpumpi error {code}: {msg}")
        self.code = code


class Config(ctypes.Structure):
    _fields_ = [("nranks", ctypes.c_int), ("threads_per_block", ctypes.c_int), ("engine_blocks", ctypes.c_int),
                ("pending_requests", ctypes.c_int), ("mailbox_depth", ctypes.c_int),
                ("unexpected_depth", ctypes.c_int), ("eager_bytes", ctypes.c_int), ("max_types", ctypes.c_int),
                ("posted_depth", ctypes.c_int), ("device", ctypes.c_int), ("stack_bytes", ctypes.c_size_t),
                ("heap_bytes", ctypes.c_size_t), ("arena_bytes", ctypes.c_size_t),
                ("copy_chunk_bytes", ctypes.c_longlong), ("engine_min_bytes", ctypes.c_longlong),
                ("timeout_s", ctypes.c_double), ("trace_capacity", ctypes.c_int),
                ("host_window_bytes", ctypes.c_longlong)]


class WorldInfo(ctypes.Structure):
    _fields_ = [("nranks", ctypes.c_int), ("threads_per_block", ctypes.c_int), ("engine_blocks", ctypes.c_int),
                ("blocks_per_sm", ctypes.c_int), ("sm_count", ctypes.c_int), ("device", ctypes.c_int),
                ("device_bytes", ctypes.c_size_t)]


class Params(ctypes.Structure):
    _fields_ = [("i", ctypes.c_longlong * 16), ("d", ctypes.c_double * 4), ("p", ctypes.c_void_p * 16)]


_lib = None


def build(force: bool = False) -> Path:
    import importlib.util
    spec = importlib.util.spec_from_file_location("gpumpi_build", PKG / "build.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force=force)


def lib():
    """Loads libgpumpi.so (raises if it was not built: there is no fallback)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build it with dphpc-gpu_mpi_gb300/build.py")
        L = ctypes.CDLL(str(LIB_PATH))
        vp, i32, i64, u64p = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.POINTER(ctypes.c_uint64)
        L.gpumpi_config_init.argtypes = [ctypes.POINTER(Config)]
        L.gpumpi_parse_args.argtypes = [i32, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(Config)]
        L.gpumpi_world_create.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(vp)]
        L.gpumpi_world_destroy.argtypes = [vp]
        L.gpumpi_world_get_info.argtypes = [vp, ctypes.POINTER(WorldInfo)]
        L.gpumpi_last_error.argtypes = [vp]
        L.gpumpi_last_error.restype = ctypes.c_char_p
        L.gpumpi_set_policy.argtypes = [vp, i32, i32]
        L.gpumpi_set_tuning.argtypes = [vp, i32, i64]
        L.gpumpi_get_tuning.argtypes = [vp, i32, ctypes.POINTER(ctypes.c_longlong)]
        L.gpumpi_set_tuned_table.argtypes = [vp, vp, ctypes.c_size_t]
        L.gpumpi_set_mlp.argtypes = [vp, vp, ctypes.c_size_t]
        L.gpumpi_read_trace.argtypes = [vp, vp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
        L.gpumpi_run_program.argtypes = [vp, i32, ctypes.POINTER(Params), vp, i32]
        L.gpumpi_graph_create.argtypes = [vp, i32, ctypes.POINTER(Params), ctypes.POINTER(vp)]
        L.gpumpi_graph_launch.argtypes = [vp, vp, i32]
        L.gpumpi_graph_destroy.argtypes = [vp]
        L.gpumpi_last_kernel_ms.argtypes = [vp]
        L.gpumpi_last_kernel_ms.restype = ctypes.c_double
        L.gpumpi_kernel_launches.restype = ctypes.c_longlong
        L.gpumpi_test_run.argtypes = [vp, i32, vp, vp, vp]
        L.gpumpi_allreduce.argtypes = [vp, vp, vp, i64, i32, i32, i32, u64p, vp]
        L.gpumpi_reduce.argtypes = [vp, vp, vp, i64, i32, i32, i32, i32, u64p, vp]
        L.gpumpi_bcast.argtypes = [vp, vp, i64, i32, i32, i32, u64p, vp]
        L.gpumpi_alltoall.argtypes = [vp, vp, vp, i64, i32, i32, u64p, vp]
        L.gpumpi_alltoallv.argtypes = [vp, vp, i64, vp, vp, vp, i64, vp, vp, i32, i32, u64p, vp]
        L.gpumpi_allgather.argtypes = [vp, vp, vp, i64, i32, i32, u64p, vp]
        L.gpumpi_pingpong.argtypes = [vp, vp, i64, i32, i32, i32, u64p, vp]
        L.gpumpi_ring.argtypes = [vp, vp, vp, i64, i32, i32, u64p, vp]
        L.gpumpi_mlp_forward.argtypes = [vp, vp, i32, vp, vp]
        L.gpumpi_mlp_loss_grad.argtypes = [vp, vp, vp, vp, i32, vp, vp, vp]
        L.gpumpi_mlp_adam_step.argtypes = [vp, vp, vp, vp, i32, ctypes.c_float, ctypes.c_float, vp]
        _lib = L
    return _lib


def _ptr(x):
    """Address of a numpy array (host) or a torch tensor (device or host)."""
    if x is None:
        return None
    if hasattr(x, "data_ptr"):
        return ctypes.c_void_p(x.data_ptr())
    if isinstance(x, np.ndarray):
        if not x.flags["C_CONTIGUOUS"]:
            raise ValueError("buffers must be C-contiguous")
        return ctypes.c_void_p(x.ctypes.data)
    if isinstance(x, int):
        return ctypes.c_void_p(x)
    raise TypeError(f"unsupported buffer type {type(x)}")


_CUDA_STREAM_LEGACY = 1   # cudaStreamLegacy: the default stream with its implicit synchronisation


def _stream(s):
    """The stream to launch on.  Default: torch's current stream when torch is in use, so a call is
    ordered after the caller's earlier work on its tensors (the world's own stream is non-blocking and
    would not be); torch's default stream (handle 0) is passed as the legacy default stream, because a
    NULL stream means the world's own stream to the C ABI."""
    if s is None:
        t = sys.modules.get("torch")
        if t is None or not t.cuda.is_available() or not t.cuda.is_initialized():
            return None
        s = t.cuda.current_stream()
    h = s.cuda_stream if hasattr(s, "cuda_stream") else int(s)
    return ctypes.c_void_p(h if h else _CUDA_STREAM_LEGACY)


class World:
    """One MPI world of `nranks` block-ranks on one GPU."""

    def __init__(self, nranks: int, **cfg):
        L = lib()
        c = Config()
        L.gpumpi_config_init(ctypes.byref(c))
        c.nranks = nranks
        for k, v in cfg.items():
            if not hasattr(c, k):
                raise TypeError(f"unknown config field {k}")
            setattr(c, k, v)
        self.cfg = c
        h = ctypes.c_void_p()
        rc = L.gpumpi_world_create(ctypes.byref(c), ctypes.byref(h))
        if rc:
            raise GpumpiError(rc, L.gpumpi_last_error(None).decode())
        self.h = h
        self.nranks = nranks

    def close(self):
        if getattr(self, "h", None):
            lib().gpumpi_world_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def last_error(self) -> str:
        return lib().gpumpi_last_error(self.h).decode()

    def _check(self, rc: int, what: str):
        if rc:
            raise GpumpiError(rc, f"{what}: {self.last_error()}")

    def info(self) -> dict:
        i = WorldInfo()
        lib().gpumpi_world_get_info(self.h, ctypes.byref(i))
        return {f: getattr(i, f) for f, _ in WorldInfo._fields_}

    def set_policy(self, variant: int = -1, mode: int = 3):
        """variant >= 0 forces one; mode 0 plain (DIRECT), 1 tuned table, 2 learned MLP, 3 heuristic."""
        self._check(lib().gpumpi_set_policy(self.h, variant, mode), "set_policy")

    def set_tuning(self, key: int, value: int):
        """Autotuner knobs (TUNE_VEC, TUNE_STAGE_GROUP, TUNE_ENGINES, TUNE_COPY_CHUNK, TUNE_ENGINE_MIN_BYTES,
        TUNE_MLP_MARGIN, TUNE_DYN_SMEM) and TUNE_HOST_DIRECT (page-locked host buffers in place or staged)."""
        self._check(lib().gpumpi_set_tuning(self.h, key, value), "set_tuning")

    def get_tuning(self, key: int) -> int:
        v = ctypes.c_longlong(0)
        self._check(lib().gpumpi_get_tuning(self.h, key, ctypes.byref(v)), "get_tuning")
        return int(v.value)

    def set_tuned_table(self, table: np.ndarray):
        t = np.ascontiguousarray(table, dtype=np.int8)
        self._check(lib().gpumpi_set_tuned_table(self.h, _ptr(t), t.nbytes), "set_tuned_table")

    def set_mlp(self, params: np.ndarray):
        p = np.ascontiguousarray(params, dtype=np.float32)
        self._check(lib().gpumpi_set_mlp(self.h, _ptr(p), p.size), "set_mlp")

    def read_trace(self, cap: int = 1 << 20) -> np.ndarray:
        dt = np.dtype([("log2_bytes", np.float32), ("log2_ranks", np.float32), ("kind", np.int32),
                       ("variant", np.int32), ("dt", np.int32), ("op", np.int32), ("us", np.float32),
                       ("aligned", np.int32)])
        out = np.zeros(cap, dtype=dt)
        n = ctypes.c_size_t()
        self._check(lib().gpumpi_read_trace(self.h, _ptr(out), cap, ctypes.byref(n)), "read_trace")
        return out[: n.value]

    def last_kernel_ms(self) -> float:
        return lib().gpumpi_last_kernel_ms(self.h)

    def run_test(self, name: str, check: bool = False):
        """TestRunner::run equivalent: returns (rc, ok[nranks], outi[nranks,64], outd[nranks,64])."""
        n = self.nranks
        ok = np.zeros(n, dtype=np.uint8)
        oi = np.zeros((n, 64), dtype=np.int64)
        od = np.zeros((n, 64), dtype=np.float64)
        rc = lib().gpumpi_test_run(self.h, TESTS[name], _ptr(ok), _ptr(oi), _ptr(od))
        if check:
            self._check(rc, name)
        return rc, ok, oi, od

    @staticmethod
    def _params(i=(), p=(), d=()) -> Params:
        prm = Params()
        for k, v in enumerate(i):
            prm.i[k] = int(v)
        for k, v in enumerate(d):
            prm.d[k] = float(v)
        for k, v in enumerate(p):
            prm.p[k] = _ptr(v).value if v is not None else None
        return prm

    def run_program(self, program: int, i=(), p=(), d=(), stream=None, sync=True) -> int:
        prm = self._params(i, p, d)
        return lib().gpumpi_run_program(self.h, program, ctypes.byref(prm), _stream(stream), int(sync))

    def graph(self, program: int, i=(), p=(), d=()) -> "Graph":
        """Records one launch of `program` into a CUDA graph (replay with Graph.launch)."""
        prm = self._params(i, p, d)
        h = ctypes.c_void_p()
        self._check(lib().gpumpi_graph_create(self.h, program, ctypes.byref(prm), ctypes.byref(h)), "graph_create")
        return Graph(self, h)

    # ---- hot path ----
    def _ns(self, iters, iter_ns):
        if iter_ns is None:
            return None
        return iter_ns.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))

    def allreduce(self, send, recv, count, dt=FLOAT, op=OP_SUM, iters=1, iter_ns=None, stream=None):
        self._check(lib().gpumpi_allreduce(self.h, _ptr(send), _ptr(recv), count, dt, op, iters,
                                           self._ns(iters, iter_ns), _stream(stream)), "allreduce")

    def reduce(self, send, recv, count, dt=FLOAT, op=OP_SUM, root=0, iters=1, iter_ns=None, stream=None):
        self._check(lib().gpumpi_reduce(self.h, _ptr(send), _ptr(recv), count, dt, op, root, iters,
                                        self._ns(iters, iter_ns), _stream(stream)), "reduce")

    def bcast(self, buf, count, dt=FLOAT, root=0, iters=1, iter_ns=None, stream=None):
        self._check(lib().gpumpi_bcast(self.h, _ptr(buf), count, dt, root, iters, self._ns(iters, iter_ns),
                                       _stream(stream)), "bcast")

    def alltoall(self, send, recv, count_per_pair, dt=FLOAT, iters=1, iter_ns=None, stream=None):
        self._check(lib().gpumpi_alltoall(self.h, _ptr(send), _ptr(recv), count_per_pair, dt, iters,
                                          self._ns(iters, iter_ns), _stream(stream)), "alltoall")

    def allgather(self, send, recv, count, dt=FLOAT, iters=1, iter_ns=None, stream=None):
        self._check(lib().gpumpi_allgather(self.h, _ptr(send), _ptr(recv), count, dt, iters,
                                           self._ns(iters, iter_ns), _stream(stream)), "allgather")

    def alltoallv(self, send, send_stride, sendcounts, sdispls, recv, recv_stride, recvcounts, rdispls,
                  dt=INT, iters=1, iter_ns=None, stream=None):
        self._check(lib().gpumpi_alltoallv(self.h, _ptr(send), send_stride, _ptr(sendcounts), _ptr(sdispls),
                                           _ptr(recv), recv_stride, _ptr(recvcounts), _ptr(rdispls), dt, iters,
                                           self._ns(iters, iter_ns), _stream(stream)), "alltoallv")

    def pingpong(self, bufs, nbytes, pairs, iters=1, nonblocking=False, iter_ns=None, stream=None):
        self._check(lib().gpumpi_pingpong(self.h, _ptr(bufs), nbytes, pairs, iters, int(nonblocking),
                                          self._ns(iters, iter_ns), _stream(stream)), "pingpong")

    def ring(self, send, recv, nbytes, iters=1, nonblocking=False, iter_ns=None, stream=None):
        self._check(lib().gpumpi_ring(self.h, _ptr(send), _ptr(recv), nbytes, iters, int(nonblocking),
                                      self._ns(iters, iter_ns), _stream(stream)), "ring")

    def coll(self, kind: str, send, recv, count, dt, op=OP_SUM, root=0, iters=1, send_stride=0, recv_stride=0,
             mats=(None, None, None, None), iter_ns=None, rcs=None, stream=None, sync=True) -> int:
        """Generic P_COLL launch on device (torch) buffers; returns the MPI code."""
        return self.run_program(P_COLL, i=(COLL[kind], count, dt, op, root, iters, send_stride, recv_stride),
                                p=(send, recv, *mats, iter_ns, rcs), stream=stream, sync=sync)


class Graph:
    """A recorded launch of one program on one world."""

    def __init__(self, world: World, h):
        self.world, self.h = world, h

    def launch(self, stream=None, sync=True) -> int:
        return lib().gpumpi_graph_launch(self.h, _stream(stream), int(sync))

    def close(self):
        if self.h:
            lib().gpumpi_graph_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def kernel_launches() -> int:
    return int(lib().gpumpi_kernel_launches())
