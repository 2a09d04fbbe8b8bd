"""GPU: the allocation-free allreduce entry point, called through the C ABI.

gpumpi_allreduce_noalloc exists for callers that cannot allocate device memory when they need a
reduction (code inside allocator or memory-pool callbacks, processes with a fixed device-memory budget
reserved up front); its scratch is a static device array of fixed size.  Its output must equal the existing entry point's
(gpumpi_allreduce, which runs inside a world with allocated state) bit for bit — both fold in the
canonical rank order — on two calls in a row that share the static scratch.  Sizes beyond the stated
maximum must be rejected with an error.  When the kernel's bounded grid barrier runs out, the caller
learns it from gpumpi_allreduce_noalloc_status (tested through the test hook that makes the barrier wait
for an arrival that never comes, with a 0.1 s limit: no fault, the GPU stays usable).  This file is
collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def noalloc_fn(gpumpi):
    L = ctypes.CDLL(str(gpumpi.LIB_PATH))
    f = L.gpumpi_allreduce_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                  ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def status_fns(gpumpi):
    L = ctypes.CDLL(str(gpumpi.LIB_PATH))
    st = L.gpumpi_allreduce_noalloc_status
    st.argtypes = []
    st.restype = ctypes.c_int
    hook = L.gpumpi_noalloc_test_hook
    hook.argtypes = [ctypes.c_double, ctypes.c_int]
    hook.restype = ctypes.c_int
    return st, hook


@pytest.mark.parametrize("n,count,dt,op,tdt", [
    (64, 4099, 12, 2, torch.float32),      # fp32 SUM, ragged tail
    (1000, 1 << 14, 12, 2, torch.float32),
    (96, 3333, 2, 2, torch.int32),         # int32 SUM
    (33, 2048, 13, 0, torch.float64),      # fp64 MAX
])
def test_noalloc_matches_existing_entry_point_twice(gpulib, n, count, dt, op, tdt):
    f = noalloc_fn(gpulib)
    g = torch.Generator(device="cuda").manual_seed(n * 7 + count)
    with gpulib.World(n, timeout_s=20.0) as w:
        for call in range(2):  # two calls in a row share the static scratch
            if tdt.is_floating_point:
                x = (torch.rand((n, count), generator=g, device="cuda", dtype=tdt) * 2 - 1).contiguous()
            else:
                x = torch.randint(-1000, 1000, (n, count), generator=g, device="cuda", dtype=tdt).contiguous()
            ref = torch.empty_like(x)
            w.allreduce(x, ref, count, dt, op)
            out = torch.full_like(x, -7)
            rc = f(x.data_ptr(), out.data_ptr(), count, dt, op, n, None)
            assert rc == 0
            torch.cuda.synchronize()
            assert torch.equal(out, ref), f"call {call}: outputs differ"
            assert status_fns(gpulib)[0]() == 0


def test_noalloc_rejects_sizes_beyond_maximum(gpulib):
    f = noalloc_fn(gpulib)
    x = torch.zeros(8, device="cuda")
    too_many = 4097  # GPUMPI_NOALLOC_MAX_RANKS + 1
    assert f(x.data_ptr(), x.data_ptr(), 1, 12, 2, too_many, None) == 10  # GPUMPI_ERR_ARG
    assert f(x.data_ptr(), x.data_ptr(), 1, 29, 2, 2, None) == 4          # MPI_BYTE: GPUMPI_ERR_TYPE
    host = np.zeros(8, np.float32)
    assert f(host.ctypes.data, host.ctypes.data, 1, 12, 2, 2, None) == 2  # host memory: GPUMPI_ERR_BUFFER


def test_noalloc_reports_barrier_timeout(gpulib):
    f = noalloc_fn(gpulib)
    status, hook = status_fns(gpulib)
    n, count = 16, 1000
    x = torch.ones((n, count), device="cuda")
    out = torch.full_like(x, -7.0)
    assert hook(0.1, 1) == 0          # the barrier waits for one arrival that never comes, 0.1 s at most
    try:
        assert f(x.data_ptr(), out.data_ptr(), count, 12, 2, n, None) == 0   # the launch itself succeeds
        torch.cuda.synchronize()
        assert status() == 15         # GPUMPI_ERR_TIMEOUT
        assert bool((out == -7.0).all())  # nothing was written
    finally:
        assert hook(0.0, 0) == 0
    # the GPU and the scratch stay usable: the next call succeeds and clears the error word
    assert f(x.data_ptr(), out.data_ptr(), count, 12, 2, n, None) == 0
    torch.cuda.synchronize()
    assert status() == 0
    assert bool((out == float(n)).all())
