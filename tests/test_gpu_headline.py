"""GPU parity at the sizes the benchmark times, against the CPU oracle, through the C ABI.

* MPI_Allreduce(SUM) fp32 among 1024 ranks x 1 MiB (the benchmark's headline): every rank's result is
  bit-identical to the oracle's canonical rank-order fold (gpu_libs/gpu_mpi/mpi.cu:209-225,
  operators.cu:216-218), for the default choice and for the canonical variants.
* MPI_Allreduce at 2048 ranks, int32 and fp32 (ragged count): bit-exact.
* MPI_Alltoallv int32 among 1024 ranks with the benchmark's counts (uniform in [0, 512] per pair, so most
  pieces sit at a different 16-byte alignment in sender and receiver): bit-exact, every variant.
* The reordered variants (TREE, RING) against an exact sum, at the stated tolerance: the error of each
  element relative to sum_r |x_r| (the scale any summation order's rounding error is proportional to)
  is at most 1e-6 for fp32 and 1e-14 for fp64, at 1024 ranks.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

THREADS = os.cpu_count() or 1


def bits(t):
    """Integer view for bit-for-bit comparison of floating-point tensors."""
    return t.view(torch.int32) if t.element_size() == 4 else t.view(torch.int64)


def check_all_ranks(gpu_out, ref_row):
    """Every rank's row of gpu_out (on the device) equals ref_row bit for bit."""
    ref = torch.from_numpy(np.ascontiguousarray(ref_row)).cuda()
    eq = bits(gpu_out) == bits(ref).unsqueeze(0)
    bad = (~eq.all(1)).nonzero().flatten()
    assert bad.numel() == 0, f"{bad.numel()} ranks differ, first {bad[:8].tolist()}"


@pytest.mark.parametrize("variant", [-1, 0, 3])   # default, DIRECT, STAGED: all canonical order
def test_headline_allreduce_fp32_1024ranks_1MiB_bit_exact(gpulib, oracle, variant):
    n, count = 1024, (1 << 20) // 4
    x = oracle.fill_f32(2026, n * count).reshape(n, count)
    ref = oracle.reduce(x, gpulib.FLOAT, gpulib.OP_SUM)
    s = torch.from_numpy(x).cuda()
    r = torch.empty_like(s)
    with gpulib.World(n, timeout_s=30.0) as w:
        if variant >= 0:
            w.set_policy(variant, 0)
        w.allreduce(s, r, count, gpulib.FLOAT, gpulib.OP_SUM, iters=2)
        torch.cuda.synchronize()
    check_all_ranks(r, ref)


@pytest.mark.parametrize("dt,count", [(2, 1 << 16), (12, (1 << 16) + 1)])
def test_allreduce_2048ranks_bit_exact(gpulib, oracle, dt, count):
    n = 2048
    if dt == 12:
        x = oracle.fill_f32(77, n * count).reshape(n, count)
    else:
        x = (oracle.fill_i32(78, n * count) % 100000).reshape(n, count)
    ref = oracle.reduce(x, dt, gpulib.OP_SUM)
    s = torch.from_numpy(x).cuda()
    r = torch.empty_like(s)
    with gpulib.World(n, timeout_s=30.0) as w:
        w.allreduce(s, r, count, dt, gpulib.OP_SUM)
        torch.cuda.synchronize()
    check_all_ranks(r, ref)


def bench_counts(n, seed=4242, hi=512):
    """The benchmark's uneven exchange: counts uniform in [0, hi] per pair, packed displacements."""
    rng = np.random.default_rng(seed)
    sc = rng.integers(0, hi + 1, (n, n)).astype(np.int32)
    rc = sc.T.copy()
    sd = (np.cumsum(sc, 1) - sc).astype(np.int32)
    rd = (np.cumsum(rc, 1) - rc).astype(np.int32)
    return sc, sd, rc, rd, int(sc.sum(1).max()), int(rc.sum(1).max())


def test_alltoallv_1024ranks_bench_counts_bit_exact(gpulib, oracle):
    n = 1024
    sc, sd, rc, rd, S, R = bench_counts(n)
    x = oracle.fill_i32(99, n * S).reshape(n, S)
    ref = oracle.alltoallv(x, sc, sd, R, rc, rd, threads=THREADS)
    s = torch.from_numpy(x).cuda()
    dsc, dsd, drc, drd = (torch.from_numpy(a).cuda() for a in (sc, sd, rc, rd))
    with gpulib.World(n, timeout_s=30.0) as w:
        for v in (-1, 0, 1, 2, 3):
            if v >= 0:
                w.set_policy(v, 0)
            r = torch.zeros((n, R), dtype=torch.int32, device="cuda")   # as the oracle's output
            w.alltoallv(s, S * 4, dsc, dsd, r, R * 4, drc, drd, gpulib.INT)
            torch.cuda.synchronize()
            got = r.cpu().numpy()
            bad = np.nonzero((got != ref).any(1))[0]
            assert bad.size == 0, (v, bad[:8].tolist())


def exact_sum(x):
    """Sum over axis 0 in double-double (Neumaier's compensated summation, with the two-sum of Knuth
    for the compensation): exact to far below fp64 rounding for these sizes."""
    s = np.zeros(x.shape[1], np.float64)
    c = np.zeros(x.shape[1], np.float64)
    for row in x.astype(np.float64):
        t = s + row
        bp = t - s
        c += (s - (t - bp)) + (row - bp)
        s = t
    return s + c


@pytest.mark.parametrize("dt,npdt,count,tol", [(12, np.float32, 1 << 16, 1e-6), (13, np.float64, 1 << 14, 1e-14)])
def test_reordered_variants_within_stated_tolerance(gpulib, oracle, dt, npdt, count, tol):
    n = 1024
    x = oracle.fill_f64(31 + dt, n * count).astype(npdt).reshape(n, count)
    exact = exact_sum(x)
    scale = np.abs(x.astype(np.float64)).sum(0)
    canon = oracle.reduce(x, dt, gpulib.OP_SUM)
    s = torch.from_numpy(x).cuda()
    with gpulib.World(n, timeout_s=30.0) as w:
        for v in (0, 1, 2):     # DIRECT (canonical) meets the same bound; TREE and RING are reordered
            w.set_policy(v, 0)
            r = torch.empty_like(s)
            w.allreduce(s, r, count, dt, gpulib.OP_SUM)
            torch.cuda.synchronize()
            got = r.cpu().numpy()
            assert (got == got[0]).all(), v                     # every rank holds the same result
            err = np.abs(got[0].astype(np.float64) - exact) / scale
            assert err.max() <= tol, (v, float(err.max()))
            if v == 0:
                assert np.array_equal(got[0].view(np.uint8), canon.view(np.uint8))
