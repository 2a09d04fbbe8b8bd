"""GPU: the application programs against the CPU oracle, bit-exact — the distributed bucket sort
(Alltoall of counts + Alltoallv of keys + local counting sort) and the 3D fp64 halo exchange with
derived-datatype faces (vector/hvector and subarray)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def oracle_keys(oracle, seed, n, kpr):
    return np.stack([oracle.bucket_keys(seed, r, kpr) for r in range(n)])


# 1001 keys per rank: rows of keys and of received keys start at every 4-byte offset modulo 16
@pytest.mark.parametrize("n,total,iters", [(16, 1 << 16, 2), (37, 37 * 1000, 1), (12, 12 * 1001, 2), (256, 1 << 25, 2)])
def test_bucket_sort_matches_oracle(gpulib, oracle, n, total, iters):
    from gpumpi import apps
    seed = 20251203
    kpr = total // n
    with gpulib.World(n, timeout_s=60.0) as w:
        rc, keys, out, counts = apps.bucket_sort(w, seed, total, iters=iters)
        assert rc == 0, w.last_error()
        keys, out, counts = keys.cpu().numpy(), out.cpu().numpy(), counts.cpu().numpy()
    ref_keys = oracle_keys(oracle, seed, n, kpr)
    assert np.array_equal(keys, ref_keys)            # device generator == oracle LCG stream
    ref_out, ref_cnt = oracle.bucket_sort(ref_keys.reshape(-1), n, out.shape[1])
    assert np.array_equal(counts, ref_cnt)
    assert counts.sum() == n * kpr
    for r in range(n):
        c = int(counts[r])
        assert np.array_equal(out[r, :c], ref_out[r, :c]), r


def test_bucket_sort_given_keys_with_empty_buckets(gpulib, oracle):
    """Keys supplied by the caller, all in the lower half of the range: half the ranks receive nothing
    (zero-count pieces in both collectives)."""
    from gpumpi import apps
    n, kpr = 32, 2048
    rng = np.random.default_rng(3)
    keys = rng.integers(0, 1 << 20, (n, kpr)).astype(np.int32)
    with gpulib.World(n, timeout_s=30.0) as w:
        rc, _, out, counts = apps.bucket_sort(w, 0, n * kpr, iters=1, keys=torch.from_numpy(keys).cuda())
        assert rc == 0, w.last_error()
        out, counts = out.cpu().numpy(), counts.cpu().numpy()
    ref_out, ref_cnt = oracle.bucket_sort(keys.reshape(-1), n, out.shape[1])
    assert np.array_equal(counts, ref_cnt) and (counts[n // 2:] == 0).all()
    for r in range(n):
        assert np.array_equal(out[r, :counts[r]], ref_out[r, :counts[r]])


@pytest.mark.parametrize("P,L,mode", [(2, 3, 0), (4, 8, 0), (4, 8, 1), (3, 5, 1)])
def test_halo_exchange_matches_oracle(gpulib, oracle, P, L, mode):
    from gpumpi import apps
    n = P ** 3
    with gpulib.World(n, timeout_s=30.0) as w:
        rc, blocks = apps.halo(w, P, L, iters=2, mode=mode)
        assert rc == 0, w.last_error()
        blocks = blocks.cpu().numpy()
    W = L + 2
    for r in range(n):
        assert np.array_equal(blocks[r].reshape(W, W, W), oracle.halo_expected(P, L, r)), r


def test_halo_exchange_full_grid_sampled(gpulib, oracle):
    """512^3 fp64 grid over 8x8x8 ranks (64^3 each): sampled ranks compared in full."""
    from gpumpi import apps
    P, L = 8, 64
    with gpulib.World(P ** 3, timeout_s=60.0) as w:
        rc, blocks = apps.halo(w, P, L, iters=1, mode=0)
        assert rc == 0, w.last_error()
        W = L + 2
        for r in (0, 7, 63, 64, 200, 448, 511):
            got = blocks[r].cpu().numpy().reshape(W, W, W)
            assert np.array_equal(got, oracle.halo_expected(P, L, r)), r
