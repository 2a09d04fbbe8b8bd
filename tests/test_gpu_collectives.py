"""GPU parity of the hot path against the CPU oracle, through the C ABI: bit-exact for integer and
byte data and for floating-point reductions in the canonical rank order."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


ALLREDUCE_CASES = [
    # ranks, count, dt, op, numpy dtype
    (2, 1, 2, 2, np.int32),
    (7, 17, 13, 2, np.float64),
    (32, 1000, 12, 2, np.float32),
    (64, 4096, 12, 2, np.float32),
    (128, 3333, 2, 2, np.int32),
    (256, 1 << 14, 13, 2, np.float64),
    (64, 2048, 12, 0, np.float32),
    (64, 2048, 2, 1, np.int32),
    (48, 777, 20, 3, np.int64),
    (33, 1025, 2, 9, np.int32),
    (16, 100, 18, 3, np.int16),      # generic path, wraps
    (16, 64, 16, 8, np.uint8),       # bool LXOR (reference semantics)
    (1024, 1 << 12, 12, 2, np.float32),
]


def make_input(oracle, n, count, npdt, seed):
    if np.issubdtype(npdt, np.floating):
        x = oracle.fill_f64(seed, n * count).astype(npdt)
    else:
        x = oracle.fill_i32(seed, n * count)
        if npdt == np.uint8:
            x = (x & 1).astype(npdt)
        else:
            x = (x % 1000).astype(npdt)
    return x.reshape(n, count)


@pytest.mark.parametrize("n,count,dt,op,npdt", ALLREDUCE_CASES)
def test_allreduce_matches_oracle_bit_exact(gpulib, oracle, n, count, dt, op, npdt):
    x = make_input(oracle, n, count, npdt, 1000 + n + count)
    ref = oracle.allreduce(x, dt, op)
    with gpulib.World(n, timeout_s=10.0) as w:
        s, r = dev(x), dev(np.zeros_like(x))
        w.allreduce(s, r, count, dt, op)
        got = host(r)
    assert np.array_equal(got.view(np.uint8), ref.view(np.uint8))


def test_allreduce_host_buffers_and_in_place(gpulib, oracle):
    n, count = 24, 5000
    x = make_input(oracle, n, count, np.float32, 5)
    ref = oracle.allreduce(x, 12, 2)
    with gpulib.World(n, timeout_s=10.0) as w:
        out = np.zeros_like(x)
        w.allreduce(x, out, count, 12, 2)          # host (numpy) buffers, staged by the library
        assert np.array_equal(out, ref)
        buf = dev(x)
        rc = w.coll("allreduce", 1, buf, count, 12, 2, send_stride=0, recv_stride=count * 4)  # MPI_IN_PLACE
        assert rc == 0, w.last_error()
        assert np.array_equal(host(buf), ref)


def test_pinned_host_buffers_in_place_and_staged(gpulib, oracle):
    """Page-locked host buffers are read and written in place by the kernel (TUNE_HOST_DIRECT 1, the
    default) or staged through device memory (0): both bit-exact, for a fold and for a pull, with every
    variant requested (STAGED runs as DIRECT on host memory: no bulk copies from the host)."""
    n, count = 64, 3000
    x = make_input(oracle, n, count, np.int32, 11)   # integers: every variant's order gives the same sum
    ref = oracle.allreduce(x, 2, 2)
    rng = np.random.default_rng(3)
    sc, sd, rc, rd, S, R = uneven_exchange(rng, n, 90, 0.2, min_c=0)
    y = oracle.fill_i32(n + 2, n * S).reshape(n, S)
    ref_v = oracle.alltoallv(y, sc, sd, R, rc, rd)
    hx = torch.from_numpy(x).pin_memory()
    hy = torch.from_numpy(y).pin_memory()
    with gpulib.World(n, timeout_s=10.0) as w:
        w.set_tuning(gpulib.TUNE_DYN_SMEM, -1)
        for direct in (1, 0):
            w.set_tuning(gpulib.TUNE_HOST_DIRECT, direct)
            for v in range(4):
                w.set_policy(v, 0)
                out = torch.zeros(n, count, dtype=torch.int32).pin_memory()
                w.allreduce(hx.numpy(), out.numpy(), count, 2, 2)
                assert np.array_equal(out.numpy(), ref), (direct, v)
                outv = torch.zeros(n, R, dtype=torch.int32).pin_memory()
                w.alltoallv(hy.numpy(), S * 4, sc, sd, outv.numpy(), R * 4, rc, rd, 2)
                assert np.array_equal(outv.numpy(), ref_v), (direct, v)


@pytest.mark.parametrize("mode", [2, 3, 4])
def test_sliced_host_allreduce_matches_oracle(gpulib, oracle, mode):
    """An Allreduce between host buffers cut into column slices (TUNE_HOST_DIRECT 2..4, one launch per
    slice, copies of later slices overlapping the folds of earlier ones) is bit-exact with the oracle:
    page-locked and pageable buffers, a ragged last slice, copies split over one or three streams,
    floating point in the canonical order."""
    n = 64
    cases = [(20000, 12, 2, np.float32), (9000, 13, 2, np.float64), (12343, 2, 0, np.int32)]
    with gpulib.World(n, timeout_s=10.0) as w:
        w.set_tuning(gpulib.TUNE_HOST_DIRECT, mode)
        w.set_tuning(gpulib.TUNE_HOST_SLICE, 16 << 10)
        assert w.get_tuning(gpulib.TUNE_HOST_DIRECT) == mode
        for count, dt, op, npdt in cases:
            w.set_tuning(gpulib.TUNE_HOST_STREAMS, 3 if dt == 13 else 1)   # row groups of 21, 21 and 22 ranks
            count -= count % (16 // np.dtype(npdt).itemsize)     # rows 16-byte aligned: the sliced path
            x = make_input(oracle, n, count, npdt, 40 + count)
            ref = oracle.allreduce(x, dt, op)
            for pinned in (True, False):
                hx = torch.from_numpy(x)
                out = torch.zeros_like(hx)
                if pinned:
                    hx, out = hx.pin_memory(), out.pin_memory()
                for _ in range(2):
                    out.zero_()
                    w.allreduce(hx.numpy(), out.numpy(), count, dt, op)
                    assert np.array_equal(out.numpy().view(np.uint8), ref.view(np.uint8)), (count, dt, pinned)
        # a rank's error reaches the caller through the slices' records: bitwise AND is illegal on floats
        x = torch.from_numpy(make_input(oracle, n, 8192, np.float32, 3)).pin_memory()
        out = torch.zeros_like(x).pin_memory()
        with pytest.raises(gpulib.GpumpiError) as e:
            w.allreduce(x.numpy(), out.numpy(), 8192, 12, gpulib.OP_BAND)
        w.set_tuning(gpulib.TUNE_HOST_DIRECT, 1)
        with pytest.raises(gpulib.GpumpiError) as e1:
            w.allreduce(x.numpy(), out.numpy(), 8192, 12, gpulib.OP_BAND)
        assert e.value.code == e1.value.code


@pytest.mark.parametrize("n,count,dt,npdt", [(32, 1000, 12, np.float32), (128, 257, 13, np.float64),
                                              (200, 1024, 2, np.int32), (513, 100, 12, np.float32)])
def test_static_split_reductions_match_the_job_path(gpulib, oracle, n, count, dt, npdt):
    """Reductions of at most TUNE_STATIC_FOLD bytes per member run without a job (the members split the
    chunks statically between two barriers): bit-exact with the oracle and with the job path, for
    Allreduce, Allreduce in place and Reduce to a non-zero root."""
    x = make_input(oracle, n, count, npdt, 77 + n)
    ref = oracle.allreduce(x, dt, 2)
    root = n // 3
    with gpulib.World(n, timeout_s=10.0) as w:
        for thr in (1 << 20, 0):           # static split, then the job path
            w.set_tuning(gpulib.TUNE_STATIC_FOLD, thr)
            assert w.get_tuning(gpulib.TUNE_STATIC_FOLD) == thr
            s, r = dev(x), dev(np.zeros_like(x))
            w.allreduce(s, r, count, dt, 2)
            assert np.array_equal(host(r).view(np.uint8), ref.view(np.uint8)), thr
            buf = dev(x)
            rc = w.coll("allreduce", 1, buf, count, dt, 2, send_stride=0, recv_stride=count * x.itemsize)
            assert rc == 0 and np.array_equal(host(buf).view(np.uint8), ref.view(np.uint8)), thr
            r = dev(np.zeros_like(x))
            w.reduce(dev(x), r, count, dt, 2, root=root)
            got = host(r)
            assert np.array_equal(got[root].view(np.uint8), ref[root].view(np.uint8)), thr


def test_allreduce_variants_agree(gpulib, oracle):
    n, count = 64, 1 << 14
    x = make_input(oracle, n, count, np.float32, 9)
    ref = oracle.allreduce(x, 12, 2)
    ref64 = x.astype(np.float64).sum(0)
    with gpulib.World(n, timeout_s=10.0) as w:
        for v in range(4):
            w.set_policy(v, 0)
            s, r = dev(x), dev(np.zeros_like(x))
            w.allreduce(s, r, count, 12, 2)
            got = host(r)
            if v in (0, 3):   # canonical order: bit-exact
                assert np.array_equal(got, ref), v
            else:
                # reordered (TREE groups, RING rotation): the error of every element against the fp64
                # sum, relative to sum_r |x_r| (the scale of any summation order's rounding error), is at
                # most 1e-6, the stated fp32 tolerance
                scale = np.abs(x).astype(np.float64).sum(0) + 1e-30
                rel = np.abs(got[0].astype(np.float64) - ref64) / scale
                assert rel.max() <= 1e-6, (v, rel.max())
                assert (got == got[0]).all()


@pytest.mark.parametrize("n,count", [(64, 1 << 14), (1024, 4096), (200, 777)])
def test_allreduce_variants_exact_on_integers(gpulib, oracle, n, count):
    x = make_input(oracle, n, count, np.int32, 17)
    ref = oracle.allreduce(x, 2, 2)
    with gpulib.World(n, timeout_s=10.0) as w:
        for v in range(4):
            w.set_policy(v, 0)
            s, r = dev(x), dev(np.zeros_like(x))
            w.allreduce(s, r, count, 2, 2)
            assert np.array_equal(host(r), ref), v


@pytest.mark.parametrize("n,count,root,dt", [(5, 14, 0, 2), (33, 1000, 7, 13), (100, 4096, 99, 12)])
def test_reduce_matches_oracle(gpulib, oracle, n, count, root, dt):
    npdt = {2: np.int32, 12: np.float32, 13: np.float64}[dt]
    x = make_input(oracle, n, count, npdt, 77)
    ref = oracle.reduce(x, dt, 2)
    with gpulib.World(n, timeout_s=10.0) as w:
        s, r = dev(x), dev(np.zeros_like(x))
        w.reduce(s, r, count, dt, 2, root)
        got = host(r)
    assert np.array_equal(got[root], ref)


@pytest.mark.parametrize("n,count,root", [(2, 1, 1), (7, 10, 3), (64, 1 << 16, 5), (300, 333, 299)])
def test_bcast(gpulib, oracle, n, count, root):
    x = np.zeros((n, count), np.int32)
    x[root] = oracle.fill_i32(3, count)
    with gpulib.World(n, timeout_s=10.0) as w:
        b = dev(x)
        w.bcast(b, count, 2, root)
        got = host(b)
    assert (got == x[root]).all()


@pytest.mark.parametrize("n,c", [(3, 1), (10, 16), (64, 256), (256, 37), (32, 20000)])
def test_alltoall(gpulib, oracle, n, c):
    x = oracle.fill_i32(11 + n, n * n * c).reshape(n, n * c)
    sc = np.full((n, n), c, np.int32)
    d = np.tile(np.arange(n, dtype=np.int32) * c, (n, 1))
    ref = oracle.alltoallv(x, sc, d, n * c, sc, d)
    with gpulib.World(n, timeout_s=10.0) as w:
        s, r = dev(x), dev(np.zeros_like(x))
        w.alltoall(s, r, c, 2)
        got = host(r)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("n,maxc,zero_frac", [(4, 5, 0.3), (37, 40, 0.5), (256, 300, 0.2), (128, 3, 0.9)])
def test_alltoallv_uneven_and_zero_counts(gpulib, oracle, n, maxc, zero_frac):
    # zero-count pairs abort the reference (hazard H2: assert(dataSize > 0), mpi.cu:548-549)
    rng = np.random.default_rng(n)
    sc = rng.integers(1, maxc + 1, (n, n)).astype(np.int32)
    sc[rng.random((n, n)) < zero_frac] = 0
    rc = sc.T.copy()
    sd = np.concatenate([np.zeros((n, 1), np.int32), np.cumsum(sc, 1)[:, :-1]], 1).astype(np.int32)
    rd = np.concatenate([np.zeros((n, 1), np.int32), np.cumsum(rc, 1)[:, :-1]], 1).astype(np.int32)
    S = int(sc.sum(1).max()) + 1
    R = int(rc.sum(1).max()) + 1
    x = oracle.fill_i32(n, n * S).reshape(n, S)
    ref = oracle.alltoallv(x, sc, sd, R, rc, rd)
    with gpulib.World(n, timeout_s=10.0) as w:
        s, r = dev(x), dev(np.zeros((n, R), np.int32))
        w.alltoallv(s, S * 4, dev(sc), dev(sd), r, R * 4, dev(rc), dev(rd), 2)
        got = host(r)
    assert np.array_equal(got, ref)


def test_alltoallv_chunks_per_worker(gpulib, oracle):
    """Pull jobs cut into 1..7 chunks per worker block (and a knob out of range refused): the pieces reach
    the same places whatever the chunking, including chunks that end inside a run of touching pieces."""
    n = 160
    rng = np.random.default_rng(31)
    sc, sd, rc, rd, S, R = uneven_exchange(rng, n, 900, 0.2, min_c=0)
    x = oracle.fill_i32(n + 3, n * S).reshape(n, S)
    ref = oracle.alltoallv(x, sc, sd, R, rc, rd)
    with gpulib.World(n, timeout_s=20.0) as w:
        with pytest.raises(gpulib.GpumpiError):
            w.set_tuning(gpulib.TUNE_PULL_CHUNKS, 0)
        for ch in (1, 3, 7):
            w.set_tuning(gpulib.TUNE_PULL_CHUNKS, ch)
            assert w.get_tuning(gpulib.TUNE_PULL_CHUNKS) == ch
            s, r = dev(x), dev(np.zeros((n, R), np.int32))
            w.alltoallv(s, S * 4, dev(sc), dev(sd), r, R * 4, dev(rc), dev(rd), 2, iters=2)
            assert np.array_equal(host(r), ref), ch


def uneven_exchange(rng, n, maxc, zero_frac, min_c=1):
    sc = rng.integers(min_c, maxc + 1, (n, n)).astype(np.int32)
    sc[rng.random((n, n)) < zero_frac] = 0
    rc = sc.T.copy()
    sd = np.concatenate([np.zeros((n, 1), np.int32), np.cumsum(sc, 1)[:, :-1]], 1).astype(np.int32)
    rd = np.concatenate([np.zeros((n, 1), np.int32), np.cumsum(rc, 1)[:, :-1]], 1).astype(np.int32)
    return sc, sd, rc, rd, int(sc.sum(1).max()) + 1, int(rc.sum(1).max()) + 1


@pytest.mark.parametrize("n,maxc,dt,npdt", [(64, 3000, 0, np.int8),       # CHAR: every byte shift 0..15
                                            (48, 700, 2, np.int32),       # int32: shifts 0/4/8/12
                                            (96, 13, 13, np.float64),     # tiny pieces, edges only
                                            (8, 40000, 2, np.int32)])     # >= 64 KiB pieces: split parts
def test_alltoallv_piece_orders_and_shifts(gpulib, oracle, n, maxc, dt, npdt):
    """Every pull variant (receiver-major, sender-major and rotated piece orders; bulk-copy staging) on
    displacements that put source and destination at every relative alignment."""
    rng = np.random.default_rng(maxc + n)
    sc, sd, rc, rd, S, R = uneven_exchange(rng, n, maxc, 0.1, min_c=0)
    x = oracle.fill_i32(n + 1, n * S).astype(npdt).reshape(n, S)
    ref = oracle.alltoallv(x, sc, sd, R, rc, rd)
    with gpulib.World(n, timeout_s=20.0, trace_capacity=64) as w:
        w.set_tuning(gpulib.TUNE_DYN_SMEM, -1)   # room for the STAGED variant's shared-memory stages
        for v in range(4):
            w.set_policy(v, 0)
            s, r = dev(x), dev(np.zeros((n, R), npdt))
            w.alltoallv(s, S * x.itemsize, dev(sc), dev(sd), r, R * x.itemsize, dev(rc), dev(rd), dt)
            got = host(r)
            assert np.array_equal(got.view(np.uint8), ref.view(np.uint8)), v
            assert set(w.read_trace()["variant"].tolist()) == {v}   # the trace covers the last launch


@pytest.mark.parametrize("n,c", [(7, 7), (100, 64), (512, 3)])
def test_allgather(gpulib, oracle, n, c):
    x = oracle.fill_i32(5, n * c).reshape(n, c)
    with gpulib.World(n, timeout_s=10.0) as w:
        s, r = dev(x), dev(np.zeros((n, n * c), np.int32))
        w.allgather(s, r, c, 2)
        got = host(r)
    assert (got == x.reshape(1, -1)).all()


@pytest.mark.parametrize("n,nbytes,nb", [(2, 8, False), (4, 4096, True), (8, 1 << 20, False), (256, 1 << 16, True),
                                         (128, 1 << 24, True)])
def test_ring_bytes_exact(gpulib, oracle, n, nbytes, nb):
    x = oracle.fill_i32(n, n * nbytes // 4).view(np.uint8).reshape(n, nbytes)
    with gpulib.World(n, timeout_s=20.0) as w:
        s, r = dev(x), dev(np.zeros_like(x))
        w.ring(s, r, nbytes, iters=2, nonblocking=nb)
        got = host(r)
    assert np.array_equal(got, np.roll(x, 1, axis=0))


@pytest.mark.parametrize("nbytes", [8, 1024, 1 << 20, 1 << 26])
def test_pingpong_round_trip_exact(gpulib, oracle, nbytes):
    n = 4
    x = oracle.fill_i32(nbytes, n * nbytes // 4).view(np.uint8).reshape(n, nbytes)
    with gpulib.World(n, timeout_s=20.0) as w:
        b = dev(x)
        w.pingpong(b, nbytes, 2, iters=3)
        got = host(b)
    # after each round trip both ranks of a pair hold the even rank's data
    for p in range(2):
        assert np.array_equal(got[2 * p], x[2 * p]) and np.array_equal(got[2 * p + 1], x[2 * p])


def test_pi_bit_exact(gpulib, oracle):
    n, pairs, seed = 64, 1 << 14, 20251203
    with gpulib.World(n, timeout_s=20.0) as w:
        hits = np.zeros(n, np.int64)
        tot = np.zeros(1, np.int64)
        hd, td = dev(hits), dev(tot)
        rc = w.run_program(gpulib.P_PI, i=(seed, pairs), p=(hd, td))
        assert rc == 0, w.last_error()
        hits, tot = host(hd), host(td)
    ref = [oracle.pi_hits(seed, r, pairs) for r in range(n)]
    assert hits.tolist() == ref and int(tot[0]) == sum(ref)


@pytest.mark.parametrize("name,n", [("p2p_matching", 5), ("datatypes", 2), ("subcomm_coll", 13), ("errors", 4)])
def test_extended_programs(gpulib, name, n):
    with gpulib.World(n, timeout_s=10.0) as w:
        rc, ok, oi, od = w.run_test(name)
    assert rc == 0 and ok.all(), (name, ok, oi[:, :10])


@pytest.mark.parametrize("n", [2, 37])
def test_attributes_and_timer(gpulib, n):
    """Keyvals and cached attributes (copy functions on MPI_Comm_dup, delete functions on MPI_Attr_delete,
    on replacement and on MPI_Comm_free; MPI_TAG_UB) and the timer: MPI_Wtime never goes backwards, is
    one clock for all ranks (every rank's reading before a world barrier precedes every rank's reading
    after it), and MPI_Wtick reports a positive step of at most 10 us."""
    with gpulib.World(n, timeout_s=10.0) as w:
        rc, ok, oi, od = w.run_test("attrs")
    assert rc == 0 and ok.all(), (ok, oi[:, 0])
    assert (oi[:, 0] == 301).all()
    assert od[:, 0].max() <= od[:, 1].min()
    assert (od[:, 2] > 0).all() and (od[:, 2] <= 1e-5).all()


def test_timeout_returns_error_not_hang(gpulib):
    # failure detection without a GPU fault: a receive that nobody matches ends in MPI_ERR_OTHER
    with gpulib.World(3, timeout_s=0.5) as w:
        rc, ok, oi, od = w.run_test("timeout")
        assert ok.all() and oi[0, 0] == gpulib.ERR_OTHER
        assert rc == gpulib.ERR_TIMEOUT
        # the world is still usable afterwards
        rc2, ok2, _, _ = w.run_test("sample")
        assert rc2 == 0 and ok2.all()


@pytest.mark.parametrize("n", [2, 33, 300, 1024])
def test_tiny_reductions_all_types_bit_exact(gpulib, oracle, n):
    """Reductions of at most 64 bytes per rank take the one-barrier path (operands inline, folded by each
    member in rank order): bit-exact with the oracle for every legal (type, op) pair tried, in place too."""
    cases = [(12, 2, np.float32, 16), (13, 2, np.float64, 8), (2, 3, np.int32, 5), (20, 0, np.int64, 3),
             (12, 1, np.float32, 1), (18, 2, np.int16, 32), (16, 8, np.uint8, 64), (2, 9, np.int32, 7)]
    with gpulib.World(n, timeout_s=10.0) as w:
        for k, (dt, op, npdt, count) in enumerate(cases):
            x = make_input(oracle, n, count, npdt, 300 + k)
            ref = oracle.allreduce(x, dt, op)
            s, r = dev(x), dev(np.zeros_like(x))
            w.allreduce(s, r, count, dt, op)
            assert np.array_equal(host(r).view(np.uint8), ref.view(np.uint8)), (dt, op, count)
        x = make_input(oracle, n, 7, np.float64, 77)
        ref = oracle.allreduce(x, 13, 2)
        buf = dev(x)
        rc = w.coll("allreduce", 1, buf, 7, 13, 2, send_stride=0, recv_stride=7 * 8)  # MPI_IN_PLACE
        assert rc == 0 and np.array_equal(host(buf), ref)
        x = make_input(oracle, n, 9, np.int32, 78)
        refr = oracle.reduce(x, 2, 2)
        s, r = dev(x), dev(np.zeros_like(x))
        w.reduce(s, r, 9, 2, 2, n - 1)
        assert np.array_equal(host(r)[n - 1], refr)


@pytest.mark.parametrize("n", [3, 64, 512])
def test_tiny_collectives_back_to_back(gpulib, n):
    # tiny Allreduce / Allreduce on a split / Bcast / Reduce / Allgather, 200 rounds, skewed ranks
    ok = torch.zeros(n, dtype=torch.uint8, device="cuda")
    oi = torch.zeros((n, 64), dtype=torch.int64, device="cuda")
    od = torch.zeros((n, 64), dtype=torch.float64, device="cuda")
    rows = torch.zeros((n, n), dtype=torch.int32, device="cuda")
    with gpulib.World(n, timeout_s=20.0) as w:
        rc = w.run_program(gpulib.TESTS["tiny_stress"], p=(ok, oi, od, rows))
    bad = host(oi)[:, 0]
    assert rc == 0 and host(ok).all(), bad[bad >= 0][:10]


@pytest.mark.parametrize("n", [2, 5, 33, 64])
def test_small_paths_mixed_buffers_and_types(gpulib, n):
    # members choose the small paths by size alone, so stack and global buffers and strided and
    # contiguous same-signature datatypes can meet in one call
    ok = torch.zeros(n, dtype=torch.uint8, device="cuda")
    oi = torch.zeros((n, 64), dtype=torch.int64, device="cuda")
    od = torch.zeros((n, 64), dtype=torch.float64, device="cuda")
    scratch = torch.zeros((n, 288), dtype=torch.int32, device="cuda")
    with gpulib.World(n, timeout_s=20.0) as w:
        rc = w.run_program(gpulib.TESTS["tiny_mixed"], p=(ok, oi, od, scratch))
    assert rc == 0 and host(ok).all(), host(ok)
