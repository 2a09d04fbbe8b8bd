"""CPU: the oracle (a C restatement of the reference's semantics) against the known answers of the
reference's own tests (tests/golden/reference_tests.json, made by tests/golden/make_golden.py from the
formulas in the reference's tests/*.cu), plus properties of the restated algorithms."""
import json
from pathlib import Path

import numpy as np
import pytest

GOLD = json.loads((Path(__file__).parent / "golden" / "reference_tests.json").read_text())


def test_reduce_int16_prod_matches_reference_test(oracle):
    # collectives_test.cu:6-54 : (r+1)(i+1), int16 PROD over 5 ranks, wraps
    g = GOLD["reduce_int16_prod"]
    x = np.array([[(r + 1) * (i + 1) for i in range(g["count"])] for r in range(g["ranks"])], dtype=np.int16)
    out = oracle.reduce(x, 18, 3)
    assert out.tolist() == g["expected"]


def test_allreduce_f64_matches_reference_test(oracle):
    g = GOLD["allreduce_f64_sum"]
    x = np.array([[(r + 1) * (i + 1) for i in range(g["count"])] for r in range(g["ranks"])], dtype=np.float64)
    out = oracle.allreduce(x, 13, 2)
    for r in range(g["ranks"]):
        assert np.allclose(out[r], g["expected"], atol=g["tol"], rtol=0)


def test_allgather_and_scatter_layouts(oracle):
    g = GOLD["allgather_int"]
    n, c = g["ranks"], g["count"]
    send = np.array([[(r + 1) * (i + 1) for i in range(c)] for r in range(n)], dtype=np.int32)
    # allgather = alltoallv where every sender sends its whole buffer to every receiver
    sc = np.full((n, n), c, np.int32)
    sd = np.zeros((n, n), np.int32)
    rd = np.tile(np.arange(n, dtype=np.int32) * c, (n, 1))
    recv = oracle.alltoallv(send, sc, sd, n * c, sc, rd)
    for r in range(n):
        assert recv[r].tolist() == g["expected"]


def test_comm_split_matches_reference_test(oracle):
    g = GOLD["comm_split"]
    nr, ns = oracle.comm_split(g["colors"], g["keys"])
    assert nr.tolist() == g["newrank"] and ns.tolist() == g["newsize"]


def test_comm_split_undefined_colour(oracle):
    nr, ns = oracle.comm_split([0, -1, 0, -1], [3, 0, 1, 0])
    assert nr.tolist() == [1, -1, 0, -1] and ns.tolist() == [2, 0, 2, 0]


def test_op_legality_table(oracle):
    # operators.cu:153-200
    assert oracle.op_allowed(2, 12) and not oracle.op_allowed(5, 12)      # SUM ok, BAND not on float
    assert oracle.op_allowed(4, 16) and not oracle.op_allowed(2, 16)      # LAND on bool, SUM not
    assert oracle.op_allowed(9, 29) and not oracle.op_allowed(2, 29)      # BXOR on byte
    assert not oracle.op_allowed(0, 0) and not oracle.op_allowed(0, 15)   # text types: nothing
    assert oracle.op_allowed(2, 27) and not oracle.op_allowed(0, 27)      # complex SUM, no MAX
    assert oracle.op_allowed(10, 30) and not oracle.op_allowed(10, 2)     # MAXLOC on pair types only


def test_reference_op_quirks(oracle):
    # LXOR is (in != inout) on raw values (operators.cu:143-144): 2 LXOR 1 -> 1
    x = np.array([[2], [1]], dtype=np.int32)
    assert oracle.reduce(x, 2, 8).tolist() == [1]
    # MAX(in, acc) = in > acc ? in : acc : a NaN accumulator stays NaN, a NaN input is skipped
    x = np.array([[np.nan], [1.0]], dtype=np.float32)
    assert np.isnan(oracle.reduce(x, 12, 0)[0])
    x = np.array([[1.0], [np.nan]], dtype=np.float32)
    assert oracle.reduce(x, 12, 0)[0] == 1.0
    # canonical order: ((x0 + x1) + x2) in float32
    x = np.array([[1e8], [1.0], [-1e8]], dtype=np.float32)
    assert oracle.reduce(x, 12, 2).tolist() == [np.float32(np.float32(1e8 + 1.0) - np.float32(1e8))]


def test_canonical_fold_equals_numpy_left_fold(oracle):
    rng = np.random.default_rng(0)
    x = rng.standard_normal((37, 1000)).astype(np.float32)
    out = oracle.reduce(x, 12, 2)
    ref = x[0].copy()
    for r in range(1, 37):
        ref = (x[r] + ref).astype(np.float32)
    assert np.array_equal(out, ref)


def test_allreduce_threads_do_not_change_bits(oracle):
    x = oracle.fill_f32(7, 64 * 4097).reshape(64, 4097)
    a = oracle.allreduce(x, 12, 2, threads=1)
    b = oracle.allreduce(x, 12, 2, threads=8)
    assert np.array_equal(a, b)


def test_alltoallv_zero_and_uneven_counts(oracle):
    n = 5
    rng = np.random.default_rng(1)
    sc = rng.integers(0, 4, (n, n)).astype(np.int32)
    rc = sc.T.copy()
    sd = np.concatenate([np.zeros((n, 1), np.int32), np.cumsum(sc, 1)[:, :-1]], 1).astype(np.int32)
    rd = np.concatenate([np.zeros((n, 1), np.int32), np.cumsum(rc, 1)[:, :-1]], 1).astype(np.int32)
    send = np.zeros((n, 16), np.int32)
    for s in range(n):
        for d in range(n):
            send[s, sd[s, d]:sd[s, d] + sc[s, d]] = 100 * s + d
    recv = oracle.alltoallv(send, sc, sd, 16, rc, rd)
    for r in range(n):
        for s in range(n):
            assert (recv[r, rd[r, s]:rd[r, s] + rc[r, s]] == 100 * s + r).all()


def test_alltoallv_truncation_is_an_error(oracle):
    sc = np.array([[1, 2], [1, 1]], np.int32)
    rc = np.array([[1, 1], [1, 1]], np.int32)  # rank 1 posts 1, rank 0 sends 2
    z = np.array([[0, 1], [0, 1]], np.int32)
    with pytest.raises(ValueError):
        oracle.alltoallv(np.zeros((2, 4), np.int32), sc, z, 4, rc, z)


def test_lcg_is_knuth_mmix(oracle):
    s = oracle.lcg_sequence(0, 2)
    a, c = 6364136223846793005, 1442695040888963407
    assert int(s[0]) == c and int(s[1]) == (a * c + c) % 2**64


def test_pi_hits_reasonable_and_deterministic(oracle):
    h = oracle.pi_hits(12345, 3, 100000)
    assert h == oracle.pi_hits(12345, 3, 100000)
    assert abs(4.0 * h / 100000 - np.pi) < 0.02


def test_vector_type_pack_unpack_roundtrip(oracle):
    d = oracle.type_basic(13)
    col = oracle.type_vector(6, 1, 6, d)
    assert col.size == 48 and col.extent == (5 * 6 + 1) * 8
    m = np.arange(36, dtype=np.float64)
    packed = oracle.pack(col, 1, m).view(np.float64)
    assert packed.tolist() == [float(6 * i) for i in range(6)]
    back = np.zeros(36)
    oracle.unpack(col, 1, packed.view(np.uint8), back)
    assert back[::6].tolist() == packed.tolist()


def test_subarray_face_matches_numpy(oracle):
    d = oracle.type_basic(13)
    face = oracle.type_subarray([6, 6, 6], [4, 4, 1], [1, 1, 4], d)
    g = np.arange(216, dtype=np.float64).reshape(6, 6, 6)
    packed = oracle.pack(face, 1, g).view(np.float64)
    assert packed.tolist() == g[1:5, 1:5, 4].ravel().tolist()


def test_bucket_sort_oracle_sorted_and_complete(oracle):
    n, kpr = 8, 4096
    keys = np.concatenate([oracle.bucket_keys(99, r, kpr) for r in range(n)])
    assert keys.min() >= 0 and keys.max() < (1 << 21)
    out, cnt = oracle.bucket_sort(keys, n, 4 * kpr)
    allk = np.concatenate([out[r, :cnt[r]] for r in range(n)])
    assert np.array_equal(allk, np.sort(keys))


def test_halo_expected_faces(oracle):
    P, L = 2, 4
    b = oracle.halo_expected(P, L, 0)
    G = P * L
    # x = 0 face of rank 0 holds the periodic neighbour's column gx = G-1
    assert b[1, 1, 0] == oracle.lib().orc_halo_value(0, 0, G - 1)
    assert b[0, 0, 0] == -1.0


def test_mlp_gradient_matches_finite_differences(oracle):
    rng = np.random.default_rng(3)
    p = rng.standard_normal(oracle.MLP_NPARAMS) * 0.1
    x = rng.standard_normal((5, 12))
    t = rng.standard_normal((5, 4))
    m = (rng.random((5, 4)) > 0.3).astype(np.float64)
    loss, g = oracle.mlp_loss_grad(p, x, t, m)
    for k in rng.choice(oracle.MLP_NPARAMS, 40, replace=False):
        e = np.zeros_like(p)
        e[k] = 1e-6
        lp, _ = oracle.mlp_loss_grad(p + e, x, t, m)
        lm, _ = oracle.mlp_loss_grad(p - e, x, t, m)
        assert abs((lp - lm) / 2e-6 - g[k]) < 1e-5 * max(1.0, abs(g[k]))


def test_dims_create_matches_the_standards_examples(oracle):
    # the MPI standard's MPI_Dims_create examples (MPI-3.1 section 7.5.2): (6, 2) -> 3x2, (7, 2) -> 7x1,
    # (6, {0,3,0}) -> 2x3x1, (7, {0,3,0}) -> erroneous
    assert oracle.dims_create(6, [0, 0]) == [3, 2]
    assert oracle.dims_create(7, [0, 0]) == [7, 1]
    assert oracle.dims_create(6, [0, 3, 0]) == [2, 3, 1]
    assert oracle.dims_create(7, [0, 3, 0]) is None
    # properties: product, non-increasing free entries, fixed entries kept
    for n in range(1, 200):
        for nd in (1, 2, 3, 4):
            d = oracle.dims_create(n, [0] * nd)
            assert int(np.prod(d)) == n and d == sorted(d, reverse=True)


def test_cart_rules(oracle):
    dims, periods = [3, 4, 2], [1, 0, 1]
    for r in range(24):
        c = oracle.cart_coords(dims, r)
        assert oracle.cart_rank(dims, periods, c) == r
    assert oracle.cart_rank(dims, periods, [-1, 0, 0]) == oracle.cart_rank(dims, periods, [2, 0, 0])
    assert oracle.cart_rank(dims, periods, [0, 4, 0]) is None
    assert oracle.cart_shift(dims, periods, 0, 1, 1) == (oracle.PROC_NULL, 2)   # non-periodic edge
    assert oracle.cart_shift(dims, periods, 0, 0, 1) == (16, 8)                 # periodic wrap
