"""GPU: Cartesian topologies (MPI_Dims_create, MPI_Cart_create/coords/rank/shift/get/sub, MPI_Topo_test)
against the oracle's restatement of the MPI standard's rules; a neighbour exchange along every dimension
checks that the grid's ranks are the ones messages reach."""
import pytest

pytestmark = pytest.mark.gpu

DIMS_CASES = [(12, 2, 0), (30, 3, 0), (16, 4, 0), (7, 2, 0), (24, 3, 3), (360, 3, 0)]


@pytest.mark.parametrize("n", [8, 24, 30, 64])
def test_cart_program(gpulib, oracle, n):
    with gpulib.World(n, timeout_s=10.0) as w:
        rc, ok, oi, _ = w.run_test("cart")
    assert rc == 0 and ok.all(), (ok, oi[:, :22])
    dims = oracle.dims_create(n, [0, 0, 0])
    periods = [1, 0, 1]
    for r in range(n):
        o = oi[r]
        c = oracle.cart_coords(dims, r)
        assert o[0:3].tolist() == dims and o[3:6].tolist() == c and o[6] == r
        for d in range(3):
            src, dst = oracle.cart_shift(dims, periods, r, d, 1)
            assert (o[7 + 2 * d], o[8 + 2 * d]) == (src, dst), (r, d)
            assert o[18 + d] == (src if src != oracle.PROC_NULL else -7), (r, d)   # the value sent up
        # Cart_sub keeping dims 0 and 2: size dims0 * dims2, rank row-major over (c0, c2)
        assert o[13] == dims[0] * dims[2] and o[14] == c[0] * dims[2] + c[2]
        assert o[15] == 3 and o[16] == gpulib.MPI_CART and o[17] == -1   # MPI_UNDEFINED for the world
        assert o[21] == gpulib.ERR_RANK   # outside the non-periodic dimension
    for k, (nn, nd, fixed2) in enumerate(DIMS_CASES):
        want = oracle.dims_create(nn, [0, fixed2, 0, 0][:nd])
        got_rc, got = oi[0][24 + 4 * k], oi[0][25 + 4 * k:25 + 4 * k + min(nd, 3)].tolist()
        if want is None:
            assert got_rc != 0
        else:
            assert got_rc == 0 and got == want[:3], (nn, nd, got, want)
