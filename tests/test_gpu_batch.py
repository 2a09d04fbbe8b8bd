"""GPU: a batch of 64 communicators of uneven sizes (8 to 512 ranks, seeded log-uniform) progressed in
one persistent launch, each running its own MPI_Allreduce; checked per communicator against the oracle,
also when the launch is recorded in a CUDA graph and replayed."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def check_batch(oracle, tab, x, got, dt, op):
    for c, (first, size, count, off) in enumerate(tab):
        xc = x[off:off + size * count].reshape(size, count)
        ref = oracle.allreduce(xc, dt, op)
        assert np.array_equal(got[off:off + size * count].reshape(size, count).view(np.uint8), ref.view(np.uint8)), c


def test_batch_of_64_communicators_matches_oracle(gpulib, oracle):
    from gpumpi import apps
    n = 512
    tab = apps.batch_layout(7, n)
    assert (tab[:, 1] >= 8).all() and (tab[:, 1] <= 512).all() and len(np.unique(tab[:, 1])) > 20
    E = apps.batch_elements(tab)
    x = oracle.fill_f32(11, E)
    with gpulib.World(n, timeout_s=60.0) as w:
        send, recv = torch.from_numpy(x).cuda(), torch.zeros(E, dtype=torch.float32, device="cuda")
        rc = apps.batch(w, tab, send, recv, iters=2, dt=gpulib.FLOAT, op=gpulib.OP_SUM)
        assert rc == 0, w.last_error()
        check_batch(oracle, tab, x, recv.cpu().numpy(), gpulib.FLOAT, gpulib.OP_SUM)


def test_batch_graph_replay_and_tuned_policy(gpulib, oracle):
    """Integer batch under a tuned table that picks RING everywhere (exact for integers), recorded once
    as a CUDA graph and replayed twice: one kernel launch per replay, same results each time."""
    from gpumpi import apps
    n = 256
    tab = apps.batch_layout(3, n, ncomms=40, max_size=256)
    E = apps.batch_elements(tab)
    x = (oracle.fill_i32(5, E) % 100000).astype(np.int32)
    with gpulib.World(n, timeout_s=60.0) as w:
        w.set_tuned_table(np.full((3, 32, 16), 2, np.int8))
        w.set_policy(-1, 1)
        send, recv = torch.from_numpy(x).cuda(), torch.zeros(E, dtype=torch.int32, device="cuda")
        with apps.batch(w, tab, send, recv, iters=1, dt=gpulib.INT, op=gpulib.OP_SUM, graph=True) as g:
            for _ in range(2):
                recv.zero_()
                torch.cuda.synchronize()
                l0 = gpulib.kernel_launches()
                rc = g.launch()
                assert rc == 0, w.last_error()
                assert gpulib.kernel_launches() - l0 == 1
                check_batch(oracle, tab, x, recv.cpu().numpy(), gpulib.INT, gpulib.OP_SUM)
