"""Host drivers of the application programs (bucket sort, 3D halo exchange) on device buffers.

The programs themselves run on the GPU (csrc/programs/prog_apps.cu); these helpers size and allocate
their buffers with torch (device memory only) and launch them through the C ABI.
"""
from __future__ import annotations

import numpy as np

from . import P_BUCKET_SORT, P_HALO, TUNE_DYN_SMEM, World

KEY_RANGE = 1 << 21


def _copy_ns(ns_dev, iter_ns):
    """Per-iteration device times (rank 0, ns) into the caller's numpy array, if any."""
    if iter_ns is not None:
        iter_ns[:] = ns_dev.cpu().numpy()[: len(iter_ns)].astype(np.uint64)


def _first_error(rc, rcs):
    if rc == 0 and int(rcs.abs().max().item()) != 0:
        rc = int(rcs[rcs != 0][0].item())
    return rc


def bucket_capacity(keys_per_rank: int) -> int:
    """Receive capacity per rank: keys are the mean of four uniforms, whose density peaks at 8/3 of the
    mean density, so three times the per-rank key count holds any bucket of a run this size."""
    return 3 * keys_per_rank + 64


def bucket_sort(world: World, seed: int, total_keys: int, iters: int = 10, keys=None, iter_ns=None):
    """Runs the distributed bucket sort (keys generated on the device unless `keys` [n, kpr] int32 is
    given).  Returns (rc, keys, sorted [n, cap], counts [n] int64)."""
    import torch
    n = world.nranks
    kpr = total_keys // n
    cap = bucket_capacity(kpr)
    dev = torch.device("cuda", torch.cuda.current_device())
    i32 = torch.int32
    gen = keys is None
    if gen:
        keys = torch.empty((n, kpr), dtype=i32, device=dev)
    send = torch.empty((n, kpr), dtype=i32, device=dev)
    recv = torch.empty((n, cap), dtype=i32, device=dev)
    out = torch.zeros((n, cap), dtype=i32, device=dev)
    counts = torch.zeros(n, dtype=torch.int64, device=dev)
    scratch = torch.zeros((n, 4 * n), dtype=i32, device=dev)
    hstride = (KEY_RANGE + n - 1) // n + 1
    hist = torch.empty((n, hstride), dtype=i32, device=dev)
    rcs = torch.zeros(n, dtype=i32, device=dev)
    ns = torch.zeros(max(1, iters), dtype=torch.int64, device=dev)
    # the local counting sort keeps its histogram (hstride ints) in the block's shared memory when the
    # launch gives it that much: raise the world's cap for this launch
    cap0 = world.get_tuning(TUNE_DYN_SMEM)
    want = 4 * hstride + 1024
    if 0 <= cap0 < want:
        world.set_tuning(TUNE_DYN_SMEM, want)
    try:
        rc = world.run_program(P_BUCKET_SORT, i=(seed, kpr, iters, cap, int(gen), hstride),
                               p=(keys, send, recv, out, counts, scratch, hist, rcs, ns))
    finally:
        world.set_tuning(TUNE_DYN_SMEM, cap0)
    torch.cuda.synchronize()
    _copy_ns(ns, iter_ns)
    return _first_error(rc, rcs), keys, out, counts


def halo(world: World, P: int, L: int, iters: int = 1, mode: int = 0, blocks=None, iter_ns=None):
    """3D halo exchange on a (P*L)^3 fp64 grid over P^3 ranks (mode 0 vector/hvector faces, 1 subarray
    faces).  Returns (rc, blocks [P^3, (L+2)^3])."""
    import torch
    n = world.nranks
    if n != P ** 3:
        raise ValueError("the world must have P^3 ranks")
    W = L + 2
    dev = torch.device("cuda", torch.cuda.current_device())
    if blocks is None:
        blocks = torch.empty((n, W ** 3), dtype=torch.float64, device=dev)
    rcs = torch.zeros(n, dtype=torch.int32, device=dev)
    ns = torch.zeros(max(1, iters), dtype=torch.int64, device=dev)
    rc = world.run_program(P_HALO, i=(P, L, iters, mode), p=(blocks, None, None, None, None, None, ns, rcs))
    torch.cuda.synchronize()
    _copy_ns(ns, iter_ns)
    return _first_error(rc, rcs), blocks


def halo_face_bytes(P: int, L: int) -> int:
    """Payload of one exchange: six faces of L*L doubles per rank."""
    return 6 * L * L * 8 * P ** 3


def batch_layout(seed: int, nranks: int, ncomms: int = 64, min_size: int = 8, max_size: int = 512,
                 min_bytes: int = 4, max_bytes: int = 1 << 16, esize: int = 4) -> np.ndarray:
    """Seeded layout of a batch of communicators: sizes log-uniform in [min_size, max_size] (capped at the
    world), each a contiguous range of world ranks at a random start, per-rank message bytes log-uniform
    in [min_bytes, max_bytes].  Returns int64 [ncomms, 4] = {first rank, size, count, element offset}."""
    rng = np.random.default_rng(seed)
    hi = min(max_size, nranks)
    tab = np.zeros((ncomms, 4), dtype=np.int64)
    off = 0
    for c in range(ncomms):
        size = int(round(np.exp(rng.uniform(np.log(min_size), np.log(hi)))))
        size = max(1, min(size, nranks))
        first = int(rng.integers(0, nranks - size + 1))
        count = max(1, int(np.exp(rng.uniform(np.log(min_bytes), np.log(max_bytes)))) // esize)
        tab[c] = (first, size, count, off)
        off += size * count
    return tab


def batch_elements(tab: np.ndarray) -> int:
    return int((tab[:, 1] * tab[:, 2]).sum())


def batch(world: World, tab: np.ndarray, send, recv, iters: int = 1, dt: int = 12, op: int = 2, iter_ns=None,
          graph: bool = False, setup_ns=None):
    """Runs the batch (every communicator's MPI_Allreduce, `iters` times) in one launch; with graph=True
    returns a recorded Graph instead of running (replay with Graph.launch).  setup_ns (2 int64, host)
    receives rank 0's time in the group calls and in MPI_Comm_create, summed over the communicators."""
    import torch
    from . import P_BATCH
    dev = torch.device("cuda", torch.cuda.current_device())
    tab_d = torch.from_numpy(np.ascontiguousarray(tab, dtype=np.int64)).to(dev)
    rcs = torch.zeros(world.nranks, dtype=torch.int32, device=dev)
    ns = torch.zeros(max(1, iters), dtype=torch.int64, device=dev)
    st = torch.zeros(2, dtype=torch.int64, device=dev)
    args = dict(i=(len(tab), iters, dt, op), p=(send, recv, tab_d, None, None, st, ns, rcs))
    if graph:
        g = world.graph(P_BATCH, **args)
        g._keep = (tab_d, rcs, ns, st)  # device buffers the recorded launch reads and writes
        return g
    rc = world.run_program(P_BATCH, **args)
    torch.cuda.synchronize()
    _copy_ns(ns, iter_ns)
    if setup_ns is not None:
        setup_ns[:2] = st.cpu().numpy()
    return _first_error(rc, rcs)
