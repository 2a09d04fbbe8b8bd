"""Autotuner and learned algorithm selector for the reduction variants (DIRECT, TREE, RING, STAGED).

No counterpart in the reference (one algorithm per collective there).  Pieces:
  * `features()` — the 12 call features; the same formula runs inside the kernel (mpi_api.cu,
    learned_variant) when a world's policy is "learned";
  * `MLP` — the 12 -> 64 -> 64 -> 4 network, trained on the GPU by the library's own forward/backward
    kernels (gpumpi_mlp_loss_grad / gpumpi_mlp_adam_step); torch only holds the device buffers;
  * `autotune()` — sweeps ranks x bytes-per-rank x datatype x variant; the per-call timings come from the
    runtime's own trace (each collective's rank 0 records its duration); produces the tuned table
    (best variant per (kind, log2 bytes, log2 ranks) cell) and the training set;
  * `evaluate()` — a held-out stream of seeded calls: time of the learned choice, the tuned table's choice
    and the plain DIRECT choice against the exhaustive best (every variant measured).

Command line (on a GPU machine):
  python dphpc-gpu_mpi_gb300/gpumpi/selector.py run --out <dir>
writes tuned_table.npy, mlp_params.npy, selector_report.json into <dir>.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import sys
import time
from pathlib import Path

import numpy as np

if __package__ in (None, ""):
    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
import gpumpi  # noqa: E402

NVAR = 4
KIND_ALLREDUCE, KIND_REDUCE, KIND_ALLTOALLV = 2, 3, 5   # JOB_* codes of the runtime
DT_SLOT = {gpumpi.FLOAT: 2, gpumpi.DOUBLE: 3, gpumpi.INT: 4, gpumpi.INT64_T: 5}
OP_SLOT = {gpumpi.OP_SUM: 6, gpumpi.OP_MAX: 7, gpumpi.OP_MIN: 8, gpumpi.OP_PROD: 9}
DT_SIZE = {gpumpi.FLOAT: 4, gpumpi.DOUBLE: 8, gpumpi.INT: 4, gpumpi.INT64_T: 8}
NP_DT = {gpumpi.FLOAT: np.float32, gpumpi.DOUBLE: np.float64, gpumpi.INT: np.int32, gpumpi.INT64_T: np.int64}


def features(kind: int, bytes_per_rank: float, n: int, dt: int, op: int, rank_share: float) -> np.ndarray:
    """The 12 features (must match learned_variant in csrc/api/mpi_api.cu)."""
    f = np.zeros(12, np.float32)
    f[0] = (math.log2(max(bytes_per_rank, 1.0)) - 16.0) / 8.0
    f[1] = (math.log2(n) - 8.0) / 3.0
    f[DT_SLOT.get(dt, 5)] = 1.0
    if op >= 0:                              # Alltoall(v) has no operator: op = -1, slots stay 0
        f[OP_SLOT.get(op, 9)] = 1.0
    f[10] = rank_share
    f[11] = 1.0 if kind == KIND_REDUCE else -1.0 if kind == KIND_ALLTOALLV else 0.0
    return f


class MLP:
    """The selector network; parameters live on the GPU as float32."""

    def __init__(self, seed: int = 0, params: np.ndarray | None = None):
        import torch
        self.torch = torch
        if params is None:
            rng = np.random.default_rng(seed)
            p = np.zeros(gpumpi.MLP_NPARAMS, np.float32)
            o = 0
            for fan_in, rows in ((12, 64), (64, 64), (64, 4)):
                p[o:o + rows * fan_in] = rng.standard_normal(rows * fan_in) * math.sqrt(2.0 / fan_in)
                o += rows * fan_in + rows  # weights then biases (biases stay 0)
            params = p
        self.p = torch.from_numpy(np.ascontiguousarray(params, np.float32)).cuda()

    def params(self) -> np.ndarray:
        self.torch.cuda.synchronize()
        return self.p.cpu().numpy()

    def loss_grad(self, x, t, m):
        torch = self.torch
        g = torch.empty_like(self.p)
        loss = torch.zeros(1, device="cuda")
        rc = gpumpi.lib().gpumpi_mlp_loss_grad(self.p.data_ptr(), x.data_ptr(), t.data_ptr(), m.data_ptr(),
                                               x.shape[0], g.data_ptr(), loss.data_ptr(), None)
        if rc:
            raise gpumpi.GpumpiError(rc, "mlp_loss_grad")
        return loss, g

    def forward(self, x):
        y = self.torch.empty((x.shape[0], 4), device="cuda")
        rc = gpumpi.lib().gpumpi_mlp_forward(self.p.data_ptr(), x.data_ptr(), x.shape[0], y.data_ptr(), None)
        if rc:
            raise gpumpi.GpumpiError(rc, "mlp_forward")
        return y

    def train(self, X: np.ndarray, T: np.ndarray, M: np.ndarray, epochs: int = 60, batch: int = 512,
              lr: float = 3e-3, wd: float = 1e-5, seed: int = 0) -> list[float]:
        torch = self.torch
        x = torch.from_numpy(np.ascontiguousarray(X, np.float32)).cuda()
        t = torch.from_numpy(np.ascontiguousarray(T, np.float32)).cuda()
        m = torch.from_numpy(np.ascontiguousarray(M, np.float32)).cuda()
        mom = torch.zeros_like(self.p)
        var = torch.zeros_like(self.p)
        g = torch.Generator(device="cpu").manual_seed(seed)
        n = x.shape[0]
        step, hist = 0, []
        for ep in range(epochs):
            perm = torch.randperm(n, generator=g).cuda()
            tot = 0.0
            for b0 in range(0, n, batch):
                idx = perm[b0:b0 + batch]
                xb, tb, mb = x[idx].contiguous(), t[idx].contiguous(), m[idx].contiguous()
                loss, grad = self.loss_grad(xb, tb, mb)
                step += 1
                rc = gpumpi.lib().gpumpi_mlp_adam_step(self.p.data_ptr(), grad.data_ptr(), mom.data_ptr(),
                                                       var.data_ptr(), step, lr, wd, None)
                if rc:
                    raise gpumpi.GpumpiError(rc, "mlp_adam_step")
                tot += float(loss.item()) * xb.shape[0]
            hist.append(tot / n)
        return hist

    def predict(self, X: np.ndarray) -> np.ndarray:
        x = self.torch.from_numpy(np.ascontiguousarray(X, np.float32)).cuda()
        y = self.forward(x)
        self.torch.cuda.synchronize()
        return y.cpu().numpy()


# ---------------------------------------------------------------------------------------------------
# measurement
# ---------------------------------------------------------------------------------------------------
RANKS = [16, 32, 64, 128, 256, 512, 1024, 2048]
LOG2_BYTES = list(range(6, 26))          # 64 B .. 32 MiB per rank
DTYPES = [gpumpi.FLOAT, gpumpi.INT, gpumpi.DOUBLE]
BUDGET = 6 << 30                          # device bytes for send + recv buffers


def _buffers(torch, n, max_bytes):
    send = torch.empty(n * max_bytes // 4, dtype=torch.int32, device="cuda")
    g = torch.Generator(device="cuda").manual_seed(n)
    send.copy_(torch.randint(-100000, 100000, send.shape, generator=g, device="cuda", dtype=torch.int32))
    recv = torch.empty_like(send)
    return send, recv


def _measure(w, torch, send, recv, n, nbytes, dt, variant, iters):
    """Per-call times (us) of `iters` calls, from the runtime's trace; plus device time per call."""
    count = max(1, nbytes // DT_SIZE[dt])
    stride = count * DT_SIZE[dt]
    w.set_policy(variant, 0)
    rc = w.coll("allreduce", send, recv, count, dt, gpumpi.OP_SUM, iters=iters, send_stride=stride,
                recv_stride=stride)
    if rc:
        raise gpumpi.GpumpiError(rc, w.last_error())
    tr = w.read_trace()
    return [float(r["us"]) for r in tr], w.last_kernel_ms() * 1e3 / iters


def autotune(iters: int = 30, log=print):
    """Sweep; returns (records, table, median grid, rank share per n).
    records: list of (n, bytes, dt, variant, us)."""
    import torch
    records = []
    grid = {}
    shares = {}
    for n in RANKS:
        max_bytes = max(b for b in (1 << lb for lb in LOG2_BYTES) if 2 * n * b <= BUDGET)
        w = gpumpi.World(n, timeout_s=60.0, trace_capacity=4096)
        send, recv = _buffers(torch, n, max_bytes)
        t0 = time.time()
        for lb in LOG2_BYTES:
            nbytes = 1 << lb
            if 2 * n * nbytes > BUDGET:
                continue
            for dt in DTYPES:
                for v in range(NVAR):
                    us, _ = _measure(w, torch, send, recv, n, nbytes, dt, v, iters)
                    us = us[2:] if len(us) > 4 else us       # drop the first calls (cold)
                    records += [(n, nbytes, dt, v, u) for u in us]
                    grid[(n, lb, dt, v)] = float(np.median(us))
        info = w.info()
        shares[n] = n / (n + info["engine_blocks"])
        log(f"autotune: {n} ranks done in {time.time() - t0:.1f}s ({len(records)} records); world {info}")
        w.close()
        del send, recv
        torch.cuda.empty_cache()
    table = np.full((2, 32, 16), -1, np.int8)
    for n in RANKS:
        for lb in LOG2_BYTES:
            best, bt = None, None
            for v in range(NVAR):
                # score over datatypes: sum of medians
                ts = [grid.get((n, lb, dt, v)) for dt in DTYPES]
                if any(t is None for t in ts):
                    continue
                s = sum(ts)
                if bt is None or s < bt:
                    best, bt = v, s
            if best is not None:
                table[0, lb, int(math.log2(n))] = best
                table[1, lb, int(math.log2(n))] = best
    return records, table, grid, shares


def dataset(records, rank_share_of):
    X = np.stack([features(KIND_ALLREDUCE, b, n, dt, gpumpi.OP_SUM, rank_share_of[n]) for n, b, dt, v, u in records])
    T = np.zeros((len(records), NVAR), np.float32)
    M = np.zeros((len(records), NVAR), np.float32)
    for i, (n, b, dt, v, u) in enumerate(records):
        T[i, v] = math.log(max(u, 1e-3))
        M[i, v] = 1.0
    return X, T, M


def evaluate(mlp_params, table, calls: int = 10000, shapes_per_rank: int = 12, seed: int = 2026, iters: int = 12,
             log=print):
    """Held-out stream: `calls` seeded Allreduce calls (sizes log-uniform 64 B .. 32 MiB, ranks 16 .. 2048,
    fp32/int32/fp64) drawn from off-grid shapes; every variant of every shape is measured."""
    import torch
    rng = np.random.default_rng(seed)
    shapes = []
    for n in RANKS:
        for _ in range(shapes_per_rank):
            while True:
                b = int(2 ** rng.uniform(6, 25))
                b -= b % 8
                if b >= 64 and 2 * n * b <= BUDGET and (b & (b - 1)) != 0:
                    break
            shapes.append((n, b, int(rng.choice(DTYPES))))
    meas = {}
    pick = {}
    shares = {}
    mlp = MLP(params=mlp_params)
    for n in RANKS:
        sub = [s for s in shapes if s[0] == n]
        max_bytes = max(b for _, b, _ in sub)
        w = gpumpi.World(n, timeout_s=60.0, trace_capacity=4096)
        send, recv = _buffers(torch, n, max_bytes)
        for (_, b, dt) in sub:
            times = []
            for v in range(NVAR):
                us, _ = _measure(w, torch, send, recv, n, b, dt, v, iters)
                us = us[2:] if len(us) > 4 else us
                times.append(float(np.median(us)))
            meas[(n, b, dt)] = times
        shares[n] = n / (n + w.info()["engine_blocks"])
        w.close()
        del send, recv
        torch.cuda.empty_cache()
    keys = list(meas)
    # the learned choice uses the same features the kernel computes (rank share = ranks / launch blocks)
    X = np.stack([features(KIND_ALLREDUCE, b, n, dt, gpumpi.OP_SUM, shares[n]) for (n, b, dt) in keys])
    pred = mlp.predict(X)
    for i, k in enumerate(keys):
        n, b, dt = k
        pick[k] = {"learned": int(np.argmin(pred[i])),
                   "tuned": int(table[0, min(31, int(math.log2(b))), int(math.log2(n))]),
                   "plain": 0}
        if pick[k]["tuned"] < 0:
            pick[k]["tuned"] = 0
    # stream of calls
    idx = rng.integers(0, len(keys), calls)
    tot = {"best": 0.0, "learned": 0.0, "tuned": 0.0, "plain": 0.0}
    regrets = {"learned": [], "tuned": [], "plain": []}
    for i in idx:
        k = keys[i]
        t = meas[k]
        best = min(t)
        tot["best"] += best
        for pol in ("learned", "tuned", "plain"):
            tp = t[pick[k][pol]]
            tot[pol] += tp
            regrets[pol].append(tp / best - 1.0)
    rep = {"calls": calls, "shapes": len(keys),
           "total_time_ms": {k: v / 1e3 for k, v in tot.items()},
           "time_over_best": {p: tot[p] / tot["best"] - 1.0 for p in ("learned", "tuned", "plain")},
           "mean_regret": {p: float(np.mean(regrets[p])) for p in regrets},
           "p90_regret": {p: float(np.percentile(regrets[p], 90)) for p in regrets},
           "learned_vs_tuned_time": tot["learned"] / tot["tuned"],
           "choices": {f"{k[0]}x{k[1]}:{k[2]}": pick[k] for k in keys}}
    log(json.dumps({k: v for k, v in rep.items() if k != "choices"}))
    return rep


def run(out: Path, iters: int = 30):
    import torch
    out.mkdir(parents=True, exist_ok=True)
    gpumpi.build()
    t0 = time.time()
    records, table, grid, shares = autotune(iters=iters)
    X, T, M = dataset(records, shares)
    print(f"dataset: {len(records)} timings, sweep {time.time() - t0:.1f}s", flush=True)
    # hold out 20% of the sweep records for a validation loss
    rng = np.random.default_rng(0)
    perm = rng.permutation(len(X))
    cut = int(0.8 * len(X))
    tr, va = perm[:cut], perm[cut:]
    mlp = MLP(seed=0)
    hist = mlp.train(X[tr], T[tr], M[tr], epochs=40)
    import torch as _t
    xv = _t.from_numpy(X[va]).cuda(); tv = _t.from_numpy(T[va]).cuda(); mv = _t.from_numpy(M[va]).cuda()
    vloss, _ = mlp.loss_grad(xv, tv, mv)
    params = mlp.params()
    np.save(out / "tuned_table.npy", table)
    np.save(out / "mlp_params.npy", params)
    rep = evaluate(params, table)
    rep.update({"train_records": int(len(tr)), "val_records": int(len(va)), "train_loss": hist,
                "val_loss": float(vloss.item()), "sweep_seconds": time.time() - t0,
                "grid_median_us": {f"{n}:{lb}:{dt}:{v}": t for (n, lb, dt, v), t in grid.items()}})
    (out / "selector_report.json").write_text(json.dumps(rep, indent=1))
    print(json.dumps({k: rep[k] for k in ("time_over_best", "mean_regret", "learned_vs_tuned_time", "val_loss")}))


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("cmd", choices=["run"])
    ap.add_argument("--out", default="gpurun_out/selector")
    ap.add_argument("--iters", type=int, default=30)
    a = ap.parse_args()
    run(Path(a.out), iters=a.iters)
