"""Autotuner and learned algorithm selector for the collective variants (DIRECT, TREE, RING, STAGED) of
MPI_Allreduce/Reduce (fold orders, TMA staging) and MPI_Alltoall(v) (piece orders, TMA staging).

No counterpart in the reference (one algorithm per collective there).  Pieces:
  * `features()` — the 12 call features; the same formula runs inside the kernel (mpi_api.cu,
    learned_decide) when a world's policy is "learned";
  * `MLP` — the 12 -> 64 -> 64 -> 4 network, trained on the GPU by the library's own forward/backward
    kernels (gpumpi_mlp_loss_grad / gpumpi_mlp_adam_step); torch only holds the device buffers;
  * `autotune()` — sweeps ranks x bytes-per-rank x datatype x variant; the per-call timings come from the
    runtime's own trace (each collective's rank 0 records its duration); produces the tuned table
    (best variant per (kind, datatype class, alignment class, log2 bytes, log2 ranks) cell) and the
    training set;
  * `evaluate()` — a held-out stream of seeded calls: time of the learned choice, the tuned table's choice
    and the plain DIRECT choice against the exhaustive best (every variant measured).

Command line (on a GPU machine):
  python dphpc-gpu_mpi_gb300/gpumpi/selector.py run --out <dir>
writes tuned_table.npy, mlp_params.npy, selector_report.json into <dir>.
"""
from __future__ import annotations

import argparse
import json
import math
import sys
import time
from pathlib import Path

import numpy as np

if __package__ in (None, ""):
    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
import gpumpi  # noqa: E402

NVAR = 4          # network outputs (one per variant)
NSEL = 3          # variants the policies choose among: DIRECT, TREE, RING (STAGED never measured fastest)
KIND_ALLREDUCE, KIND_REDUCE, KIND_ALLTOALLV = 2, 3, 5   # JOB_* codes of the runtime
DT_SLOT = {gpumpi.FLOAT: 2, gpumpi.DOUBLE: 3, gpumpi.INT: 4, gpumpi.INT64_T: 5}
OP_SLOT = {gpumpi.OP_SUM: 6, gpumpi.OP_MAX: 7, gpumpi.OP_MIN: 8, gpumpi.OP_PROD: 9}
DT_SIZE = {gpumpi.FLOAT: 4, gpumpi.DOUBLE: 8, gpumpi.INT: 4, gpumpi.INT64_T: 8}
NP_DT = {gpumpi.FLOAT: np.float32, gpumpi.DOUBLE: np.float64, gpumpi.INT: np.int32, gpumpi.INT64_T: np.int64}


def features(kind: int, bytes_per_rank: float, n: int, dt: int, op: int, rank_share: float,
             aligned: int = 16) -> np.ndarray:
    """The 12 features (must match learned_decide in csrc/api/mpi_api.cu): log2 bytes per rank, log2
    ranks, datatype one-hot, SUM flag (Alltoall(v) has no operator: op = -1), 16-byte and 8-byte alignment
    flags of the members' buffers, rank share of the launch's blocks, kind."""
    f = np.zeros(12, np.float32)
    f[0] = (math.log2(max(bytes_per_rank, 1.0)) - 16.0) / 8.0
    f[1] = (math.log2(n) - 8.0) / 3.0
    f[DT_SLOT.get(dt, 5)] = 1.0
    f[6] = 1.0 if op == gpumpi.OP_SUM else 0.0
    f[7] = 1.0 if aligned >= 16 else 0.0
    f[8] = 1.0 if aligned >= 8 else 0.0
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
KINDS = (KIND_ALLREDUCE, KIND_ALLTOALLV)
MARGIN = 0.05   # default predicted log-time gain the network needs to override the tuned table (5%)
KIND_NAME = {KIND_ALLREDUCE: "allreduce", KIND_REDUCE: "allreduce", KIND_ALLTOALLV: "alltoallv"}
TABLE_ROW = {KIND_ALLREDUCE: 0, KIND_REDUCE: 1, KIND_ALLTOALLV: 2}
DATA = Path(__file__).resolve().parent / "data"


def _buffers(torch, n, max_bytes):
    send = torch.empty(2 * n * max_bytes // 4 + 2 * n * n, dtype=torch.int32, device="cuda")
    g = torch.Generator(device="cuda").manual_seed(n)
    send.copy_(torch.randint(-100000, 100000, send.shape, generator=g, device="cuda", dtype=torch.int32))
    recv = torch.empty_like(send)
    return send, recv


class Exchange:
    """Seeded uneven Alltoallv layout: every pair's count uniform in [0, 2m] int32, m = bytes / (4 n)."""

    def __init__(self, torch, n, nbytes, seed):
        rng = np.random.default_rng(seed)
        m = nbytes / (4.0 * n)
        sc = rng.integers(0, int(2 * m) + 1, (n, n)).astype(np.int32)
        rc = sc.T.copy()
        self.S, self.R = max(1, int(sc.sum(1).max())), max(1, int(rc.sum(1).max()))
        sd, rd = (np.cumsum(sc, 1) - sc).astype(np.int32), (np.cumsum(rc, 1) - rc).astype(np.int32)
        self.dev = [torch.from_numpy(a).cuda() for a in (sc, sd, rc, rd)]


def _measure(w, torch, send, recv, n, nbytes, dt, kind, variant, iters, ex=None):
    """Per-call records (log2 bytes seen by the kernel, us, buffer alignment) of `iters` calls, from the
    runtime's trace."""
    w.set_policy(variant, 0)
    if kind == KIND_ALLTOALLV:
        sc, sd, rc, rd = ex.dev
        w.alltoallv(send, ex.S * 4, sc, sd, recv, ex.R * 4, rc, rd, gpumpi.INT, iters=iters)
    else:
        count = max(1, nbytes // DT_SIZE[dt])
        stride = count * DT_SIZE[dt]
        code = w.coll("allreduce", send, recv, count, dt, gpumpi.OP_SUM, iters=iters, send_stride=stride,
                      recv_stride=stride)
        if code:
            raise gpumpi.GpumpiError(code, w.last_error())
    tr = w.read_trace()
    return [(float(r["log2_bytes"]), float(r["us"]), int(r["aligned"])) for r in tr]


def _shapes_for(kind):
    return DTYPES if kind == KIND_ALLREDUCE else [gpumpi.INT]


def _sizes_for(lb):
    """The power of two 2^lb and two off-grid sizes in the same octave, 8 and 4 mod 16 bytes, so rank buffers
    laid end to end lose 16-byte (and 8-byte) alignment: vector width and variant ranking change with it."""
    b = 1 << lb
    out = [b]
    for f, rem in ((1.41, 8), (1.19, 4)):
        off = int(round(b * f / 16)) * 16 + rem
        if b < off < 2 * b:
            out.append(off)
    return out


def autotune(iters: int = 30, log=print):
    """Sweep of Allreduce (SUM; fp32, int32, fp64) and uneven int32 Alltoallv over ranks x bytes per rank
    x variant.  Returns (records, table, median grid, rank share per n); a record is
    (kind, n, log2 bytes seen by the kernel, dt, variant, us, buffer alignment, bytes per rank asked)."""
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
            for nbytes in _sizes_for(lb):
                if 2 * n * nbytes > BUDGET:
                    continue
                for kind in KINDS:
                    ex = Exchange(torch, n, nbytes, seed=n * 100 + nbytes) if kind == KIND_ALLTOALLV else None
                    for dt in _shapes_for(kind):
                        for v in range(NSEL):
                            recs = _measure(w, torch, send, recv, n, nbytes, dt, kind, v, iters, ex)
                            recs = recs[2:] if len(recs) > 4 else recs    # drop the first calls (cold)
                            records += [(kind, n, l2b, dt, v, u, al, nbytes) for l2b, u, al in recs]
                            # table cell: log2 bytes as the kernel sees them, alignment class
                            cell = int(math.floor(recs[0][0])) if recs and recs[0][0] > 0 else 0
                            cls = 0 if recs and recs[0][2] >= 16 else 1
                            grid[(kind, n, nbytes, dt, v)] = (cell, cls, float(np.median([u for _, u, _ in recs])),
                                                              recs[0][0] if recs else 0.0)
        info = w.info()
        shares[n] = n / (n + info["engine_blocks"])
        log(f"autotune: {n} ranks done in {time.time() - t0:.1f}s ({len(records)} records); world {info}")
        w.close()
        del send, recv
        torch.cuda.empty_cache()
    return records, build_table(grid), grid, shares


NDCLASS = 3   # datatype classes of the tuned table: 0 float, 1 double / long double, 2 every other type


def dclass(dt: int) -> int:
    """Datatype class of the tuned table (sel_dclass in rt_select.cuh)."""
    return 0 if dt == gpumpi.FLOAT else 1 if dt in (gpumpi.DOUBLE, gpumpi.LONG_DOUBLE) else 2


def table_choice(table, kind: int, dt: int, aligned: int, log2_bytes: float, col: int) -> int:
    """The tuned table's variant for a call, indexed as the kernel does (tuned_cell in rt_select.cuh):
    datatype class, alignment class, floor of log2 bytes per rank, rank column `col`; -1 when unset."""
    cell = min(31, max(0, int(math.floor(log2_bytes))))
    return int(table[TABLE_ROW[kind], dclass(dt), 0 if aligned >= 16 else 1, cell, col])


def build_table(grid):
    """The tuned table: per (kind, datatype class, alignment class, cell of log2 bytes, log2 ranks) the
    variant with the least summed median time over the shapes of `grid` in the cell; alignment class 0 =
    16-byte aligned buffers (the power-of-two sizes), 1 = not (the off-grid sizes, 8 or 4 mod 16 bytes).
    A cell the sweep did not reach in one alignment class takes the same datatype class's other alignment
    class; a datatype class the sweep did not time at all (Alltoall(v) is timed with int32 only) takes the
    choice over every datatype."""
    per, pooled = {}, {}
    for (kind, n, nbytes, dt, v), (cell, cls, t, _) in grid.items():
        per.setdefault((kind, dclass(dt), n, cell, cls), np.zeros(NSEL))[v] += t
        pooled.setdefault((kind, n, cell, cls), np.zeros(NSEL))[v] += t

    def fill(tab, sums, dcls_of):
        for key, tv in sums.items():
            kind, n, cell, cls = key[0], key[-3], key[-2], key[-1]
            rows = (TABLE_ROW[kind],) + ((TABLE_ROW[KIND_REDUCE],) if kind == KIND_ALLREDUCE else ())
            for row in rows:
                for d in dcls_of(key):
                    tab[row, d, cls, min(31, cell), int(math.log2(n))] = int(np.argmin(tv))
        for cls in (0, 1):
            mine, other = tab[:, :, cls], tab[:, :, 1 - cls]
            mine[mine < 0] = other[mine < 0]
        return tab

    table = fill(np.full((3, NDCLASS, 2, 32, 16), -1, np.int8), per, lambda key: (key[1],))
    every = fill(np.full((3, NDCLASS, 2, 32, 16), -1, np.int8), pooled, lambda key: range(NDCLASS))
    table[table < 0] = every[table < 0]
    return table


MARGIN_CANDIDATES = (0.0, 0.02, 0.05, 0.1, 0.2, 0.3, 0.5, 1.0, 2.0)


def margin_totals(mlp, table, grid, shares, candidates=MARGIN_CANDIDATES, rank_col=None):
    """Per kind and candidate margin, the total median time over the complete shapes of `grid` of the learned
    policy: "the table's choice unless the network predicts at least the margin lower log-time".  The table
    column of a rank count is rank_col(n) (default: its log2, as the kernel indexes it)."""
    rank_col = rank_col or (lambda n: int(math.log2(n)))
    shapes = {}
    for (kind, n, nbytes, dt, v), (cell, cls, t, l2b) in grid.items():
        sh = shapes.setdefault((kind, n, nbytes, dt), {"t": [np.inf] * NSEL, "cell": cell, "cls": cls, "l2b": l2b})
        sh["t"][v] = t
    keys = [k for k in shapes if all(np.isfinite(shapes[k]["t"]))]
    tot = {"allreduce": {}, "alltoallv": {}}
    if not keys:
        return tot
    X = np.stack([features(k, 2.0 ** shapes[(k, n, b, dt)]["l2b"], n, dt,
                           gpumpi.OP_SUM if k == KIND_ALLREDUCE else -1, shares[n],
                           16 if shapes[(k, n, b, dt)]["cls"] == 0 else 8) for (k, n, b, dt) in keys])
    pred = mlp.predict(X)
    for m in candidates:
        for i, key in enumerate(keys):
            sh = shapes[key]
            tv = table_choice(table, key[0], key[3], 16 if sh["cls"] == 0 else 8, sh["cell"], rank_col(key[1]))
            kn = KIND_NAME[key[0]]
            tot[kn][m] = tot[kn].get(m, 0.0) + sh["t"][policy_pick(pred[i], tv, m)]
    return tot


def pick_margins(totals):
    """Per kind, the candidate with the least total (ties go to the larger margin); the default without data."""
    out = {}
    for kname in ("allreduce", "alltoallv"):
        t = totals.get(kname, {})
        out[kname] = min(t, key=lambda m: (t[m], -m)) if t else MARGIN
    return out


def choose_margin(mlp, table, grid, shares, candidates=MARGIN_CANDIDATES):
    """The override margins of the learned policy, one for Allreduce and one for Alltoall(v): per kind, the
    margin with the least total time over the shapes of `grid` (margin_totals; ties go to the larger
    margin)."""
    return pick_margins(margin_totals(mlp, table, grid, shares, candidates))


def policy_pick(pred_row, tv: int, margin: float) -> int:
    """The learned policy's choice, as the kernel makes it (select_variant in rt_select.cuh): the network's
    best selectable variant, unless the tuned table's choice is predicted within `margin`."""
    pure = int(np.argmin(pred_row[:NSEL]))
    return tv if (tv >= 0 and pred_row[tv] <= pred_row[pure] + margin) else pure


def dataset(records, rank_share_of):
    """Features and targets of the timing records.  The target of a record is its log-time relative to its
    shape: minus the mean over the shape's variants of their median log-times.  Only the differences
    between variants decide the choice, and without the shape's own scale (microseconds to milliseconds)
    the network spends its capacity on them."""
    X = np.stack([features(k, 2.0 ** l2b, n, dt, gpumpi.OP_SUM if k == KIND_ALLREDUCE else -1, rank_share_of[n], al)
                  for k, n, l2b, dt, v, u, al, _ in records])
    per = {}
    for k, n, l2b, dt, v, u, al, _ in records:
        per.setdefault((k, n, round(l2b, 4), dt, al), {}).setdefault(v, []).append(math.log(max(u, 1e-3)))
    base = {key: float(np.mean([np.median(x) for x in d.values()])) for key, d in per.items()}
    T = np.zeros((len(records), NVAR), np.float32)
    M = np.zeros((len(records), NVAR), np.float32)
    for i, (k, n, l2b, dt, v, u, al, _) in enumerate(records):
        T[i, v] = math.log(max(u, 1e-3)) - base[(k, n, round(l2b, 4), dt, al)]
        M[i, v] = 1.0
    return X, T, M


def heldout_ranks(seed: int = 2026, count: int = 24) -> list:
    """Rank counts of the held-out stream, drawn independently of the sweep's powers of two: log-uniform
    integers in [16, 2048], every one off the grid (a power of two is redrawn)."""
    rng = np.random.default_rng(seed + 1)
    out = set()
    while len(out) < count:
        n = int(round(2 ** rng.uniform(4, 11)))
        if 16 <= n <= 2048 and (n & (n - 1)) != 0:
            out.add(n)
    return sorted(out)


def evaluate(mlp_params, table, calls: int = 10000, shapes_per_rank: int = 16, seed: int = 2026, iters: int = 12,
             log=print, margins: dict = None):
    """Held-out stream: `calls` seeded calls, half Allreduce (fp32/int32/fp64 SUM) and half uneven int32
    Alltoallv, over shapes drawn independently of the sweep: rank counts off the power-of-two grid
    (heldout_ranks), sizes log-uniform 64 B .. 32 MiB per rank and not powers of two.  Every selectable
    variant of every shape is measured, so the exhaustive best is known."""
    import torch
    margins = margins or {"allreduce": MARGIN, "alltoallv": MARGIN}
    rng = np.random.default_rng(seed)
    shapes = []
    for n in heldout_ranks(seed):
        for j in range(shapes_per_rank):
            kind = KINDS[j % 2]
            dt = int(rng.choice(DTYPES)) if kind == KIND_ALLREDUCE else gpumpi.INT
            while True:
                b = int(2 ** rng.uniform(6, 25))
                b -= b % DT_SIZE[dt]
                if b >= 64 and 2 * n * b <= BUDGET and (b & (b - 1)) != 0:
                    break
            shapes.append((kind, n, b, dt))
    meas, seen, shares = {}, {}, {}
    mlp = MLP(params=mlp_params)
    for n in sorted({s_[1] for s_ in shapes}):
        sub = [s_ for s_ in shapes if s_[1] == n]
        max_bytes = max(b for _, _, b, _ in sub)
        w = gpumpi.World(n, timeout_s=60.0, trace_capacity=4096)
        send, recv = _buffers(torch, n, max_bytes)
        for k, (kind, _, b, dt) in enumerate(sub):
            ex = Exchange(torch, n, b, seed=seed + 7 * k + n) if kind == KIND_ALLTOALLV else None
            times = []
            for v in range(NSEL):
                recs = _measure(w, torch, send, recv, n, b, dt, kind, v, iters, ex)
                recs = recs[2:] if len(recs) > 4 else recs
                times.append(float(np.median([u for _, u, _ in recs])))
                seen[(kind, n, b, dt)] = (recs[0][0], recs[0][2])   # log2 bytes and alignment the kernel saw
            meas[(kind, n, b, dt)] = times
        shares[n] = n / (n + w.info()["engine_blocks"])
        w.close()
        del send, recv
        torch.cuda.empty_cache()
    keys = list(meas)
    # the learned and tuned choices use what the kernel computes per call (bytes estimate, rank share,
    # alignment of the members' buffers)
    X = np.stack([features(k, 2.0 ** seen[(k, n, b, dt)][0], n, dt, gpumpi.OP_SUM if k == KIND_ALLREDUCE else -1,
                           shares[n], seen[(k, n, b, dt)][1]) for (k, n, b, dt) in keys])
    pred = mlp.predict(X)
    pick = {}
    for i, key in enumerate(keys):
        kind, n, b, dt = key
        l2b, al = seen[key]
        tv = table_choice(table, kind, dt, al, l2b, int(math.log2(n)))
        pick[key] = {"learned": policy_pick(pred[i], tv, margins[KIND_NAME[kind]]),
                     "learned_pure": int(np.argmin(pred[i][:NSEL])), "tuned": tv if tv >= 0 else 0, "plain": 0}
    rep = summarize(keys, meas, pick, rng.integers(0, len(keys), calls))
    rep["calls"] = calls
    rep["shapes"] = len(keys)
    rep["ranks"] = sorted({k[1] for k in keys})
    rep["choices"] = {f"{k[0]}:{k[1]}x{k[2]}:{k[3]}": pick[k] for k in keys}
    rep["measured_us"] = {f"{k[0]}:{k[1]}x{k[2]}:{k[3]}": meas[k] for k in keys}
    rep["kernel_seen"] = {f"{k[0]}:{k[1]}x{k[2]}:{k[3]}": list(seen[k]) + [shares[k[1]]] for k in keys}
    log(json.dumps({k: rep[k] for k in ("all", "allreduce", "alltoallv")}))
    return rep


POLICIES = ("learned", "learned_pure", "tuned", "plain")


def summarize(keys, meas, pick, idx):
    """Total and per-call regret of each policy over the calls `idx` (indices into keys)."""
    rep = {}
    for label, kinds in (("all", KINDS), ("allreduce", (KIND_ALLREDUCE,)), ("alltoallv", (KIND_ALLTOALLV,))):
        tot = {p_: 0.0 for p_ in ("best",) + POLICIES}
        regrets = {p_: [] for p_ in POLICIES}
        for i in idx:
            key = keys[i]
            if key[0] not in kinds:
                continue
            t = meas[key]
            best = min(t)
            tot["best"] += best
            for pol in POLICIES:
                tp = t[pick[key][pol]]
                tot[pol] += tp
                regrets[pol].append(tp / best - 1.0)
        rep[label] = {"calls": len(regrets["plain"]),
                      "total_time_ms": {k: v / 1e3 for k, v in tot.items()},
                      "time_over_best": {p_: tot[p_] / tot["best"] - 1.0 for p_ in POLICIES},
                      "mean_regret": {p_: float(np.mean(regrets[p_])) for p_ in POLICIES},
                      "p90_regret": {p_: float(np.percentile(regrets[p_], 90)) for p_ in POLICIES},
                      "learned_vs_tuned_time": tot["learned"] / tot["tuned"]}
    return rep


def split_margins(records, grid, shares, epochs: int = 60):
    """Override margins chosen without the held-out stream and without judging either side on shapes it
    was fitted to: two folds over the sweep's rank counts (even and odd powers of two); in each, a table and
    a network are fitted to one half and the other half is served as an off-grid rank count is at run time,
    from the table column of the next lower fitted rank count."""
    totals = {"allreduce": {}, "alltoallv": {}}
    for fit in (RANKS[0::2], RANKS[1::2]):
        score = [n for n in RANKS if n not in fit and any(f < n for f in fit)]
        rec_f = [r for r in records if r[1] in fit]
        X, T, M = dataset(rec_f, shares)
        net = MLP(seed=1)
        net.train(X, T, M, epochs=epochs)
        table = build_table({k: g for k, g in grid.items() if k[1] in fit})
        lower = {n: int(math.log2(max(f for f in fit if f < n))) for n in score}
        t = margin_totals(net, table, {k: g for k, g in grid.items() if k[1] in score}, shares,
                          rank_col=lambda n: lower[n])
        for kname, d in t.items():
            for m, v in d.items():
                totals[kname][m] = totals[kname].get(m, 0.0) + v
    return pick_margins(totals)


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
    hist = mlp.train(X[tr], T[tr], M[tr], epochs=100)
    xv = torch.from_numpy(X[va]).cuda()
    tv = torch.from_numpy(T[va]).cuda()
    mv = torch.from_numpy(M[va]).cuda()
    vloss, _ = mlp.loss_grad(xv, tv, mv)
    params = mlp.params()
    margins = split_margins(records, grid, shares)
    print(f"override margins chosen by the rank-count split of the sweep: {margins}", flush=True)
    np.save(out / "tuned_table.npy", table)
    np.save(out / "mlp_params.npy", params)
    rep = evaluate(params, table, margins=margins)
    rep.update({"train_records": int(len(tr)), "val_records": int(len(va)), "train_loss": hist,
                "val_loss": float(vloss.item()), "sweep_seconds": time.time() - t0,
                "records_by_kind": {str(k): int(sum(1 for r in records if r[0] == k)) for k in KINDS},
                "grid_median_us": {f"{k[0]}:{k[1]}:{k[2]}:{k[3]}:{k[4]}": g[2] for k, g in grid.items()}})
    rep["margins"] = margins
    (out / "selector_report.json").write_text(json.dumps(rep, indent=1))
    print(json.dumps({k: rep[k] for k in ("all", "allreduce", "alltoallv", "val_loss", "train_records")}))


def load_packaged():
    """(tuned table, MLP parameters) shipped with the package, or (None, None)."""
    t, p = DATA / "tuned_table.npy", DATA / "mlp_params.npy"
    if not (t.exists() and p.exists()):
        return None, None
    return np.load(t), np.load(p)


def packaged_margins() -> dict:
    """The override margins (per kind) the packaged network was evaluated with (chosen on its sweep)."""
    rep = DATA / "selector_report.json"
    if rep.exists():
        r = json.loads(rep.read_text())
        if "margins" in r:
            return {k: float(v) for k, v in r["margins"].items()}
        m = float(r.get("margin", MARGIN))
        return {"allreduce": m, "alltoallv": m}
    return {"allreduce": MARGIN, "alltoallv": MARGIN}


def apply_policy(world, policy: str):
    """Sets a world's selection policy: "plain" (DIRECT), "tuned" (packaged table), "learned" (packaged
    network evaluated in the kernel once per call shape, its choice cached), "heuristic" (the library
    default)."""
    if policy == "plain":
        world.set_policy(-1, 0)
        return
    if policy == "heuristic":
        world.set_policy(-1, 3)
        return
    table, params = load_packaged()
    if table is None:
        raise FileNotFoundError(f"no trained selector in {DATA}")
    if policy == "tuned":
        world.set_tuned_table(table)
        world.set_policy(-1, 1)
    elif policy == "learned":
        world.set_tuned_table(table)
        world.set_mlp(params)
        m = packaged_margins()
        world.set_tuning(gpumpi.TUNE_MLP_MARGIN, int(round(m["allreduce"] * 1000)))
        world.set_tuning(gpumpi.TUNE_MLP_MARGIN_PULL, int(round(m["alltoallv"] * 1000)))
        world.set_policy(-1, 2)
    else:
        raise ValueError(policy)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("cmd", choices=["run"])
    ap.add_argument("--out", required=True, help="folder for the recorded timings, table, network and report")
    ap.add_argument("--iters", type=int, default=30)
    a = ap.parse_args()
    run(Path(a.out), iters=a.iters)
