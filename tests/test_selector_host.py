"""CPU: the host side of the selector — the override-margin rule chosen on the sweep's shapes, the
packaged artifacts and their recorded held-out figures, and the calls apply_policy makes on a world."""
import json

import numpy as np
import pytest

import gpumpi
from gpumpi import selector as sel


class TableNet:
    """Stand-in for the trained network: predicted log-times per variant, looked up by the bytes feature."""

    def __init__(self, rows):
        self.rows = rows                      # {log2 bytes: [4 predicted log-times]}

    def predict(self, X):
        return np.stack([np.asarray(self.rows[int(round(x[0] * 8 + 16))], np.float32) for x in X])


def grid_entry(grid, n, nbytes, times):
    l2b = float(np.log2(nbytes))
    for v, t in enumerate(times):
        grid[(sel.KIND_ALLREDUCE, n, nbytes, gpumpi.FLOAT, v)] = (int(l2b), 0, float(t), l2b)


def test_margin_keeps_table_where_network_is_unsure_and_overrides_where_sure():
    n = 64
    grid = {}
    grid_entry(grid, n, 1 << 10, [1.0, 2.0, 2.0])   # the table is right (variant 0)
    grid_entry(grid, n, 1 << 12, [3.0, 1.0, 3.0])   # the table is wrong; variant 1 is 3x faster
    table = np.full((3, sel.NDCLASS, 2, 32, 16), -1, np.int8)
    table[0, :, :, 10, 6] = 0
    table[0, :, :, 12, 6] = 0
    # shape 1 KiB: the network prefers variant 1 by 0.08 (wrongly); shape 4 KiB: by 0.8 (rightly)
    net = TableNet({10: [0.50, 0.42, 1.0, 1.0], 12: [1.0, 0.2, 1.0, 1.0]})
    # margins 0.1 .. 0.5 keep the table at 1 KiB and override at 4 KiB (total 2.0); 0.05 overrides both
    # (3.0); 1.0 and 2.0 override neither (4.0); ties go to the larger margin.  Margins are per kind: the
    # Alltoall(v) margin has no shapes here and keeps the default.
    m = sel.choose_margin(net, table, grid, {n: 0.8})
    assert m == {"allreduce": 0.5, "alltoallv": sel.MARGIN}
    assert sel.choose_margin(net, table, grid, {n: 0.8}, candidates=(0.05, 1.0))["allreduce"] == 0.05
    assert sel.choose_margin(net, table, grid, {n: 0.8}, candidates=(1.0, 2.0))["allreduce"] == 2.0


def test_table_separates_datatypes_and_fills_untimed_classes():
    # one cell (1024 ranks, 2^20 bytes, 16-byte aligned): float and int32 favour DIRECT, double favours RING
    # by enough that the pooled sum would pick RING for every type
    n, grid = 1024, {}
    for dt, times in ((gpumpi.FLOAT, [367.5, 527.8, 403.2]), (gpumpi.INT, [377.7, 530.7, 400.6]),
                      (gpumpi.DOUBLE, [962.1, 904.8, 601.9])):
        for v, t in enumerate(times):
            grid[(sel.KIND_ALLREDUCE, n, 1 << 20, dt, v)] = (20, 0, t, 20.0)
    # Alltoall(v) timed with int32 only, and only its misaligned class
    for v, t in enumerate([5.0, 6.0, 4.0]):
        grid[(sel.KIND_ALLTOALLV, n, 3 << 19, gpumpi.INT, v)] = (20, 1, t, 20.58)
    t = sel.build_table(grid)
    assert t.shape == (3, sel.NDCLASS, 2, 32, 16)
    assert t[0, sel.dclass(gpumpi.FLOAT), 0, 20, 10] == 0
    assert t[0, sel.dclass(gpumpi.INT), 0, 20, 10] == 0
    assert t[0, sel.dclass(gpumpi.DOUBLE), 0, 20, 10] == 2
    assert sel.dclass(gpumpi.INT64_T) == sel.dclass(gpumpi.INT) == 2 and sel.dclass(gpumpi.LONG_DOUBLE) == 1
    assert np.array_equal(t[0], t[1])                                  # Reduce follows Allreduce
    assert (t[0, :, 1, 20, 10] == t[0, :, 0, 20, 10]).all()            # untimed alignment class: the other one
    assert (t[2, :, :, 20, 10] == 2).all()                             # every datatype and alignment class
    assert sel.table_choice(t, sel.KIND_ALLREDUCE, gpumpi.DOUBLE, 16, 20.3, 10) == 2
    assert sel.table_choice(t, sel.KIND_ALLREDUCE, gpumpi.FLOAT, 8, 20.3, 10) == 0
    assert sel.table_choice(t, sel.KIND_ALLREDUCE, gpumpi.FLOAT, 16, 21.0, 10) == -1


def test_policy_pick_never_chooses_staged():
    # the network's output for STAGED (variant 3) is not a choice, however low it is
    pred = np.array([1.0, 0.9, 0.8, -5.0], np.float32)
    assert sel.policy_pick(pred, 0, 0.05) == 2
    assert sel.policy_pick(pred, 0, 0.3) == 0      # within the margin: the table's choice stands
    assert sel.policy_pick(pred, -1, 0.3) == 2     # no table cell: the network's choice


def test_margin_defaults_without_complete_shapes():
    grid = {}
    grid[(sel.KIND_ALLREDUCE, 64, 1024, gpumpi.FLOAT, 0)] = (10, 0, 1.0, 10.0)   # one variant only
    table = np.zeros((3, sel.NDCLASS, 2, 32, 16), np.int8)
    assert sel.choose_margin(TableNet({}), table, grid, {64: 0.8}) == {"allreduce": sel.MARGIN,
                                                                        "alltoallv": sel.MARGIN}


def test_packaged_artifacts_and_recorded_figures():
    table, params = sel.load_packaged()
    if table is None:
        pytest.skip("no packaged selector")
    assert table.shape == (3, sel.NDCLASS, 2, 32, 16) and table.dtype == np.int8
    assert set(np.unique(table)) <= {-1, 0, 1, 2}        # STAGED is not a choice
    assert np.array_equal(table[0], table[1])          # Reduce follows the Allreduce sweep
    assert params.shape == (gpumpi.MLP_NPARAMS,) and params.dtype == np.float32
    assert np.isfinite(params).all()
    rep = json.loads((sel.DATA / "selector_report.json").read_text())
    allr = rep["all"]
    assert allr["calls"] >= 10000
    # the claim the artifacts ship with: learned within 5% of exhaustive best, not slower than the table
    assert allr["time_over_best"]["learned"] <= 0.05
    assert allr["learned_vs_tuned_time"] <= 1.0
    assert allr["time_over_best"]["learned"] <= allr["time_over_best"]["plain"]
    assert rep["margins"] == sel.packaged_margins()
    assert min(rep["ranks"]) >= 16 and all(n & (n - 1) for n in rep["ranks"])   # off-grid rank counts
    assert rep["shapes"] >= 300


class FakeWorld:
    def __init__(self):
        self.calls = []

    def set_policy(self, v, mode):
        self.calls.append(("policy", v, mode))

    def set_tuned_table(self, t):
        self.calls.append(("table", t.shape))

    def set_mlp(self, p):
        self.calls.append(("mlp", p.shape))

    def set_tuning(self, key, value):
        self.calls.append(("tuning", key, value))


def test_apply_policy_calls():
    w = FakeWorld()
    sel.apply_policy(w, "plain")
    assert w.calls == [("policy", -1, 0)]
    if sel.load_packaged()[0] is None:
        pytest.skip("no packaged selector")
    w = FakeWorld()
    sel.apply_policy(w, "tuned")
    assert w.calls == [("table", (3, sel.NDCLASS, 2, 32, 16)), ("policy", -1, 1)]
    w = FakeWorld()
    sel.apply_policy(w, "learned")
    assert w.calls == [("table", (3, sel.NDCLASS, 2, 32, 16)), ("mlp", (gpumpi.MLP_NPARAMS,)),
                       ("tuning", gpumpi.TUNE_MLP_MARGIN, int(round(sel.packaged_margins()["allreduce"] * 1000))),
                       ("tuning", gpumpi.TUNE_MLP_MARGIN_PULL,
                        int(round(sel.packaged_margins()["alltoallv"] * 1000))),
                       ("policy", -1, 2)]
    with pytest.raises(ValueError):
        sel.apply_policy(FakeWorld(), "nonsense")
