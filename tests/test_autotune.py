"""The autotuner's search on the CPU, over a fake context whose device times
depend on the tuning (the real timings come from a GB300 run): coordinate
descent picks the cheapest value per field, fields only time the patterns
whose kernels they steer, a count that changes with a setting is an error, and
the JSON record round-trips."""
import os
import sys

import pytest

import fsgc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "fringe-sgc_gb300"))
import autotune  # noqa: E402


class R:
    def __init__(self, count, core, ms):
        self.count, self.raw_total, self.core_type, self.device_ms = count, count, core, ms


class FakeCtx:
    """Pattern i has core type cores[i]; its time is a function of the tuning."""

    def __init__(self, cores, cost, break_on=None):
        self.cores, self.cost, self.break_on = cores, cost, break_on
        self.t = fsgc.Tuning.default().as_dict()
        self.timed = []

    def set_tuning(self, t=None, **fields):
        if t is not None:
            self.t = t.as_dict()
        self.t.update(fields)

    def count(self, gid, mo):
        i = mo
        self.timed.append((i, dict(self.t)))
        c = 100 + i
        if self.break_on and self.t[self.break_on[0]] == self.break_on[1]:
            c += 1
        return R(c, self.cores[i], self.cost(i, self.t))


def test_picks_the_cheapest_value_per_field():
    cores = [3, 4, 5, 1]

    def cost(i, t):
        if cores[i] == 3:
            return abs(t["wedge_small_max_degree"] - 512) / 100 + 1
        if cores[i] == 4:
            return abs(t["triangle_walk_ratio"] - 4) + (0 if t["triangle_stage_max"] == 8192 else 3)
        if cores[i] == 5:
            return abs(t["general_lane_venn_max"] - 32) / 10 + abs(t["general_blocks_per_sm"] - 4)
        return 1.0
    ctx = FakeCtx(cores, cost)
    values, report = autotune.tune(ctx, 0, [0, 1, 2, 3], repeats=1)
    assert values["wedge_small_max_degree"] == 512
    assert values["triangle_walk_ratio"] == 4 and values["triangle_stage_max"] == 8192
    assert values["general_lane_venn_max"] == 32 and values["general_blocks_per_sm"] == 4
    assert ctx.t == values
    # the vertex-core pattern (core 1) is steered by no field and only timed once, for the reference counts
    assert sum(1 for i, _ in ctx.timed if i == 3) == 1


def test_a_count_that_changes_is_an_error():
    ctx = FakeCtx([3], lambda i, t: 1.0, break_on=("wedge_small_max_degree", 256))
    with pytest.raises(RuntimeError):
        autotune.tune(ctx, 0, [0], repeats=1)


def test_json_record_round_trip(tmp_path):
    p = str(tmp_path / "tuning.json")
    key = autotune.graph_key(10, 20, 3)
    values = fsgc.Tuning.default().as_dict()
    values["triangle_walk_ratio"] = 4
    autotune.save(p, key, values, {"triangle_walk_ratio": {4: 1.5, 16: 2.0}}, note="x")
    assert autotune.load(p, key) == values
    assert autotune.load(p, "other") is None
