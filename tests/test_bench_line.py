"""bench.py's JSON line, assembled on the CPU from a stand-in of the GPU run
(the measured values are made up; only the line's keys, units and arithmetic
are checked): the fields of the benchmark contract, roofline, e2e, CPU baseline,
edges/s and exact counts."""
import json
import os
import sys

import pytest

import fsgc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


class _Ctx:
    def close(self):
        pass


def test_default_line_has_the_contract_fields(monkeypatch, capsys):
    g = fsgc.gen_rmat(10, 8, seed=3)
    mos = bench.matching_orders()
    names = [n for n, _ in mos]
    per = {n: 10.0 + i for i, n in enumerate(names)}
    out = {"per_task_ms": per, "prep_ms": 1.5, "counts": {n: 7 for n in names},
           "cores": {n: (3 if "wedge_1_on_each_end" in n else 1) for n in names},
           "exact": {n: {"exact": "7", "u64_wrapped": False} for n in names},
           "t_dev": 0.2, "t_e2e": 0.25, "launches": 21, "clocks": {"sm_mhz": 2000.0, "sm_max_mhz": 2070.0,
                                                                     "reasons": [], "samples": 9},
           "gen_s": 0.1, "graph": {"n": g.n, "m": g.m, "max_degree": int(g.degrees().max())}}
    monkeypatch.setattr(bench, "run_gpu", lambda args, rank, world: (out, g, mos, _Ctx()))
    monkeypatch.setattr(bench, "cpu_sample", lambda g, mos, budget, threads: (100.0, {n: 1 for n in names}))
    monkeypatch.setattr(sys, "argv", ["bench.py", "--steps", "2", "--warmup", "3"])
    bench.main()
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "roofline", "cpu_baseline", "e2e",
                "gpu_launches", "clocks"):
        assert key in line, key
    assert line["value"] == pytest.approx(len(mos) * 2 / 0.2)
    assert line["e2e"]["value"] == pytest.approx(len(mos) * 2 / 0.25)
    assert line["e2e"]["h2d_bytes_per_step"] == 8 * (g.n + 1) + 4 * g.m
    r = line["roofline"]
    assert r["kernel"] == max(per, key=per.get) and r["unit"] == "GB/s" and r["peak"] > 0
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"], rel=1e-3)
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == pytest.approx(len(mos) / 100.0)
    c = line["config"]
    assert c["workload"].startswith("RMAT") and set(c["edges_per_s"]) == set(names)
    assert c["exact_counts"][names[0]]["exact"] == "7"


def _fake_refrun(monkeypatch, ms_per_pattern, available=True):
    import refrun
    calls = []
    monkeypatch.setattr(refrun, "available", lambda: available)

    def write(path, *a):
        with open(path, "wb") as f:
            f.write((1024).to_bytes(4, "little") + (20000).to_bytes(4, "little"))
    monkeypatch.setattr(refrun, "write_rmat_egr", write)

    def run(egr, paths, timeout=None):
        calls.append(paths[0])
        return [{"core": 3, "aut": 2, "raw": 10, "count": 5, "ms": ms_per_pattern}]
    monkeypatch.setattr(refrun, "run", run)
    return calls


def test_reference_arm_line(monkeypatch, capsys):
    """The reference arm's line: the reference's kernels' times (faked here),
    full passes repeated within the budget, the first ones untimed."""
    calls = _fake_refrun(monkeypatch, 250.0)
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--steps", "2", "--warmup", "3",
                                      "--ref-budget", "100000"])
    bench.main()
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "patterns/s"
    assert len(calls) == 8 * 5 and line["steps"] == 2 and line["warmup"] == 3
    assert line["value"] == pytest.approx(8 / 2.0)  # 8 patterns x 250 ms per step
    assert line["e2e"] == {"value": line["value"], "unit": "patterns/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["cpu_baseline"]["kind"] == "reference" and line["config"]["value_bound"] is None
    assert line["config"]["counts"]["edge_5_5"]["count"] == "5"


def test_reference_arm_takes_recorded_times_for_patterns_beyond_its_budget(monkeypatch, capsys):
    """With the recorded RMAT-22 run, the shortest patterns run first and the
    ones whose recorded time does not fit the budget are counted at that time."""
    rec = bench.reference_golden(22)
    assert rec is not None
    ran = []
    import refrun
    _fake_refrun(monkeypatch, 0.0)

    def run(egr, paths, timeout=None):
        ran.append(paths[0])
        return [{"core": 1, "aut": 1, "raw": 1, "count": 1, "ms": 100.0}]
    monkeypatch.setattr(refrun, "run", run)
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0",
                                      "--ref-budget", "300"])
    bench.main()
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["steps"] == 0 and line["config"]["value_bound"].startswith("upper")
    skipped = [k for k, v in rec["patterns"].items() if v["ms"] > 200000]
    assert len(ran) == 8 - len(skipped) and all(k in line["config"]["value_bound"] for k in skipped)
    want = 8 / ((8 - len(skipped)) * 0.1 + sum(rec["patterns"][k]["ms"] / 1000.0 for k in skipped))
    assert line["value"] == pytest.approx(want)


def test_reference_arm_stops_within_its_budget(monkeypatch, capsys):
    """Passes stop once the next would not end within the budget; one full pass
    is then the timed step."""
    import time as _time
    clock = [1000.0]
    monkeypatch.setattr(bench.time, "time", lambda: clock[0])
    import refrun

    def run(egr, paths, timeout=None):
        clock[0] += 60.0
        return [{"core": 3, "aut": 1, "raw": 1, "count": 1, "ms": 60000.0}]
    _fake_refrun(monkeypatch, 0.0)
    monkeypatch.setattr(refrun, "run", run)
    monkeypatch.setattr(bench, "reference_golden", lambda scale: None)  # no recorded run to predict from
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--steps", "20", "--warmup", "5",
                                      "--ref-budget", "700"])
    bench.main()
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["steps"] == 1 and line["warmup"] == 0 and line["value"] == pytest.approx(8 / 480.0)
    assert _time is not None


def test_reference_arm_unavailable_without_the_cubin(monkeypatch, capsys):
    _fake_refrun(monkeypatch, 1.0, available=False)
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference"])
    bench.main()
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and "unavailable" in line


class _CountingCtx:
    """fsgc.Context stand-in for the mixed workload: a count's result is a
    function of the pattern bytes, so single counts and sets agree."""

    launches = 0

    def __init__(self, *_):
        self.tuning = fsgc.Tuning.default()

    def upload(self, g):
        return 7

    def prepare(self, gid):
        pass

    def set_tuning(self, t=None, **kw):
        pass

    def get_tuning(self):
        return self.tuning

    def _res(self, mo):
        b = mo.to_bytes()

        class R:
            count = sum(b) * 1000003
            raw_total = count
            automorphisms = 1
            core_type = min(mo.nodes, 5)
            flags = 0
            device_ms = 0.5
        return R()

    def count(self, gid, mo):
        self.launches += 1
        return self._res(mo)

    def count_set(self, gid, mos):
        self.launches += 1
        return [self._res(mo) for mo in mos]

    def synchronize(self):
        pass

    def release(self, gid):
        pass

    def close(self):
        pass


def test_mixed_line_splits_patterns_and_reports_both_modes(monkeypatch, capsys):
    """The mixed workload's line: patterns without per-match work on the main
    graph, general cores and fringed-centre wedges on the small one, both modes
    timed, every batched count checked against its single count."""
    monkeypatch.setattr(fsgc, "Context", _CountingCtx)
    monkeypatch.setattr(sys, "argv", ["bench.py", "--workload", "mixed", "--mixed-patterns", "16",
                                      "--mixed-scale", "8", "--general-scale", "5", "--steps", "1", "--warmup", "2"])
    bench.main()
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    main, gen = line["config"]["main"], line["config"]["general"]
    assert main["scale"] == 8 and main["patterns"] + (gen["patterns"] if gen else 0) == 16
    assert not main["not_timed"]
    assert line["value"] == main["batched_queries_per_s"] > 0
    assert line["one_query_per_launch"]["value"] == main["single_queries_per_s"]
    assert line["batched_over_single"] == main["batched_over_single"]
    pats = dict(bench.draw_patterns(16, 20251208, max_core=6))
    for name in main["single_per_pattern_ms"]:
        assert not bench.per_match_family(pats[name])
    if gen:
        for name in gen["single_per_pattern_ms"]:
            assert bench.per_match_family(pats[name])
