"""Autotuner of the counting kernels' method thresholds and launch shapes.

The reference fixes its method switches at compile time (src/fringeCount.cu:70,
80-84, 1237, 1328-1334, 1797-1804).  Here they are fields of fsgc_tuning, set
per context, and this module picks them per graph by timing:

  wedge_small_max_degree  endpoint degree up to which the wedge-pair counting
                          runs in the shared-memory counter kernel (higher
                          degrees go to the hub kernel)
  triangle_walk_ratio     triangle bitmaps: walk N(b) against the staged N(a)
                          when deg b <= ratio * deg a, else binary-search N(b)
  triangle_stage_max      longest N(a) staged in shared memory by bulk copy
  general_lane_venn_max   general cores: Venn rows up to this many list
                          entries are built by one lane, longer ones by a warp
  general_blocks_per_sm   general cores: the task granularity of the grid

Coordinate descent: each field in turn takes each candidate value while the
others keep their best so far; a candidate's cost is the smallest, over
`repeats` runs, of the summed device time of the patterns whose kernels the
field steers.  Every candidate's counts must equal the default setting's
(the fields change speed only); a difference is an error.  The chosen values
are written to a JSON file keyed by the graph's (n, m, maximum degree), which
bench.py reads.

    python fringe-sgc_gb300/autotune.py --scale 22 --out fringe-sgc_gb300/tuning.json
"""
import argparse
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))

CANDIDATES = {
    "wedge_small_max_degree": [256, 512, 1024, 2048],
    "triangle_walk_ratio": [0, 1, 2, 4, 16],
    "triangle_stage_max": [0, 2048, 8192],
    "general_lane_venn_max": [0, 32, 96, 256, 1 << 20],
    "general_blocks_per_sm": [2, 4, 8, 12],
}
# core types (fsgc_result.core_type) whose kernels each field steers
STEERS = {
    "wedge_small_max_degree": {3},
    "triangle_walk_ratio": {4},
    "triangle_stage_max": {4},
    "general_lane_venn_max": {5},
    "general_blocks_per_sm": {5},
}


def graph_key(n, m, max_degree):
    return f"n{n}_m{m}_d{max_degree}"


def _timed(ctx, gid, mos, repeats):
    """(min over repeats of the summed device ms, results of the last run)."""
    best, res = None, None
    for _ in range(repeats):
        res = [ctx.count(gid, mo) for mo in mos]
        t = sum(r.device_ms for r in res)
        best = t if best is None else min(best, t)
    return best, res


def tune(ctx, gid, mos, repeats=2, fields=None, log=None):
    """Picks the context's tuning for graph `gid` and patterns `mos`.  Returns
    (values dict, report {field: {value: ms}}); leaves the context set to the
    chosen values."""
    import fsgc
    base = fsgc.Tuning.default()
    ctx.set_tuning(base)
    ref = [ctx.count(gid, mo) for mo in mos]  # the default setting's counts
    kinds = [r.core_type for r in ref]
    best = base.as_dict()
    report = {}
    for field in fields or list(CANDIDATES):
        sel = [mo for mo, k in zip(mos, kinds) if k in STEERS[field]]
        if not sel:
            continue
        want = [(r.count, r.raw_total) for r, k in zip(ref, kinds) if k in STEERS[field]]
        report[field] = {}
        for value in CANDIDATES[field]:
            ctx.set_tuning(None, **{**best, field: value})
            ms, res = _timed(ctx, gid, sel, repeats)
            got = [(r.count, r.raw_total) for r in res]
            if got != want:
                raise RuntimeError(f"{field}={value} changed a count: {got} vs {want}")
            report[field][value] = ms
            if log:
                log(f"autotune: {field}={value}: {ms:.2f} ms")
        best[field] = min(report[field], key=report[field].get)
    ctx.set_tuning(None, **best)
    return best, report


def load(path, key):
    """The tuned values recorded for graph `key`, or None."""
    if not os.path.exists(path):
        return None
    with open(path) as f:
        return json.load(f).get(key, {}).get("values")


def save(path, key, values, report, note=""):
    rec = {}
    if os.path.exists(path):
        with open(path) as f:
            rec = json.load(f)
    rec[key] = {"values": values, "ms": {f: {str(v): round(ms, 3) for v, ms in r.items()} for f, r in report.items()},
                "note": note}
    with open(path, "w") as f:
        json.dump(rec, f, indent=1, sort_keys=True)


def main():
    sys.path.insert(0, HERE)
    sys.path.insert(0, os.path.dirname(HERE))
    import fsgc
    import bench
    ap = argparse.ArgumentParser()
    ap.add_argument("--scale", type=int, default=22)
    ap.add_argument("--repeats", type=int, default=2)
    ap.add_argument("--mixed", type=int, default=0, help="also tune on this many mixed-workload patterns")
    ap.add_argument("--out", default=os.path.join(HERE, "tuning.json"))
    args = ap.parse_args()
    R = bench.RMAT
    g = fsgc.gen_rmat(args.scale, R["edge_factor"], R["a"], R["b"], R["c"], R["seed"])
    mos = [mo for _, mo in bench.matching_orders()]
    if args.mixed:
        mos += [mo for _, mo in bench.draw_patterns(args.mixed, 20251208, max_core=3)]
    with fsgc.Context(0) as ctx:
        gid = ctx.upload(g)
        ctx.prepare(gid)
        values, report = tune(ctx, gid, mos, args.repeats, log=lambda s: print(s, file=sys.stderr, flush=True))
        ctx.release(gid)
    key = graph_key(g.n, g.m, int(g.degrees().max()))
    save(args.out, key, values, report, note=f"RMAT scale {args.scale}, {len(mos)} patterns")
    print(json.dumps({"key": key, "values": values, "ms": report}))


if __name__ == "__main__":
    main()
