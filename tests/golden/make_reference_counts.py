"""Pin the benchmark's counts to the reference's own kernels.

Runs on a GB300 (or any GPU the cubin was compiled for): generates the seeded
RMAT graph of the benchmark with oracle/_build/graphgen, counts the eight
workload patterns with the reference's own kernels (oracle/_ref/fringeCount.cubin
driven by oracle/_build/ref_runner), and writes, per pattern, the core type, the
divisor, the raw u64 total, the count and the reference's occurrences() time:

    python tests/golden/make_reference_counts.py --scale 22 --out tests/golden/reference_rmat22.json

bench.py asserts its own counts against the file for its scale, and the GPU
tests do the same at the smaller scales.  The graph parameters are those of the
benchmark: edge factor 16, (a, b, c) = (0.57, 0.19, 0.19), seed 20251203.
"""
import argparse
import json
import os
import platform
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import refrun  # noqa: E402

RMAT = dict(edge_factor=16, a=0.57, b=0.19, c=0.19, seed=20251203)
PATTERNS = ["wedge_1_on_centre", "wedge_2_on_centre", "wedge_4_on_centre", "wedge_1_on_each_end",
            "triangle_3_on_one", "4cycle_opposite", "4clique_3_distinct", "edge_5_5"]


def gpu_name():
    try:
        r = subprocess.run(["nvidia-smi", "--query-gpu=name", "--format=csv,noheader"], capture_output=True,
                           text=True, timeout=30)
        return r.stdout.strip().splitlines()[0]
    except (OSError, IndexError, subprocess.SubprocessError):
        return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scale", type=int, required=True)
    ap.add_argument("--patterns", default=",".join(PATTERNS))
    ap.add_argument("--out", required=True)
    args = ap.parse_args()
    if not refrun.available():
        raise SystemExit("the reference's cubin is not built (oracle/_ref/fringeCount.cubin)")
    names = args.patterns.split(",")
    mos = refrun.workload_matching_orders(names)
    with tempfile.TemporaryDirectory() as tmp:
        egr = os.path.join(tmp, "g.egr")
        t = time.time()
        refrun.write_rmat_egr(egr, args.scale, RMAT["edge_factor"], RMAT["a"], RMAT["b"], RMAT["c"], RMAT["seed"])
        gen_s = time.time() - t
        n, m = refrun.egr_header(egr)
        paths = refrun.write_mo_files(mos, tmp)
        res = {}
        for name, p in zip(names, paths):  # one pattern per process, as the reference's harness runs them
            r = refrun.run(egr, [p])[0]
            res[name] = r
            print(name, r, file=sys.stderr, flush=True)
    rec = {"generator": "reference kernels (oracle/_ref/fringeCount.cubin via oracle/_build/ref_runner)",
           "graph": {"kind": "rmat", "scale": args.scale, **RMAT, "n": n, "m_directed": m},
           "gpu": gpu_name(), "host": platform.machine(), "graph_gen_s": round(gen_s, 1),
           "patterns": {k: {"core": v["core"], "aut": v["aut"], "raw": str(v["raw"]), "count": str(v["count"]),
                            "ms": v["ms"], "mo": mos[k].hex()} for k, v in res.items()}}
    with open(args.out, "w") as f:
        json.dump(rec, f, indent=1)
    print(json.dumps(rec["patterns"]))


if __name__ == "__main__":
    main()
