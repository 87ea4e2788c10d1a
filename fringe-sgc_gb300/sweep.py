"""Edges-per-second sweep over a pattern family, in one process.

Counterpart of the reference's reproduce.py, which runs one fringePreprocess
and one fringeCount process per (graph, pattern) and writes, per graph, the
directed CSR entries divided by each count's runtime (reproduce.py:20-98).
Here every count goes through the library on resident graphs.  Patterns are
read from files in the reference's format: a first line `# Nodes: N ...`, then
one `a b` pair per line (both directions may appear; pairs are deduplicated).

    python fringe-sgc_gb300/sweep.py edge --patterns /path/to/patterns \\
        --graphs graphs/a.egr graphs/b.egr --out edge.csv
    python fringe-sgc_gb300/sweep.py fig3 --patterns /path/to/patterns/wedge \\
        --stand-ins all --shrink 4

Without .egr files, --stand-ins builds seeded synthetic graphs of the shapes of
the reference's eight evaluation graphs (road network, co-purchase, RMAT-16,
web crawl, co-authorship, social network, internet topology, Delaunay mesh);
--shrink k divides their vertex counts by k.
"""
import argparse
import csv
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import fsgc  # noqa: E402


def read_pattern_file(path):
    """(n, sorted undirected pairs) of a pattern file."""
    with open(path) as f:
        m = re.search(r"Nodes:\s*(\d+)", f.readline())
        if not m:
            raise ValueError(f"{path}: first line has no 'Nodes: N'")
        n = int(m.group(1))
        pairs = set()
        for line in f:
            if line.strip():
                a, b = map(int, line.split())
                pairs.add((min(a, b), max(a, b)))
    return n, sorted(pairs)


def family_patterns(pattern_dir, family):
    """The family's pattern files in pattern_dir (names starting with the
    family, as reproduce.py selects them), sorted by name."""
    out = []
    for f in sorted(os.listdir(pattern_dir)):
        if f.endswith(".txt") and f.startswith(family):
            n, pairs = read_pattern_file(os.path.join(pattern_dir, f))
            out.append((os.path.splitext(f)[0], n, pairs))
    return out


def lattice(rows, cols, diagonals, drop, seed):
    """rows x cols grid, optionally triangulated, with a seeded fraction of
    edges dropped (planar stand-ins)."""
    rng = np.random.default_rng(seed)
    idx = np.arange(rows * cols, dtype=np.int64).reshape(rows, cols)
    e = [np.stack([idx[:, :-1].ravel(), idx[:, 1:].ravel()], 1), np.stack([idx[:-1, :].ravel(), idx[1:, :].ravel()], 1)]
    if diagonals:
        e.append(np.stack([idx[:-1, :-1].ravel(), idx[1:, 1:].ravel()], 1))
    e = np.concatenate(e)
    if drop > 0:
        e = e[rng.random(len(e)) >= drop]
    return fsgc.csr_from_edges(rows * cols, e.astype(np.int32))


def stand_ins(shrink=1):
    """Seeded synthetic graphs with the vertex counts and average degrees of the
    reference's evaluation graphs (generators: lattice, Chung-Lu, RMAT)."""
    s = max(1, int(shrink))
    side = lambda n: max(2, int(round((n / s) ** 0.5)))  # noqa: E731
    return {
        "USA-road-d.NY": lambda: lattice(side(264346), side(264346), False, 0.3, 1),
        "amazon0601": lambda: fsgc.gen_chung_lu(403394 // s, 12.2, 2.6, 2),
        "rmat16.sym": lambda: fsgc.gen_rmat(max(8, 16 - (s.bit_length() - 1)), 16, seed=3),
        "in-2004": lambda: fsgc.gen_chung_lu(1382908 // s, 19.8, 2.1, 4),
        "coPapersDBLP": lambda: fsgc.gen_chung_lu(540486 // s, 56.4, 2.5, 5),
        "soc-LiveJournal1": lambda: fsgc.gen_chung_lu(4847571 // s, 17.7, 2.3, 6),
        "internet": lambda: fsgc.gen_chung_lu(124651 // s, 3.1, 2.2, 7),
        "delaunay_n22": lambda: lattice(side(4194304), side(4194304), True, 0.0, 8),
    }


def sweep(ctx, graphs, patterns, writer=None):
    """graphs: [(name, Graph)]; patterns: [(name, n, pairs)].  Returns rows of
    [graph, edges/s per pattern ...] (directed entries / count seconds)."""
    mos = [(name, fsgc.preprocess(n, pairs)) for name, n, pairs in patterns]
    rows = []
    for gname, g in graphs:
        gid = ctx.upload(g)
        ctx.prepare(gid)
        row = [gname]
        for _, mo in mos:
            r = ctx.count(gid, mo)
            row.append(g.m / (r.device_ms / 1000.0) if r.device_ms > 0 else float("inf"))
        ctx.release(gid)
        rows.append(row)
        if writer is not None:
            writer.writerow(row)
    return rows


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("family", help="pattern-file prefix, e.g. vertex, edge, triangle, wedge, fig3")
    ap.add_argument("--patterns", required=True, help="directory of pattern files")
    ap.add_argument("--graphs", nargs="*", default=[], help=".egr files")
    ap.add_argument("--stand-ins", default="", help="'all' or comma-separated stand-in names")
    ap.add_argument("--shrink", type=int, default=1, help="divide the stand-ins' vertex counts by this")
    ap.add_argument("--out", default=None, help="CSV file (default: <family>.csv)")
    ap.add_argument("--device", type=int, default=0)
    args = ap.parse_args(argv)
    patterns = family_patterns(args.patterns, args.family)
    if not patterns:
        raise SystemExit(f"no pattern files starting with {args.family!r} in {args.patterns}")
    graphs = [(os.path.splitext(os.path.basename(p))[0], fsgc.egr_read(p)) for p in args.graphs]
    if args.stand_ins:
        si = stand_ins(args.shrink)
        names = list(si) if args.stand_ins == "all" else args.stand_ins.split(",")
        graphs += [(name, si[name]()) for name in names]
    out = args.out or f"{args.family}.csv"
    with open(out, "w", newline="") as f, fsgc.Context(args.device) as ctx:
        w = csv.writer(f)
        w.writerow(["Graph File"] + [f"fsgc GB300 {name}" for name, _, _ in patterns])
        for row in sweep(ctx, graphs, patterns, w):
            print(row[0], " ".join(f"{x:.4g}" for x in row[1:]), flush=True)
    print(f"wrote {out}")


if __name__ == "__main__":
    main()
