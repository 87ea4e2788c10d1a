"""Generate tests/golden/matching_orders.json with the reference's own decomposer.

Runs the reference's fringePreprocess (compiled from its sources by
oracle/Makefile into oracle/_ref/) on
  - every pattern file of the reference's pattern corpus (patterns/**.txt),
    turned into a command line the way its harness does (reproduce.py:54-66);
  - the 31 predefined motifs (`fringePreprocess <number>`);
  - the workload patterns (ER triangle + 2 fringes, the eight RMAT patterns);
  - seeded random patterns drawn like the batching workload (core from
    {edge, wedge, triangle, 4-path, 4-cycle, diamond, 4-clique, 5-cycle},
    0-12 fringes, each on a uniform random non-empty subset of the core).
and records the bytes of motif.mo that the reference defines (undefined bytes
of its uninitialised struct are stored as zero) or the rejection.

Usage (where the reference tree is available):
    python tests/golden/make_golden.py /path/to/reference
"""
import json
import os
import random
import re
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle  # noqa: E402

CORES = {
    "edge": (2, [(0, 1)]),
    "wedge": (3, [(0, 1), (0, 2)]),
    "triangle": (3, [(0, 1), (1, 2), (0, 2)]),
    "4-path": (4, [(0, 1), (1, 2), (2, 3)]),
    "4-cycle": (4, [(0, 1), (1, 2), (2, 3), (3, 0)]),
    "diamond": (4, [(0, 1), (1, 2), (2, 3), (3, 0), (0, 2)]),
    "4-clique": (4, [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]),
    "5-cycle": (5, [(0, 1), (1, 2), (2, 3), (3, 4), (4, 0)]),
}

WORKLOAD = {
    "er_triangle_2fringes": (5, [(0, 1), (1, 2), (0, 2), (0, 3), (1, 4)]),
    "wedge_1_on_centre": (4, [(0, 1), (0, 2), (0, 3)]),
    "wedge_2_on_centre": (5, [(0, 1), (0, 2), (0, 3), (0, 4)]),
    "wedge_4_on_centre": (7, [(0, 1), (0, 2), (0, 3), (0, 4), (0, 5), (0, 6)]),
    "wedge_1_on_each_end": (5, [(0, 1), (0, 2), (1, 3), (2, 4)]),
    "triangle_3_on_one": (6, [(0, 1), (1, 2), (0, 2), (0, 3), (0, 4), (0, 5)]),
    "4cycle_opposite": (6, [(0, 1), (1, 2), (2, 3), (3, 0), (0, 4), (2, 5)]),
    "4clique_3_distinct": (7, [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3), (0, 4), (1, 5), (2, 6)]),
    "edge_5_5": (12, [(0, 1)] + [(0, i) for i in range(2, 7)] + [(1, i) for i in range(7, 12)]),
}


def random_pattern(rng):
    name = rng.choice(sorted(CORES))
    k, edges = CORES[name]
    edges = list(edges)
    f = rng.randint(0, 12)
    for i in range(f):
        v = k + i
        sub = []
        while not sub:
            sub = [c for c in range(k) if rng.random() < 0.5]
        edges += [(c, v) for c in sub]
    return name, k + f, edges


def defined_bytes(mo):
    """Zero the bytes the reference does not write (its struct is uninitialised)."""
    b = bytearray(mo)
    nodes, sets = b[0], b[1]
    keep = {0, 1, 2}
    keep |= {3 + i for i in range(max(0, nodes - 1))}
    keep |= {8 + i for i in range(max(0, nodes - 1))}
    keep |= {13 + i for i in range(sets)}
    keep |= {76 + i for i in range(sets)}
    return bytes(b[i] if i in keep else 0 for i in range(len(b)))


def corpus(refroot):
    out = []
    pdir = os.path.join(refroot, "patterns")
    for dirpath, _, files in os.walk(pdir):
        for f in sorted(files):
            if not f.endswith(".txt"):
                continue
            with open(os.path.join(dirpath, f)) as fh:
                first = fh.readline()
                m = re.search(r"Nodes:\s*(\d+)", first)
                n = int(m.group(1))
                pairs = set()
                for line in fh:
                    if line.strip():
                        a, b = map(int, line.split())
                        pairs.add(tuple(sorted((a, b))))
            out.append((os.path.relpath(os.path.join(dirpath, f), pdir), n, sorted(pairs)))
    return sorted(out)


def run(args, tmp):
    try:
        return defined_bytes(oracle.reference_preprocess(args, tmp)).hex(), None
    except RuntimeError as e:
        return None, str(e).strip().splitlines()[-1]


def main():
    if len(sys.argv) != 2 or not os.path.isdir(os.path.join(sys.argv[1], "src")):
        raise SystemExit("usage: make_golden.py <reference tree> (the directory holding src/ and patterns/)")
    refroot = sys.argv[1]
    oracle.build(os.path.join(refroot, "src"))
    cases = []
    with tempfile.TemporaryDirectory() as tmp:
        for rel, n, pairs in corpus(refroot):
            args = [n] + [x for p in pairs for x in p]
            mo, err = run(args, tmp)
            cases.append({"kind": "corpus", "name": rel, "n": n, "edges": pairs, "mo": mo, "error": err})
        for k in range(31):
            mo, err = run([k], tmp)
            cases.append({"kind": "predefined", "name": str(k), "number": k, "mo": mo, "error": err})
        for name, (n, edges) in WORKLOAD.items():
            args = [n] + [x for e in edges for x in e]
            mo, err = run(args, tmp)
            cases.append({"kind": "workload", "name": name, "n": n, "edges": edges, "mo": mo, "error": err})
        # inputs the reference rejects: a core of more than six vertices (a
        # 14-cycle), a disconnected pattern, out-of-range vertex ids
        rejects = {
            "cycle14": [14] + [x for i in range(14) for x in (i, (i + 1) % 14)],
            "disconnected": [4, 0, 1, 2, 3],
            "bad_id": [3, 0, 1, 1, 5],
            "too_many_nodes": [33, 0, 1],
        }
        for name, args in rejects.items():
            mo, err = run(args, tmp)
            n = args[0]
            edges = [(args[i], args[i + 1]) for i in range(1, len(args) - 1, 2)]
            cases.append({"kind": "reject", "name": name, "n": n, "edges": edges, "mo": mo, "error": err})
        rng = random.Random(20251203)
        for i in range(400):
            core, n, edges = random_pattern(rng)
            args = [n] + [x for e in edges for x in e]
            mo, err = run(args, tmp)
            cases.append({"kind": "random", "name": f"r{i}-{core}", "n": n, "edges": edges, "mo": mo, "error": err})
    with open(os.path.join(HERE, "matching_orders.json"), "w") as f:
        json.dump({"generator": "reference fringePreprocess (oracle/_ref)", "cases": cases}, f, indent=0)
    print(len(cases), "cases;", sum(c["error"] is not None for c in cases), "rejected")


if __name__ == "__main__":
    main()
