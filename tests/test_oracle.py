"""The oracle (CPU restatement of the reference's counting path) pinned against
an independent brute-force enumerator and closed-form counts.  CPU only."""
import math
import random

import pytest

import fsgc
import oracle
from helpers import EXTRA, WORKLOAD, complete_graph, star_graph

MASK = (1 << 64) - 1


def nck_ref_py(n, k):
    """The reference's u64 binomial (src/fringeCount.cu:189-197) in Python."""
    k = min(k, n - k)
    if k < 0:
        return 0
    if k == 0:
        return 1
    r = n
    for i in range(2, k + 1):
        r = ((r * (n + 1 - i)) & MASK) // i
    return r


def small_graphs():
    yield "er12", fsgc.gen_er(12, 30, 3)
    yield "er16", fsgc.gen_er(16, 45, 5)
    yield "rmat5", fsgc.gen_rmat(5, 4, seed=7)
    yield "cl30", fsgc.gen_chung_lu(30, 5.0, 2.3, 11)
    yield "k7", complete_graph(7)


PATTERNS = {**WORKLOAD, **EXTRA}
PATTERNS.update({f"pre{k}": fsgc.predefined_pattern(k) for k in range(1, 31)})


@pytest.mark.parametrize("gname,g", list(small_graphs()), ids=lambda x: x if isinstance(x, str) else "")
def test_oracle_matches_bruteforce(gname, g):
    for name, (n, edges) in PATTERNS.items():
        if n > 8:  # |Aut| by enumeration grows like n! (stars)
            continue
        mo = fsgc.preprocess(n, edges).to_bytes()
        o = oracle.count(g.nindex, g.nlist, mo, exact_placements=True)
        b, _ = oracle.bruteforce(g.nindex, g.nlist, n, edges)
        assert o["count"] == b, (gname, name, o, b)


def test_reference_placements_differ_only_in_general_cores():
    """The reference's functionX leaves a region reduced after backing up from
    a step, so for general cores with several fringes per anchor set it differs
    from the exact placement count; every other core type is unaffected."""
    g = fsgc.gen_er(60, 300, 2)
    from helpers import golden_cases
    differs = 0
    for c in golden_cases("random")[:120]:
        if c["mo"] is None:
            continue
        mo = bytes.fromhex(c["mo"])
        a = oracle.count(g.nindex, g.nlist, mo)
        b = oracle.count(g.nindex, g.nlist, mo, exact_placements=True)
        if mo[0] <= 3:
            assert a == b
        differs += a != b
    assert differs > 0


def test_closed_forms():
    k9 = complete_graph(9)
    tri = fsgc.preprocess(3, [(0, 1), (1, 2), (0, 2)]).to_bytes()
    assert oracle.count(k9.nindex, k9.nlist, tri)["count"] == math.comb(9, 3)
    k4 = fsgc.preprocess(4, [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]).to_bytes()
    assert oracle.count(k9.nindex, k9.nlist, k4)["count"] == math.comb(9, 4)
    st = star_graph(40)
    for k in (2, 3, 5):
        mo = fsgc.preprocess(k + 1, [(0, i) for i in range(1, k + 1)]).to_bytes()
        assert oracle.count(st.nindex, st.nlist, mo)["count"] == math.comb(40, k)
    # bipartite: no odd cycles
    bip = fsgc.csr_from_edges(12, [(i, j) for i in range(6) for j in range(6, 12) if (i + j) % 3])
    c5 = fsgc.preprocess(5, [(0, 1), (1, 2), (2, 3), (3, 4), (4, 0)]).to_bytes()
    assert oracle.count(bip.nindex, bip.nlist, c5)["count"] == 0
    assert oracle.count(bip.nindex, bip.nlist, tri)["count"] == 0


def test_nck_wraps_like_the_reference():
    rng = random.Random(5)
    for _ in range(3000):
        k = rng.randint(0, 31)
        n = rng.choice([rng.randint(-3, 40), rng.randint(0, 5000), rng.randint(0, 200000), rng.randint(0, 2**31 - 1)])
        assert oracle.nck(n, k) == nck_ref_py(n, k)
    # below the wrap thresholds the value is exact
    assert oracle.nck(3000, 6) == math.comb(3000, 6)
    assert oracle.nck(13467, 5) == math.comb(13467, 5)
    assert oracle.nck(13468, 5) != math.comb(13468, 5) % (1 << 64)


def fc3_brute(fr, venn):
    """Exact placements of fringe types into the exclusive regions containing them."""
    regions = [r for r in range(1, 8)]
    types = [t for t in range(1, 8) for _ in range(fr[t])]
    cap = {r: venn[r] for r in regions}

    def rec(i):
        if i == len(types):
            return 1
        t = types[i]
        s = 0
        for r in regions:
            if (r & t) == t and cap[r] > 0:
                c = cap[r]  # choose one of the region's free vertices
                cap[r] -= 1
                s += c * rec(i + 1)
                cap[r] += 1
        return s

    # identical fringes of the same type are interchangeable
    div = 1
    for t in range(1, 8):
        div *= math.factorial(fr[t])
    return rec(0) // div


def test_fc3_counts_placements():
    rng = random.Random(9)
    for _ in range(150):
        fr = [0] + [rng.randint(0, 2) for _ in range(7)]
        if sum(fr) > 5:
            continue
        venn = [0] + [rng.randint(0, 4) for _ in range(7)]
        assert oracle.fc3(fr, venn) == fc3_brute(fr, venn), (fr, venn)


def test_oracle_matches_bruteforce_on_mixed_draws():
    """Patterns drawn as the mixed-pattern workloads draw them (every core
    shape, fringes on random nonempty core subsets), up to 8 vertices so that
    the enumerator stays fast: the oracle's exact-placement count equals brute
    force on small graphs, and its reference-semantics count equals it for
    cores of at most three vertices."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from bench import CORE_SHAPES
    rng = random.Random(20251210)
    graphs = [fsgc.gen_er(14, 40, 21), fsgc.gen_rmat(5, 4, seed=22), fsgc.gen_chung_lu(24, 5.0, 2.3, 23)]
    shapes = sorted(CORE_SHAPES)
    seen = {}
    while len(seen) < 150:
        k, core = CORE_SHAPES[rng.choice(shapes)]
        nf = rng.randint(0, 8 - k)
        edges = list(core)
        for i in range(nf):
            sub = rng.randrange(1, 1 << k)
            edges += [(j, k + i) for j in range(k) if sub >> j & 1]
        try:
            mo = fsgc.preprocess(k + nf, edges).to_bytes()
        except fsgc.FsgcError:
            continue
        seen[mo] = (k + nf, edges)
    cores = set()
    for mo, (n, edges) in seen.items():
        cores.add(mo[0])
        for g in graphs:
            b, _ = oracle.bruteforce(g.nindex, g.nlist, n, edges)
            o = oracle.count(g.nindex, g.nlist, mo, exact_placements=True)
            assert o["count"] == b, (n, edges, o, b)
            if mo[0] <= 3:
                assert oracle.count(g.nindex, g.nlist, mo)["count"] == b, (n, edges)
    assert {1, 2, 3, 4, 5} <= cores  # vertex, edge, three-, four- and five-vertex cores


def test_oracle_reproduces_the_reference_kernels_recorded_counts():
    """tests/golden/reference_rmat16.json holds what the reference's own
    kernels computed on the benchmark's RMAT-16 graph (count, raw total,
    divisor, core type).  The oracle reproduces the five light patterns here;
    the three heavy ones take minutes each on the CPU and are compared on the
    GPU path instead."""
    import json
    import os
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    with open(os.path.join(root, "tests", "golden", "reference_rmat16.json")) as f:
        rec = json.load(f)["patterns"]
    R = bench.RMAT
    g = fsgc.gen_rmat(16, R["edge_factor"], R["a"], R["b"], R["c"], R["seed"])
    heavy = {"wedge_1_on_each_end", "4cycle_opposite", "4clique_3_distinct"}
    checked = 0
    for name, mo in bench.matching_orders():
        if name in heavy:
            continue
        o = oracle.count(g.nindex, g.nlist, mo.to_bytes())
        r = rec[name]
        assert (o["count"], o["raw"], o["aut"], o["core"]) == (int(r["count"]), int(r["raw"]), r["aut"], r["core"]), name
        checked += 1
    assert checked == 5
