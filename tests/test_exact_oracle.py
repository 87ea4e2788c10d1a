"""Exact (128-bit, saturating) counting in the oracle: binomials against
Python's integers, counts against the brute-force enumerator on small graphs,
and on hub graphs -- where the reference's u64 arithmetic wraps -- against
closed forms computed with Python's integers."""
import math

import pytest

import fsgc
import oracle
from helpers import EXTRA, WORKLOAD, complete_graph, star_graph

U128_MAX = (1 << 128) - 1


@pytest.mark.parametrize("n,k", [(0, 0), (5, 0), (5, 5), (5, 6), (-3, 2), (7, -1), (40, 20), (162739, 6),
                                 (162739, 7), (162739, 8), (200000, 12), (1000000, 31), (3000, 300), (2000, 13)])
def test_nck_exact_matches_python(n, k):
    v, sat = oracle.nck_exact(n, k)
    want = math.comb(n, k) if 0 <= k <= n else 0
    if want >= U128_MAX:
        assert sat
    else:
        assert not sat and v == want


SMALL = {
    "er40": lambda: fsgc.gen_er(40, 120, 3),
    "k7": lambda: complete_graph(7),
    "rmat6": lambda: fsgc.gen_rmat(6, 4, seed=2),
}


@pytest.mark.parametrize("gname", sorted(SMALL))
def test_exact_matches_bruteforce_and_compat(gname):
    g = SMALL[gname]()
    for name, (n, edges) in {**WORKLOAD, **EXTRA}.items():
        mo = fsgc.preprocess(n, edges).to_bytes()
        x = oracle.count_exact(g.nindex, g.nlist, mo)
        c = oracle.count(g.nindex, g.nlist, mo, exact_placements=True)
        assert not x["saturated"]
        # small graphs: nothing wraps, so the exact count is the compat count
        assert (x["count"], x["raw"], x["aut"], x["core"]) == (c["count"], c["raw"], c["aut"], c["core"]), name
        if n <= 8:
            b, _ = oracle.bruteforce(g.nindex, g.nlist, n, edges)
            assert x["count"] == b, (gname, name)


def test_exact_closed_forms_where_u64_wraps():
    # a star with 2300 leaves plus a few extra edges: C(2300, k) passes 2^64 for k >= 8
    L = 2300
    g = star_graph(L)
    d = g.degrees()
    for k in (3, 6, 8, 10, 12):
        mo = fsgc.preprocess(k + 1, [(0, i) for i in range(1, k + 1)]).to_bytes()
        x = oracle.count_exact(g.nindex, g.nlist, mo)
        want = sum(math.comb(int(dv), k) for dv in d)
        assert x["count"] == want and not x["saturated"], k
        c = oracle.count(g.nindex, g.nlist, mo)
        assert c["count"] == (want if want < 1 << 64 else c["count"])  # compat only agrees below 2^64
        if want >= 1 << 64:
            assert c["raw"] != want
    # two joined hubs: vertex 0 has L-2 private leaves, vertex 1 has L; an edge
    # with f fringes on each end occurs C(L-2, f) * C(L, f) times
    g2 = fsgc.csr_from_edges(2 * L, [(0, 1)] + [(0, i) for i in range(2, L)] + [(1, i) for i in range(L, 2 * L)])
    for f, saturates in ((4, False), (8, True)):
        edges = [(0, 1)] + [(0, i) for i in range(2, 2 + f)] + [(1, i) for i in range(2 + f, 2 + 2 * f)]
        x = oracle.count_exact(g2.nindex, g2.nlist, fsgc.preprocess(2 + 2 * f, edges).to_bytes())
        want = math.comb(L - 2, f) * math.comb(L, f)
        assert (want >= U128_MAX) == saturates
        assert x["saturated"] if saturates else (x["count"] == want and not x["saturated"]), f


def test_exact_matches_bruteforce_on_random_and_predefined_patterns():
    from helpers import golden_cases
    g = fsgc.gen_er(30, 90, 11)
    cases = [(f"pre{k}", fsgc.predefined_pattern(k)) for k in range(31)]
    cases += [(c["name"], (c["n"], [tuple(e) for e in c["edges"]])) for c in golden_cases("random")
              if c["mo"] is not None and c["n"] <= 8][:40]
    checked = 0
    for name, (n, edges) in cases:
        if n > 8:
            continue
        mo = fsgc.preprocess(n, edges).to_bytes()
        x = oracle.count_exact(g.nindex, g.nlist, mo)
        b, _ = oracle.bruteforce(g.nindex, g.nlist, n, edges)
        assert x["count"] == b and not x["saturated"], name
        checked += 1
    assert checked >= 30
