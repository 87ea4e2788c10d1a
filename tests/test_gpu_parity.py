"""GPU counts against the oracle, bit for bit (count, raw u64 total, divisor,
core type), through the C ABI.  Graphs are small enough for the oracle to
finish in seconds and include hubs whose degrees make the reference's u64
binomials wrap, so the wrapping arithmetic itself is compared."""
import numpy as np
import pytest

import fsgc
import oracle
from helpers import EXTRA, WORKLOAD, complete_graph, golden_cases, star_graph

pytestmark = pytest.mark.gpu


def hub_graph(n=3000, hub=2000, extra=8000, seed=3, hub_id=0):
    """A star of `hub` leaves around vertex hub_id plus random edges."""
    rng = np.random.default_rng(seed)
    leaves = [x for x in range(n) if x != hub_id][:hub]
    pairs = [(hub_id, i) for i in leaves]
    a = rng.integers(0, n, size=extra)
    b = rng.integers(0, n, size=extra)
    pairs += list(zip(a.tolist(), b.tolist()))
    return fsgc.csr_from_edges(n, pairs)


GRAPHS = {
    "er300": lambda: fsgc.gen_er(300, 2400, 7),
    "rmat10": lambda: fsgc.gen_rmat(10, 8, seed=5),
    "cl2000": lambda: fsgc.gen_chung_lu(2000, 8.0, 2.2, 9),
    "k12": lambda: complete_graph(12),
    "star300": lambda: star_graph(300),
    "hub3000": hub_graph,
}
# General cores (4-6 core vertices) enumerate every ordered core match and every
# fringe placement; on graphs with hubs that takes the oracle (and the
# reference's algorithm) minutes per pattern, so they run on the sparse graphs.
ALL_CORES = {"er300", "k12", "star300"}

RANDOM = [c for c in golden_cases("random") if c["mo"] is not None]
PATTERNS = {**WORKLOAD, **EXTRA}
PATTERNS.update({f"pre{k}": fsgc.predefined_pattern(k) for k in range(1, 31)})


def mos():
    out = [(name, fsgc.preprocess(n, e)) for name, (n, e) in PATTERNS.items()]
    out += [(c["name"], fsgc.MatchingOrder.from_bytes(bytes.fromhex(c["mo"]))) for c in RANDOM[:60]]
    return out


_cache = {}


def graph(name):
    if name not in _cache:
        _cache[name] = GRAPHS[name]()
    return _cache[name]


def check(ctx, g, gid, name, mo, threads=0):
    r = ctx.count(gid, mo)
    o = oracle.count(g.nindex, g.nlist, mo.to_bytes(), threads=threads)
    got = (r.count, r.raw_total, r.automorphisms, r.core_type)
    want = (o["count"], o["raw"], o["aut"], o["core"])
    assert got == want, (name, got, want)


@pytest.mark.parametrize("gname", list(GRAPHS))
def test_counts_match_oracle(ctx, gname):
    g = graph(gname)
    gid = ctx.upload(g)
    try:
        for name, mo in mos():
            if gname not in ALL_CORES and mo.nodes >= 4:
                continue
            check(ctx, g, gid, name, mo)
    finally:
        ctx.release(gid)


@pytest.mark.parametrize("hub_id", [0, 2999])
def test_wrapping_patterns_on_hub(ctx, hub_id):
    """Many fringes on one anchor: nck(2000, k) wraps for k >= 7.  With the hub
    at the largest id and degree above 2048 the wedge core also runs its
    high-degree endpoint kernel."""
    g = graph("hub3000") if hub_id == 0 else hub_graph(3000, 2100, 8000, 4, hub_id)
    gid = ctx.upload(g)
    try:
        deg = g.degrees()
        assert deg.max() >= 2000
        pats = {
            "star7": (8, [(0, i) for i in range(1, 8)]),
            "star12": (13, [(0, i) for i in range(1, 13)]),
            "edge_8_3": EXTRA["edge_8_3"],
            "edge_7_7": (16, [(0, 1)] + [(0, i) for i in range(2, 9)] + [(1, i) for i in range(9, 16)]),
            "triangle_7_on_one": (10, [(0, 1), (1, 2), (0, 2)] + [(0, i) for i in range(3, 10)]),
            "wedge_ends_7_1": (11, [(0, 1), (0, 2)] + [(1, i) for i in range(3, 10)] + [(2, 10)]),
            "wedge_centre_7": (11, [(0, 1), (0, 2)] + [(0, i) for i in range(3, 10)] + [(1, 10), (2, 10)]),
            "triangle_core_7": (12, [(0, 1), (1, 2), (0, 2)] + [e for i in range(3, 10) for e in ((0, i), (1, i))]
                                + [(1, 10), (2, 10), (0, 11), (2, 11)]),
        }
        for name, (n, e) in pats.items():
            check(ctx, g, gid, name, fsgc.preprocess(n, e))
    finally:
        ctx.release(gid)


def test_exact_placement_mode(ctx):
    """With exact placements, general-core counts equal the oracle's exact mode
    (and so the brute-force count on small graphs)."""
    g = graph("er300")
    gid = ctx.upload(g)
    ctx.set_exact_placements(True)
    try:
        for name, mo in mos():
            if mo.nodes < 4:
                continue
            r = ctx.count(gid, mo)
            o = oracle.count(g.nindex, g.nlist, mo.to_bytes(), exact_placements=True)
            assert (r.count, r.raw_total, r.automorphisms) == (o["count"], o["raw"], o["aut"]), name
    finally:
        ctx.set_exact_placements(False)
        ctx.release(gid)
    small = fsgc.gen_er(14, 40, 9)
    gid = ctx.upload(small)
    ctx.set_exact_placements(True)
    try:
        for name, (n, e) in {**WORKLOAD, **EXTRA}.items():
            if n > 8:
                continue
            mo = fsgc.preprocess(n, e)
            b, _ = oracle.bruteforce(small.nindex, small.nlist, n, e)
            assert ctx.count(gid, mo).count == b, name
    finally:
        ctx.set_exact_placements(False)
        ctx.release(gid)


def test_wedge_chunks_over_large_id_ranges(ctx):
    """Vertex ids beyond 64K and hubs above degree 512/2048: the wedge kernels
    sweep several id chunks per endpoint and read the chunk-boundary table."""
    rng = np.random.default_rng(11)
    n = 100000
    hubs = {99999: 2100, 50000: 1500, 70001: 900}
    pairs = []
    for h, k in hubs.items():
        leaves = rng.choice(n, size=k, replace=False)
        pairs += [(h, int(x)) for x in leaves if x != h]
    pairs += list(zip(rng.integers(0, n, 60000).tolist(), rng.integers(0, n, 60000).tolist()))
    g = fsgc.csr_from_edges(n, pairs)
    gid = ctx.upload(g)
    try:
        for name in ("wedge_1_on_each_end", "4cycle_opposite"):
            check(ctx, g, gid, name, fsgc.preprocess(*WORKLOAD[name]))
        for name in ("edge_8_3", "star_12"):
            check(ctx, g, gid, name, fsgc.preprocess(*EXTRA[name]))
        wedge_ends = fsgc.preprocess(11, [(0, 1), (0, 2)] + [(1, i) for i in range(3, 10)] + [(2, 10)])
        check(ctx, g, gid, "wedge_ends_7_1", wedge_ends)
    finally:
        ctx.release(gid)


def test_batch_equals_single_counts(ctx):
    g = graph("rmat10")
    g2 = graph("er300")
    a, b = ctx.upload(g), ctx.upload(g2)
    try:
        ms = [mo for _, mo in mos()[:40] if mo.nodes <= 3]
        tasks = [(a, mo) for mo in ms] + [(b, mo) for mo in ms]
        res = ctx.count_batch(tasks)
        for (gid, mo), r in zip(tasks, res):
            s = ctx.count(gid, mo)
            assert (r.count, r.raw_total, r.automorphisms) == (s.count, s.raw_total, s.automorphisms)
    finally:
        ctx.release(a)
        ctx.release(b)


def test_edge_cases(ctx):
    tri = fsgc.preprocess(3, [(0, 1), (1, 2), (0, 2)])
    k4p3 = fsgc.preprocess(*WORKLOAD["4clique_3_distinct"])
    # graph without edges, isolated vertices, a single edge
    for g in (fsgc.Graph(np.zeros(6, np.int64), np.zeros(0, np.int32)), fsgc.csr_from_edges(2, [(0, 1)]),
              fsgc.csr_from_edges(50, [(0, 1), (1, 2), (0, 2)])):
        gid = ctx.upload(g)
        for name, (n, e) in {**WORKLOAD, **EXTRA}.items():
            check(ctx, g, gid, name, fsgc.preprocess(n, e))
        r = ctx.count(gid, k4p3)
        assert r.count == 0
        ctx.release(gid)
    # pattern larger than the graph: the reference returns 0 early
    g = complete_graph(5)
    gid = ctx.upload(g)
    r = ctx.count(gid, k4p3)
    assert r.count == 0 and (r.flags & 1)
    assert ctx.count(gid, tri).count == 10
    ctx.release(gid)
    with pytest.raises(fsgc.FsgcError):
        ctx.count(12345, tri)


def test_config1_full_size(ctx):
    """ER n=20,000, m=200,000 with the triangle + 2 single fringes pattern,
    against the oracle and the brute-force enumerator."""
    g = fsgc.gen_er(20000, 200000, seed=1)
    n, e = WORKLOAD["er_triangle_2fringes"]
    mo = fsgc.preprocess(n, e)
    gid = ctx.upload(g)
    try:
        r = ctx.count(gid, mo)
        o = oracle.count(g.nindex, g.nlist, mo.to_bytes())
        assert (r.count, r.raw_total) == (o["count"], o["raw"])
        b, _ = oracle.bruteforce(g.nindex, g.nlist, n, e)
        assert r.count == b
    finally:
        ctx.release(gid)


def test_device_resident_input(ctx):
    torch = pytest.importorskip("torch")
    g = graph("rmat10")
    d_idx = torch.from_numpy(g.nindex).cuda()
    d_adj = torch.from_numpy(g.nlist).cuda()
    torch.cuda.synchronize()
    gid = ctx.upload_device(g.n, g.m, d_idx.data_ptr(), d_adj.data_ptr())
    try:
        mo = fsgc.preprocess(*WORKLOAD["4clique_3_distinct"])
        check(ctx, g, gid, "k4p3", mo)
    finally:
        ctx.release(gid)


def test_cli_drop_in(tmp_path):
    import os
    import re
    import subprocess
    g = graph("rmat10")
    p = str(tmp_path / "g.egr")
    fsgc.egr_write(p, g)
    exe = os.path.dirname(fsgc.LIB_PATH)
    n, e = WORKLOAD["triangle_3_on_one"]
    args = [str(n)] + [str(x) for ed in e for x in ed]
    subprocess.run([os.path.join(exe, "fringePreprocess"), *args], cwd=tmp_path, check=True, capture_output=True)
    r = subprocess.run([os.path.join(exe, "fringeCount"), p, "motif.mo"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert re.search(r"runtime: \d+\.\d{6} s", r.stdout)
    cnt = int(re.search(r"(-?\d+) occurrences", r.stdout).group(1))
    o = oracle.count(g.nindex, g.nlist, (tmp_path / "motif.mo").read_bytes())
    assert cnt % (1 << 64) == o["count"]


GENERAL_HUB = {
    "5cycle": EXTRA["5cycle"],
    "5cycle_chord_fringe": EXTRA["5cycle_chord_fringe"],
    "4cycle_3": (7, [(0, 1), (1, 2), (2, 3), (3, 0), (0, 4), (1, 4), (2, 5), (3, 6), (0, 6)]),
    "diamond_2": (6, [(0, 1), (1, 2), (2, 3), (3, 0), (0, 2), (1, 4), (3, 4), (0, 5), (1, 5), (2, 5)]),
    "4path_ends": (6, [(0, 1), (1, 2), (2, 3), (0, 4), (3, 4), (1, 5)]),
    "6cycle": (6, [(0, 1), (1, 2), (2, 3), (3, 4), (4, 5), (5, 0)]),
}


@pytest.mark.parametrize("hub_id", [0, 1199])
def test_general_cores_on_hub_graph(ctx, hub_id):
    """General cores (4-5 core vertices, few anchor sets) on a graph whose hub
    has degree 600: the hub's list is the longest anchor list of many matches,
    the one the Venn rows never walk, and it sends warps into long candidate
    loops."""
    rng = np.random.default_rng(11)
    leaves = [x for x in range(1200) if x != hub_id][:600]
    pairs = [(hub_id, i) for i in leaves]
    pairs += list(zip(rng.integers(0, 1200, 2400).tolist(), rng.integers(0, 1200, 2400).tolist()))
    g = fsgc.csr_from_edges(1200, pairs)
    assert g.degrees().max() >= 600
    gid = ctx.upload(g)
    try:
        pats = [(name, fsgc.preprocess(n, e)) for name, (n, e) in GENERAL_HUB.items()]
        pats += [(c["name"], fsgc.MatchingOrder.from_bytes(bytes.fromhex(c["mo"]))) for c in RANDOM
                 if bytes.fromhex(c["mo"])[0] >= 4 and bytes.fromhex(c["mo"])[1] <= 3][:12]
        assert sum(mo.nodes >= 4 for _, mo in pats) >= 12
        for name, mo in pats:
            check(ctx, g, gid, name, mo)
    finally:
        ctx.release(gid)
