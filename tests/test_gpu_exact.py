"""Exact (128-bit, saturating) counts through the C ABI against the oracle's
exact mode: count, raw total, divisor, core type and saturation, on the parity
graphs -- including hubs where the reference's u64 binomials wrap and the exact
totals pass 2^64 -- and a saturating case."""
import math

import pytest

import fsgc
import oracle
from helpers import EXTRA, WORKLOAD
from test_gpu_parity import ALL_CORES, GRAPHS, RANDOM, graph

pytestmark = pytest.mark.gpu

PATTERNS = {**WORKLOAD, **EXTRA}
PATTERNS.update({f"pre{k}": fsgc.predefined_pattern(k) for k in range(1, 31)})


def mos():
    out = [(name, fsgc.preprocess(n, e)) for name, (n, e) in PATTERNS.items()]
    out += [(c["name"], fsgc.MatchingOrder.from_bytes(bytes.fromhex(c["mo"]))) for c in RANDOM[:30]]
    return out


@pytest.mark.parametrize("gname", list(GRAPHS))
def test_exact_counts_match_oracle(ctx, gname):
    g = graph(gname)
    gid = ctx.upload(g)
    wrapped = 0
    try:
        for name, mo in mos():
            if gname not in ALL_CORES and mo.nodes >= 4:
                continue
            r = ctx.count_exact(gid, mo)
            o = oracle.count_exact(g.nindex, g.nlist, mo.to_bytes())
            got = (r.saturated, r.core_type, bool(r.flags & 1))
            want = (o["saturated"], o["core"], o["too_large"])
            assert got == want, (gname, name, got, want)
            if not o["saturated"] and not o["too_large"]:
                assert (r.count, r.raw_total, r.automorphisms) == (o["count"], o["raw"], o["aut"]), (gname, name)
                wrapped += r.raw_total >= 1 << 64
    finally:
        ctx.release(gid)
    if gname == "hub3000":
        assert wrapped > 0  # the exact totals there pass 2^64


def test_exact_saturates_and_rejects_packed(ctx):
    L = 2300
    g = fsgc.csr_from_edges(2 * L, [(0, 1)] + [(0, i) for i in range(2, L)] + [(1, i) for i in range(L, 2 * L)])
    gid = ctx.upload(g)
    try:
        for f, saturates in ((4, False), (8, True)):
            edges = [(0, 1)] + [(0, i) for i in range(2, 2 + f)] + [(1, i) for i in range(2 + f, 2 + 2 * f)]
            r = ctx.count_exact(gid, fsgc.preprocess(2 + 2 * f, edges))
            assert r.saturated == saturates
            if not saturates:
                assert r.count == math.comb(L - 2, f) * math.comb(L, f)
    finally:
        ctx.release(gid)
    pid = ctx.upload_packed([fsgc.gen_er(50, 100, 1), fsgc.gen_er(60, 120, 2)])
    try:
        with pytest.raises(fsgc.FsgcError):
            ctx.count_exact(pid, fsgc.preprocess(3, [(0, 1), (1, 2)]))
    finally:
        ctx.release(pid)


@pytest.mark.parametrize("scale", [14, 16])
def test_exact_bench_patterns_on_rmat(ctx, scale):
    """The benchmark's eight patterns on its RMAT graph family in exact
    arithmetic against the oracle's exact mode: all eight at scale 14, and at
    scale 16 the five whose oracle run takes seconds (the wedge-pair and
    4-clique ones take it minutes there)."""
    from helpers import CONFIG2
    heavy = {"wedge_1_on_each_end", "4cycle_opposite", "4clique_3_distinct"}
    g = fsgc.gen_rmat(scale, 16, 0.57, 0.19, 0.19, 20251203)
    gid = ctx.upload(g)
    try:
        for name in CONFIG2:
            if scale > 14 and name in heavy:
                continue
            mo = fsgc.preprocess(*WORKLOAD[name])
            r = ctx.count_exact(gid, mo)
            o = oracle.count_exact(g.nindex, g.nlist, mo.to_bytes())
            assert (r.saturated, r.core_type) == (o["saturated"], o["core"]), (scale, name)
            if not o["saturated"]:
                assert (r.count, r.raw_total, r.automorphisms) == (o["count"], o["raw"], o["aut"]), (scale, name)
    finally:
        ctx.release(gid)
