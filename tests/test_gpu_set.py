"""Many patterns on one graph in shared passes (fsgc_count_set) against one
fsgc_count per pattern: every result (count, raw u64 total, divisor, core
type) must be identical, on the first call (direct launches), the second
(captured into a CUDA graph) and the third (replayed).  The sets are large
enough to split into several shared passes per core family."""
import pytest

import fsgc
from helpers import EXTRA, WORKLOAD, golden_cases
from test_gpu_parity import graph

pytestmark = pytest.mark.gpu


def pattern_set():
    pats = [fsgc.preprocess(n, e) for n, e in {**WORKLOAD, **EXTRA}.values()]
    pats += [fsgc.preprocess_predefined(k) for k in range(1, 31)]
    pats += [fsgc.MatchingOrder.from_bytes(bytes.fromhex(c["mo"])) for c in golden_cases("random")
             if c["mo"] is not None][:80]
    return pats


@pytest.mark.parametrize("gname", ["er300", "rmat10", "cl2000", "hub3000"])
def test_count_set_equals_single_counts(ctx, gname):
    g = graph(gname)
    gid = ctx.upload(g)
    try:
        pats = [mo for mo in pattern_set() if gname == "er300" or mo.nodes <= 3]
        fam = {}
        for mo in pats:
            fam[mo.nodes] = fam.get(mo.nodes, 0) + 1
        assert fam.get(2, 0) > 8 and fam.get(3, 0) > 8  # several shared passes per family
        want = [ctx.count(gid, mo) for mo in pats]
        for call in range(3):  # direct, captured, replayed
            got = ctx.count_set(gid, pats)
            for i, (a, b) in enumerate(zip(got, want)):
                assert (a.count, a.raw_total, a.automorphisms, a.core_type, a.flags) == \
                       (b.count, b.raw_total, b.automorphisms, b.core_type, b.flags), (gname, call, i)
    finally:
        ctx.release(gid)


def test_count_set_after_arena_growth_recaptures(ctx):
    """A captured set whose work arena was reallocated by another count is
    captured again instead of replaying stale pointers."""
    small = fsgc.gen_rmat(9, 8, seed=3)
    big = fsgc.gen_rmat(12, 16, seed=4)
    gs, gb = ctx.upload(small), ctx.upload(big)
    try:
        pats = [fsgc.preprocess(*WORKLOAD[n]) for n in ("wedge_1_on_each_end", "4clique_3_distinct",
                                                         "4cycle_opposite", "edge_5_5")]
        want = [ctx.count(gs, mo) for mo in pats]
        for _ in range(2):
            ctx.count_set(gs, pats)
        ctx.count(gb, pats[1])  # grows the triangle bitmap arena
        got = ctx.count_set(gs, pats)
        assert [(r.count, r.raw_total) for r in got] == [(r.count, r.raw_total) for r in want]
    finally:
        ctx.release(gs)
        ctx.release(gb)


def test_count_set_rejects_packed_and_unknown(ctx):
    pid = ctx.upload_packed([fsgc.gen_er(50, 100, 1), fsgc.gen_er(60, 120, 2)])
    mo = fsgc.preprocess(3, [(0, 1), (1, 2)])
    try:
        with pytest.raises(fsgc.FsgcError):
            ctx.count_set(pid, [mo])
        with pytest.raises(fsgc.FsgcError):
            ctx.count_set(987654, [mo])
    finally:
        ctx.release(pid)
    gid = ctx.upload(fsgc.gen_er(40, 80, 3))
    try:
        assert ctx.count_set(gid, []) == []
    finally:
        ctx.release(gid)
