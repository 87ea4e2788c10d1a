"""Batching across graphs: many member graphs packed into one resident CSR and
counted together must give, member by member, exactly the count of that
member alone (count, raw u64 total, divisor, core type, size flag)."""
import numpy as np
import pytest

import fsgc
from helpers import EXTRA, WORKLOAD, complete_graph, golden_cases, star_graph

pytestmark = pytest.mark.gpu


def hub_graph(n=3000, hub=2000, extra=8000, seed=3):
    rng = np.random.default_rng(seed)
    pairs = [(0, i) for i in range(1, hub + 1)]
    pairs += list(zip(rng.integers(0, n, extra).tolist(), rng.integers(0, n, extra).tolist()))
    return fsgc.csr_from_edges(n, pairs)


def patterns(all_cores):
    pats = [(name, fsgc.preprocess(n, e)) for name, (n, e) in {**WORKLOAD, **EXTRA}.items()]
    pats += [(f"pre{k}", fsgc.preprocess_predefined(k)) for k in range(1, 31)]
    pats += [(c["name"], fsgc.MatchingOrder.from_bytes(bytes.fromhex(c["mo"])))
             for c in golden_cases("random") if c["mo"] is not None][:40]
    return [(n, mo) for n, mo in pats if all_cores or mo.nodes <= 3]


SPARSE = [lambda: fsgc.gen_er(300, 2400, 7), lambda: complete_graph(12), lambda: star_graph(300),
          lambda: fsgc.gen_er(40, 80, 3), lambda: fsgc.csr_from_edges(1, []), lambda: complete_graph(5),
          lambda: fsgc.gen_rmat(6, 4, seed=2)]
HUBS = [lambda: fsgc.gen_rmat(10, 8, seed=5), lambda: fsgc.gen_chung_lu(2000, 8.0, 2.2, 9), hub_graph,
        lambda: fsgc.gen_er(20000, 200000, seed=1), lambda: star_graph(50)]


@pytest.mark.parametrize("kind", ["sparse", "hubs"])
def test_packed_counts_equal_single_counts(ctx, kind):
    members = [f() for f in (SPARSE if kind == "sparse" else HUBS)]
    pid = ctx.upload_packed(members)
    gids = [ctx.upload(g) for g in members]
    try:
        for name, mo in patterns(kind == "sparse"):
            packed = ctx.count_packed(pid, mo)
            for i, (gid, r) in enumerate(zip(gids, packed)):
                s = ctx.count(gid, mo)
                assert (r.count, r.raw_total, r.automorphisms, r.core_type, r.flags) == \
                       (s.count, s.raw_total, s.automorphisms, s.core_type, s.flags), (kind, name, i)
    finally:
        ctx.release(pid)
        for gid in gids:
            ctx.release(gid)


def test_packed_rejects_crossing_edges(ctx):
    g = fsgc.csr_from_edges(4, [(0, 1), (1, 2), (2, 3)])
    import ctypes as C
    gid = C.c_int()
    vstart = np.array([0, 2, 4], np.int32)
    st = fsgc.lib().fsgc_graph_from_packed_csr(ctx.ptr, g.n, g.m, g.nindex.ctypes.data, g.nlist.ctypes.data, 2,
                                               vstart.ctypes.data, C.byref(gid))
    assert st != 0
