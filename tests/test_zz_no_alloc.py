"""The allocation-free entry point against the regular one.

fsgc_count_wedge_noalloc exists for callers that cannot allocate device memory
while they count; it keeps every intermediate in a fixed array inside the
library.  This file is collected last so that a failure here leaves every other
test already run.  Each check calls the new entry point twice in a row through
the C ABI on the caller's own device arrays and compares both results with
fsgc_count on the same graph: the counts are integers and must be equal.
"""
import numpy as np
import pytest

import fsgc

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

PATTERNS = {
    "5-path": (5, [(0, 1), (0, 2), (1, 3), (2, 4)]),
    "4-cycle + 2 opposite": (6, [(0, 1), (1, 2), (2, 3), (3, 0), (0, 4), (2, 5)]),
    "4-cycle": (4, [(0, 2), (0, 3), (1, 2), (1, 3)]),
    "wedge ends 7 + 1": (11, [(0, 1), (0, 2)] + [(1, i) for i in range(3, 10)] + [(2, 10)]),
}


def hub_graph(n=3000, hub=2300, extra=8000, seed=4):
    rng = np.random.default_rng(seed)
    hub_id = n - 1
    pairs = [(hub_id, i) for i in range(hub)]
    pairs += list(zip(rng.integers(0, n, extra).tolist(), rng.integers(0, n, extra).tolist()))
    return fsgc.csr_from_edges(n, pairs)


@pytest.mark.parametrize("graph", ["rmat11", "hub"])
def test_noalloc_matches_regular_entry_point(graph):
    g = fsgc.gen_rmat(11, 8, seed=7) if graph == "rmat11" else hub_graph()
    d_idx = torch.from_numpy(g.nindex).cuda()
    d_adj = torch.from_numpy(g.nlist).cuda()
    torch.cuda.synchronize()
    with fsgc.Context(0) as ctx:
        gid = ctx.upload(g)
        for name, (n, e) in PATTERNS.items():
            mo = fsgc.preprocess(n, e)
            want = ctx.count(gid, mo)
            for call in range(2):
                got = fsgc.count_wedge_noalloc(g.n, g.m, d_idx.data_ptr(), d_adj.data_ptr(), mo)
                assert (got.count, got.raw_total, got.automorphisms, got.core_type) == \
                       (want.count, want.raw_total, want.automorphisms, want.core_type), (graph, name, call)
        ctx.release(gid)
    if graph == "hub":
        assert g.degrees().max() > 2048  # the hub-endpoint pass ran as well


def test_noalloc_allocates_nothing_and_runs_on_the_callers_stream():
    """After one warm-up call, a second call leaves the device's free memory
    unchanged; the count is the same on a non-default stream."""
    g = fsgc.gen_rmat(11, 8, seed=7)
    d_idx = torch.from_numpy(g.nindex).cuda()
    d_adj = torch.from_numpy(g.nlist).cuda()
    mo = fsgc.preprocess(*PATTERNS["5-path"])
    torch.cuda.synchronize()
    first = fsgc.count_wedge_noalloc(g.n, g.m, d_idx.data_ptr(), d_adj.data_ptr(), mo)
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    again = fsgc.count_wedge_noalloc(g.n, g.m, d_idx.data_ptr(), d_adj.data_ptr(), mo)
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        on_side = fsgc.count_wedge_noalloc(g.n, g.m, d_idx.data_ptr(), d_adj.data_ptr(), mo,
                                           stream=side.cuda_stream)
    side.synchronize()
    assert (first.count, first.raw_total) == (again.count, again.raw_total) == (on_side.count, on_side.raw_total)


def test_noalloc_rejects_other_shapes():
    g = fsgc.gen_rmat(8, 4, seed=1)
    d_idx = torch.from_numpy(g.nindex).cuda()
    d_adj = torch.from_numpy(g.nlist).cuda()
    tri = fsgc.preprocess(3, [(0, 1), (1, 2), (0, 2)])
    with pytest.raises(fsgc.FsgcError):
        fsgc.count_wedge_noalloc(g.n, g.m, d_idx.data_ptr(), d_adj.data_ptr(), tri)
    centre = fsgc.preprocess(6, [(0, 1), (0, 2), (0, 3), (1, 4), (2, 5)])  # fringe on the centre
    with pytest.raises(fsgc.FsgcError):
        fsgc.count_wedge_noalloc(g.n, g.m, d_idx.data_ptr(), d_adj.data_ptr(), centre)
    # malformed orders the regular entry point refuses: core vertex B not joined
    # to A (list[0] == 0), and C joined to a vertex that does not precede it
    wedge = fsgc.preprocess(5, [(0, 1), (0, 2), (1, 3), (2, 4)])
    for pos, val in [(8, 0), (9, 4), (9, 0)]:
        b = bytearray(wedge.to_bytes())
        b[pos] = val
        bad = fsgc.MatchingOrder.from_bytes(bytes(b))
        with pytest.raises(fsgc.FsgcError):
            fsgc.count_wedge_noalloc(g.n, g.m, d_idx.data_ptr(), d_adj.data_ptr(), bad)
