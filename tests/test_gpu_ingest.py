"""Edge-list ingestion on the GPU (fsgc_graph_from_edges) against the host's
fsgc_csr_from_edges: the same cleaned CSR (loops dropped, duplicates merged,
symmetric, sorted), byte for byte, for host and device pair arrays; an id
outside [0, n) is refused; counts on the ingested graph equal counts on the
uploaded one."""
import numpy as np
import pytest

import fsgc
from helpers import WORKLOAD

pytestmark = pytest.mark.gpu


def messy_pairs(n, E, seed):
    rng = np.random.default_rng(seed)
    a = rng.integers(0, n, E)
    b = (a + rng.integers(-50, 50, E)) % n  # local, with duplicates and loops
    pairs = np.stack([a, b], 1).astype(np.int32)
    pairs[: E // 50, 1] = pairs[: E // 50, 0]  # explicit loops
    pairs = np.concatenate([pairs, pairs[::7, ::-1], pairs[::11]])  # reversed and repeated copies
    return pairs


@pytest.mark.parametrize("n,E,seed", [(1, 0, 1), (10, 30, 2), (5000, 80000, 3), (200000, 3000000, 4)])
def test_ingested_csr_equals_host_cleaning(ctx, n, E, seed):
    pairs = messy_pairs(n, E, seed) if E else np.zeros((0, 2), np.int32)
    want = fsgc.csr_from_edges(n, pairs)
    gid = ctx.upload_edges(n, pairs)
    try:
        got = ctx.download(gid)
        assert got.n == want.n and got.m == want.m
        assert np.array_equal(got.nindex, want.nindex) and np.array_equal(got.nlist, want.nlist)
    finally:
        ctx.release(gid)


def test_ingest_from_device_pairs_and_counts(ctx):
    torch = pytest.importorskip("torch")
    g = fsgc.gen_rmat(12, 16, seed=6)
    # one direction of every edge plus duplicates, from device memory
    src = np.repeat(np.arange(g.n), np.diff(g.nindex))
    pairs = np.stack([src, g.nlist], 1).astype(np.int32)
    pairs = pairs[pairs[:, 0] < pairs[:, 1]]
    pairs = np.concatenate([pairs, pairs[::3]])
    d = torch.from_numpy(pairs.copy()).cuda()
    torch.cuda.synchronize()
    gid = ctx.upload_edges(g.n, (d.data_ptr(), len(pairs)), on_device=True)
    ref = ctx.upload(g)
    try:
        got = ctx.download(gid)
        assert np.array_equal(got.nindex, g.nindex) and np.array_equal(got.nlist, g.nlist)
        for name in ("wedge_1_on_each_end", "4clique_3_distinct", "edge_5_5"):
            mo = fsgc.preprocess(*WORKLOAD[name])
            a, b = ctx.count(gid, mo), ctx.count(ref, mo)
            assert (a.count, a.raw_total) == (b.count, b.raw_total), name
    finally:
        ctx.release(gid)
        ctx.release(ref)


def test_ingest_refuses_out_of_range_ids(ctx):
    with pytest.raises(fsgc.FsgcError):
        ctx.upload_edges(10, [(0, 1), (2, 10)])
    with pytest.raises(fsgc.FsgcError):
        ctx.upload_edges(10, [(0, 1), (-1, 3)])
