"""Lanes and the serving loop: counts submitted on several lanes at once, and
queries submitted concurrently from several threads to a server with
continuous batching, each complete with exactly the count of a direct
fsgc_count (itself checked against the oracle elsewhere) -- the same result
alone and in the mix.  A bad query fails alone; admission refuses queries
larger than the memory budget."""
import ctypes as C
import threading

import pytest

import fsgc
import oracle
from helpers import EXTRA, WORKLOAD

pytestmark = pytest.mark.gpu

GRAPHS = [lambda: fsgc.gen_er(300, 2400, 7), lambda: fsgc.gen_rmat(10, 8, seed=5),
          lambda: fsgc.gen_chung_lu(2000, 8.0, 2.2, 9)]


def test_concurrent_queries_match_direct_counts(ctx):
    graphs = [f() for f in GRAPHS]
    gids = [ctx.upload(g) for g in graphs]
    pats = [fsgc.preprocess(n, e) for n, e in {**WORKLOAD, **EXTRA}.values()]
    pats = [mo for mo in pats if mo.nodes <= 3]
    queries = [(gi, pi) for gi in range(len(gids)) for pi in range(len(pats))] * 2
    direct = {(gi, pi): ctx.count(gids[gi], pats[pi]) for gi in range(len(gids)) for pi in range(len(pats))}
    got = {}
    try:
        with fsgc.Server(ctx, memory_budget=1 << 34, lanes=4, max_batch=16) as srv:
            for gid in gids:
                srv.add_graph(gid)

            def client(part):
                for k in part:
                    gi, pi = queries[k]
                    t = srv.submit(gids[gi], pats[pi])
                    got[k] = srv.wait(t, timeout_s=300)

            threads = [threading.Thread(target=client, args=(range(i, len(queries), 4),)) for i in range(4)]
            for t in threads:
                t.start()
            for t in threads:
                t.join()
            st = srv.stats()
            assert st.completed == len(queries)
            assert 1 <= st.rounds <= len(queries)
            assert st.queued == 0 and st.in_use_bytes <= 1 << 34
            assert 0 < st.p50_ms <= st.p99_ms
        for k, (gi, pi) in enumerate(queries):
            r, lat = got[k]
            d = direct[(gi, pi)]
            assert (r.count, r.raw_total, r.automorphisms, r.core_type) == \
                   (d.count, d.raw_total, d.automorphisms, d.core_type), (gi, pi)
            assert lat > 0
        # one graph checked against the oracle through the served path as well
        for pi, mo in enumerate(pats):
            o = oracle.count(graphs[0].nindex, graphs[0].nlist, bytes(mo))
            assert direct[(0, pi)].count == o["count"]
    finally:
        for gid in gids:
            ctx.release(gid)


def test_bad_query_fails_alone_and_admission_refuses(ctx):
    g = fsgc.gen_er(300, 2400, 7)
    gid = ctx.upload(g)
    good = fsgc.preprocess(3, [(0, 1), (1, 2)])
    # passes the submission checks, fails when counted: a general core (a
    # 4-path) with no anchor set, which the decomposition never produces
    bad = fsgc.MatchingOrder()
    bad.nodes, bad.anchorsets = 4, 0
    bad.list[0], bad.list[1], bad.list[2] = 1, 2, 4
    try:
        with fsgc.Server(ctx, memory_budget=1 << 34, lanes=1, max_batch=8) as srv:
            srv.add_graph(gid)
            with pytest.raises(fsgc.FsgcError):
                srv.submit(gid, fsgc.MatchingOrder())  # nodes == 0: refused at submission
            ts = [srv.submit(gid, good), srv.submit(gid, bad), srv.submit(gid, good)]
            r0, _ = srv.wait(ts[0])
            with pytest.raises(fsgc.FsgcError):
                srv.wait(ts[1])
            r2, _ = srv.wait(ts[2])
            assert r0.count == r2.count == ctx.count(gid, good).count
            # a repeated query is answered from the result cache at submission
            hits = srv.stats().cache_hits
            r3, _ = srv.wait(srv.submit(gid, good))
            assert r3.count == r0.count and srv.stats().cache_hits == hits + 1
            with pytest.raises(fsgc.FsgcError):  # failures are not cached
                srv.wait(srv.submit(gid, bad))
            with pytest.raises(fsgc.FsgcError):
                srv.submit(gid + 1000, good)  # unregistered graph
        # a hub graph whose wedge count needs a hub-cursor arena
        hub = fsgc.csr_from_edges(5000, [(0, i) for i in range(1, 4000)] + [(1, i) for i in range(2, 4000)])
        hid = ctx.upload(hub)
        wedge = fsgc.preprocess(*WORKLOAD["wedge_1_on_each_end"])
        assert ctx.count(hid, wedge).core_type == 3
        need = fsgc.task_footprint(ctx, hid, wedge)
        assert need > 0
        # the registered graph's device bytes count against the budget too
        ctx.prepare_all(hid)
        resident = ctx.info(hid).device_bytes
        with fsgc.Server(ctx, memory_budget=resident + need - 1, lanes=2, max_batch=8) as tiny:
            tiny.add_graph(hid)
            t = C.c_uint64()
            st = fsgc.lib().fsgc_server_submit(tiny.ptr, hid, C.byref(wedge), C.byref(t))
            assert st == 8  # FSGC_EBUSY: footprint above the whole budget
        # a budget for one such query at a time: they queue and all complete
        with fsgc.Server(ctx, memory_budget=resident + need, lanes=3, max_batch=1) as one:
            one.add_graph(hid)
            ts = [one.submit(hid, wedge) for _ in range(6)]
            outs = [one.wait(t, timeout_s=120)[0].count for t in ts]
            assert outs == [ctx.count(hid, wedge).count] * 6
            assert one.stats().in_use_bytes <= resident + need
        # a graph that does not fit beside the registered ones is refused
        with fsgc.Server(ctx, memory_budget=resident - 1, lanes=1, max_batch=1) as small:
            with pytest.raises(fsgc.FsgcError):
                small.add_graph(hid)
        ctx.release(hid)
    finally:
        ctx.release(gid)


def test_lanes_overlap_and_match_batch(ctx):
    # cores of four or more vertices enumerate every core match, which takes
    # minutes on hub graphs: they run on the sparse graphs only
    graphs = [fsgc.gen_rmat(12, 8, seed=1), fsgc.gen_er(2000, 16000, 2), fsgc.gen_er(3000, 9000, 3)]
    gids = [ctx.upload(g) for g in graphs]
    pats = [fsgc.preprocess(n, e) for n, e in {**WORKLOAD, **EXTRA}.values()]
    tasks = [(gid, mo) for gid in gids for mo in pats if gid != gids[0] or mo.nodes <= 3]
    try:
        want = ctx.count_batch(tasks)
        lanes = [fsgc.Lane(ctx) for _ in range(3)]
        parts = [tasks[i::3] for i in range(3)]
        for lane, part in zip(lanes, parts):
            lane.submit(part)
        # lane 1 hands its results out one task at a time, the others all at once
        got = [lanes[0].wait(), [lanes[1].wait_task(i) for i in range(len(parts[1]))], lanes[2].wait()]
        lanes[1].submit(parts[1][:1])  # free again once its last result was taken
        assert lanes[1].wait()[0].count == want[1].count
        for i, part in enumerate(parts):
            assert len(got[i]) == len(part)
            for j, r in enumerate(got[i]):
                w = want[3 * j + i]
                assert (r.count, r.raw_total, r.automorphisms, r.core_type, r.flags) == \
                       (w.count, w.raw_total, w.automorphisms, w.core_type, w.flags)
        # a lane holds one submission at a time
        lanes[0].submit(parts[0][:1])
        with pytest.raises(fsgc.FsgcError):
            lanes[0].submit(parts[0][:1])
        lanes[0].wait()
        for lane in lanes:
            lane.close()
    finally:
        for gid in gids:
            ctx.release(gid)
