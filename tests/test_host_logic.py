"""Host-side logic that needs no GPU: the exact 128-bit arithmetic of the
counting kernels (the same host/device code), argument checks of the lane,
server and exact-count entry points, and the seeded workload generators and
traffic record used by bench.py."""
import ctypes as C
import math
import os
import random
import sys

import pytest

import fsgc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
M128 = (1 << 128) - 1


def x128(op, a=0, b=0, n=0, k=0):
    L = fsgc.lib()
    L.fsgc_x128_host.restype = None
    L.fsgc_x128_host.argtypes = [C.c_int] + [C.c_ulonglong] * 4 + [C.c_int, C.c_int, C.POINTER(C.c_ulonglong)]
    out = (C.c_ulonglong * 3)()
    L.fsgc_x128_host(op, a & (2**64 - 1), a >> 64, b & (2**64 - 1), b >> 64, n, k, out)
    return out[0] | (out[1] << 64), bool(out[2])


def test_x128_add_mul_saturate_like_python():
    rng = random.Random(5)
    cases = [(0, 0), (1, M128 - 1), (M128 - 1, 1), (2**64 - 1, 1), (2**127, 2**127), (3, 2**126)]
    for _ in range(3000):
        bits_a, bits_b = rng.choice([8, 40, 64, 65, 100, 127, 128]), rng.choice([8, 40, 64, 65, 100, 127, 128])
        cases.append((rng.getrandbits(bits_a), rng.getrandbits(bits_b)))
    for a, b in cases:
        if a == M128 or b == M128:
            continue  # the saturated value itself
        v, sat = x128(0, a, b)
        assert (sat, v) == ((True, M128) if a + b >= M128 else (False, a + b)), (a, b)
        v, sat = x128(1, a, b)
        want = a * b
        if a == 0 or b == 0:
            assert (v, sat) == (0, False)
        else:
            assert (sat, v) == ((True, M128) if want >= M128 else (False, want)), (a, b)


def test_x128_binomial_like_python():
    for n, k in [(0, 0), (10, 3), (10, 11), (-4, 2), (9, -1), (162739, 6), (162739, 8), (200000, 12),
                 (4000, 20), (3000, 300), (67, 33), (130, 65), (2**31 - 1, 4), (2**31 - 1, 5)]:
        v, sat = x128(2, n=n, k=k)
        want = math.comb(n, k) if 0 <= k <= n else 0
        assert (sat, v) == ((True, M128) if want >= M128 else (False, want)), (n, k)


def test_entry_points_reject_null_arguments():
    L = fsgc.lib()
    p = C.c_void_p()
    assert L.fsgc_server_create(None, 1 << 30, 2, 8, C.byref(p)) != 0
    assert L.fsgc_lane_create(None, C.byref(p)) != 0
    assert L.fsgc_lane_submit(None, None, 1) != 0
    assert L.fsgc_lane_wait(None, None) != 0
    assert L.fsgc_lane_wait_task(None, 0, None) != 0
    assert L.fsgc_lane_query(None) != 0
    assert L.fsgc_lane_scratch_bytes(None) == 0
    assert L.fsgc_server_stats_get(None, None) != 0
    assert L.fsgc_server_poll(None, 1, None, None) != 0
    assert L.fsgc_count_exact(None, 1, None, None) != 0
    assert L.fsgc_task_footprint(None, None, None) != 0
    L.fsgc_server_destroy(None)
    L.fsgc_lane_destroy(None)


def test_workload_generators_are_seeded():
    sys.path.insert(0, ROOT)
    import bench
    a = [(n, mo.to_bytes()) for n, mo in bench.draw_patterns(16, 11, max_core=3)]
    b = [(n, mo.to_bytes()) for n, mo in bench.draw_patterns(16, 11, max_core=3)]
    assert a == b and all(mo[0] <= 3 for _, mo in a)
    assert len(bench.draw_patterns(24, 12)) == 24
    g1 = bench.mixed_graphs(3, 3000, 7)
    g2 = bench.mixed_graphs(3, 3000, 7)
    for x, y in zip(g1, g2):
        assert (x.nindex == y.nindex).all() and (x.nlist == y.nlist).all() and 1000 <= x.n <= 3000


def test_traffic_record_only_for_its_own_workload():
    sys.path.insert(0, ROOT)
    import bench

    class G:
        n, m = 4194304, 128312556
    assert bench.measured_traffic("wedge_1_on_each_end", G) == 461885000000
    assert bench.measured_traffic("4cycle_opposite", G) is None
    G.n = 1048576
    assert bench.measured_traffic("wedge_1_on_each_end", G) is None


def test_edges_per_second_is_entries_over_seconds():
    sys.path.insert(0, ROOT)
    import bench
    e = bench.edges_per_second(128312556, {"a": 1000.0, "b": 0.0, "c": 250.0})
    assert e == {"a": 128312556.0, "b": None, "c": 513250224.0}
