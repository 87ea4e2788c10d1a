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


def wedge_formula(dx, dy, adj, fx, fxy, fy, c, k01, exact):
    L = fsgc.lib()
    L.fsgc_wedge_formula_host.restype = None
    L.fsgc_wedge_formula_host.argtypes = [C.c_int] * 9 + [C.POINTER(C.c_ulonglong)]
    out = (C.c_ulonglong * 2)()
    L.fsgc_wedge_formula_host(dx, dy, adj, fx, fxy, fy, c, k01, exact, out)
    return out[0] | (out[1] << 64)


def wedge_formula_python(dx, dy, adj, fx, fxy, fy, c):
    """wedge() of the reference (src/fringeCount.cu:1381-1406) in Python
    integers, binomials 0 outside 0 <= k <= n."""
    def comb(n, k):
        return math.comb(n, k) if 0 <= k <= n else 0
    a_xy = c - fxy
    if a_xy < 0:
        return 0
    corr = 2 if adj else 1
    a_x, a_y = dx - (corr + c), dy - (corr + c)
    s = 0
    for j in range(min(fx, a_xy) + 1):
        k = fx - j
        t = comb(a_x, k) * comb(a_xy + a_y - j, fy)
        if fx != fy:
            t += comb(a_y, k) * comb(a_xy + a_x - j, fy)
        s += t * comb(a_xy, j)
    return s * comb(c, fxy)


def test_wedge_formula_k01_form_equals_general_binomials():
    """The kernels evaluate wedge() with two-case binomials when every fringe
    count is 0 or 1; that must give the general form's value bit for bit,
    including where the u64 products wrap and for arguments outside the
    kernels' range (negative Venn sizes)."""
    rng = random.Random(11)
    cases = [(dx, dy, adj, c) for dx in range(0, 9) for dy in range(0, 9) for adj in (0, 1) for c in range(-2, 8)]
    for _ in range(3000):
        big = rng.choice([100, 70000, 2**20, 2**31 - 1])
        c = rng.randrange(0, min(big, 3000))
        cases.append((rng.randrange(c, big), rng.randrange(c, big), rng.randrange(2), c))
    for fx in (0, 1):
        for fxy in (0, 1):
            for fy in (0, 1):
                for dx, dy, adj, c in cases:
                    u = wedge_formula(dx, dy, adj, fx, fxy, fy, c, 0, 0)
                    assert wedge_formula(dx, dy, adj, fx, fxy, fy, c, 1, 0) == u, (dx, dy, adj, fx, fxy, fy, c)
                    x = wedge_formula(dx, dy, adj, fx, fxy, fy, c, 1, 1)
                    assert wedge_formula(dx, dy, adj, fx, fxy, fy, c, 0, 1) == x
                    want = wedge_formula_python(dx, dy, adj, fx, fxy, fy, c)
                    assert x == min(want, M128) and u == want % 2**64, (dx, dy, adj, fx, fxy, fy, c)


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
