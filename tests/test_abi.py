"""C ABI surface and host-side logic of libfsgc (no GPU needed)."""
import os
import random
import re

import numpy as np
import pytest

import fsgc
import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "fsgc.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fsgc_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    L = fsgc.lib()
    names = declared_symbols()
    assert len(names) >= 25
    for name in names:
        assert hasattr(L, name), name


def test_device_binomial_arithmetic_on_host():
    # the magic-number division used on the device, evaluated on the host
    L = fsgc.lib()
    rng = random.Random(1)
    for _ in range(20000):
        d = rng.randint(2, 63)
        x = rng.getrandbits(64) if rng.random() < 0.8 else rng.choice([0, 1, d - 1, d, (1 << 64) - 1, (1 << 63)])
        assert L.fsgc_div_small_host(x, d) == x // d
    for _ in range(5000):
        k = rng.randint(0, 31)
        n = rng.choice([rng.randint(-2, 60), rng.randint(0, 20000), rng.randint(0, 2**31 - 1)])
        assert L.fsgc_nck_host(n, k) == oracle.nck(n, k), (n, k)


def test_generators_are_deterministic_and_valid():
    a = fsgc.gen_rmat(10, 8, seed=3)
    b = fsgc.gen_rmat(10, 8, seed=3)
    assert np.array_equal(a.nindex, b.nindex) and np.array_equal(a.nlist, b.nlist)
    assert fsgc.validate(a)[0] == 0
    er = fsgc.gen_er(2000, 15000, seed=4)
    assert er.m == 30000 and fsgc.validate(er)[0] == 0
    cl = fsgc.gen_chung_lu(3000, 10.0, 2.4, seed=5)
    assert fsgc.validate(cl)[0] == 0
    assert cl.degrees().max() > 5 * cl.degrees().mean()


def test_egr_round_trip_and_errors(tmp_path):
    g = fsgc.gen_er(500, 2000, seed=2)
    p = str(tmp_path / "g.egr")
    fsgc.egr_write(p, g)
    h = fsgc.egr_read(p)
    assert np.array_equal(g.nindex, h.nindex) and np.array_equal(g.nlist, h.nlist)
    raw = open(p, "rb").read()
    # the ECLgraph layout: int32 n, int32 m, nindex[n+1], nlist[m]
    hdr = np.frombuffer(raw[:8], dtype=np.int32)
    assert hdr[0] == 500 and hdr[1] == 4000 and len(raw) == 8 + 4 * 501 + 4 * 4000
    (tmp_path / "t.egr").write_bytes(raw[: len(raw) // 2])
    with pytest.raises(fsgc.FsgcError):
        fsgc.egr_read(str(tmp_path / "t.egr"))
    with pytest.raises(fsgc.FsgcError):
        fsgc.egr_read(str(tmp_path / "missing.egr"))


def test_validate_catches_broken_inputs():
    g = fsgc.csr_from_edges(4, [(0, 1), (1, 2), (2, 3)])
    assert fsgc.validate(g)[0] == 0
    bad = fsgc.Graph(g.nindex.copy(), g.nlist.copy())
    bad.nlist[0] = 0  # self loop on vertex 0
    assert fsgc.validate(bad)[0] != 0
    asym = fsgc.Graph(np.array([0, 1, 1], np.int64), np.array([1], np.int32))
    assert "symmetric" in fsgc.validate(asym)[1]


def test_edges_to_csr_cleans_input():
    g = fsgc.csr_from_edges(5, [(0, 1), (1, 0), (2, 2), (3, 4), (0, 1), (4, 3)])
    assert g.m == 4 and list(g.nlist) == [1, 0, 4, 3]


def test_context_without_gpu_fails_loudly():
    import subprocess
    r = subprocess.run(["nvidia-smi"], capture_output=True) if os.path.exists("/usr/bin/nvidia-smi") else None
    if r is not None and r.returncode == 0:
        pytest.skip("a GPU is present")
    with pytest.raises(fsgc.FsgcError):
        fsgc.Context(0)


def test_struct_layouts_match_the_header():
    import ctypes as C
    # fsgc_matching_order is the reference's 139-byte MatchingOrder; fsgc_task
    # pads to 4-byte alignment (int32 gid first)
    assert C.sizeof(fsgc.MatchingOrder) == 139
    assert C.sizeof(fsgc.Task) == 144
    assert C.sizeof(fsgc.Result) == 40
    assert C.sizeof(fsgc.ServerStats) == 64
    assert C.sizeof(fsgc.ExactResult) == 56


def test_divisor_follows_the_references_int_and_assertion():
    """occurrences() keeps a pattern's count in itself in an int and asserts it
    is positive (src/fringeCount.cu:2230-2232): the divisor is that int, and a
    self-count whose low 32 bits are zero or negative as an int is an error,
    not a large positive divisor."""
    import ctypes as C
    L = fsgc.lib()
    L.fsgc_divisor_from_self_count.restype = C.c_int
    L.fsgc_divisor_from_self_count.argtypes = [C.c_ulonglong, C.POINTER(C.c_ulonglong)]
    out = C.c_ulonglong()
    for raw, want in [(1, 1), (24, 24), (2**31 - 1, 2**31 - 1), ((1 << 32) + 5, 5), ((7 << 40) + 12, 12)]:
        assert L.fsgc_divisor_from_self_count(raw, C.byref(out)) == 0, raw
        assert out.value == want
    for raw in [0, 2**31, 2**32 - 1, (1 << 32) + 2**31 + 3, 1 << 32, 2**64 - 1]:
        assert L.fsgc_divisor_from_self_count(raw, C.byref(out)) == 1, raw  # FSGC_EINVAL
        assert out.value == 0
    assert L.fsgc_divisor_from_self_count(1, None) == 1  # FSGC_EINVAL


def test_standalone_graph_writer_equals_the_product_generator(tmp_path):
    """oracle/graphgen (the reference arm's graph, written without the product
    library) and fsgc_gen_rmat give the same .egr bytes."""
    import refrun
    for scale, ef, seed in [(9, 8, 1), (12, 16, 20251203), (14, 16, 20251203)]:
        a, b = str(tmp_path / "a.egr"), str(tmp_path / "b.egr")
        refrun.write_rmat_egr(a, scale, ef, 0.57, 0.19, 0.19, seed)
        fsgc.egr_write(b, fsgc.gen_rmat(scale, ef, 0.57, 0.19, 0.19, seed))
        assert open(a, "rb").read() == open(b, "rb").read(), (scale, ef, seed)
        assert refrun.egr_header(a)[0] == 1 << scale


def test_reference_arm_matching_orders_are_the_references():
    """The reference arm takes the eight workload patterns' .mo bytes from the
    reference CLI's own output; they equal fsgc_preprocess's."""
    import refrun
    sys_path_bench()
    import bench
    mos = refrun.workload_matching_orders(list(bench.WORKLOAD))
    for name, (n, e) in bench.WORKLOAD.items():
        assert mos[name] == fsgc.preprocess(n, e).to_bytes(), name


def sys_path_bench():
    import sys
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)


def test_egr_int64_extension_round_trip(tmp_path):
    """Graphs of 2^31 or more directed entries are written in the int64
    extension (int32 n, int32 -1, int64 m, int64 offsets, int32 lists); the
    reader takes both layouts and the reference's own reader refuses the
    extension's negative edge count (src/ECLgraph.h:64-66)."""
    g = fsgc.gen_rmat(11, 8, seed=9)
    p64, p32 = str(tmp_path / "g64.egr"), str(tmp_path / "g32.egr")
    fsgc.egr_write(p64, g, int64=True)
    fsgc.egr_write(p32, g)
    raw = open(p64, "rb").read()
    assert int.from_bytes(raw[0:4], "little") == g.n and int.from_bytes(raw[4:8], "little", signed=True) == -1
    assert int.from_bytes(raw[8:16], "little") == g.m
    assert len(raw) == 16 + 8 * (g.n + 1) + 4 * g.m
    for p in (p64, p32):
        h = fsgc.egr_read(p)
        assert np.array_equal(h.nindex, g.nindex) and np.array_equal(h.nlist, g.nlist)
    bad = str(tmp_path / "bad.egr")
    with open(bad, "wb") as f:
        f.write(raw[:40])  # truncated
    with pytest.raises(fsgc.FsgcError):
        fsgc.egr_read(bad)


def test_recorded_reference_counts_are_for_the_bench_graph_and_patterns():
    """tests/golden/reference_rmat<scale>.json: the reference's own kernels'
    counts on the benchmark graph; their graph sizes equal the generator's and
    their matching orders the reference CLI's."""
    import glob
    import json
    import refrun
    files = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "reference_rmat*.json")))
    assert len(files) >= 4
    mos = refrun.workload_matching_orders()
    for p in files:
        rec = json.load(open(p))
        gr = rec["graph"]
        assert len(rec["patterns"]) == 8 and rec["gpu"] and "GB300" in rec["gpu"]
        for name, r in rec["patterns"].items():
            assert bytes.fromhex(r["mo"]) == mos[name], (p, name)
            assert int(r["count"]) == int(r["raw"]) // r["aut"]
        if gr["scale"] <= 18:
            g = fsgc.gen_rmat(gr["scale"], gr["edge_factor"], gr["a"], gr["b"], gr["c"], gr["seed"])
            assert (g.n, g.m) == (gr["n"], gr["m_directed"])
