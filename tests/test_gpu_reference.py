"""fsgc against the reference's own kernels on the same GPU.

oracle/_ref/fringeCount.cubin is the reference's src/fringeCount.cu device
code, compiled for sm_103a from its sources; oracle/_build/ref_runner performs
the reference's host steps around it (see oracle/ref_runner.cpp).  For every
(graph, pattern) the count, the raw u64 total, the divisor and the core type
must be identical, including on graphs whose hubs make the reference's u64
binomials wrap.  Skipped where the cubin is not present (it can only be
compiled where the reference sources are)."""
import os
import re
import subprocess

import pytest

import fsgc
from helpers import EXTRA, WORKLOAD, complete_graph, golden_cases, star_graph

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUBIN = os.path.join(ROOT, "oracle", "_ref", "fringeCount.cubin")
RUNNER = os.path.join(ROOT, "oracle", "_build", "ref_runner")

if not os.path.exists(CUBIN):
    pytest.skip("reference cubin not built here", allow_module_level=True)


def run_reference(egr, mo_paths, timeout=900):
    if not os.path.exists(RUNNER):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    r = subprocess.run([RUNNER, CUBIN, egr, *mo_paths], capture_output=True, text=True, timeout=timeout)
    assert r.returncode == 0, r.stderr
    out = []
    for line in r.stdout.splitlines():
        m = re.match(r"core=(\d+) aut=(\d+) raw=(\d+) count=(\d+) ms=([\d.]+)", line)
        out.append({k: (float(v) if k == "ms" else int(v)) for k, v in zip(("core", "aut", "raw", "count", "ms"), m.groups())})
    return out


def hub_graph(n=3000, hub=2000, extra=8000, seed=3):
    import numpy as np
    rng = np.random.default_rng(seed)
    pairs = [(0, i) for i in range(1, hub + 1)]
    pairs += list(zip(rng.integers(0, n, extra).tolist(), rng.integers(0, n, extra).tolist()))
    return fsgc.csr_from_edges(n, pairs)


GRAPHS = {
    "er300": (lambda: fsgc.gen_er(300, 2400, 7), True),
    "k12": (lambda: complete_graph(12), True),
    "star300": (lambda: star_graph(300), True),
    "rmat10": (lambda: fsgc.gen_rmat(10, 8, seed=5), False),
    "hub3000": (hub_graph, False),
    "er20k_config1": (lambda: fsgc.gen_er(20000, 200000, seed=1), False),
}

WRAP = {
    "star12": (13, [(0, i) for i in range(1, 13)]),
    "edge_7_7": (16, [(0, 1)] + [(0, i) for i in range(2, 9)] + [(1, i) for i in range(9, 16)]),
    "triangle_7_on_one": (10, [(0, 1), (1, 2), (0, 2)] + [(0, i) for i in range(3, 10)]),
    "wedge_ends_7_1": (11, [(0, 1), (0, 2)] + [(1, i) for i in range(3, 10)] + [(2, 10)]),
    "triangle_core_7": (12, [(0, 1), (1, 2), (0, 2)] + [e for i in range(3, 10) for e in ((0, i), (1, i))]
                        + [(1, 10), (2, 10), (0, 11), (2, 11)]),
}


def patterns(all_cores):
    pats = [(n_, fsgc.preprocess(n, e)) for n_, (n, e) in {**WORKLOAD, **EXTRA, **WRAP}.items()]
    pats += [(f"pre{k}", fsgc.preprocess_predefined(k)) for k in range(1, 31)]
    pats += [(c["name"], fsgc.MatchingOrder.from_bytes(bytes.fromhex(c["mo"])))
             for c in golden_cases("random") if c["mo"] is not None][:40]
    return [(name, mo) for name, mo in pats if all_cores or mo.nodes <= 3]


@pytest.mark.parametrize("gname", list(GRAPHS))
def test_counts_match_reference_kernels(ctx, gname, tmp_path):
    make, all_cores = GRAPHS[gname]
    g = make()
    egr = str(tmp_path / "g.egr")
    fsgc.egr_write(egr, g)
    pats = patterns(all_cores) if gname != "er20k_config1" else [("config1", fsgc.preprocess(*WORKLOAD["er_triangle_2fringes"]))]
    paths = []
    for i, (_, mo) in enumerate(pats):
        p = str(tmp_path / f"p{i}.mo")
        with open(p, "wb") as f:
            f.write(mo.to_bytes())
        paths.append(p)
    ref = run_reference(egr, paths)
    gid = ctx.upload(g)
    try:
        for (name, mo), r in zip(pats, ref):
            got = ctx.count(gid, mo)
            want_core = r["core"] if r["core"] else got.core_type
            assert (got.count, got.raw_total, got.automorphisms, got.core_type) == \
                   (r["count"], r["raw"], r["aut"], want_core), (gname, name, r)
    finally:
        ctx.release(gid)


@pytest.mark.parametrize("scale", [16, 18])
def test_bench_patterns_match_reference_kernels(ctx, tmp_path, scale):
    """The eight RMAT workload patterns at scales 16 and 18 (n = 65,536 and
    262,144, hubs of degree ~9,700 and ~25,000): fsgc and the reference's
    kernels, run here, agree bit for bit."""
    g = fsgc.gen_rmat(scale, 16, 0.57, 0.19, 0.19, 20251203)
    egr = str(tmp_path / "g.egr")
    fsgc.egr_write(egr, g)
    names = ["wedge_1_on_centre", "wedge_2_on_centre", "wedge_4_on_centre", "wedge_1_on_each_end",
             "triangle_3_on_one", "4cycle_opposite", "4clique_3_distinct", "edge_5_5"]
    mos = [fsgc.preprocess(*WORKLOAD[n]) for n in names]
    paths = []
    for i, mo in enumerate(mos):
        p = str(tmp_path / f"b{i}.mo")
        with open(p, "wb") as f:
            f.write(mo.to_bytes())
        paths.append(p)
    ref = run_reference(egr, paths)
    gid = ctx.upload(g)
    try:
        for name, mo, r in zip(names, mos, ref):
            got = ctx.count(gid, mo)
            assert (got.count, got.raw_total, got.automorphisms, got.core_type) == \
                   (r["count"], r["raw"], r["aut"], r["core"]), name
    finally:
        ctx.release(gid)

