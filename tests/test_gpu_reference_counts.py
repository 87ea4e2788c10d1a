"""fsgc against counts recorded from the reference's own kernels.

tests/golden/reference_rmat<scale>.json hold, per benchmark pattern, the count,
raw u64 total, divisor and core type that the reference's kernels (its
src/fringeCount.cu compiled for sm_103a, run by oracle/ref_runner) produced on
a GB300 for the benchmark's seeded RMAT graph at that scale; the script that
wrote them is tests/golden/make_reference_counts.py.  These tests need no
reference build, so they run wherever a GPU is."""
import os
import re

import pytest

import fsgc
from helpers import WORKLOAD

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _golden_scales():
    import glob
    out = []
    for p in sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "reference_rmat*.json"))):
        out.append(int(re.search(r"rmat(\d+)", p).group(1)))
    return out


@pytest.mark.parametrize("scale", _golden_scales())
def test_bench_patterns_match_recorded_reference_counts(ctx, scale):
    """The benchmark graph's counts recorded from the reference's own kernels
    on a GB300 (tests/golden/reference_rmat<scale>.json, written by
    tests/golden/make_reference_counts.py): fsgc must reproduce each
    pattern's count, raw u64 total, divisor and core type, up to the benchmark's
    own scale, where the reference's run takes minutes per pattern."""
    import json
    with open(os.path.join(ROOT, "tests", "golden", f"reference_rmat{scale}.json")) as f:
        rec = json.load(f)
    gr = rec["graph"]
    g = fsgc.gen_rmat(scale, gr["edge_factor"], gr["a"], gr["b"], gr["c"], gr["seed"])
    assert (g.n, g.m) == (gr["n"], gr["m_directed"])
    gid = ctx.upload(g)
    try:
        for name, r in rec["patterns"].items():
            mo = fsgc.MatchingOrder.from_bytes(bytes.fromhex(r["mo"]))
            assert mo.to_bytes() == fsgc.preprocess(*WORKLOAD[name]).to_bytes()
            got = ctx.count(gid, mo)
            assert (got.count, got.raw_total, got.automorphisms, got.core_type) == \
                   (int(r["count"]), int(r["raw"]), r["aut"], r["core"]), (scale, name)
    finally:
        ctx.release(gid)
