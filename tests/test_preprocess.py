"""Pattern decomposition: byte parity with the reference's own fringePreprocess.

The fixtures in tests/golden/matching_orders.json were produced by the
reference CLI itself (tests/golden/make_golden.py): its pattern corpus, its 31
predefined motifs, the workload patterns, 400 seeded random patterns and four
inputs it rejects.
"""
import os
import subprocess

import pytest

import fsgc
from helpers import golden_cases

CASES = golden_cases()


@pytest.mark.parametrize("case", CASES, ids=[f"{c['kind']}:{c['name']}" for c in CASES])
def test_matching_order_bytes(case):
    if case["kind"] == "predefined":
        call = lambda: fsgc.preprocess_predefined(case["number"])  # noqa: E731
    else:
        call = lambda: fsgc.preprocess(case["n"], case["edges"])  # noqa: E731
    if case["mo"] is None:
        with pytest.raises(fsgc.FsgcError):
            call()
        return
    assert call().to_bytes().hex() == case["mo"]


def test_predefined_table_matches_numbers():
    for k in range(31):
        n, edges = fsgc.predefined_pattern(k)
        assert fsgc.preprocess(n, edges).to_bytes() == fsgc.preprocess_predefined(k).to_bytes()


def test_rejects_self_loop_and_bad_arguments():
    with pytest.raises(fsgc.FsgcError):
        fsgc.preprocess(3, [(0, 0), (0, 1), (1, 2)])
    with pytest.raises(fsgc.FsgcError):
        fsgc.preprocess(1, [])
    with pytest.raises(fsgc.FsgcError):
        fsgc.preprocess_predefined(31)


def test_cli_writes_reference_bytes(tmp_path):
    exe = os.path.join(os.path.dirname(fsgc.LIB_PATH), "fringePreprocess")
    case = [c for c in CASES if c["kind"] == "workload" and c["name"] == "edge_5_5"][0]
    args = [str(case["n"])] + [str(x) for e in case["edges"] for x in e]
    r = subprocess.run([exe, *args], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert (tmp_path / "motif.mo").read_bytes().hex() == case["mo"]
    assert (tmp_path / "motif.dot").exists()
    r = subprocess.run([exe, "9"], cwd=tmp_path, capture_output=True, text=True)
    pre = [c for c in CASES if c["kind"] == "predefined" and c["number"] == 9][0]
    assert (tmp_path / "motif.mo").read_bytes().hex() == pre["mo"]
    r = subprocess.run([exe, "14", *[str(x) for i in range(14) for x in (i, (i + 1) % 14)]], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode != 0 and "core" in r.stderr


def _random_connected(rng, n, extra):
    """A random spanning tree on n vertices plus `extra` random edges."""
    edges = set()
    for v in range(1, n):
        u = rng.randrange(v)
        edges.add((u, v))
    for _ in range(extra):
        a, b = rng.randrange(n), rng.randrange(n)
        if a != b:
            edges.add((min(a, b), max(a, b)))
    return sorted(edges)


def test_random_patterns_against_the_reference_decomposer(tmp_path):
    """Where the reference's own fringePreprocess was built from its sources
    (oracle/_ref), 600 more seeded random patterns -- trees, sparse and dense
    graphs of 2-24 vertices, relabelled at random -- decompose to the same
    defined bytes, or are rejected by both."""
    import random
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import oracle
    from make_golden import defined_bytes
    if not os.path.exists(oracle.REF_PREPROCESS):
        pytest.skip("the reference's fringePreprocess is not built here")
    rng = random.Random(20251207)
    checked = rejected = 0
    for i in range(600):
        n = rng.randint(2, 24)
        edges = _random_connected(rng, n, rng.choice([0, 1, 2, n // 2, n, 2 * n]))
        perm = list(range(n))
        rng.shuffle(perm)
        edges = sorted((min(perm[a], perm[b]), max(perm[a], perm[b])) for a, b in edges)
        args = [n] + [x for e in edges for x in e]
        try:
            want = defined_bytes(oracle.reference_preprocess(args, str(tmp_path))).hex()
        except RuntimeError:
            want = None
        if want is None:
            with pytest.raises(fsgc.FsgcError):
                fsgc.preprocess(n, edges)
            rejected += 1
        else:
            assert fsgc.preprocess(n, edges).to_bytes().hex() == want, (i, n, edges)
            checked += 1
    assert checked > 200 and rejected > 0  # dense draws often need a core above six vertices


def test_ten_thousand_mixed_draws_against_the_reference_decomposer(tmp_path):
    """Where the reference's own fringePreprocess is built: 10,000 seeded
    patterns drawn as the mixed-pattern workloads draw them (a core from edge,
    wedge, triangle, 4-path, 4-cycle, diamond, 4-clique, 5-cycle; 0-12 fringe
    vertices, each joined to a uniformly random nonempty subset of the core),
    with the vertex ids shuffled, decompose to the same defined bytes or are
    rejected by both."""
    import concurrent.futures as cf
    import random
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "tests", "golden"))
    sys.path.insert(0, root)
    import oracle
    from bench import CORE_SHAPES
    from make_golden import defined_bytes
    if not os.path.exists(oracle.REF_PREPROCESS):
        pytest.skip("the reference's fringePreprocess is not built here")
    rng = random.Random(20251209)
    shapes = sorted(CORE_SHAPES)
    draws = []
    for _ in range(10000):
        k, core = CORE_SHAPES[rng.choice(shapes)]
        nf = rng.randint(0, 12)
        edges = list(core)
        for i in range(nf):
            sub = rng.randrange(1, 1 << k)
            edges += [(j, k + i) for j in range(k) if sub >> j & 1]
        n = k + nf
        perm = list(range(n))
        rng.shuffle(perm)
        draws.append((n, sorted((min(perm[a], perm[b]), max(perm[a], perm[b])) for a, b in edges)))

    def reference(job):
        worker, chunk = job
        wd = tmp_path / f"w{worker}"
        wd.mkdir()
        out = []
        for n, edges in chunk:
            try:
                out.append(defined_bytes(oracle.reference_preprocess([n] + [x for e in edges for x in e], str(wd))).hex())
            except RuntimeError:
                out.append(None)
        return out

    workers = 8
    jobs = [(w, draws[w::workers]) for w in range(workers)]
    with cf.ThreadPoolExecutor(workers) as ex:
        parts = list(ex.map(reference, jobs))
    want = [None] * len(draws)
    for w, part in enumerate(parts):
        want[w::workers] = part
    checked = rejected = 0
    for i, ((n, edges), ref) in enumerate(zip(draws, want)):
        if ref is None:
            with pytest.raises(fsgc.FsgcError):
                fsgc.preprocess(n, edges)
            rejected += 1
        else:
            assert fsgc.preprocess(n, edges).to_bytes().hex() == ref, (i, n, edges)
            checked += 1
    assert checked + rejected == 10000 and checked > 5000
