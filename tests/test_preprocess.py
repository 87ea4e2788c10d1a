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
