"""The edges/s sweep's host side: pattern files in the reference's format,
family selection as its harness makes it, and the seeded stand-in graphs."""
import os
import sys

import fsgc

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "fringe-sgc_gb300"))
import sweep  # noqa: E402


def write(path, text):
    with open(path, "w") as f:
        f.write(text)


def test_pattern_files_and_families(tmp_path):
    # both directions listed, as in the reference's files
    write(tmp_path / "edge_1.txt", "# Nodes: 4 Edges: 6\n0 1\n1 0\n0 2\n2 0\n1 3\n3 1\n")
    write(tmp_path / "edge_0.txt", "# Nodes: 2 Edges: 2\n0 1\n1 0\n")
    write(tmp_path / "wedge_1.txt", "# Nodes: 3 Edges: 4\n0 1\n0 2\n1 0\n2 0\n")
    write(tmp_path / "notes.md", "not a pattern")
    assert sweep.read_pattern_file(tmp_path / "edge_1.txt") == (4, [(0, 1), (0, 2), (1, 3)])
    fam = sweep.family_patterns(str(tmp_path), "edge")
    assert [name for name, _, _ in fam] == ["edge_0", "edge_1"]
    # each one decomposes like any other pattern
    for _, n, pairs in fam:
        fsgc.preprocess(n, pairs)


def test_stand_ins_have_the_shapes(tmp_path):
    si = sweep.stand_ins(shrink=64)
    assert len(si) == 8
    for name in ("USA-road-d.NY", "internet", "amazon0601", "delaunay_n22"):
        g = si[name]()
        assert g.n > 1000 and g.m > 0
        assert fsgc.validate(g)[0] == 0  # sorted, duplicate-free, loop-free, symmetric
        d = g.m / g.n
        if name == "delaunay_n22":
            assert 5.5 < d < 6.1  # triangulated grid
        if name == "USA-road-d.NY":
            assert 2.0 < d < 3.2
    a, b = si["internet"](), sweep.stand_ins(shrink=64)["internet"]()
    assert (a.nindex == b.nindex).all() and (a.nlist == b.nlist).all()
