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


class FakeContext:
    """Stands in for fsgc.Context on the CPU: counts take a fixed device time
    per pattern, and every upload is released again."""

    def __init__(self, *_):
        self.live = set()
        self.next = 1
        self.counted = []

    def __enter__(self):
        return self

    def __exit__(self, *a):
        assert not self.live  # every graph released
        return False

    def upload(self, g):
        gid = self.next
        self.next += 1
        self.live.add(gid)
        return gid

    def prepare(self, gid):
        assert gid in self.live

    def count(self, gid, mo):
        assert gid in self.live
        self.counted.append((gid, mo.nodes))

        class R:
            device_ms = 2.0 * mo.nodes

        return R()

    def release(self, gid):
        self.live.remove(gid)


def test_sweep_rows_are_entries_over_count_seconds(tmp_path, monkeypatch):
    """The sweep's CSV: one row per graph, directed CSR entries divided by each
    pattern's count time, columns in pattern-file order, as the reference's
    harness writes them; run through main() with the GPU context faked."""
    import csv
    pats = tmp_path / "pats"
    pats.mkdir()
    write(pats / "edge_1.txt", "# Nodes: 3 Edges: 4\n0 1\n1 0\n0 2\n2 0\n")
    write(pats / "edge_0.txt", "# Nodes: 2 Edges: 2\n0 1\n1 0\n")
    g1, g2 = fsgc.gen_er(50, 120, 1), fsgc.gen_er(80, 300, 2)
    egr = tmp_path / "g1.egr"
    fsgc.egr_write(str(egr), g1)
    fake = FakeContext()
    monkeypatch.setattr(fsgc, "Context", lambda *a: fake)
    monkeypatch.setattr(sweep, "stand_ins", lambda shrink=1: {"tiny": lambda: g2})
    out = tmp_path / "edge.csv"
    sweep.main(["edge", "--patterns", str(pats), "--graphs", str(egr), "--stand-ins", "tiny", "--out", str(out)])
    rows = list(csv.reader(open(out)))
    names = [p[0] for p in sweep.family_patterns(str(pats), "edge")]
    assert rows[0] == ["Graph File"] + [f"fsgc GB300 {n}" for n in names]
    assert [r[0] for r in rows[1:]] == ["g1", "tiny"]
    nodes = [fsgc.preprocess(n, e).nodes for _, n, e in sweep.family_patterns(str(pats), "edge")]
    for r, g in zip(rows[1:], (g1, g2)):
        for cell, k in zip(r[1:], nodes):
            assert abs(float(cell) - g.m / (2.0 * k / 1000.0)) <= 1e-6 * float(cell)
    assert len(fake.counted) == 2 * len(names)
