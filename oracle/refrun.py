"""Running the reference's own kernels (TEST INFRASTRUCTURE ONLY).

oracle/_ref/fringeCount.cubin is the reference's src/fringeCount.cu compiled
for sm_103a from its own sources; oracle/_build/ref_runner performs the host
steps of the reference's occurrences() around those kernels and times each
count the way the reference's `runtime:` line does (src/fringeCount.cu:2317-2321:
wall clock around occurrences(), which includes the automorphism self-count,
the worklist build and the scratch allocation, and excludes reading the graph
and copying it to the GPU).  oracle/_build/graphgen writes the seeded RMAT
graphs as .egr files.

Nothing here loads the product library: the matching orders are the bytes the
reference's own fringePreprocess wrote (tests/golden/matching_orders.json), and
the graphs come from graphgen.  Used by the GPU parity tests, the script that
pins the benchmark's counts, and bench.py's reference arm.
"""
import json
import os
import re
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CUBIN = os.path.join(HERE, "_ref", "fringeCount.cubin")
RUNNER = os.path.join(HERE, "_build", "ref_runner")
GRAPHGEN = os.path.join(HERE, "_build", "graphgen")
GOLDEN_MO = os.path.join(ROOT, "tests", "golden", "matching_orders.json")

LINE = re.compile(r"core=(\d+) aut=(\d+) raw=(\d+) count=(\d+) ms=([\d.]+)")


def available():
    """True where the reference's kernels can run: the cubin was compiled (it
    can only be compiled where the reference sources are) and travelled here."""
    return os.path.exists(CUBIN)


def ensure_tools():
    if not (os.path.exists(RUNNER) and os.path.exists(GRAPHGEN)):
        subprocess.run(["make", "-s", "-C", HERE], check=True)


def workload_matching_orders(names=None):
    """{name: 139 bytes} of the workload patterns, as the reference's
    fringePreprocess wrote them."""
    with open(GOLDEN_MO) as f:
        cases = json.load(f)["cases"]
    out = {c["name"]: bytes.fromhex(c["mo"]) for c in cases if c["kind"] == "workload"}
    if names is not None:
        out = {n: out[n] for n in names}
    return out


def write_rmat_egr(path, scale, edge_factor, a, b, c, seed):
    ensure_tools()
    subprocess.run([GRAPHGEN, "rmat", str(scale), str(edge_factor), repr(float(a)), repr(float(b)),
                    repr(float(c)), str(int(seed)), path], check=True)


def egr_header(path):
    """(n, m) of an .egr file."""
    with open(path, "rb") as f:
        h = f.read(8)
    return int.from_bytes(h[:4], "little", signed=True), int.from_bytes(h[4:], "little", signed=True)


def write_mo_files(mos, directory):
    paths = []
    for i, (name, b) in enumerate(mos.items()):
        p = os.path.join(directory, f"{i:03d}.mo")
        with open(p, "wb") as f:
            f.write(b)
        paths.append(p)
    return paths


def parse(stdout):
    out = []
    for line in stdout.splitlines():
        m = LINE.match(line)
        if m:
            out.append({k: (float(v) if k == "ms" else int(v))
                        for k, v in zip(("core", "aut", "raw", "count", "ms"), m.groups())})
    return out


def run(egr, mo_paths, timeout=None):
    """Count every matching order on the graph with the reference's kernels, in
    one process (each count starts from the original graph and zeroed device
    state, as a fresh fringeCount process would).  Returns one dict per order:
    core, aut, raw, count, ms."""
    ensure_tools()
    r = subprocess.run([RUNNER, CUBIN, egr, *mo_paths], capture_output=True, text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError(f"ref_runner failed ({r.returncode}): {r.stderr.strip()[-400:]}")
    out = parse(r.stdout)
    if len(out) != len(mo_paths):
        raise RuntimeError(f"ref_runner printed {len(out)} results for {len(mo_paths)} orders")
    return out
