"""ctypes front end of the oracle library (TEST INFRASTRUCTURE ONLY).

liboracle.so holds the CPU restatement of the reference's counting path and an
independent brute-force enumerator (see fsgc_oracle.cpp).  Only tests, the
smoke check and bench.py's CPU-baseline legs use it; it is never part of the
product path.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_PREPROCESS = os.path.join(HERE, "_ref", "fringePreprocess")

_lib = None


def build(refsrc=None):
    """Compile the oracle; with `refsrc` (the reference's src/ directory) also
    the reference's own preprocessor and kernels into _ref/."""
    cmd = ["make", "-s", "-C", HERE]
    if refsrc:
        cmd.append("REFSRC=" + refsrc)
    subprocess.run(cmd, check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.oracle_count.restype = C.c_int
        L.oracle_count.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_char_p, C.c_int, C.c_int, C.c_int,
                                   C.POINTER(C.c_ulonglong)]
        L.oracle_set_exact_placements.restype = None
        L.oracle_set_exact_placements.argtypes = [C.c_int]
        L.oracle_nck.restype = C.c_ulonglong
        L.oracle_nck.argtypes = [C.c_int, C.c_int]
        L.oracle_fc3.restype = C.c_ulonglong
        L.oracle_fc3.argtypes = [C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.oracle_rotations.restype = C.c_int
        L.oracle_rotations.argtypes = [C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_int)]
        L.oracle_count_exact.restype = C.c_int
        L.oracle_count_exact.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_char_p, C.c_int,
                                         C.POINTER(C.c_ulonglong)]
        L.oracle_nck_exact.restype = None
        L.oracle_nck_exact.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_ulonglong)]
        L.oracle_bruteforce.restype = C.c_int
        L.oracle_bruteforce.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.c_int), C.c_int,
                                        C.POINTER(C.c_ulonglong)]
        _lib = L
    return _lib


def count(nindex, nlist, mo_bytes, stride=1, phase=0, threads=0, exact_placements=False):
    """Reference-semantics count: dict(count, raw, aut, core).  With
    exact_placements the general core sums the exact number of fringe
    placements instead of following the reference's functionX."""
    lib().oracle_set_exact_placements(1 if exact_placements else 0)
    idx = np.ascontiguousarray(nindex, dtype=np.int64)
    adj = np.ascontiguousarray(nlist, dtype=np.int32)
    if len(adj) == 0:
        adj = np.zeros(1, np.int32)
    out = (C.c_ulonglong * 4)()
    st = lib().oracle_count(len(idx) - 1, idx.ctypes.data, adj.ctypes.data, bytes(mo_bytes), stride, phase,
                            threads, out)
    lib().oracle_set_exact_placements(0)
    if st != 0:
        raise RuntimeError(f"oracle_count failed ({st})")
    return {"count": out[0], "raw": out[1], "aut": out[2], "core": out[3]}


def count_exact(nindex, nlist, mo_bytes, threads=0):
    """Exact count in 128 bits: dict(count, raw, aut, core, too_large, saturated);
    the same per-match formulas in exact arithmetic, exact fringe placements."""
    idx = np.ascontiguousarray(nindex, dtype=np.int64)
    adj = np.ascontiguousarray(nlist, dtype=np.int32)
    if len(adj) == 0:
        adj = np.zeros(1, np.int32)
    out = (C.c_ulonglong * 7)()
    st = lib().oracle_count_exact(len(idx) - 1, idx.ctypes.data, adj.ctypes.data, bytes(mo_bytes), threads, out)
    if st != 0:
        raise RuntimeError(f"oracle_count_exact failed ({st})")
    return {"count": out[0] | (out[1] << 64), "raw": out[2] | (out[3] << 64), "aut": out[4], "core": out[5],
            "too_large": bool(out[6] & 1), "saturated": bool(out[6] & 2)}


def nck_exact(n, k):
    """Exact binomial in 128 bits: (value, saturated)."""
    out = (C.c_ulonglong * 3)()
    lib().oracle_nck_exact(n, k, out)
    return out[0] | (out[1] << 64), bool(out[2])


def bruteforce(nindex, nlist, n_pattern, edges):
    """Exact number of (non-induced) occurrences of the pattern, by enumeration."""
    idx = np.ascontiguousarray(nindex, dtype=np.int64)
    adj = np.ascontiguousarray(nlist, dtype=np.int32)
    if len(adj) == 0:
        adj = np.zeros(1, np.int32)
    pe = (C.c_int * (2 * len(edges) or 1))(*[int(x) for e in edges for x in e])
    out = (C.c_ulonglong * 4)()
    st = lib().oracle_bruteforce(len(idx) - 1, idx.ctypes.data, adj.ctypes.data, n_pattern, pe, len(edges), out)
    if st != 0:
        raise RuntimeError("oracle_bruteforce failed")
    return out[0] | (out[1] << 64), out[2] | (out[3] << 64)


def nck(n, k):
    return lib().oracle_nck(n, k)


def fc3(fr, venn):
    a = (C.c_int * 8)(*fr)
    b = (C.c_int * 8)(*venn)
    return lib().oracle_fc3(a, b)


def reference_preprocess(args, workdir):
    """Run the reference's own fringePreprocess (built by oracle/Makefile) in
    `workdir`; returns the 139 bytes it wrote to motif.mo, or raises."""
    if not os.path.exists(REF_PREPROCESS):
        raise FileNotFoundError(REF_PREPROCESS)
    r = subprocess.run([REF_PREPROCESS, *[str(a) for a in args]], cwd=workdir, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stdout + r.stderr)
    with open(os.path.join(workdir, "motif.mo"), "rb") as f:
        return f.read()
