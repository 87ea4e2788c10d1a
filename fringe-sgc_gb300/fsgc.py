"""ctypes binding of libfsgc (include/fsgc.h) for tests, benchmarks and scripts.

The binding only marshals arguments; all counting happens in the CUDA library.
Loading fails loudly when libfsgc.so has not been built.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfsgc.so")

MO_SIZE = 139
CORE_NAMES = {1: "vertex", 2: "edge", 3: "wedge", 4: "triangle", 5: "general"}


class MatchingOrder(C.Structure):
    _pack_ = 1
    _fields_ = [("nodes", C.c_uint8), ("anchorsets", C.c_uint8), ("startdeg", C.c_uint8),
                ("destdeg", C.c_uint8 * 5), ("list", C.c_uint8 * 5), ("anch", C.c_uint8 * 63),
                ("fcnt", C.c_uint8 * 63)]

    def to_bytes(self):
        return bytes(C.string_at(C.addressof(self), MO_SIZE))

    @classmethod
    def from_bytes(cls, b):
        assert len(b) == MO_SIZE
        mo = cls()
        C.memmove(C.addressof(mo), b, MO_SIZE)
        return mo


assert C.sizeof(MatchingOrder) == MO_SIZE


class Result(C.Structure):
    _fields_ = [("count", C.c_uint64), ("raw_total", C.c_uint64), ("automorphisms", C.c_uint64),
                ("flags", C.c_uint32), ("core_type", C.c_int32), ("device_ms", C.c_double)]


class Task(C.Structure):
    _fields_ = [("gid", C.c_int32), ("mo", MatchingOrder)]


class HostCSR(C.Structure):
    _fields_ = [("n", C.c_int32), ("m", C.c_int64), ("nindex", C.POINTER(C.c_int64)),
                ("nlist", C.POINTER(C.c_int32))]


class GraphInfo(C.Structure):
    _fields_ = [("n", C.c_int32), ("m", C.c_int64), ("max_degree", C.c_int32), ("triangles", C.c_int64),
                ("device_bytes", C.c_int64)]


class ExactResult(C.Structure):
    _fields_ = [("count_lo", C.c_uint64), ("count_hi", C.c_uint64), ("raw_lo", C.c_uint64), ("raw_hi", C.c_uint64),
                ("automorphisms", C.c_uint64), ("flags", C.c_uint32), ("core_type", C.c_int32),
                ("device_ms", C.c_double)]

    @property
    def count(self):
        return self.count_lo | (self.count_hi << 64)

    @property
    def raw_total(self):
        return self.raw_lo | (self.raw_hi << 64)

    @property
    def saturated(self):
        return bool(self.flags & 2)


class ServerStats(C.Structure):
    _fields_ = [("completed", C.c_uint64), ("rounds", C.c_uint64), ("queued", C.c_uint64),
                ("in_use_bytes", C.c_uint64), ("p50_ms", C.c_double), ("p99_ms", C.c_double),
                ("queries_per_s", C.c_double), ("cache_hits", C.c_uint64)]


class FsgcError(RuntimeError):
    pass


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FsgcError(f"libfsgc.so not built at {LIB_PATH}; run fringe-sgc_gb300/build.py")
        L = C.CDLL(LIB_PATH)
        P, I, I64, U64 = C.c_void_p, C.c_int, C.c_int64, C.c_uint64
        sig = {
            "fsgc_preprocess": (I, [I, C.POINTER(C.c_int), I, C.POINTER(MatchingOrder), C.c_char_p, I]),
            "fsgc_preprocess_predefined": (I, [I, C.POINTER(MatchingOrder), C.c_char_p, I]),
            "fsgc_predefined_pattern": (I, [I, C.POINTER(C.c_int), C.POINTER(C.c_int), I, C.POINTER(C.c_int)]),
            "fsgc_predefined_name": (C.c_char_p, [I]),
            "fsgc_egr_read": (I, [C.c_char_p, C.POINTER(HostCSR)]),
            "fsgc_egr_write": (I, [C.c_char_p, C.POINTER(HostCSR)]),
            "fsgc_egr_write64": (I, [C.c_char_p, C.POINTER(HostCSR)]),
            "fsgc_csr_validate": (I, [C.POINTER(HostCSR), C.c_char_p, I]),
            "fsgc_gen_rmat": (I, [I, I, C.c_double, C.c_double, C.c_double, U64, C.POINTER(HostCSR)]),
            "fsgc_gen_er": (I, [I, I64, U64, C.POINTER(HostCSR)]),
            "fsgc_gen_chung_lu": (I, [I, C.c_double, C.c_double, U64, C.POINTER(HostCSR)]),
            "fsgc_csr_from_edges": (I, [I, I64, C.POINTER(C.c_int32), C.POINTER(HostCSR)]),
            "fsgc_host_csr_pin": (I, [C.POINTER(HostCSR)]),
            "fsgc_host_csr_free": (None, [C.POINTER(HostCSR)]),
            "fsgc_ctx_create": (I, [I, C.POINTER(P)]),
            "fsgc_ctx_destroy": (None, [P]),
            "fsgc_ctx_last_error": (C.c_char_p, [P]),
            "fsgc_ctx_stream": (P, [P]),
            "fsgc_ctx_launches": (U64, [P]),
            "fsgc_graph_from_csr": (I, [P, I, I64, P, P, C.POINTER(C.c_int)]),
            "fsgc_graph_from_csr32": (I, [P, I, I, P, P, C.POINTER(C.c_int)]),
            "fsgc_graph_from_device_csr": (I, [P, I, I64, P, P, C.POINTER(C.c_int)]),
            "fsgc_graph_from_edges": (I, [P, I, I64, P, I, C.POINTER(C.c_int)]),
            "fsgc_graph_copy_csr": (I, [P, I, P, P]),
            "fsgc_graph_prepare_all": (I, [P, I]),
            "fsgc_tuning_default": (I, [C.POINTER(Tuning)]),
            "fsgc_ctx_set_tuning": (I, [P, C.POINTER(Tuning)]),
            "fsgc_ctx_get_tuning": (I, [P, C.POINTER(Tuning)]),
            "fsgc_graph_load_egr": (I, [P, C.c_char_p, C.POINTER(C.c_int)]),
            "fsgc_graph_release": (I, [P, I]),
            "fsgc_graph_prepare": (I, [P, I]),
            "fsgc_graph_info_get": (I, [P, I, C.POINTER(GraphInfo)]),
            "fsgc_count": (I, [P, I, C.POINTER(MatchingOrder), C.POINTER(Result)]),
            "fsgc_count_batch": (I, [P, C.POINTER(Task), I, C.POINTER(Result)]),
            "fsgc_count_set": (I, [P, I, C.POINTER(MatchingOrder), I, C.POINTER(Result)]),
            "fsgc_divisor_from_self_count": (I, [C.c_ulonglong, C.POINTER(C.c_ulonglong)]),
            "fsgc_count_exact": (I, [P, I, C.POINTER(MatchingOrder), C.POINTER(ExactResult)]),
            "fsgc_graph_from_packed_csr": (I, [P, I, I64, P, P, I, P, C.POINTER(C.c_int)]),
            "fsgc_count_packed": (I, [P, I, C.POINTER(MatchingOrder), C.POINTER(Result)]),
            "fsgc_ctx_timer_start": (I, [P]),
            "fsgc_ctx_timer_stop": (I, [P, C.POINTER(C.c_double)]),
            "fsgc_ctx_flush_l2": (I, [P, C.c_size_t]),
            "fsgc_ctx_synchronize": (I, [P]),
            "fsgc_ctx_set_exact_placements": (I, [P, I]),
            "fsgc_count_wedge_noalloc": (I, [I, I64, P, P, C.POINTER(MatchingOrder), P, C.POINTER(Result),
                                             C.c_char_p, I]),
            "fsgc_lane_create": (I, [P, C.POINTER(P)]),
            "fsgc_lane_destroy": (None, [P]),
            "fsgc_lane_submit": (I, [P, C.POINTER(Task), I]),
            "fsgc_lane_wait": (I, [P, C.POINTER(Result)]),
            "fsgc_lane_wait_task": (I, [P, I, C.POINTER(Result)]),
            "fsgc_lane_query": (I, [P]),
            "fsgc_lane_scratch_bytes": (C.c_size_t, [P]),
            "fsgc_lane_trim": (I, [P]),
            "fsgc_task_footprint": (I, [P, C.POINTER(Task), C.POINTER(C.c_size_t)]),
            "fsgc_server_create": (I, [P, C.c_size_t, I, I, C.POINTER(P)]),
            "fsgc_server_destroy": (None, [P]),
            "fsgc_server_add_graph": (I, [P, I]),
            "fsgc_server_submit": (I, [P, I, C.POINTER(MatchingOrder), C.POINTER(U64)]),
            "fsgc_server_poll": (I, [P, U64, C.POINTER(Result), C.POINTER(C.c_double)]),
            "fsgc_server_wait": (I, [P, U64, C.c_double, C.POINTER(Result), C.POINTER(C.c_double)]),
            "fsgc_server_stats_get": (I, [P, C.POINTER(ServerStats)]),
            "fsgc_nck_host": (C.c_ulonglong, [I, I]),
            "fsgc_div_small_host": (C.c_ulonglong, [C.c_ulonglong, C.c_uint]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(st, what, ctx=None):
    if st != 0:
        msg = ""
        if ctx is not None:
            msg = lib().fsgc_ctx_last_error(ctx).decode(errors="replace")
        raise FsgcError(f"{what} failed with status {st}: {msg}")


# ----------------------------------------------------------------- patterns
def preprocess(n, edges):
    """Decompose a pattern (n vertices, list of (s, d) edges) into a MatchingOrder."""
    flat = (C.c_int * (2 * len(edges) or 1))(*[int(x) for e in edges for x in e])
    mo = MatchingOrder()
    err = C.create_string_buffer(256)
    st = lib().fsgc_preprocess(int(n), flat, len(edges), C.byref(mo), err, 256)
    if st != 0:
        raise FsgcError(f"preprocess: {err.value.decode()} (status {st})")
    return mo


def preprocess_predefined(number):
    mo = MatchingOrder()
    err = C.create_string_buffer(256)
    st = lib().fsgc_preprocess_predefined(int(number), C.byref(mo), err, 256)
    if st != 0:
        raise FsgcError(f"preprocess_predefined: {err.value.decode()} (status {st})")
    return mo


def predefined_pattern(number):
    n, ne = C.c_int(), C.c_int()
    _check(lib().fsgc_predefined_pattern(number, C.byref(n), None, 0, C.byref(ne)), "predefined_pattern")
    buf = (C.c_int * (2 * ne.value))()
    _check(lib().fsgc_predefined_pattern(number, C.byref(n), buf, ne.value, C.byref(ne)), "predefined_pattern")
    return n.value, [(buf[2 * i], buf[2 * i + 1]) for i in range(ne.value)]


# ----------------------------------------------------------------- host graphs
class Tuning(C.Structure):
    """fsgc_tuning: method thresholds and launch shapes (speed only, never results)."""
    _fields_ = [("wedge_small_max_degree", C.c_int32), ("triangle_walk_ratio", C.c_int32),
                ("triangle_stage_max", C.c_int32), ("general_lane_venn_max", C.c_int32),
                ("general_blocks_per_sm", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}

    @classmethod
    def default(cls):
        t = cls()
        _check(lib().fsgc_tuning_default(C.byref(t)), "tuning_default")
        return t


class Graph:
    """Host CSR as numpy arrays: nindex int64[n+1], nlist int32[m]."""

    def __init__(self, nindex, nlist):
        self.nindex = np.ascontiguousarray(nindex, dtype=np.int64)
        self.nlist = np.ascontiguousarray(nlist, dtype=np.int32)
        self.n = len(self.nindex) - 1
        self.m = int(self.nindex[-1])

    def degrees(self):
        return np.diff(self.nindex)

    def as_host_csr(self):
        h = HostCSR()
        h.n = self.n
        h.m = self.m
        h.nindex = self.nindex.ctypes.data_as(C.POINTER(C.c_int64))
        h.nlist = self.nlist.ctypes.data_as(C.POINTER(C.c_int32))
        return h


def _take(h):
    n, m = h.n, h.m
    idx = np.ctypeslib.as_array(h.nindex, shape=(n + 1,)).copy()
    adj = np.ctypeslib.as_array(h.nlist, shape=(max(m, 1),))[:m].copy() if m > 0 else np.zeros(0, np.int32)
    lib().fsgc_host_csr_free(C.byref(h))
    return Graph(idx, adj)


def gen_rmat(scale, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=1):
    h = HostCSR()
    _check(lib().fsgc_gen_rmat(scale, edge_factor, a, b, c, seed, C.byref(h)), "gen_rmat")
    return _take(h)


def gen_er(n, m, seed=1):
    h = HostCSR()
    _check(lib().fsgc_gen_er(n, m, seed, C.byref(h)), "gen_er")
    return _take(h)


def gen_chung_lu(n, avg_degree, exponent, seed=1):
    h = HostCSR()
    _check(lib().fsgc_gen_chung_lu(n, avg_degree, exponent, seed, C.byref(h)), "gen_chung_lu")
    return _take(h)


def csr_from_edges(n, pairs):
    arr = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).reshape(-1, 2))
    h = HostCSR()
    _check(lib().fsgc_csr_from_edges(n, len(arr), arr.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(h)),
           "csr_from_edges")
    return _take(h)


def egr_read(path):
    h = HostCSR()
    _check(lib().fsgc_egr_read(path.encode(), C.byref(h)), "egr_read")
    return _take(h)


def egr_write(path, g, int64=False):
    """Writes the reference's .egr layout, or its int64 extension when the graph
    needs it (m >= 2^31) or `int64` is set."""
    h = g.as_host_csr()
    fn = lib().fsgc_egr_write64 if int64 else lib().fsgc_egr_write
    _check(fn(path.encode(), C.byref(h)), "egr_write")


def validate(g):
    h = g.as_host_csr()
    err = C.create_string_buffer(256)
    st = lib().fsgc_csr_validate(C.byref(h), err, 256)
    return st, err.value.decode()


# ----------------------------------------------------------------- device
def count_wedge_noalloc(n, m, d_nindex, d_nlist, mo, stream=None):
    """Allocation-free wedge-core count over a caller-owned device CSR
    (fsgc_count_wedge_noalloc); returns a Result."""
    r = Result()
    err = C.create_string_buffer(256)
    st = lib().fsgc_count_wedge_noalloc(n, m, d_nindex, d_nlist, C.byref(mo), stream, C.byref(r), err, 256)
    if st != 0:
        raise FsgcError(f"count_wedge_noalloc failed with status {st}: {err.value.decode()}")
    return r


class Context:
    def __init__(self, device=0):
        self.ptr = C.c_void_p()
        st = lib().fsgc_ctx_create(device, C.byref(self.ptr))
        if st != 0:
            raise FsgcError(f"fsgc_ctx_create failed with status {st} (no usable GB300 device or kernels)")

    def close(self):
        if self.ptr:
            lib().fsgc_ctx_destroy(self.ptr)
            self.ptr = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def launches(self):
        return int(lib().fsgc_ctx_launches(self.ptr))

    @property
    def stream(self):
        return lib().fsgc_ctx_stream(self.ptr)

    def timer_start(self):
        _check(lib().fsgc_ctx_timer_start(self.ptr), "timer_start", self.ptr)

    def timer_stop(self):
        ms = C.c_double()
        _check(lib().fsgc_ctx_timer_stop(self.ptr, C.byref(ms)), "timer_stop", self.ptr)
        return ms.value

    def flush_l2(self, nbytes=0):
        _check(lib().fsgc_ctx_flush_l2(self.ptr, nbytes), "flush_l2", self.ptr)

    def set_exact_placements(self, on):
        _check(lib().fsgc_ctx_set_exact_placements(self.ptr, 1 if on else 0), "set_exact_placements", self.ptr)

    def synchronize(self):
        _check(lib().fsgc_ctx_synchronize(self.ptr), "synchronize", self.ptr)

    def upload(self, g):
        gid = C.c_int()
        _check(lib().fsgc_graph_from_csr(self.ptr, g.n, g.m, g.nindex.ctypes.data, g.nlist.ctypes.data,
                                         C.byref(gid)), "graph_from_csr", self.ptr)
        return gid.value

    def upload_device(self, n, m, d_nindex, d_nlist):
        gid = C.c_int()
        _check(lib().fsgc_graph_from_device_csr(self.ptr, n, m, d_nindex, d_nlist, C.byref(gid)),
               "graph_from_device_csr", self.ptr)
        return gid.value

    def upload_edges(self, n, pairs, on_device=False):
        """Edge-list ingestion on the GPU (fsgc_graph_from_edges): `pairs` is
        an (E, 2) int32 array, or a device pointer to 2E int32 when on_device
        (then pass E as len via a tuple (ptr, E))."""
        gid = C.c_int()
        if on_device:
            ptr, E = pairs
        else:
            arr = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).reshape(-1, 2))
            ptr, E = arr.ctypes.data, len(arr)
        _check(lib().fsgc_graph_from_edges(self.ptr, n, E, ptr, 1 if on_device else 0, C.byref(gid)),
               "graph_from_edges", self.ptr)
        return gid.value

    def download(self, gid):
        """The resident graph's CSR, read back (a Graph)."""
        info = self.info(gid)
        idx = np.zeros(info.n + 1, np.int64)
        adj = np.zeros(max(1, info.m), np.int32)
        _check(lib().fsgc_graph_copy_csr(self.ptr, gid, idx.ctypes.data, adj.ctypes.data), "graph_copy_csr",
               self.ptr)
        return Graph(idx, adj[:info.m])

    def get_tuning(self):
        t = Tuning()
        _check(lib().fsgc_ctx_get_tuning(self.ptr, C.byref(t)), "get_tuning", self.ptr)
        return t

    def set_tuning(self, t=None, **fields):
        """Sets the context's method thresholds: a Tuning, or fields over the current ones."""
        cur = t if t is not None else self.get_tuning()
        for k, v in fields.items():
            setattr(cur, k, int(v))
        _check(lib().fsgc_ctx_set_tuning(self.ptr, C.byref(cur)), "set_tuning", self.ptr)

    def prepare_all(self, gid):
        _check(lib().fsgc_graph_prepare_all(self.ptr, gid), "graph_prepare_all", self.ptr)

    def load_egr(self, path):
        gid = C.c_int()
        _check(lib().fsgc_graph_load_egr(self.ptr, path.encode(), C.byref(gid)), "graph_load_egr", self.ptr)
        return gid.value

    def release(self, gid):
        _check(lib().fsgc_graph_release(self.ptr, gid), "graph_release", self.ptr)

    def prepare(self, gid):
        _check(lib().fsgc_graph_prepare(self.ptr, gid), "graph_prepare", self.ptr)

    def info(self, gid):
        gi = GraphInfo()
        _check(lib().fsgc_graph_info_get(self.ptr, gid, C.byref(gi)), "graph_info", self.ptr)
        return gi

    def count(self, gid, mo):
        r = Result()
        _check(lib().fsgc_count(self.ptr, gid, C.byref(mo), C.byref(r)), "count", self.ptr)
        return r

    def upload_packed(self, graphs):
        """Pack member graphs (list of Graph) into one resident graph; returns (gid, ngraphs)."""
        sizes = np.array([g.n for g in graphs], dtype=np.int64)
        vstart = np.zeros(len(graphs) + 1, dtype=np.int32)
        vstart[1:] = np.cumsum(sizes)
        idx = [np.zeros(1, np.int64)]
        adj = []
        base_e = 0
        for g, v0 in zip(graphs, vstart[:-1]):
            idx.append(g.nindex[1:] + base_e)
            adj.append(g.nlist + v0)
            base_e += g.m
        packed = Graph(np.concatenate(idx), np.concatenate(adj) if adj else np.zeros(0, np.int32))
        gid = C.c_int()
        _check(lib().fsgc_graph_from_packed_csr(self.ptr, packed.n, packed.m, packed.nindex.ctypes.data,
                                                packed.nlist.ctypes.data, len(graphs), vstart.ctypes.data,
                                                C.byref(gid)), "graph_from_packed_csr", self.ptr)
        self._packed_sizes = getattr(self, "_packed_sizes", {})
        self._packed_sizes[gid.value] = len(graphs)
        return gid.value

    def count_exact(self, gid, mo):
        """Exact 128-bit count (ExactResult: .count, .raw_total, .saturated)."""
        r = ExactResult()
        _check(lib().fsgc_count_exact(self.ptr, gid, C.byref(mo), C.byref(r)), "count_exact", self.ptr)
        return r

    def count_packed(self, gid, mo):
        ng = self._packed_sizes[gid]
        res = (Result * ng)()
        _check(lib().fsgc_count_packed(self.ptr, gid, C.byref(mo), res), "count_packed", self.ptr)
        return list(res)

    def count_batch(self, tasks):
        """tasks: list of (gid, MatchingOrder)."""
        arr = (Task * len(tasks))()
        for i, (gid, mo) in enumerate(tasks):
            arr[i].gid = gid
            arr[i].mo = mo
        res = (Result * len(tasks))()
        _check(lib().fsgc_count_batch(self.ptr, arr, len(tasks), res), "count_batch", self.ptr)
        return list(res)

    def count_set(self, gid, mos):
        """Many patterns on one graph in shared passes (fsgc_count_set); the
        second call with the same patterns captures a CUDA graph, later calls
        replay it."""
        arr = (MatchingOrder * len(mos))(*mos)
        res = (Result * len(mos))()
        _check(lib().fsgc_count_set(self.ptr, gid, arr, len(mos), res), "count_set", self.ptr)
        return list(res)


# ----------------------------------------------------------------- lanes, serving
class Lane:
    """Asynchronous counts on their own stream: submit(tasks) returns at once,
    wait() returns the results (as Context.count_batch would)."""

    def __init__(self, ctx):
        self.ctx = ctx
        p = C.c_void_p()
        _check(lib().fsgc_lane_create(ctx.ptr, C.byref(p)), "lane_create", ctx.ptr)
        self.ptr = p
        self.n = 0

    def submit(self, tasks):
        arr = (Task * len(tasks))()
        for i, (gid, mo) in enumerate(tasks):
            arr[i].gid = gid
            arr[i].mo = mo
        _check(lib().fsgc_lane_submit(self.ptr, arr, len(tasks)), "lane_submit", self.ctx.ptr)
        self.n = len(tasks)

    def done(self):
        return lib().fsgc_lane_query(self.ptr) == 0

    def wait_task(self, index):
        r = Result()
        _check(lib().fsgc_lane_wait_task(self.ptr, int(index), C.byref(r)), "lane_wait_task", self.ctx.ptr)
        return r

    def wait(self):
        res = (Result * self.n)()
        _check(lib().fsgc_lane_wait(self.ptr, res), "lane_wait", self.ctx.ptr)
        return list(res)

    def scratch_bytes(self):
        return lib().fsgc_lane_scratch_bytes(self.ptr)

    def close(self):
        if self.ptr:
            lib().fsgc_lane_destroy(self.ptr)
            self.ptr = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def task_footprint(ctx, gid, mo):
    t = Task()
    t.gid = gid
    t.mo = mo
    b = C.c_size_t()
    _check(lib().fsgc_task_footprint(ctx.ptr, C.byref(t), C.byref(b)), "task_footprint", ctx.ptr)
    return b.value


class Server:
    """Serving loop over a Context with continuous batching on `lanes` lanes:
    submit() queues a count query and returns a ticket, wait() returns
    (Result, latency_ms)."""

    def __init__(self, ctx, memory_budget, lanes=4, max_batch=64):
        self.ctx = ctx
        p = C.c_void_p()
        st = lib().fsgc_server_create(ctx.ptr, int(memory_budget), int(lanes), int(max_batch), C.byref(p))
        _check(st, "server_create")
        self.ptr = p

    def add_graph(self, gid):
        _check(lib().fsgc_server_add_graph(self.ptr, gid), "server_add_graph", self.ctx.ptr)

    def submit(self, gid, mo):
        t = C.c_uint64()
        _check(lib().fsgc_server_submit(self.ptr, gid, C.byref(mo), C.byref(t)), "server_submit")
        return t.value

    def poll(self, ticket):
        """None while the query runs, else (Result, latency_ms)."""
        r, lat = Result(), C.c_double()
        st = lib().fsgc_server_poll(self.ptr, ticket, C.byref(r), C.byref(lat))
        if st == 8:  # FSGC_EBUSY
            return None
        _check(st, "server_poll", self.ctx.ptr)
        return r, lat.value

    def wait(self, ticket, timeout_s=600.0):
        r, lat = Result(), C.c_double()
        _check(lib().fsgc_server_wait(self.ptr, ticket, float(timeout_s), C.byref(r), C.byref(lat)), "server_wait",
               self.ctx.ptr)
        return r, lat.value

    def stats(self):
        s = ServerStats()
        _check(lib().fsgc_server_stats_get(self.ptr, C.byref(s)), "server_stats")
        return s

    def close(self):
        if self.ptr:
            lib().fsgc_server_destroy(self.ptr)
            self.ptr = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
