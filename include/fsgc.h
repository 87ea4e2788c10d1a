/*
 * fsgc.h -- C ABI of the GB300-native fringe subgraph counter (libfsgc.so).
 *
 * The reference (Fringe-SGC) has no library interface: its boundary is two
 * command-line programs and two binary formats.  Each entry point below names
 * the reference code it stands in for.  Conventions:
 *   - every call returns an fsgc_status (0 = success); nothing calls exit() or
 *     traps on the device; fsgc_ctx_last_error() has the message;
 *   - callers own host buffers, a context owns device memory;
 *   - a context serialises its own calls with an internal lock, and any number
 *     of contexts may live in one process.
 */
#ifndef FSGC_H
#define FSGC_H

#include <stddef.h>
#include <stdint.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FSGC_MAX_CORE 6     /* src/fringes.h:44 */
#define FSGC_MAX_PATTERN 32 /* src/patterns.h:45 */

typedef enum fsgc_status {
  FSGC_OK = 0,
  FSGC_EINVAL = 1,       /* bad argument or malformed input */
  FSGC_ENOMEM = 2,       /* device or host allocation failed */
  FSGC_ECUDA = 3,        /* CUDA runtime error */
  FSGC_EIO = 4,          /* file could not be read or written */
  FSGC_EUNSUPPORTED = 5, /* e.g. a core of more than six vertices */
  FSGC_ETIMEDOUT = 6,    /* a bounded device wait gave up */
  FSGC_ENOTFOUND = 7,    /* unknown graph id or ticket */
  FSGC_EBUSY = 8,        /* result not ready / admission refused */
  FSGC_ENODEV = 9        /* no usable CUDA device or kernels not loaded */
} fsgc_status;

/* Matching order: byte-for-byte the reference's MatchingOrder
 * (src/fringes.h:50-58), 139 packed bytes, the content of a `.mo` file. */
typedef struct fsgc_matching_order {
  uint8_t nodes;      /* core vertices (1..6) */
  uint8_t anchorsets; /* number of distinct anchor sets */
  uint8_t startdeg;   /* pattern degree of core vertex A */
  uint8_t destdeg[FSGC_MAX_CORE - 1];
  uint8_t list[FSGC_MAX_CORE - 1];               /* earlier core vertices each must touch */
  uint8_t anch[(1 << FSGC_MAX_CORE) - 1];        /* anchor-set bitmaps */
  uint8_t fcnt[(1 << FSGC_MAX_CORE) - 1];        /* fringes per anchor set */
} fsgc_matching_order;

typedef enum fsgc_core_type {
  FSGC_CORE_VERTEX = 1,   /* vertexCore, src/fringeCount.cu:2172 */
  FSGC_CORE_EDGE = 2,     /* edgeCore, :2106 */
  FSGC_CORE_WEDGE = 3,    /* wedgeCore, :1783 */
  FSGC_CORE_TRIANGLE = 4, /* triangleCore, :1320 */
  FSGC_CORE_GENERAL = 5   /* generalCore, :666 */
} fsgc_core_type;

/* fsgc_result.flags */
#define FSGC_FLAG_PATTERN_TOO_LARGE 0x1u /* pattern has more vertices/edges than the graph: count 0 */

typedef struct fsgc_result {
  uint64_t count;         /* the reference's printed count, as u64: raw_total / automorphisms */
  uint64_t raw_total;     /* u64 total of the per-match formulas (the reference's `total`) */
  uint64_t automorphisms; /* divisor: the pattern counted in itself (1 for vertex and edge cores) */
  uint32_t flags;
  int32_t core_type;      /* fsgc_core_type */
  double device_ms;       /* device time of this count (CUDA events on the context stream) */
} fsgc_result;

typedef struct fsgc_ctx fsgc_ctx;

/* ---- pattern decomposition (replaces fringePreprocess, src/fringePreprocess.cpp:287-365) ---- */

/* n pattern vertices (2..32), nedges undirected edges as pairs in `edges`.
 * Fills *out with the same matching order the reference CLI writes to motif.mo
 * (bytes the reference leaves unwritten are zero). */
int fsgc_preprocess(int n, const int* edges, int nedges, fsgc_matching_order* out, char* errbuf, int errlen);
/* `fringePreprocess <motif_number>`: predefined motif 0..30 (src/patterns.h:57-354). */
int fsgc_preprocess_predefined(int number, fsgc_matching_order* out, char* errbuf, int errlen);
/* Same as fsgc_preprocess, writing the reference CLI's progress lines to `log`. */
int fsgc_preprocess_log(int n, const int* edges, int nedges, fsgc_matching_order* out, char* errbuf, int errlen,
                        FILE* log);
/* Predefined motif as an edge list (edges may be NULL to query the size). */
int fsgc_predefined_pattern(int number, int* n, int* edges, int max_edges, int* nedges);
const char* fsgc_predefined_name(int number);

/* ---- host-side graphs, ECLgraph files, generators (src/ECLgraph.h:45-96) ---- */

/* Host CSR with 64-bit offsets: nindex[n+1], nlist[m] (m directed entries). */
typedef struct fsgc_host_csr {
  int32_t n;
  int64_t m;
  int64_t* nindex;
  int32_t* nlist;
} fsgc_host_csr;

/* readECLgraph (src/ECLgraph.h:58-85): int32 header and arrays; weights ignored.
 * Also reads the int64 extension below. */
int fsgc_egr_read(const char* path, fsgc_host_csr* out);
/* Writes the same format; graphs of m >= 2^31 directed entries, which its int32
 * fields cannot hold, in an extension: int32 n, int32 -1 (refused by the
 * reference's reader), int64 m, int64 nindex[n+1], int32 nlist[m]. */
int fsgc_egr_write(const char* path, const fsgc_host_csr* g);
/* Writes the int64 extension whatever m is (for tests and tools). */
int fsgc_egr_write64(const char* path, const fsgc_host_csr* g);
/* Checks the reference's documented preconditions (src/fringeCount.cu:50-56):
 * sorted, duplicate-free, loop-free, symmetric lists. */
int fsgc_csr_validate(const fsgc_host_csr* g, char* errbuf, int errlen);
/* Seeded synthetic graphs, symmetrised, deduplicated, self loops dropped. */
int fsgc_gen_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t seed, fsgc_host_csr* out);
int fsgc_gen_er(int n, int64_t undirected_edges, uint64_t seed, fsgc_host_csr* out);
int fsgc_gen_chung_lu(int n, double avg_degree, double exponent, uint64_t seed, fsgc_host_csr* out);
/* Builds a cleaned CSR from an arbitrary undirected edge list (pairs). */
int fsgc_csr_from_edges(int n, int64_t nedges, const int32_t* pairs, fsgc_host_csr* out);
/* Page-locks a host CSR for fast uploads (optional). */
int fsgc_host_csr_pin(fsgc_host_csr* g);
void fsgc_host_csr_free(fsgc_host_csr* g);

/* ---- contexts ---- */

int fsgc_ctx_create(int device, fsgc_ctx** out);
void fsgc_ctx_destroy(fsgc_ctx* ctx);
const char* fsgc_ctx_last_error(const fsgc_ctx* ctx);
/* The cudaStream_t on which the context runs all of its work. */
void* fsgc_ctx_stream(fsgc_ctx* ctx);
/* Number of this library's kernels launched by the context so far. */
uint64_t fsgc_ctx_launches(const fsgc_ctx* ctx);
/* Benchmark support: CUDA events on the context stream around a region, and a
 * write of `bytes` (0 = 512 MiB, larger than the 126 MB L2) to evict caches. */
int fsgc_ctx_timer_start(fsgc_ctx* ctx);
int fsgc_ctx_timer_stop(fsgc_ctx* ctx, double* ms);
int fsgc_ctx_flush_l2(fsgc_ctx* ctx, size_t bytes);
int fsgc_ctx_synchronize(fsgc_ctx* ctx);
/* General cores (4-6 core vertices): 0 (default) sums fringe placements the
 * way the reference's functionX does (src/fringeCount.cu:408-486), which for
 * anchor sets with two or more fringes can differ from the exact number of
 * placements; 1 sums the exact number.  Other core types are unaffected. */
int fsgc_ctx_set_exact_placements(fsgc_ctx* ctx, int on);

/* Method thresholds and launch shapes of the counting kernels (no counterpart
 * in the reference, whose thresholds are compile-time constants,
 * src/fringeCount.cu:70, 80-84, 1237, 1328-1334, 1797-1804).  They change speed,
 * never results.  fringe-sgc_gb300/autotune.py picks them per graph by timing. */
typedef struct fsgc_tuning {
  int32_t wedge_small_max_degree; /* wedge pairs: endpoints up to this degree (16..2048) count in the
                                     shared-memory kernel, higher ones in the hub kernel */
  int32_t triangle_walk_ratio;    /* triangle bitmaps: a row walks N(b) against the staged N(a) when
                                     deg b <= ratio * deg a, else searches N(b) (0: always search) */
  int32_t triangle_stage_max;     /* longest N(a) staged in shared memory by bulk copy (0..8192, x32) */
  int32_t general_lane_venn_max;  /* general core: a lane builds its own Venn row up to this many
                                     list entries, longer rows are built by the whole warp */
  int32_t general_blocks_per_sm;  /* general core: resident blocks of 4 warps per SM (1..16) */
} fsgc_tuning;
/* Defaults: 2048, 16, 8192, 96, 8. */
int fsgc_tuning_default(fsgc_tuning* out);
int fsgc_ctx_set_tuning(fsgc_ctx* ctx, const fsgc_tuning* t);
int fsgc_ctx_get_tuning(fsgc_ctx* ctx, fsgc_tuning* out);

/* ---- resident graphs (CSR upload + loader: src/fringeCount.cu:2286-2297) ---- */

/* Uploads a host CSR (offsets 64-bit) and prepares it for counting. */
int fsgc_graph_from_csr(fsgc_ctx* ctx, int n, int64_t m, const int64_t* nindex, const int32_t* nlist, int* gid);
/* Same with the reference's int32 offsets (ECLgraph layout). */
int fsgc_graph_from_csr32(fsgc_ctx* ctx, int n, int m, const int32_t* nindex, const int32_t* nlist, int* gid);
/* Device-resident input (context's device): the arrays are copied, not adopted. */
int fsgc_graph_from_device_csr(fsgc_ctx* ctx, int n, int64_t m, const int64_t* d_nindex, const int32_t* d_nlist,
                               int* gid);
int fsgc_graph_load_egr(fsgc_ctx* ctx, const char* path, int* gid);
/* Edge-list ingestion on the GPU (the reference has none: its loader reads a
 * CSR that must already be clean, src/ECLgraph.h:58-85, src/fringeCount.cu:50-56):
 * nedges undirected pairs (2 x int32 each, host memory, or device memory of
 * the context's device when pairs_on_device) become the resident CSR with
 * self loops dropped, duplicates merged, both directions and sorted lists --
 * the same graph fsgc_csr_from_edges builds on the host.  FSGC_EINVAL for an
 * id outside [0, n). */
int fsgc_graph_from_edges(fsgc_ctx* ctx, int n, int64_t nedges, const int32_t* pairs, int pairs_on_device, int* gid);
/* Copies a resident graph's CSR back to host buffers (nindex[n+1], nlist[m]). */
int fsgc_graph_copy_csr(fsgc_ctx* ctx, int gid, int64_t* nindex, int32_t* nlist);
int fsgc_graph_release(fsgc_ctx* ctx, int gid);
/* Runs the loader's derived passes now (degree orientation, triangle supports)
 * instead of on the first count that needs them (the reference's relabel and
 * worklist builders, src/fringeCount.cu:1221-1288, 617-663, 1167-1218). */
int fsgc_graph_prepare(fsgc_ctx* ctx, int gid);
/* Builds, now, every derived structure any count on this graph could need:
 * the passes above plus the wedge core's chunk table, the per-vertex triangle
 * counts and the per-entry supports (their bytes show in device_bytes). */
int fsgc_graph_prepare_all(fsgc_ctx* ctx, int gid);

typedef struct fsgc_graph_info {
  int32_t n;
  int64_t m;            /* directed CSR entries */
  int32_t max_degree;
  int64_t triangles;    /* -1 until the triangle pass has run */
  int64_t device_bytes; /* HBM held by this graph */
} fsgc_graph_info;
int fsgc_graph_info_get(fsgc_ctx* ctx, int gid, fsgc_graph_info* out);

/* ---- packed graphs: many member graphs in one resident CSR (the batching-across-
 *      graphs workload; the reference runs one fringeCount process per graph) ----
 * Member i owns vertices [vstart[i], vstart[i+1]) (vstart[0] = 0, vstart[ngraphs]
 * = n); no edge may cross members.  One count covers every member: each
 * member's result equals a count on that member alone (its own relabel gate,
 * vertex order and pattern-size check).  results[] has ngraphs entries. */
int fsgc_graph_from_packed_csr(fsgc_ctx* ctx, int n, int64_t m, const int64_t* nindex, const int32_t* nlist,
                               int ngraphs, const int32_t* vstart, int* gid);
int fsgc_count_packed(fsgc_ctx* ctx, int gid, const fsgc_matching_order* mo, fsgc_result* results);

/* ---- counting (replaces `fringeCount <graph> <motif.mo>`, src/fringeCount.cu:2265-2331,
 *      and occurrences(), :2199-2262) ---- */

/* The divisor occurrences() takes from a pattern's count in itself
 * (src/fringeCount.cu:2230-2232, 2250-2261): the reference stores that u64
 * count in an int and asserts the int is positive.  *out = that int when it
 * is positive; FSGC_EINVAL where the reference's assertion would stop the
 * program (counts of cores with 3+ vertices then fail with FSGC_EINVAL). */
int fsgc_divisor_from_self_count(uint64_t self_count, uint64_t* out);

int fsgc_count(fsgc_ctx* ctx, int gid, const fsgc_matching_order* mo, fsgc_result* out);

/* ---- exact counts (the reference has none: its u64 binomials wrap silently,
 *      src/fringeCount.cu:189-197) ----
 * The same per-match formulas evaluated in exact 128-bit arithmetic, with
 * general cores summing the exact number of fringe placements; values that
 * reach 2^128 - 1 saturate (FSGC_FLAG_SATURATED, all words set).  The divisor
 * is the pattern counted in itself with exact placements.  Ordinary (not
 * packed) graphs only. */
#define FSGC_FLAG_SATURATED 0x2u /* the exact total needs more than 128 bits */
typedef struct fsgc_exact_result {
  uint64_t count_lo, count_hi; /* exact count = raw / automorphisms */
  uint64_t raw_lo, raw_hi;     /* exact total of the per-match formulas */
  uint64_t automorphisms;
  uint32_t flags;              /* FSGC_FLAG_PATTERN_TOO_LARGE, FSGC_FLAG_SATURATED */
  int32_t core_type;
  double device_ms;
} fsgc_exact_result;
int fsgc_count_exact(fsgc_ctx* ctx, int gid, const fsgc_matching_order* mo, fsgc_exact_result* out);

/* Many patterns on one resident graph in one call (the batching-on-one-graph
 * workload; the reference runs one fringeCount process per pattern).  Patterns
 * whose kernels share their match enumeration are counted in shared passes:
 * stars and tailed triangles in one pass over the vertices, edge-core
 * formulas in one pass over the edges, fringe-free-centre wedge cores over
 * one set of centre counts, triangle cores over one set of per-vertex
 * bitmaps; the rest one by one.  Every result equals fsgc_count's.  The
 * second call with the same graph and patterns captures the launches into a
 * CUDA graph and later calls replay it.  device_ms is the whole set's device
 * time divided by n.  Ordinary (not packed) graphs; u64 counts. */
int fsgc_count_set(fsgc_ctx* ctx, int gid, const fsgc_matching_order* mos, int n, fsgc_result* results);

/* Many (graph, pattern) tasks in one call; results in task order. */
typedef struct fsgc_task {
  int32_t gid;
  fsgc_matching_order mo;
} fsgc_task;
int fsgc_count_batch(fsgc_ctx* ctx, const fsgc_task* tasks, int ntasks, fsgc_result* results);

/* ---- lanes: asynchronous counts (no counterpart in the reference) ----
 * A lane is a CUDA stream of the context with its own work areas and result
 * slots.  fsgc_lane_submit checks a batch of tasks, builds any one-time
 * per-graph structure they need (on the context's stream, synchronously) and
 * enqueues the counts on the lane, then returns; fsgc_lane_wait sleeps until
 * they finish and writes ntasks results (same values as fsgc_count_batch).
 * Submissions on different lanes run concurrently on the device.  A lane holds
 * one submission at a time (FSGC_EBUSY otherwise) and is used by one host
 * thread at a time; destroy lanes before their context. */
typedef struct fsgc_lane fsgc_lane;
int fsgc_lane_create(fsgc_ctx* ctx, fsgc_lane** out);
void fsgc_lane_destroy(fsgc_lane* lane);
int fsgc_lane_submit(fsgc_lane* lane, const fsgc_task* tasks, int ntasks);
int fsgc_lane_wait(fsgc_lane* lane, fsgc_result* results);
/* Sleeps until task `index` of the submission has finished (tasks finish in
 * order) and writes its result; take results in increasing index order.  The
 * lane is free again once the last task's result has been taken. */
int fsgc_lane_wait_task(fsgc_lane* lane, int index, fsgc_result* out);
/* FSGC_OK when the submission has finished, FSGC_EBUSY while it runs. */
int fsgc_lane_query(fsgc_lane* lane);
/* Device bytes of the lane's growable work arena, and its release (idle lane). */
size_t fsgc_lane_scratch_bytes(const fsgc_lane* lane);
int fsgc_lane_trim(fsgc_lane* lane);
/* Work-arena bytes a count of this task needs beyond its resident graph
 * (hub cursors of the wedge core, the triangle core's bitmaps); prepares the
 * graph if it is not prepared yet. */
int fsgc_task_footprint(fsgc_ctx* ctx, const fsgc_task* task, size_t* bytes);

/* ---- serving loop (no counterpart in the reference, which runs one fringeCount
 *      process per query: src/fringeCount.cu:2265-2331) ----
 * Continuous batching over `lanes` lanes of `ctx`, one worker thread each.
 * Graphs are uploaded to the context first and registered with
 * fsgc_server_add_graph, which builds every derived structure a count could
 * need (fsgc_graph_prepare_all) and counts the graph's device bytes against
 * `memory_budget` while it is registered (FSGC_EBUSY when it does not fit).
 * Submitted queries wait in arrival order.  Whenever a lane is free, its
 * worker admits queries from the head of the queue (at most `max_batch`)
 * while the registered graphs and the lanes' work arenas, with this batch's
 * need, fit `memory_budget`; it submits them to its lane and
 * completes them when they finish, while the other lanes keep admitting and
 * running queries that arrived in the meantime.  A query whose footprint alone
 * exceeds the budget is refused at submission (FSGC_EBUSY); a query that fails
 * fails alone.  Latency is submission to completion.  Completed counts are
 * cached by (graph, matching-order bytes); a repeated query completes at
 * submission. */
typedef struct fsgc_server fsgc_server;
typedef struct fsgc_server_stats {
  uint64_t completed;    /* queries finished */
  uint64_t rounds;       /* lane submissions (batches) run */
  uint64_t queued;       /* queries waiting for admission */
  uint64_t in_use_bytes; /* work-arena bytes the lanes hold or have reserved */
  double p50_ms, p99_ms; /* latency percentiles over completed queries */
  double queries_per_s;  /* completed / (last completion - first submission) */
  uint64_t cache_hits;   /* queries answered from the result cache at submission */
} fsgc_server_stats;
int fsgc_server_create(fsgc_ctx* ctx, size_t memory_budget, int lanes, int max_batch, fsgc_server** out);
/* Finishes every submitted query, then stops the worker. */
void fsgc_server_destroy(fsgc_server* srv);
int fsgc_server_add_graph(fsgc_server* srv, int gid);
int fsgc_server_submit(fsgc_server* srv, int gid, const fsgc_matching_order* mo, uint64_t* ticket);
/* FSGC_EBUSY while the query runs; otherwise the query's own status, its result
 * and latency, after which the ticket is forgotten. */
int fsgc_server_poll(fsgc_server* srv, uint64_t ticket, fsgc_result* out, double* latency_ms);
/* Blocks up to timeout_s seconds (FSGC_ETIMEDOUT), else as fsgc_server_poll. */
int fsgc_server_wait(fsgc_server* srv, uint64_t ticket, double timeout_s, fsgc_result* out, double* latency_ms);
int fsgc_server_stats_get(fsgc_server* srv, fsgc_server_stats* out);

/* ---- allocation-free count (no counterpart in the reference) ----
 * For callers that cannot allocate device memory when they count -- code
 * running where a host framework forbids cudaMalloc after start-up, or inside
 * another library's memory pool.  The caller passes its own device CSR
 * (d_nindex[n+1] int64, d_nlist[m] int32 on the current device) and a stream
 * (NULL = default stream); the count of a wedge-core pattern whose centre
 * carries no fringes is written to *out.  Every intermediate lives in one fixed
 * 64 MiB device array inside the library (held by each GPU that loads it until
 * the process exits); graphs that do not fit (about 16M vertices, fewer when
 * hub endpoints are large) and other pattern shapes return FSGC_EUNSUPPORTED.
 * The caller's CSR is used as given, without the checks of the upload entry
 * points: each list sorted ascending, no duplicates, no self loops, symmetric,
 * every neighbour id in [0, n) (the reference's preconditions,
 * src/fringeCount.cu:50-56).  Unsorted lists give a wrong count and no error;
 * run fsgc_csr_validate on a host copy once if in doubt.
 * The first call on a device looks up that array's device address and loads a
 * constant table; make that first call before any stream capture.  Both stay
 * valid for the life of the device's primary context: do not call this after
 * a cudaDeviceReset on that device.  Each call reads the graph's maximum degree
 * back to the host and waits for `stream` to finish the count before it
 * returns, so no call can be captured into a CUDA graph.  All calls share the
 * array, so calls that overlap on the GPU race: serialise them. */
int fsgc_count_wedge_noalloc(int n, int64_t m, const int64_t* d_nindex, const int32_t* d_nlist,
                             const fsgc_matching_order* mo, void* stream, fsgc_result* out, char* errbuf,
                             int errlen);

#ifdef __cplusplus
}
#endif
#endif /* FSGC_H */
