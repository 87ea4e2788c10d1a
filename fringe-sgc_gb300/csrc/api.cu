// C ABI: contexts, resident graphs, counting.
//
// A count follows occurrences() (src/fringeCount.cu:2199-2262): vertex and edge
// cores return their raw total; larger cores divide it by the pattern's count
// in itself, computed with the same kernels on the pattern graph built from the
// matching order (matchingOrder2ECLgraph, :121-186) and cached per pattern.
// Unlike the reference, all device state lives in the context (no file-scope
// device globals), so any number of counts and contexts can coexist.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "fsgc_internal.h"

using fsgc::DevGraph;
typedef unsigned long long u64;

struct fsgc_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::mutex mu;
  std::string err;
  uint64_t launches = 0;
  std::map<int, DevGraph*> graphs;
  int next_gid = 1;
  fsgc::DevWork work;
  u64* d_slots = nullptr;
  u64* h_slots = nullptr;
  int slot_cap = 0;
  std::vector<cudaEvent_t> events;
  std::map<std::string, u64> aut_cache;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  int exact_placements = 0;
  u64* d_member = nullptr;  // per-member result slots of packed counts
  u64* h_member = nullptr;
  int member_cap = 0;
  void* flush_buf = nullptr;
  size_t flush_bytes = 0;
  uint64_t slot_gen = 0;  // bumped whenever d_slots changes
  // captured launch sequences of pattern sets, by (graph, matching orders)
  struct SetGraph {
    int gid;
    uint64_t slot_gen, arena_gen;
    cudaGraphExec_t exec;
    std::vector<fsgc::CountJob> plan;  // host-side results of planning (core types, host values)
  };
  std::map<std::string, SetGraph> set_graphs;
  std::map<std::string, int> set_seen;
};

struct fsgc_lane {
  fsgc_ctx* ctx = nullptr;
  cudaStream_t stream = nullptr;
  fsgc::DevWork work;
  u64* d_slots = nullptr;
  u64* h_slots = nullptr;
  int cap = 0;
  std::vector<cudaEvent_t> events;  // blocking-sync: waiting threads sleep
  std::vector<fsgc_task> tasks;     // the submission in flight (jobs point here)
  std::vector<fsgc::CountJob> jobs;
  std::vector<u64> aut;
  std::vector<fsgc_result> res;
  int pending = 0;   // tasks of the submission in flight (0: the lane is free)
  int finished = 0;  // tasks whose results have been taken
};

namespace {

std::mutex g_init_mu;
bool g_magic_uploaded[64] = {false};

int fail(fsgc_ctx* c, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  return code;
}

int cuda_fail(fsgc_ctx* c, cudaError_t e, const char* what) {
  return fail(c, e == cudaErrorMemoryAllocation ? FSGC_ENOMEM : FSGC_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(expr, what)                              \
  do {                                              \
    cudaError_t e__ = (expr);                       \
    if (e__ != cudaSuccess) return cuda_fail(c, e__, what); \
  } while (0)

void free_graph(DevGraph* g) {
  if (!g) return;
  cudaFree(g->off);
  cudaFree(g->adj);
  cudaFree(g->deg);
  cudaFree(g->ooff);
  cudaFree(g->oadj);
  cudaFree(g->osrc);
  cudaFree(g->osup);
  cudaFree(g->vtri2);
  cudaFree(g->esup);
  cudaFree(g->ctab_id);
  cudaFree(g->ctab_rows);
  cudaFree(g->ctab_pos);
  cudaFree(g->comp);
  cudaFree(g->comp_relabel);
  delete g;
}

int ensure_slots(fsgc_ctx* c, int n) {
  if (n <= c->slot_cap) return FSGC_OK;
  int cap = std::max(n, 2 * c->slot_cap);
  cudaStreamSynchronize(c->stream);
  cudaFree(c->d_slots);
  cudaFreeHost(c->h_slots);
  cudaFree(c->d_member);
  cudaFreeHost(c->h_member);
  c->d_slots = nullptr;
  c->h_slots = nullptr;
  CK(cudaMalloc((void**)&c->d_slots, sizeof(u64) * (size_t)cap), "slot allocation");
  CK(cudaMallocHost((void**)&c->h_slots, sizeof(u64) * (size_t)cap), "slot allocation");
  c->slot_cap = cap;
  c->slot_gen++;
  return FSGC_OK;
}

int ensure_events(fsgc_ctx* c, size_t n) {
  while (c->events.size() < n) {
    cudaEvent_t e;
    CK(cudaEventCreate(&e), "event creation");
    c->events.push_back(e);
  }
  return FSGC_OK;
}

// Upload a host CSR (64-bit offsets) as a new DevGraph.
int upload_graph(fsgc_ctx* c, int n, long long m, const long long* off, const int* adj, bool device_src,
                 DevGraph** out) {
  DevGraph* g = new DevGraph();
  g->n = n;
  g->m = m;
  cudaError_t e = cudaMalloc((void**)&g->off, sizeof(long long) * ((size_t)n + 1));
  // the neighbour lists are padded by 16 bytes: bulk copies into shared memory
  // round a list's end up to a 16-byte boundary
  if (e == cudaSuccess) e = cudaMalloc((void**)&g->adj, sizeof(int) * (size_t)std::max(1LL, m) + 16);
  if (e == cudaSuccess) e = cudaMalloc((void**)&g->deg, sizeof(int) * (size_t)std::max(1, n));
  if (e != cudaSuccess) {
    free_graph(g);
    cudaGetLastError();
    return cuda_fail(c, e, "graph allocation");
  }
  const cudaMemcpyKind kind = device_src ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  e = cudaMemcpyAsync(g->off, off, sizeof(long long) * ((size_t)n + 1), kind, c->stream);
  if (e == cudaSuccess && m > 0) e = cudaMemcpyAsync(g->adj, adj, sizeof(int) * (size_t)m, kind, c->stream);
  if (e != cudaSuccess) {
    free_graph(g);
    return cuda_fail(c, e, "graph upload");
  }
  g->bytes = sizeof(long long) * ((size_t)n + 1) + sizeof(int) * ((size_t)m + (size_t)n);
  const int st = fsgc::graph_degrees(*g, c->stream, &c->launches, c->work.small);
  if (st != FSGC_OK) {
    free_graph(g);
    return fail(c, st, "degree pass failed: %s", cudaGetErrorString(cudaGetLastError()));
  }
  *out = g;
  return FSGC_OK;
}

// Pattern graph of a matching order (src/fringeCount.cu:121-186): core vertices
// 0..k-1 joined as mo.list says, then each anchor set's fringes.
void pattern_csr(const fsgc_matching_order& mo, std::vector<long long>& off, std::vector<int>& adj) {
  int n = mo.nodes;
  for (int i = 0; i < mo.anchorsets; i++) n += mo.fcnt[i];
  std::vector<std::vector<int>> nb(n);
  for (int i = 0; i < mo.nodes - 1; i++)
    for (int j = 0; j <= i; j++)
      if (mo.list[i] & (1 << j)) { nb[i + 1].push_back(j); nb[j].push_back(i + 1); }
  int v = mo.nodes;
  for (int i = 0; i < mo.anchorsets; i++)
    for (int t = 0; t < mo.fcnt[i]; t++, v++)
      for (int j = 0; j < FSGC_MAX_CORE; j++)
        if (mo.anch[i] & (1 << j)) { nb[j].push_back(v); nb[v].push_back(j); }
  off.assign((size_t)n + 1, 0);
  adj.clear();
  for (int x = 0; x < n; x++) {
    std::sort(nb[x].begin(), nb[x].end());
    adj.insert(adj.end(), nb[x].begin(), nb[x].end());
    off[x + 1] = (long long)adj.size();
  }
}

bool mo_valid(const fsgc_matching_order& mo) { return fsgc::matching_order_valid(mo); }

// The divisor for cores of 3+ vertices: the pattern counted in itself with the
// same kernels.  The reference stores it in an int (src/fringeCount.cu:2213).
int automorphisms(fsgc_ctx* c, const fsgc_matching_order& mo, u64* out, int exact_placements) {
  std::string key(reinterpret_cast<const char*>(&mo), sizeof(mo));
  key.push_back(exact_placements ? 'x' : 'r');
  auto it = c->aut_cache.find(key);
  if (it != c->aut_cache.end()) {
    *out = it->second;
    return FSGC_OK;
  }
  std::vector<long long> off;
  std::vector<int> adj;
  pattern_csr(mo, off, adj);
  const int pn = (int)off.size() - 1;
  DevGraph* pg = nullptr;
  int st = upload_graph(c, pn, off[pn], off.data(), adj.data(), false, &pg);
  if (st != FSGC_OK) return st;
  st = ensure_slots(c, 1);
  if (st != FSGC_OK) { free_graph(pg); return st; }
  cudaMemsetAsync(c->d_slots, 0, sizeof(u64), c->stream);
  fsgc::CountJob job{&mo, pg, c->d_slots, 0, 0, false, exact_placements, nullptr, 1};
  st = fsgc::enqueue_count(job, c->stream, &c->launches, c->work);
  u64 raw = 0;
  if (st == FSGC_OK) {
    if (job.host_only) raw = job.host_value;
    else {
      cudaMemcpyAsync(c->h_slots, c->d_slots, sizeof(u64), cudaMemcpyDeviceToHost, c->stream);
      cudaError_t e = cudaStreamSynchronize(c->stream);
      if (e != cudaSuccess) st = cuda_fail(c, e, "automorphism count");
      else if (fsgc::take_kernel_error(c->work, c->stream) != FSGC_OK)
        st = fail(c, FSGC_ETIMEDOUT, "the automorphism count's kernel gave up a bounded wait");
      raw = c->h_slots[0];
    }
  } else {
    fail(c, st, "automorphism count failed (%d)", st);
  }
  cudaStreamSynchronize(c->stream);
  free_graph(pg);
  if (st != FSGC_OK) return st;
  uint64_t aut = 0;
  if (fsgc_divisor_from_self_count(raw, &aut) != FSGC_OK)
    return fail(c, FSGC_EINVAL, "the pattern's count in itself (%llu) is not a positive int: no divisor", raw);
  c->aut_cache[key] = aut;
  *out = aut;
  return FSGC_OK;
}

// Size check of occurrences() (src/fringeCount.cu:2216-2219).
bool pattern_too_large(const fsgc_matching_order& mo, const DevGraph& g) {
  if (mo.nodes < 3) return false;
  long long pn = mo.nodes, pm = 0;
  for (int i = 0; i + 1 < mo.nodes; i++) pm += 2 * __builtin_popcount(mo.list[i]);
  for (int i = 0; i < mo.anchorsets; i++) {
    pn += mo.fcnt[i];
    pm += 2LL * mo.fcnt[i] * __builtin_popcount(mo.anch[i]);
  }
  return pn > g.n || pm > g.m;
}

DevGraph* find_graph(fsgc_ctx* c, int gid) {
  auto it = c->graphs.find(gid);
  return it == c->graphs.end() ? nullptr : it->second;
}

// Host checks of a batch and the divisors of its patterns (context lock held).
int plan_tasks(fsgc_ctx* c, const fsgc_task* tasks, int nt, std::vector<u64>& aut) {
  aut.assign((size_t)nt, 1);
  for (int t = 0; t < nt; t++) {
    const fsgc_matching_order& mo = tasks[t].mo;
    if (!mo_valid(mo)) return fail(c, FSGC_EINVAL, "task %d: malformed matching order", t);
    DevGraph* g = find_graph(c, tasks[t].gid);
    if (!g) return fail(c, FSGC_ENOTFOUND, "task %d: unknown graph %d", t, tasks[t].gid);
    if (g->ngraphs > 0) return fail(c, FSGC_EINVAL, "task %d: graph %d is packed; use fsgc_count_packed", t, tasks[t].gid);
    if (mo.nodes >= 3 && !pattern_too_large(mo, *g)) {
      const int st = automorphisms(c, mo, &aut[(size_t)t], c->exact_placements);
      if (st != FSGC_OK) return st;
    }
  }
  return FSGC_OK;
}

// Enqueues a planned batch on `s`: slot reset, each task's kernels between
// events ev[t] and ev[t+1], and the read-back of the raw totals into h_slots
// (per task before its closing event when per_task_copy, else once at the end).
int enqueue_tasks(fsgc_ctx* c, const fsgc_task* tasks, int nt, cudaStream_t s, fsgc::DevWork& work, u64* d_slots,
                  u64* h_slots, const cudaEvent_t* ev, std::vector<fsgc::CountJob>& jobs, fsgc_result* res,
                  bool per_task_copy) {
  jobs.assign((size_t)nt, fsgc::CountJob{});
  CK(cudaMemsetAsync(d_slots, 0, sizeof(u64) * (size_t)nt, s), "slot reset");
  CK(cudaEventRecord(ev[0], s), "event");
  for (int t = 0; t < nt; t++) {
    const fsgc_matching_order& mo = tasks[t].mo;
    DevGraph* g = find_graph(c, tasks[t].gid);
    memset(&res[t], 0, sizeof(fsgc_result));
    jobs[t] = fsgc::CountJob{&tasks[t].mo, g, d_slots + t, 0, 0, false, c->exact_placements, nullptr, 1};
    if (pattern_too_large(mo, *g)) {
      jobs[t].host_only = true;
      jobs[t].host_value = 0;
      jobs[t].core_type = (mo.nodes == 3) ? ((__builtin_popcount(mo.list[1]) == 1) ? FSGC_CORE_WEDGE : FSGC_CORE_TRIANGLE)
                                          : FSGC_CORE_GENERAL;
      res[t].flags |= FSGC_FLAG_PATTERN_TOO_LARGE;
    } else {
      const int st = fsgc::enqueue_count(jobs[t], s, &c->launches, work);
      if (st != FSGC_OK) {
        cudaStreamSynchronize(s);
        return fail(c, st, "task %d: count failed (%s)", t, cudaGetErrorString(cudaGetLastError()));
      }
    }
    if (per_task_copy)
      CK(cudaMemcpyAsync(h_slots + t, d_slots + t, sizeof(u64), cudaMemcpyDeviceToHost, s), "readback");
    CK(cudaEventRecord(ev[t + 1], s), "event");
  }
  if (!per_task_copy)
    CK(cudaMemcpyAsync(h_slots, d_slots, sizeof(u64) * (size_t)nt, cudaMemcpyDeviceToHost, s), "readback");
  return FSGC_OK;
}

// Result of finished task t (its closing event and read-back have completed).
void finish_task(int t, const std::vector<fsgc::CountJob>& jobs, const std::vector<u64>& aut, const u64* h_slots,
                 const cudaEvent_t* ev, fsgc_result* res) {
  const u64 raw = jobs[t].host_only ? jobs[t].host_value : h_slots[t];
  const bool too_large = (res[t].flags & FSGC_FLAG_PATTERN_TOO_LARGE) != 0;
  res[t].raw_total = raw;
  // no divisor is computed when the pattern does not fit the graph
  res[t].automorphisms = too_large ? 0 : aut[t];
  res[t].count = too_large ? 0 : raw / aut[t];
  res[t].core_type = jobs[t].core_type;
  float ms = 0;
  cudaEventElapsedTime(&ms, ev[t], ev[t + 1]);
  res[t].device_ms = ms;
}

int count_tasks(fsgc_ctx* c, const fsgc_task* tasks, int nt, fsgc_result* res) {
  if (nt <= 0) return FSGC_OK;
  for (int t = 0; t < nt; t++) memset(&res[t], 0, sizeof(fsgc_result));
  int st = ensure_slots(c, nt);
  if (st != FSGC_OK) return st;
  st = ensure_events(c, (size_t)nt + 1);
  if (st != FSGC_OK) return st;
  std::vector<u64> aut;
  st = plan_tasks(c, tasks, nt, aut);
  if (st != FSGC_OK) return st;
  std::vector<fsgc::CountJob> jobs;
  st = enqueue_tasks(c, tasks, nt, c->stream, c->work, c->d_slots, c->h_slots, c->events.data(), jobs, res, false);
  if (st != FSGC_OK) return st;
  CK(cudaStreamSynchronize(c->stream), "count");
  st = fsgc::take_kernel_error(c->work, c->stream);
  if (st != FSGC_OK) return fail(c, st, "a counting kernel gave up a bounded wait; the counts are void");
  for (int t = 0; t < nt; t++) finish_task(t, jobs, aut, c->h_slots, c->events.data(), res);
  return FSGC_OK;
}

// Captured pattern-set launches of graph `gid` (all graphs when gid < 0).
void drop_set_graphs(fsgc_ctx* c, int gid) {
  for (auto it = c->set_graphs.begin(); it != c->set_graphs.end();) {
    if (gid < 0 || it->second.gid == gid) {
      cudaGraphExecDestroy(it->second.exec);
      it = c->set_graphs.erase(it);
    } else {
      ++it;
    }
  }
  if (gid < 0) c->set_seen.clear();
}

}  // namespace

namespace fsgc {

int take_kernel_error(DevWork& w, cudaStream_t s) {
  if (!w.h_err || *w.h_err == 0) return FSGC_OK;
  *w.h_err = 0;
  cudaMemsetAsync(w.small + kErrWord, 0, sizeof(u64), s);
  cudaStreamSynchronize(s);
  return FSGC_ETIMEDOUT;
}

}  // namespace fsgc

namespace fsgc {

// A matching order the kernels can take: 1-6 core vertices, every later core
// vertex joined to at least one earlier one (list[i] a non-empty subset of the
// i+1 earlier vertices, so list[0] == 1), anchor sets non-empty subsets of the
// core, at most 32 pattern vertices.
bool matching_order_valid(const fsgc_matching_order& mo) {
  if (mo.nodes < 1 || mo.nodes > FSGC_MAX_CORE || mo.anchorsets > 63) return false;
  int total = mo.nodes;
  for (int i = 0; i < mo.anchorsets; i++) {
    if (mo.anch[i] == 0 || mo.anch[i] >= (1 << mo.nodes)) return false;
    total += mo.fcnt[i];
  }
  for (int i = 0; i + 1 < mo.nodes; i++)
    if (mo.list[i] == 0 || mo.list[i] >= (2 << i)) return false;
  return total <= FSGC_MAX_PATTERN;
}

}  // namespace fsgc

extern "C" {

int fsgc_divisor_from_self_count(uint64_t self_count, uint64_t* out) {
  if (!out) return FSGC_EINVAL;
  *out = 0;
  // the reference keeps the count in an int and asserts it is positive
  const int as_int = (int)(unsigned int)(self_count & 0xffffffffULL);
  if (as_int <= 0) return FSGC_EINVAL;
  *out = (uint64_t)as_int;
  return FSGC_OK;
}

int fsgc_ctx_create(int device, fsgc_ctx** out) {
  if (!out) return FSGC_EINVAL;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return FSGC_ENODEV;
  }
  if (device < 0 || device >= ndev) return FSGC_EINVAL;
  if (cudaSetDevice(device) != cudaSuccess) return FSGC_ECUDA;
  fsgc_ctx* c = new fsgc_ctx();
  c->device = device;
  {
    std::lock_guard<std::mutex> lk(g_init_mu);
    if (device < 64 && !g_magic_uploaded[device]) {
      fsgc::upload_div_magic();
      g_magic_uploaded[device] = true;
    }
  }
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc((void**)&c->work.small, 32 * sizeof(u64)) != cudaSuccess ||
      cudaMallocHost((void**)&c->work.h_err, sizeof(u64)) != cudaSuccess || ensure_slots(c, 64) != FSGC_OK) {
    cudaGetLastError();
    fsgc_ctx_destroy(c);
    return FSGC_ECUDA;
  }
  cudaMemset(c->work.small, 0, 32 * sizeof(u64));
  *c->work.h_err = 0;
  if (cudaDeviceSynchronize() != cudaSuccess) {
    // kernels for this architecture missing or device unusable
    cudaGetLastError();
    fsgc_ctx_destroy(c);
    return FSGC_ENODEV;
  }
  *out = c;
  return FSGC_OK;
}

void fsgc_ctx_destroy(fsgc_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (auto& kv : c->graphs) free_graph(kv.second);
  c->graphs.clear();
  for (auto e : c->events) cudaEventDestroy(e);
  if (c->t0) cudaEventDestroy(c->t0);
  if (c->t1) cudaEventDestroy(c->t1);
  drop_set_graphs(c, -1);
  cudaFree(c->flush_buf);
  cudaFree(c->work.small);
  cudaFreeHost(c->work.h_err);
  cudaFree(c->work.tri.ptr);
  cudaFree(c->d_slots);
  cudaFreeHost(c->h_slots);
  cudaFree(c->d_member);
  cudaFreeHost(c->h_member);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char* fsgc_ctx_last_error(const fsgc_ctx* c) { return c ? c->err.c_str() : "null context"; }
void* fsgc_ctx_stream(fsgc_ctx* c) { return c ? (void*)c->stream : nullptr; }
uint64_t fsgc_ctx_launches(const fsgc_ctx* c) { return c ? c->launches : 0; }

int fsgc_ctx_timer_start(fsgc_ctx* c) {
  if (!c) return FSGC_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  if (!c->t0) {
    CK(cudaEventCreate(&c->t0), "event creation");
    CK(cudaEventCreate(&c->t1), "event creation");
  }
  CK(cudaEventRecord(c->t0, c->stream), "event record");
  return FSGC_OK;
}

int fsgc_ctx_timer_stop(fsgc_ctx* c, double* ms) {
  if (!c || !ms || !c->t0) return FSGC_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  CK(cudaEventRecord(c->t1, c->stream), "event record");
  CK(cudaEventSynchronize(c->t1), "event sync");
  float f = 0;
  CK(cudaEventElapsedTime(&f, c->t0, c->t1), "event time");
  *ms = f;
  return FSGC_OK;
}

int fsgc_ctx_flush_l2(fsgc_ctx* c, size_t bytes) {
  if (!c) return FSGC_EINVAL;
  if (bytes == 0) bytes = (size_t)512 << 20;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  if (c->flush_bytes < bytes) {
    cudaStreamSynchronize(c->stream);
    cudaFree(c->flush_buf);
    c->flush_buf = nullptr;
    c->flush_bytes = 0;
    CK(cudaMalloc(&c->flush_buf, bytes), "flush buffer");
    c->flush_bytes = bytes;
  }
  static unsigned char pattern = 0;
  pattern++;
  CK(cudaMemsetAsync(c->flush_buf, pattern, bytes, c->stream), "flush");
  return FSGC_OK;
}

int fsgc_tuning_default(fsgc_tuning* out) {
  if (!out) return FSGC_EINVAL;
  *out = fsgc::DevWork().tune;
  return FSGC_OK;
}

int fsgc_ctx_set_tuning(fsgc_ctx* c, const fsgc_tuning* t) {
  if (!c || !t) return FSGC_EINVAL;
  if (fsgc::check_tuning(*t) != FSGC_OK) return fail(c, FSGC_EINVAL, "tuning value out of range");
  std::lock_guard<std::mutex> lk(c->mu);
  c->work.tune = *t;
  drop_set_graphs(c, -1);  // captured launches hold the old shapes
  return FSGC_OK;
}

int fsgc_ctx_get_tuning(fsgc_ctx* c, fsgc_tuning* out) {
  if (!c || !out) return FSGC_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  *out = c->work.tune;
  return FSGC_OK;
}

int fsgc_ctx_set_exact_placements(fsgc_ctx* c, int on) {
  if (!c) return FSGC_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  c->exact_placements = on ? 1 : 0;
  return FSGC_OK;
}

int fsgc_ctx_synchronize(fsgc_ctx* c) {
  if (!c) return FSGC_EINVAL;
  cudaSetDevice(c->device);
  CK(cudaStreamSynchronize(c->stream), "synchronize");
  return FSGC_OK;
}

int fsgc_graph_from_csr(fsgc_ctx* c, int n, int64_t m, const int64_t* nindex, const int32_t* nlist, int* gid) {
  if (!c || !gid || n < 1 || m < 0 || !nindex || (m > 0 && !nlist)) return fail(c, FSGC_EINVAL, "bad graph arguments");
  if (nindex[0] != 0 || nindex[n] != m) return fail(c, FSGC_EINVAL, "offsets must start at 0 and end at m");
  for (int v = 0; v < n; v++)
    if (nindex[v + 1] < nindex[v]) return fail(c, FSGC_EINVAL, "offsets decrease at vertex %d", v);
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  DevGraph* g = nullptr;
  int st = upload_graph(c, n, m, (const long long*)nindex, nlist, false, &g);
  if (st != FSGC_OK) return st;
  CK(cudaStreamSynchronize(c->stream), "graph upload");
  *gid = c->next_gid++;
  c->graphs[*gid] = g;
  return FSGC_OK;
}

int fsgc_graph_from_csr32(fsgc_ctx* c, int n, int m, const int32_t* nindex, const int32_t* nlist, int* gid) {
  if (!c || n < 1 || m < 0 || !nindex) return fail(c, FSGC_EINVAL, "bad graph arguments");
  std::vector<int64_t> off((size_t)n + 1);
  for (int v = 0; v <= n; v++) off[v] = nindex[v];
  return fsgc_graph_from_csr(c, n, m, off.data(), nlist, gid);
}

int fsgc_graph_from_device_csr(fsgc_ctx* c, int n, int64_t m, const int64_t* d_nindex, const int32_t* d_nlist,
                               int* gid) {
  if (!c || !gid || n < 1 || m < 0 || !d_nindex || (m > 0 && !d_nlist)) return fail(c, FSGC_EINVAL, "bad graph arguments");
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  DevGraph* g = nullptr;
  int st = upload_graph(c, n, m, (const long long*)d_nindex, d_nlist, true, &g);
  if (st != FSGC_OK) return st;
  *gid = c->next_gid++;
  c->graphs[*gid] = g;
  return FSGC_OK;
}

int fsgc_graph_from_edges(fsgc_ctx* c, int n, int64_t nedges, const int32_t* pairs, int pairs_on_device, int* gid) {
  if (!c || !gid || n < 1 || nedges < 0 || (nedges > 0 && !pairs)) return fail(c, FSGC_EINVAL, "bad edge-list arguments");
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  const int* d_pairs = pairs;
  int* owned = nullptr;
  if (!pairs_on_device && nedges > 0) {
    CK(cudaMallocAsync((void**)&owned, sizeof(int32_t) * 2 * (size_t)nedges, c->stream), "edge-list upload");
    CK(cudaMemcpyAsync(owned, pairs, sizeof(int32_t) * 2 * (size_t)nedges, cudaMemcpyHostToDevice, c->stream),
       "edge-list upload");
    d_pairs = owned;
  }
  long long* off = nullptr;
  int* adj = nullptr;
  long long m = 0;
  int st = fsgc::csr_from_device_edges(n, nedges, d_pairs, c->stream, &off, &adj, &m, c->work.small);
  if (owned) cudaFreeAsync(owned, c->stream);
  if (st != FSGC_OK) {
    cudaStreamSynchronize(c->stream);
    return fail(c, st, st == FSGC_EINVAL ? "edge list has a vertex id outside [0, n)" : "edge-list ingestion failed");
  }
  DevGraph* g = new DevGraph();
  g->n = n;
  g->m = m;
  g->off = off;
  g->adj = adj;
  if (cudaMalloc((void**)&g->deg, sizeof(int) * (size_t)n) != cudaSuccess) {
    free_graph(g);
    cudaGetLastError();
    return fail(c, FSGC_ENOMEM, "graph allocation");
  }
  g->bytes = sizeof(long long) * ((size_t)n + 1) + sizeof(int) * ((size_t)m + (size_t)n);
  st = fsgc::graph_degrees(*g, c->stream, &c->launches, c->work.small);
  if (st != FSGC_OK) {
    free_graph(g);
    return fail(c, st, "degree pass failed");
  }
  *gid = c->next_gid++;
  c->graphs[*gid] = g;
  return FSGC_OK;
}

int fsgc_graph_copy_csr(fsgc_ctx* c, int gid, int64_t* nindex, int32_t* nlist) {
  if (!c || !nindex) return FSGC_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  DevGraph* g = find_graph(c, gid);
  if (!g) return fail(c, FSGC_ENOTFOUND, "unknown graph %d", gid);
  if (g->m > 0 && !nlist) return fail(c, FSGC_EINVAL, "no list buffer");
  CK(cudaMemcpyAsync(nindex, g->off, sizeof(long long) * ((size_t)g->n + 1), cudaMemcpyDeviceToHost, c->stream),
     "graph read-back");
  if (g->m > 0)
    CK(cudaMemcpyAsync(nlist, g->adj, sizeof(int) * (size_t)g->m, cudaMemcpyDeviceToHost, c->stream), "graph read-back");
  CK(cudaStreamSynchronize(c->stream), "graph read-back");
  return FSGC_OK;
}

int fsgc_graph_load_egr(fsgc_ctx* c, const char* path, int* gid) {
  fsgc_host_csr h;
  const int st = fsgc_egr_read(path, &h);
  if (st != FSGC_OK) return fail(c, st, "could not read graph file %s", path ? path : "(null)");
  const int r = fsgc_graph_from_csr(c, h.n, h.m, h.nindex, h.nlist, gid);
  if (c) cudaStreamSynchronize(c->stream);
  fsgc_host_csr_free(&h);
  return r;
}

int fsgc_graph_release(fsgc_ctx* c, int gid) {
  if (!c) return FSGC_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  auto it = c->graphs.find(gid);
  if (it == c->graphs.end()) return fail(c, FSGC_ENOTFOUND, "unknown graph %d", gid);
  cudaStreamSynchronize(c->stream);
  drop_set_graphs(c, gid);
  free_graph(it->second);
  c->graphs.erase(it);
  return FSGC_OK;
}

int fsgc_graph_from_packed_csr(fsgc_ctx* c, int n, int64_t m, const int64_t* nindex, const int32_t* nlist,
                               int ngraphs, const int32_t* vstart, int* gid) {
  if (!c || !gid || n < 1 || m < 0 || !nindex || (m > 0 && !nlist) || ngraphs < 1 || !vstart)
    return fail(c, FSGC_EINVAL, "bad packed graph arguments");
  if (vstart[0] != 0 || vstart[ngraphs] != n) return fail(c, FSGC_EINVAL, "member ranges must cover [0, n)");
  if (nindex[0] != 0 || nindex[n] != m) return fail(c, FSGC_EINVAL, "offsets must start at 0 and end at m");
  std::vector<int> comp((size_t)n);
  std::vector<unsigned char> relabel((size_t)ngraphs);
  std::vector<int> mn((size_t)ngraphs);
  std::vector<long long> mm((size_t)ngraphs);
  for (int gi = 0; gi < ngraphs; gi++) {
    const int a = vstart[gi], b = vstart[gi + 1];
    if (b <= a) return fail(c, FSGC_EINVAL, "member graph %d is empty", gi);
    int maxd = 0;
    for (int v = a; v < b; v++) {
      comp[v] = gi;
      if (nindex[v + 1] < nindex[v]) return fail(c, FSGC_EINVAL, "offsets decrease at vertex %d", v);
      maxd = std::max(maxd, (int)(nindex[v + 1] - nindex[v]));
      for (int64_t j = nindex[v]; j < nindex[v + 1]; j++)
        if (nlist[j] < a || nlist[j] >= b) return fail(c, FSGC_EINVAL, "edge %d-%d crosses member graphs", v, nlist[j]);
    }
    mn[gi] = b - a;
    mm[gi] = nindex[b] - nindex[a];
    // the triangle core's relabel gate, per member (src/fringeCount.cu:1237, 1342-1344)
    relabel[gi] = (mn[gi] > 10000) && !((long long)mn[gi] > mm[gi] / 10) && (maxd > 16);
  }
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  DevGraph* g = nullptr;
  int st = upload_graph(c, n, m, (const long long*)nindex, nlist, false, &g);
  if (st != FSGC_OK) return st;
  cudaError_t e = cudaMalloc((void**)&g->comp, sizeof(int) * (size_t)n);
  if (e == cudaSuccess) e = cudaMalloc((void**)&g->comp_relabel, (size_t)ngraphs);
  if (e == cudaSuccess) e = cudaMemcpyAsync(g->comp, comp.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(g->comp_relabel, relabel.data(), (size_t)ngraphs, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    free_graph(g);
    return cuda_fail(c, e, "packed graph upload");
  }
  g->ngraphs = ngraphs;
  g->member_n = mn;
  g->member_m = mm;
  g->bytes += sizeof(int) * (size_t)n + (size_t)ngraphs;
  *gid = c->next_gid++;
  c->graphs[*gid] = g;
  return FSGC_OK;
}

int fsgc_count_packed(fsgc_ctx* c, int gid, const fsgc_matching_order* mo, fsgc_result* results) {
  if (!c || !mo || !results) return fail(c, FSGC_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  DevGraph* g = find_graph(c, gid);
  if (!g) return fail(c, FSGC_ENOTFOUND, "unknown graph %d", gid);
  if (g->ngraphs == 0) return fail(c, FSGC_EINVAL, "graph %d is not packed", gid);
  if (!mo_valid(*mo)) return fail(c, FSGC_EINVAL, "malformed matching order");
  const int ng = g->ngraphs;
  // pattern size (vertices, directed entries) for the per-member early return
  long long pn = mo->nodes, pm = 0;
  for (int i = 0; i + 1 < mo->nodes; i++) pm += 2 * __builtin_popcount(mo->list[i]);
  for (int i = 0; i < mo->anchorsets; i++) {
    pn += mo->fcnt[i];
    pm += 2LL * mo->fcnt[i] * __builtin_popcount(mo->anch[i]);
  }
  bool any_fits = false;
  for (int i = 0; i < ng; i++) any_fits = any_fits || !(pn > g->member_n[i] || pm > g->member_m[i]);
  u64 aut = 1;
  if (mo->nodes >= 3 && any_fits) {
    const int st = automorphisms(c, *mo, &aut, c->exact_placements);
    if (st != FSGC_OK) return st;
  }
  if (ng > c->member_cap) {
    cudaStreamSynchronize(c->stream);
    cudaFree(c->d_member);
    cudaFreeHost(c->h_member);
    c->d_member = nullptr;
    c->h_member = nullptr;
    c->member_cap = 0;
    CK(cudaMalloc((void**)&c->d_member, sizeof(u64) * (size_t)ng), "member slots");
    CK(cudaMallocHost((void**)&c->h_member, sizeof(u64) * (size_t)ng), "member slots");
    c->member_cap = ng;
  }
  int st = ensure_events(c, 2);
  if (st != FSGC_OK) return st;
  st = ensure_slots(c, 1);
  if (st != FSGC_OK) return st;
  CK(cudaMemsetAsync(c->d_member, 0, sizeof(u64) * (size_t)ng, c->stream), "slot reset");
  CK(cudaEventRecord(c->events[0], c->stream), "event");
  fsgc::CountJob job{mo, g, c->d_slots, 0, 0, false, c->exact_placements, c->d_member, 1};
  if (any_fits) {
    st = fsgc::enqueue_count(job, c->stream, &c->launches, c->work);
    if (st != FSGC_OK) {
      cudaStreamSynchronize(c->stream);
      return fail(c, st, "packed count failed (%s)", cudaGetErrorString(cudaGetLastError()));
    }
  } else {
    job.core_type = mo->nodes == 1 ? FSGC_CORE_VERTEX : mo->nodes == 2 ? FSGC_CORE_EDGE
                   : mo->nodes == 3 ? ((__builtin_popcount(mo->list[1]) == 1) ? FSGC_CORE_WEDGE : FSGC_CORE_TRIANGLE)
                   : FSGC_CORE_GENERAL;
  }
  CK(cudaEventRecord(c->events[1], c->stream), "event");
  CK(cudaMemcpyAsync(c->h_member, c->d_member, sizeof(u64) * (size_t)ng, cudaMemcpyDeviceToHost, c->stream), "readback");
  CK(cudaStreamSynchronize(c->stream), "packed count");
  st = fsgc::take_kernel_error(c->work, c->stream);
  if (st != FSGC_OK) return fail(c, st, "a counting kernel gave up a bounded wait; the counts are void");
  float ms = 0;
  cudaEventElapsedTime(&ms, c->events[0], c->events[1]);
  for (int i = 0; i < ng; i++) {
    fsgc_result& r = results[i];
    memset(&r, 0, sizeof(r));
    r.core_type = job.core_type;
    r.device_ms = ms;
    if (mo->nodes >= 3 && (pn > g->member_n[i] || pm > g->member_m[i])) {
      r.flags = FSGC_FLAG_PATTERN_TOO_LARGE;
      continue;
    }
    u64 raw;
    if (job.host_only) raw = (mo->anchorsets == 0) ? (u64)g->member_n[i] : (u64)(g->member_m[i] / 2);
    else raw = c->h_member[i] / (u64)job.per_member_div;
    r.raw_total = raw;
    r.automorphisms = aut;
    r.count = raw / aut;
  }
  return FSGC_OK;
}

int fsgc_graph_prepare(fsgc_ctx* c, int gid) {
  if (!c) return FSGC_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  DevGraph* g = find_graph(c, gid);
  if (!g) return fail(c, FSGC_ENOTFOUND, "unknown graph %d", gid);
  const int st = fsgc::prepare_graph(*g, c->stream, &c->launches, c->work.small);
  if (st != FSGC_OK) return fail(c, st, "graph preparation failed: %s", cudaGetErrorString(cudaGetLastError()));
  return FSGC_OK;
}

int fsgc_graph_prepare_all(fsgc_ctx* c, int gid) {
  if (!c) return FSGC_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  DevGraph* g = find_graph(c, gid);
  if (!g) return fail(c, FSGC_ENOTFOUND, "unknown graph %d", gid);
  const int st = fsgc::prepare_all(*g, c->stream, &c->launches, c->work);
  if (st != FSGC_OK) return fail(c, st, "graph preparation failed: %s", cudaGetErrorString(cudaGetLastError()));
  return FSGC_OK;
}

int fsgc_graph_info_get(fsgc_ctx* c, int gid, fsgc_graph_info* out) {
  if (!c || !out) return FSGC_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  DevGraph* g = find_graph(c, gid);
  if (!g) return fail(c, FSGC_ENOTFOUND, "unknown graph %d", gid);
  out->n = g->n;
  out->m = g->m;
  out->max_degree = g->maxdeg;
  out->triangles = g->prepared ? g->triangles : -1;
  out->device_bytes = (int64_t)g->bytes;
  return FSGC_OK;
}

int fsgc_count_exact(fsgc_ctx* c, int gid, const fsgc_matching_order* mo, fsgc_exact_result* out) {
  if (!c || !mo || !out) return fail(c, FSGC_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  memset(out, 0, sizeof(*out));
  if (!mo_valid(*mo)) return fail(c, FSGC_EINVAL, "malformed matching order");
  DevGraph* g = find_graph(c, gid);
  if (!g) return fail(c, FSGC_ENOTFOUND, "unknown graph %d", gid);
  if (g->ngraphs > 0) return fail(c, FSGC_EUNSUPPORTED, "exact counts of packed graphs are not supported");
  if (pattern_too_large(*mo, *g)) {
    out->flags = FSGC_FLAG_PATTERN_TOO_LARGE;
    out->core_type = (mo->nodes == 3) ? ((__builtin_popcount(mo->list[1]) == 1) ? FSGC_CORE_WEDGE : FSGC_CORE_TRIANGLE)
                                      : FSGC_CORE_GENERAL;
    return FSGC_OK;
  }
  // the divisor is the pattern counted in itself with exact placements (small, exact in u64)
  u64 aut = 1;
  int st = FSGC_OK;
  if (mo->nodes >= 3) {
    st = automorphisms(c, *mo, &aut, 1);
    if (st != FSGC_OK) return st;
  }
  st = ensure_slots(c, 3);
  if (st != FSGC_OK) return st;
  st = ensure_events(c, 2);
  if (st != FSGC_OK) return st;
  CK(cudaMemsetAsync(c->d_slots, 0, 3 * sizeof(u64), c->stream), "slot reset");
  CK(cudaEventRecord(c->events[0], c->stream), "event");
  fsgc::CountJob job{mo, g, c->d_slots, 0, 0, false, 1, nullptr, 1};
  job.exact_count = true;
  st = fsgc::enqueue_count(job, c->stream, &c->launches, c->work);
  if (st != FSGC_OK) {
    cudaStreamSynchronize(c->stream);
    return fail(c, st, "exact count failed (%s)", cudaGetErrorString(cudaGetLastError()));
  }
  CK(cudaEventRecord(c->events[1], c->stream), "event");
  CK(cudaMemcpyAsync(c->h_slots, c->d_slots, 3 * sizeof(u64), cudaMemcpyDeviceToHost, c->stream), "readback");
  CK(cudaStreamSynchronize(c->stream), "exact count");
  st = fsgc::take_kernel_error(c->work, c->stream);
  if (st != FSGC_OK) return fail(c, st, "a counting kernel gave up a bounded wait; the count is void");
  unsigned __int128 raw;
  bool sat = false;
  if (job.host_only) {
    raw = job.host_value;
  } else {
    raw = ((unsigned __int128)c->h_slots[1] << 64) | c->h_slots[0];
    sat = c->h_slots[2] != 0 || raw == ~(unsigned __int128)0;
  }
  out->core_type = job.core_type;
  out->automorphisms = aut;
  float ms = 0;
  cudaEventElapsedTime(&ms, c->events[0], c->events[1]);
  out->device_ms = ms;
  if (sat) {
    out->flags |= FSGC_FLAG_SATURATED;
    out->raw_lo = out->raw_hi = out->count_lo = out->count_hi = ~0ULL;
    return FSGC_OK;
  }
  const unsigned __int128 q = raw / aut;
  out->raw_lo = (u64)raw;
  out->raw_hi = (u64)(raw >> 64);
  out->count_lo = (u64)q;
  out->count_hi = (u64)(q >> 64);
  return FSGC_OK;
}

int fsgc_count(fsgc_ctx* c, int gid, const fsgc_matching_order* mo, fsgc_result* out) {
  if (!c || !mo || !out) return fail(c, FSGC_EINVAL, "null argument");
  fsgc_task t;
  t.gid = gid;
  t.mo = *mo;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  return count_tasks(c, &t, 1, out);
}

int fsgc_count_batch(fsgc_ctx* c, const fsgc_task* tasks, int ntasks, fsgc_result* results) {
  if (!c || ntasks < 0 || (ntasks > 0 && (!tasks || !results))) return fail(c, FSGC_EINVAL, "bad batch arguments");
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  return count_tasks(c, tasks, ntasks, results);
}

// Many patterns on one graph in shared passes.  The first call with a given
// (graph, matching orders) runs the launches directly and builds whatever the
// graph still lacks; the second captures the launch sequence into a CUDA
// graph; later calls replay it (one launch of the whole set) while the slot
// array and the work arena stay where they were at capture.
int fsgc_count_set(fsgc_ctx* c, int gid, const fsgc_matching_order* mos, int n, fsgc_result* results) {
  if (!c || n < 0 || (n > 0 && (!mos || !results))) return fail(c, FSGC_EINVAL, "bad pattern-set arguments");
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  if (n == 0) return FSGC_OK;
  DevGraph* g = find_graph(c, gid);
  if (!g) return fail(c, FSGC_ENOTFOUND, "unknown graph %d", gid);
  if (g->ngraphs > 0) return fail(c, FSGC_EINVAL, "graph %d is packed; use fsgc_count_packed", gid);
  std::vector<fsgc_task> tasks((size_t)n);
  for (int t = 0; t < n; t++) {
    tasks[t].gid = gid;
    tasks[t].mo = mos[t];
    memset(&results[t], 0, sizeof(fsgc_result));
  }
  std::vector<u64> aut;
  int st = plan_tasks(c, tasks.data(), n, aut);
  if (st != FSGC_OK) return st;
  st = ensure_slots(c, n);
  if (st != FSGC_OK) return st;
  st = ensure_events(c, 2);
  if (st != FSGC_OK) return st;
  std::vector<fsgc::CountJob> jobs((size_t)n);
  std::vector<fsgc::CountJob*> run;
  for (int t = 0; t < n; t++) {
    jobs[t] = fsgc::CountJob{&tasks[t].mo, g, c->d_slots + t, 0, 0, false, c->exact_placements, nullptr, 1};
    if (pattern_too_large(tasks[t].mo, *g)) {
      jobs[t].host_only = true;
      jobs[t].core_type = (tasks[t].mo.nodes == 3)
                              ? ((__builtin_popcount(tasks[t].mo.list[1]) == 1) ? FSGC_CORE_WEDGE : FSGC_CORE_TRIANGLE)
                              : FSGC_CORE_GENERAL;
      results[t].flags |= FSGC_FLAG_PATTERN_TOO_LARGE;
    } else {
      run.push_back(&jobs[t]);
    }
  }
  std::string key(reinterpret_cast<const char*>(&gid), sizeof(gid));
  key.append(reinterpret_cast<const char*>(mos), sizeof(fsgc_matching_order) * (size_t)n);
  key.push_back(c->exact_placements ? 'x' : 'r');
  CK(cudaMemsetAsync(c->d_slots, 0, sizeof(u64) * (size_t)n, c->stream), "slot reset");
  CK(cudaEventRecord(c->events[0], c->stream), "event");
  auto it = c->set_graphs.find(key);
  if (it != c->set_graphs.end() &&
      (it->second.slot_gen != c->slot_gen || it->second.arena_gen != c->work.tri.gen)) {
    cudaGraphExecDestroy(it->second.exec);
    c->set_graphs.erase(it);
    it = c->set_graphs.end();
  }
  if (it != c->set_graphs.end()) {
    // the plan's host-side fields (core types, host values) as at capture
    for (int t = 0; t < n; t++) {
      if (jobs[t].host_only) continue;  // too large for the graph: decided above
      jobs[t].core_type = it->second.plan[t].core_type;
      jobs[t].host_only = it->second.plan[t].host_only;
      jobs[t].host_value = it->second.plan[t].host_value;
    }
    CK(cudaGraphLaunch(it->second.exec, c->stream), "pattern-set replay");
    c->launches += 1;
  } else if (c->set_seen[key]++ > 0) {
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "capture");
    uint64_t launches = 0;
    st = fsgc::enqueue_count_set(run, c->stream, &launches, c->work);
    const cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
    if (st != FSGC_OK || ce != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      cudaGetLastError();
      return fail(c, st != FSGC_OK ? st : FSGC_ECUDA, "capturing the pattern set failed");
    }
    cudaGraphExec_t exec = nullptr;
    const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) return cuda_fail(c, ie, "instantiating the pattern set");
    c->set_graphs[key] = fsgc_ctx::SetGraph{gid, c->slot_gen, c->work.tri.gen, exec, jobs};
    CK(cudaGraphLaunch(exec, c->stream), "pattern-set launch");
    c->launches += launches;
  } else {
    st = fsgc::enqueue_count_set(run, c->stream, &c->launches, c->work);
    if (st != FSGC_OK) {
      cudaStreamSynchronize(c->stream);
      return fail(c, st, "pattern-set count failed (%s)", cudaGetErrorString(cudaGetLastError()));
    }
  }
  CK(cudaEventRecord(c->events[1], c->stream), "event");
  CK(cudaMemcpyAsync(c->h_slots, c->d_slots, sizeof(u64) * (size_t)n, cudaMemcpyDeviceToHost, c->stream), "readback");
  CK(cudaStreamSynchronize(c->stream), "pattern-set count");
  st = fsgc::take_kernel_error(c->work, c->stream);
  if (st != FSGC_OK) return fail(c, st, "a counting kernel gave up a bounded wait; the counts are void");
  float ms = 0;
  cudaEventElapsedTime(&ms, c->events[0], c->events[1]);
  for (int t = 0; t < n; t++) {
    fsgc_result& r = results[t];
    const bool too_large = (r.flags & FSGC_FLAG_PATTERN_TOO_LARGE) != 0;
    const u64 raw = jobs[t].host_only ? jobs[t].host_value : c->h_slots[t];
    r.raw_total = too_large ? 0 : raw;
    r.automorphisms = too_large ? 0 : aut[t];
    r.count = too_large ? 0 : raw / aut[t];
    r.core_type = jobs[t].core_type;
    r.device_ms = ms / n;
  }
  return FSGC_OK;
}

// ---- lanes: asynchronous counts on their own streams.  The context lock is
// held while a submission is checked and enqueued, never while it runs, so
// submissions on different lanes overlap on the device.
int fsgc_lane_create(fsgc_ctx* c, fsgc_lane** out) {
  if (!c || !out) return FSGC_EINVAL;
  *out = nullptr;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  fsgc_lane* L = new fsgc_lane();
  L->ctx = c;
  cudaError_t e = cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc((void**)&L->work.small, 32 * sizeof(u64));
  if (e == cudaSuccess) e = cudaMallocHost((void**)&L->work.h_err, sizeof(u64));
  if (e == cudaSuccess) *L->work.h_err = 0;
  if (e == cudaSuccess) e = cudaMemsetAsync(L->work.small, 0, 32 * sizeof(u64), L->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(L->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    fsgc_lane_destroy(L);
    return cuda_fail(c, e, "lane creation");
  }
  *out = L;
  return FSGC_OK;
}

void fsgc_lane_destroy(fsgc_lane* L) {
  if (!L) return;
  cudaSetDevice(L->ctx->device);
  if (L->stream) cudaStreamSynchronize(L->stream);
  for (auto e : L->events) cudaEventDestroy(e);
  cudaFree(L->work.small);
  cudaFreeHost(L->work.h_err);
  cudaFree(L->work.tri.ptr);
  cudaFree(L->d_slots);
  cudaFreeHost(L->h_slots);
  if (L->stream) cudaStreamDestroy(L->stream);
  delete L;
}

int fsgc_lane_submit(fsgc_lane* L, const fsgc_task* tasks, int ntasks) {
  if (!L || ntasks < 1 || !tasks) return FSGC_EINVAL;
  fsgc_ctx* c = L->ctx;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  if (L->pending > 0) return fail(c, FSGC_EBUSY, "lane has a submission in flight");
  L->work.tune = c->work.tune;  // the context's method thresholds
  L->tasks.assign(tasks, tasks + ntasks);
  int st = plan_tasks(c, L->tasks.data(), ntasks, L->aut);
  if (st != FSGC_OK) return st;
  // one-time per-graph structures are built on the context's stream before
  // any lane reads them
  for (int t = 0; t < ntasks; t++) {
    DevGraph* g = find_graph(c, L->tasks[t].gid);
    if (pattern_too_large(L->tasks[t].mo, *g)) continue;
    st = fsgc::prepare_for_count(L->tasks[t].mo, *g, c->stream, &c->launches, c->work);
    if (st != FSGC_OK) return fail(c, st, "graph preparation failed: %s", cudaGetErrorString(cudaGetLastError()));
  }
  if (ntasks > L->cap) {
    cudaStreamSynchronize(L->stream);
    cudaFree(L->d_slots);
    cudaFreeHost(L->h_slots);
    L->d_slots = nullptr;
    L->h_slots = nullptr;
    L->cap = 0;
    CK(cudaMalloc((void**)&L->d_slots, sizeof(u64) * (size_t)ntasks), "lane slots");
    CK(cudaMallocHost((void**)&L->h_slots, sizeof(u64) * (size_t)ntasks), "lane slots");
    L->cap = ntasks;
  }
  while (L->events.size() < (size_t)ntasks + 1) {
    cudaEvent_t e;
    CK(cudaEventCreateWithFlags(&e, cudaEventBlockingSync), "event creation");
    L->events.push_back(e);
  }
  L->res.assign((size_t)ntasks, fsgc_result{});
  st = enqueue_tasks(c, L->tasks.data(), ntasks, L->stream, L->work, L->d_slots, L->h_slots, L->events.data(),
                     L->jobs, L->res.data(), true);
  if (st != FSGC_OK) return st;
  L->pending = ntasks;
  L->finished = 0;
  return FSGC_OK;
}

int fsgc_lane_wait_task(fsgc_lane* L, int index, fsgc_result* out) {
  if (!L) return FSGC_EINVAL;
  if (L->pending <= 0 || index < L->finished || index >= L->pending) return FSGC_ENOTFOUND;
  cudaSetDevice(L->ctx->device);
  // the host thread sleeps until the task's closing event (blocking-sync event)
  const cudaError_t e = cudaEventSynchronize(L->events[(size_t)index + 1]);
  if (e != cudaSuccess) {
    L->pending = 0;
    std::lock_guard<std::mutex> lk(L->ctx->mu);
    return cuda_fail(L->ctx, e, "lane count");
  }
  if (L->work.h_err && *L->work.h_err) {
    // a kernel of this submission gave up a bounded wait: its counts are void
    L->pending = 0;
    fsgc::take_kernel_error(L->work, L->stream);
    std::lock_guard<std::mutex> lk(L->ctx->mu);
    return fail(L->ctx, FSGC_ETIMEDOUT, "a counting kernel gave up a bounded wait; the counts are void");
  }
  for (int t = L->finished; t <= index; t++) finish_task(t, L->jobs, L->aut, L->h_slots, L->events.data(), L->res.data());
  L->finished = index + 1;
  if (out) *out = L->res[(size_t)index];
  if (L->finished == L->pending) L->pending = 0;  // the lane is free again
  return FSGC_OK;
}

int fsgc_lane_wait(fsgc_lane* L, fsgc_result* results) {
  if (!L) return FSGC_EINVAL;
  if (L->pending <= 0) return FSGC_ENOTFOUND;
  const int nt = L->pending;
  const int st = fsgc_lane_wait_task(L, nt - 1, nullptr);
  if (st != FSGC_OK) return st;
  if (results) memcpy(results, L->res.data(), sizeof(fsgc_result) * (size_t)nt);
  return FSGC_OK;
}

int fsgc_lane_query(fsgc_lane* L) {
  if (!L) return FSGC_EINVAL;
  if (L->pending <= 0) return FSGC_ENOTFOUND;
  const cudaError_t e = cudaEventQuery(L->events[(size_t)L->pending]);  // the last task's closing event
  if (e == cudaErrorNotReady) return FSGC_EBUSY;
  return e == cudaSuccess ? FSGC_OK : FSGC_ECUDA;
}

size_t fsgc_lane_scratch_bytes(const fsgc_lane* L) { return L ? L->work.tri.bytes : 0; }

int fsgc_lane_trim(fsgc_lane* L) {
  if (!L) return FSGC_EINVAL;
  if (L->pending > 0) return FSGC_EBUSY;
  if (L->work.tri.ptr) {
    cudaSetDevice(L->ctx->device);
    cudaFreeAsync(L->work.tri.ptr, L->stream);
    L->work.tri.ptr = nullptr;
    L->work.tri.bytes = 0;
  }
  return FSGC_OK;
}

int fsgc_task_footprint(fsgc_ctx* c, const fsgc_task* task, size_t* bytes) {
  if (!c || !task || !bytes) return FSGC_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  *bytes = 0;
  if (!mo_valid(task->mo)) return fail(c, FSGC_EINVAL, "malformed matching order");
  DevGraph* g = find_graph(c, task->gid);
  if (!g) return fail(c, FSGC_ENOTFOUND, "unknown graph %d", task->gid);
  if (g->ngraphs > 0) return fail(c, FSGC_EINVAL, "graph %d is packed", task->gid);
  if (pattern_too_large(task->mo, *g) || task->mo.nodes < 2) return FSGC_OK;
  const int st = fsgc::prepare_graph(*g, c->stream, &c->launches, c->work.small);
  if (st != FSGC_OK) return fail(c, st, "graph preparation failed: %s", cudaGetErrorString(cudaGetLastError()));
  *bytes = fsgc::count_scratch_bytes(task->mo, *g, c->work.tune);
  return FSGC_OK;
}

// Host evaluation of the device binomial (same magic-number division) so that
// the arithmetic can be checked without a GPU.
unsigned long long fsgc_nck_host(int n, int k) {
  static fsgc::DivMagic tab[fsgc::kMaxDiv];
  static bool init = false;
  if (!init) {
    for (int d = 2; d < fsgc::kMaxDiv; d++) tab[d] = fsgc::make_div_magic((unsigned)d);
    init = true;
  }
  return fsgc::nck_ref(n, k, tab);
}

// Host evaluation of the exact 128-bit arithmetic of the counting kernels (the
// same __host__ __device__ code), for tests without a GPU: op 0 = a + b,
// 1 = a * b, 2 = C(n, k).  out = (lo, hi, saturated).
void fsgc_x128_host(int op, unsigned long long a_lo, unsigned long long a_hi, unsigned long long b_lo,
                    unsigned long long b_hi, int n, int k, unsigned long long* out) {
  const fsgc::X128 a(a_lo, a_hi), b(b_lo, b_hi);
  const fsgc::X128 r = (op == 0) ? a + b : (op == 1) ? a * b : fsgc::nck_x(n, k);
  out[0] = r.lo;
  out[1] = r.hi;
  out[2] = r.is_saturated() ? 1 : 0;
}

// Host evaluation of the wedge-pair formula (the same __host__ __device__
// code as the kernels) with the general binomials (k01 = 0) or the k <= 1
// form the kernels take when every fringe count is 0 or 1 (k01 = 1), in u64
// (exact = 0) or exact 128-bit arithmetic (exact = 1).  out = (lo, hi).
void fsgc_wedge_formula_host(int dx, int dy, int adj, int f_x, int f_xy, int f_y, int c, int k01, int exact,
                             unsigned long long* out) {
  static fsgc::DivMagic tab[fsgc::kMaxDiv];
  static bool init = false;
  if (!init) {
    for (int d = 2; d < fsgc::kMaxDiv; d++) tab[d] = fsgc::make_div_magic((unsigned)d);
    init = true;
  }
  if (exact) {
    const fsgc::X128 r =
        k01 ? fsgc::wedge_formula_with<fsgc::X128>(dx, dy, adj != 0, f_x, f_xy, f_y, c,
                                                   [](int n, int k) { return fsgc::X128(fsgc::nck01(n, k)); })
            : fsgc::wedge_formula_with<fsgc::X128>(dx, dy, adj != 0, f_x, f_xy, f_y, c,
                                                   [](int n, int k) { return fsgc::nck_x(n, k); });
    out[0] = r.lo;
    out[1] = r.hi;
  } else {
    out[0] = k01 ? fsgc::wedge_formula_with<uint64_t>(dx, dy, adj != 0, f_x, f_xy, f_y, c,
                                                      [](int n, int k) { return (uint64_t)fsgc::nck01(n, k); })
                 : fsgc::wedge_formula_with<uint64_t>(dx, dy, adj != 0, f_x, f_xy, f_y, c,
                                                      [](int n, int k) { return (uint64_t)fsgc::nck_ref(n, k, tab); });
    out[1] = 0;
  }
}

unsigned long long fsgc_div_small_host(unsigned long long x, unsigned d) {
  if (d < 2 || d >= (unsigned)fsgc::kMaxDiv) return 0;
  return fsgc::div_magic(x, fsgc::make_div_magic(d));
}

}  // extern "C"
