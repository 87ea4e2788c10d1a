// Host-only stand-ins for the lane and graph calls the serving loop makes
// (TEST INFRASTRUCTURE: linked with csrc/server.cpp to test its admission,
// batching, caching and completion logic without a GPU).
//
// A task on graph `gid` needs a work arena of gid MiB and takes `mo.nodes`
// milliseconds; its count is gid * 1000 + nodes.  A matching order with
// nodes == 6 fails the submission checks; startdeg == 99 passes them and
// fails when its count is waited for; nodes == 0 or > 6 is malformed; graphs
// above 100 do not exist.  The fake records the
// peak sum of the lanes' arenas and the peak number of lanes counting at once.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include "fsgc.h"

using Clock = std::chrono::steady_clock;

struct fsgc_ctx {
  std::mutex mu;
  size_t live = 0, peak = 0;
  int busy = 0, peak_busy = 0;
};

struct fsgc_lane {
  fsgc_ctx* ctx = nullptr;
  size_t scratch = 0;
  std::vector<fsgc_task> tasks;
  std::vector<Clock::time_point> done_at;
  int pending = 0, finished = 0;
};

namespace {
const size_t kMiB = (size_t)1 << 20;
bool malformed(const fsgc_matching_order& mo) { return mo.nodes == 0 || mo.nodes > 6; }
}  // namespace

extern "C" {

fsgc_ctx* sim_ctx_create() { return new fsgc_ctx(); }
void sim_ctx_destroy(fsgc_ctx* c) { delete c; }
void sim_ctx_peaks(fsgc_ctx* c, size_t* peak_bytes, int* peak_busy) {
  std::lock_guard<std::mutex> lk(c->mu);
  *peak_bytes = c->peak;
  *peak_busy = c->peak_busy;
}

int fsgc_graph_prepare(fsgc_ctx*, int gid) { return (gid >= 1 && gid <= 100) ? FSGC_OK : FSGC_ENOTFOUND; }
int fsgc_graph_prepare_all(fsgc_ctx* c, int gid) { return fsgc_graph_prepare(c, gid); }

// Graphs hold no device memory except 90 and 91, which hold 40 MiB each.
int fsgc_graph_info_get(fsgc_ctx*, int gid, fsgc_graph_info* out) {
  if (gid < 1 || gid > 100) return FSGC_ENOTFOUND;
  memset(out, 0, sizeof(*out));
  out->device_bytes = (gid == 90 || gid == 91) ? (int64_t)40 << 20 : 0;
  return FSGC_OK;
}

int fsgc_task_footprint(fsgc_ctx*, const fsgc_task* t, size_t* bytes) {
  if (malformed(t->mo)) return FSGC_EINVAL;
  if (t->gid < 1 || t->gid > 100) return FSGC_ENOTFOUND;
  *bytes = (size_t)t->gid * kMiB;
  return FSGC_OK;
}

int fsgc_lane_create(fsgc_ctx* c, fsgc_lane** out) {
  *out = new fsgc_lane();
  (*out)->ctx = c;
  return FSGC_OK;
}

void fsgc_lane_destroy(fsgc_lane* l) { delete l; }

int fsgc_lane_submit(fsgc_lane* l, const fsgc_task* tasks, int n) {
  if (!l || n < 1) return FSGC_EINVAL;
  if (l->pending) return FSGC_EBUSY;
  size_t need = 0;
  for (int i = 0; i < n; i++) {
    if (malformed(tasks[i].mo) || tasks[i].mo.nodes == 6) return FSGC_EINVAL;
    need = std::max(need, (size_t)tasks[i].gid * kMiB);
  }
  {
    std::lock_guard<std::mutex> lk(l->ctx->mu);
    if (need > l->scratch) {
      l->ctx->live += need - l->scratch;
      l->scratch = need;
      l->ctx->peak = std::max(l->ctx->peak, l->ctx->live);
    }
    l->ctx->busy++;
    l->ctx->peak_busy = std::max(l->ctx->peak_busy, l->ctx->busy);
  }
  l->tasks.assign(tasks, tasks + n);
  l->done_at.clear();
  auto t = Clock::now();
  for (int i = 0; i < n; i++) {
    t += std::chrono::milliseconds(tasks[i].mo.nodes);
    l->done_at.push_back(t);
  }
  l->pending = n;
  l->finished = 0;
  return FSGC_OK;
}

int fsgc_lane_wait_task(fsgc_lane* l, int i, fsgc_result* out) {
  if (!l || l->pending <= 0 || i < l->finished || i >= l->pending) return FSGC_ENOTFOUND;
  std::this_thread::sleep_until(l->done_at[(size_t)i]);
  if (l->tasks[(size_t)i].mo.startdeg == 99) {
    // a count that fails on the device: the submission is abandoned
    l->pending = 0;
    std::lock_guard<std::mutex> lk(l->ctx->mu);
    l->ctx->busy--;
    return FSGC_ECUDA;
  }
  if (out) {
    memset(out, 0, sizeof(*out));
    out->count = out->raw_total = (uint64_t)l->tasks[(size_t)i].gid * 1000 + l->tasks[(size_t)i].mo.nodes;
    out->automorphisms = 1;
  }
  l->finished = i + 1;
  if (l->finished == l->pending) {
    l->pending = 0;
    std::lock_guard<std::mutex> lk(l->ctx->mu);
    l->ctx->busy--;
  }
  return FSGC_OK;
}

int fsgc_lane_wait(fsgc_lane* l, fsgc_result* results) {
  if (!l || l->pending <= 0) return FSGC_ENOTFOUND;
  const int n = l->pending;
  for (int i = l->finished; i < n; i++) {
    const int st = fsgc_lane_wait_task(l, i, results ? &results[i] : nullptr);
    if (st != FSGC_OK) return st;
  }
  return FSGC_OK;
}

size_t fsgc_lane_scratch_bytes(const fsgc_lane* l) { return l ? l->scratch : 0; }

int fsgc_lane_trim(fsgc_lane* l) {
  if (!l || l->pending) return FSGC_EBUSY;
  std::lock_guard<std::mutex> lk(l->ctx->mu);
  l->ctx->live -= l->scratch;
  l->scratch = 0;
  return FSGC_OK;
}

}  // extern "C"
