// Serving loop: resident graphs, count queries admitted by memory footprint,
// continuous batching over lanes.
//
// The reference has no serving mode (one fringeCount process per query).  Here
// each of the server's lanes (a CUDA stream of the context with its own work
// arena, see fsgc_lane_*) has a worker thread.  Queries arrive from any thread
// through fsgc_server_submit and wait in arrival order.  A free worker admits
// queries from the head of the queue -- its share of what is waiting, at most
// max_batch -- while the lanes' work arenas, grown to this batch's need, stay
// within the memory budget, submits them to its lane and sleeps until they
// finish, completing each query as soon as its own counts are done.
// Meanwhile the other workers admit and submit what arrives, so work from
// different batches overlaps on the device and no query waits for a batch
// that was already running when it arrived.  A batch the checks refuse is
// re-run one query at a time, so that a bad query fails alone, and when a
// count fails inside a batch the queries after it are re-run one at a time.
// Registering a graph builds every derived structure any count could need
// (orientation, supports, chunk table, per-vertex triangles, per-entry
// supports), so no query builds one under the context lock while other lanes
// wait, and the graph's device bytes count against the budget for as long as
// it is registered, beside the lanes' work arenas.  Latency is
// submission to completion.  Results are cached by (graph, matching-order
// bytes): resident graphs never change and graph ids are never reused, so a
// repeated query completes at submission without device work.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <thread>
#include <vector>

#include "fsgc.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Query {
  uint64_t ticket;
  int gid;
  fsgc_matching_order mo;
  size_t footprint;
  Clock::time_point submitted;
  bool done = false;
  int status = FSGC_OK;
  fsgc_result result{};
  double latency_ms = 0;
};

struct LaneSlot {
  fsgc_lane* lane = nullptr;
  size_t held = 0;  // arena bytes this lane holds or has reserved
  bool busy = false;
};

}  // namespace

struct fsgc_server {
  fsgc_ctx* ctx = nullptr;
  size_t budget = 0;
  size_t resident = 0;    // device bytes of the registered graphs
  size_t held_total = 0;  // sum of LaneSlot::held
  int max_batch = 64;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<uint64_t> waiting;  // admission queue (submission order)
  std::map<uint64_t, Query> queries;
  uint64_t next_ticket = 1;
  bool stop = false;
  std::vector<LaneSlot> lanes;
  std::vector<std::thread> workers;
  std::map<int, int> graphs;  // registered graph ids
  std::map<std::pair<int, std::string>, fsgc_result> cache;  // completed counts
  static constexpr size_t kCacheCap = 1 << 16;               // entries; cleared when full
  uint64_t cache_hits = 0;
  // statistics
  std::vector<double> latencies;
  uint64_t completed = 0, rounds = 0;
  Clock::time_point first_submit, last_done;
  bool any = false;
};

namespace {

// Takes this lane's batch from the head of the queue (server lock held).
// Returns false when nothing fits the budget now.
bool admit(fsgc_server* s, LaneSlot& ls, std::vector<uint64_t>& batch) {
  int idle = 0;
  for (const LaneSlot& l : s->lanes) idle += l.busy ? 0 : 1;
  const size_t share = (s->waiting.size() + (size_t)std::max(1, idle) - 1) / (size_t)std::max(1, idle);
  const size_t take = std::min<size_t>((size_t)s->max_batch, std::max<size_t>(1, share));
  size_t need = 0;
  while (!s->waiting.empty() && batch.size() < take) {
    const Query& q = s->queries[s->waiting.front()];
    const size_t nneed = std::max(need, q.footprint);
    const size_t mine = std::max(ls.held, nneed);
    if (s->resident + s->held_total - ls.held + mine > s->budget) break;
    need = nneed;
    batch.push_back(q.ticket);
    s->waiting.pop_front();
  }
  if (batch.empty()) return false;
  const size_t mine = std::max(ls.held, need);
  s->held_total += mine - ls.held;
  ls.held = mine;
  ls.busy = true;
  return true;
}

void worker_loop(fsgc_server* s, int li) {
  std::vector<uint64_t> batch;
  std::vector<fsgc_task> tasks;
  std::vector<fsgc_result> results;
  std::vector<int> status;
  for (;;) {
    batch.clear();
    {
      std::unique_lock<std::mutex> lk(s->mu);
      LaneSlot& ls = s->lanes[(size_t)li];
      for (;;) {
        if (s->waiting.empty() && s->stop) return;
        if (!s->waiting.empty()) {
          if (admit(s, ls, batch)) break;
          if (ls.held > 0) {
            // the head does not fit: give back this idle lane's arena and let
            // the other idle lanes do the same
            fsgc_lane_trim(ls.lane);
            s->held_total -= ls.held;
            ls.held = 0;
            s->cv_work.notify_all();
            continue;
          }
          // nothing of ours to give back: wake the idle lanes that hold an
          // arena (each either admits the head with it or gives it back);
          // lanes that are counting wake everyone when they finish
          bool others_hold = false;
          for (const LaneSlot& l : s->lanes) others_hold = others_hold || (&l != &ls && !l.busy && l.held > 0);
          if (others_hold) s->cv_work.notify_all();
        }
        s->cv_work.wait(lk);
      }
      tasks.resize(batch.size());
      for (size_t i = 0; i < batch.size(); i++) {
        const Query& q = s->queries[batch[i]];
        tasks[i].gid = q.gid;
        tasks[i].mo = q.mo;
      }
    }
    fsgc_lane* lane = s->lanes[(size_t)li].lane;
    results.assign(batch.size(), fsgc_result{});
    status.assign(batch.size(), FSGC_OK);
    // each query completes as soon as its own counts have finished
    auto complete = [&](size_t i) {
      const auto now = Clock::now();
      {
        std::lock_guard<std::mutex> lk(s->mu);
        Query& q = s->queries[batch[i]];
        q.status = status[i];
        q.result = results[i];
        q.done = true;
        if (q.status == FSGC_OK) {
          if (s->cache.size() >= fsgc_server::kCacheCap) s->cache.clear();
          s->cache[{q.gid, std::string(reinterpret_cast<const char*>(&q.mo), sizeof(q.mo))}] = q.result;
        }
        q.latency_ms = std::chrono::duration<double, std::milli>(now - q.submitted).count();
        s->latencies.push_back(q.latency_ms);
        s->completed++;
        s->last_done = now;
      }
      s->cv_done.notify_all();
    };
    int st = fsgc_lane_submit(lane, tasks.data(), (int)tasks.size());
    if (st == FSGC_OK) {
      size_t i = 0;
      for (; i < batch.size(); i++) {
        status[i] = fsgc_lane_wait_task(lane, (int)i, &results[i]);
        complete(i);
        if (status[i] != FSGC_OK) break;
      }
      // a count failed inside the batch (its submission is abandoned): the
      // queries after it run one at a time, so each gets its own outcome
      for (i = i + 1; i < batch.size(); i++) {
        status[i] = fsgc_lane_submit(lane, &tasks[i], 1);
        if (status[i] == FSGC_OK) status[i] = fsgc_lane_wait(lane, &results[i]);
        complete(i);
      }
    } else if (batch.size() > 1) {
      // a batch the checks refused: each query on its own, so a bad one fails alone
      for (size_t i = 0; i < batch.size(); i++) {
        status[i] = fsgc_lane_submit(lane, &tasks[i], 1);
        if (status[i] == FSGC_OK) status[i] = fsgc_lane_wait(lane, &results[i]);
        complete(i);
      }
    } else {
      status[0] = st;
      complete(0);
    }
    {
      std::lock_guard<std::mutex> lk(s->mu);
      LaneSlot& ls = s->lanes[(size_t)li];
      s->rounds++;
      // Keep the arena for the next batch only while nothing waits: with
      // queries queued, an idle lane holding budget would keep the other lanes
      // from admitting them (the arena is stream-ordered, so regrowing it is cheap).
      if (!s->waiting.empty()) fsgc_lane_trim(lane);
      const size_t real = fsgc_lane_scratch_bytes(lane);
      s->held_total = s->held_total - ls.held + real;
      ls.held = real;
      ls.busy = false;
    }
    s->cv_work.notify_all();
  }
}

double percentile(std::vector<double> v, double p) {
  if (v.empty()) return 0;
  std::sort(v.begin(), v.end());
  const double idx = p * (double)(v.size() - 1);
  const size_t lo = (size_t)idx;
  const size_t hi = std::min(lo + 1, v.size() - 1);
  return v[lo] + (v[hi] - v[lo]) * (idx - (double)lo);
}

}  // namespace

extern "C" {

int fsgc_server_create(fsgc_ctx* ctx, size_t memory_budget, int lanes, int max_batch, fsgc_server** out) {
  if (!ctx || !out || memory_budget == 0 || lanes < 1 || lanes > 64 || max_batch < 1) return FSGC_EINVAL;
  *out = nullptr;
  fsgc_server* s = new fsgc_server();
  s->ctx = ctx;
  s->budget = memory_budget;
  s->max_batch = max_batch;
  s->lanes.resize((size_t)lanes);
  for (int i = 0; i < lanes; i++) {
    const int st = fsgc_lane_create(ctx, &s->lanes[(size_t)i].lane);
    if (st != FSGC_OK) {
      for (int j = 0; j < i; j++) fsgc_lane_destroy(s->lanes[(size_t)j].lane);
      delete s;
      return st;
    }
  }
  for (int i = 0; i < lanes; i++) s->workers.emplace_back(worker_loop, s, i);
  *out = s;
  return FSGC_OK;
}

void fsgc_server_destroy(fsgc_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  for (auto& w : s->workers)
    if (w.joinable()) w.join();
  for (auto& l : s->lanes) fsgc_lane_destroy(l.lane);
  delete s;
}

int fsgc_server_add_graph(fsgc_server* s, int gid) {
  if (!s) return FSGC_EINVAL;
  int st = fsgc_graph_prepare_all(s->ctx, gid);
  if (st != FSGC_OK) return st;
  fsgc_graph_info info;
  st = fsgc_graph_info_get(s->ctx, gid, &info);
  if (st != FSGC_OK) return st;
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->graphs.count(gid)) return FSGC_OK;
  const size_t bytes = (size_t)std::max<int64_t>(0, info.device_bytes);
  if (s->resident + s->held_total + bytes > s->budget) return FSGC_EBUSY;  // does not fit beside what is there
  s->resident += bytes;
  s->graphs[gid] = 1;
  return FSGC_OK;
}

int fsgc_server_submit(fsgc_server* s, int gid, const fsgc_matching_order* mo, uint64_t* ticket) {
  if (!s || !mo || !ticket) return FSGC_EINVAL;
  const auto t0 = Clock::now();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->graphs.find(gid) == s->graphs.end()) return FSGC_ENOTFOUND;
    auto hit = s->cache.find({gid, std::string(reinterpret_cast<const char*>(mo), sizeof(*mo))});
    if (hit != s->cache.end()) {
      Query q;
      q.ticket = s->next_ticket++;
      q.gid = gid;
      q.mo = *mo;
      q.footprint = 0;
      q.submitted = t0;
      q.done = true;
      q.result = hit->second;
      const auto now = Clock::now();
      q.latency_ms = std::chrono::duration<double, std::milli>(now - t0).count();
      if (!s->any) {
        s->first_submit = t0;
        s->any = true;
      }
      s->latencies.push_back(q.latency_ms);
      s->completed++;
      s->cache_hits++;
      s->last_done = now;
      s->queries[q.ticket] = q;
      *ticket = q.ticket;
      return FSGC_OK;
    }
  }
  fsgc_task task;
  task.gid = gid;
  task.mo = *mo;
  size_t fp = 0;
  const int st = fsgc_task_footprint(s->ctx, &task, &fp);
  if (st != FSGC_OK) return st;
  std::lock_guard<std::mutex> lk(s->mu);
  // can never be admitted beside the registered graphs
  if (s->resident + fp > s->budget) return FSGC_EBUSY;
  Query q;
  q.ticket = s->next_ticket++;
  q.gid = gid;
  q.mo = *mo;
  q.footprint = fp;
  q.submitted = t0;
  if (!s->any) {
    s->first_submit = t0;
    s->any = true;
  }
  s->queries[q.ticket] = q;
  s->waiting.push_back(q.ticket);
  *ticket = q.ticket;
  s->cv_work.notify_one();
  return FSGC_OK;
}

static int take_result(fsgc_server* s, uint64_t ticket, fsgc_result* out, double* latency_ms) {
  auto it = s->queries.find(ticket);
  Query& q = it->second;
  const int st = q.status;
  if (out) *out = q.result;
  if (latency_ms) *latency_ms = q.latency_ms;
  s->queries.erase(it);
  return st;
}

int fsgc_server_poll(fsgc_server* s, uint64_t ticket, fsgc_result* out, double* latency_ms) {
  if (!s) return FSGC_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->queries.find(ticket);
  if (it == s->queries.end()) return FSGC_ENOTFOUND;
  if (!it->second.done) return FSGC_EBUSY;
  return take_result(s, ticket, out, latency_ms);
}

int fsgc_server_wait(fsgc_server* s, uint64_t ticket, double timeout_s, fsgc_result* out, double* latency_ms) {
  if (!s) return FSGC_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  auto ready = [&] {
    auto it = s->queries.find(ticket);
    return it == s->queries.end() || it->second.done;
  };
  if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), ready)) return FSGC_ETIMEDOUT;
  if (s->queries.find(ticket) == s->queries.end()) return FSGC_ENOTFOUND;
  return take_result(s, ticket, out, latency_ms);
}

int fsgc_server_stats_get(fsgc_server* s, fsgc_server_stats* out) {
  if (!s || !out) return FSGC_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  memset(out, 0, sizeof(*out));
  out->completed = s->completed;
  out->rounds = s->rounds;
  out->queued = s->waiting.size();
  out->in_use_bytes = s->held_total + s->resident;
  out->cache_hits = s->cache_hits;
  out->p50_ms = percentile(s->latencies, 0.50);
  out->p99_ms = percentile(s->latencies, 0.99);
  if (s->completed > 0 && s->any) {
    const double secs = std::chrono::duration<double>(s->last_done - s->first_submit).count();
    out->queries_per_s = secs > 0 ? (double)s->completed / secs : 0;
  }
  return FSGC_OK;
}

}  // extern "C"
