// Drives csrc/server.cpp over the host-only fake lanes (TEST INFRASTRUCTURE).
// Exits non-zero with a message at the first failed check.
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <thread>
#include <vector>

#include "fsgc.h"

extern "C" {
fsgc_ctx* sim_ctx_create();
void sim_ctx_destroy(fsgc_ctx* c);
void sim_ctx_peaks(fsgc_ctx* c, size_t* peak_bytes, int* peak_busy);
}

#define CHECK(cond, ...)                                        \
  do {                                                          \
    if (!(cond)) {                                              \
      fprintf(stderr, "FAIL %s:%d: ", __FILE__, __LINE__);      \
      fprintf(stderr, __VA_ARGS__);                             \
      fprintf(stderr, "\n");                                    \
      exit(1);                                                  \
    }                                                           \
  } while (0)

static fsgc_matching_order order(int nodes, int tag) {
  fsgc_matching_order mo;
  memset(&mo, 0, sizeof(mo));
  mo.nodes = (uint8_t)nodes;
  mo.anch[0] = (uint8_t)tag;  // distinguishes cache keys
  return mo;
}

int main() {
  const size_t MiB = (size_t)1 << 20;
  fsgc_ctx* ctx = sim_ctx_create();

  // 1. concurrent clients, 3 lanes, a 16 MiB budget (arenas of 1-8 MiB per
  //    query): every count right, the lanes' arenas never above the budget,
  //    lanes counting at once
  {
    fsgc_server* srv = nullptr;
    CHECK(fsgc_server_create(ctx, 16 * MiB, 3, 4, &srv) == FSGC_OK, "create");
    for (int g = 1; g <= 9; g++) CHECK(fsgc_server_add_graph(srv, g) == FSGC_OK, "add_graph %d", g);
    CHECK(fsgc_server_add_graph(srv, 1000) == FSGC_ENOTFOUND, "unknown graph registered");
    const int nq = 240;
    std::atomic<int> bad{0};
    std::vector<std::thread> th;
    for (int t = 0; t < 4; t++) {
      th.emplace_back([&, t] {
        std::mt19937 rng(100 + t);
        for (int k = t; k < nq; k += 4) {
          const int gid = 1 + (int)(rng() % 8), nodes = 1 + (int)(rng() % 5), tag = (int)(rng() % 6);
          const fsgc_matching_order mo = order(nodes, tag);
          uint64_t ticket = 0;
          if (fsgc_server_submit(srv, gid, &mo, &ticket) != FSGC_OK) { bad++; continue; }
          fsgc_result r;
          double ms = -1;
          if (fsgc_server_wait(srv, ticket, 60.0, &r, &ms) != FSGC_OK) { bad++; continue; }
          if (r.count != (uint64_t)gid * 1000 + nodes || ms < 0) bad++;
        }
      });
    }
    for (auto& x : th) x.join();
    CHECK(bad == 0, "%d wrong or failed queries", bad.load());
    fsgc_server_stats st;
    CHECK(fsgc_server_stats_get(srv, &st) == FSGC_OK, "stats");
    CHECK(st.completed == (uint64_t)nq, "completed %llu", (unsigned long long)st.completed);
    CHECK(st.queued == 0 && st.in_use_bytes <= 16 * MiB, "queued %llu in use %llu", (unsigned long long)st.queued,
          (unsigned long long)st.in_use_bytes);
    CHECK(st.cache_hits > 0 && st.cache_hits < (uint64_t)nq, "cache hits %llu", (unsigned long long)st.cache_hits);
    CHECK(st.p50_ms <= st.p99_ms && st.queries_per_s > 0, "latency stats");
    size_t peak = 0;
    int peak_busy = 0;
    sim_ctx_peaks(ctx, &peak, &peak_busy);
    CHECK(peak <= 16 * MiB, "arenas peaked at %zu bytes, budget %zu", peak, 16 * MiB);
    CHECK(peak_busy >= 2 && peak_busy <= 3, "lanes counting at once: %d", peak_busy);

    // 2. a query larger than the whole budget is refused; malformed ones too
    fsgc_matching_order mo = order(2, 0);
    uint64_t ticket;
    CHECK(fsgc_server_add_graph(srv, 17) == FSGC_OK, "add 17");
    CHECK(fsgc_server_submit(srv, 17, &mo, &ticket) == FSGC_EBUSY, "oversize accepted");
    mo = order(0, 0);
    CHECK(fsgc_server_submit(srv, 1, &mo, &ticket) == FSGC_EINVAL, "malformed accepted");
    mo = order(2, 0);
    CHECK(fsgc_server_submit(srv, 77, &mo, &ticket) == FSGC_ENOTFOUND, "unregistered graph accepted");
    fsgc_server_destroy(srv);
  }

  // 3. one lane, batches: a query that fails when counted fails alone and is
  //    not cached; a repeated query is answered at submission
  {
    fsgc_server* srv = nullptr;
    CHECK(fsgc_server_create(ctx, 64 * MiB, 1, 8, &srv) == FSGC_OK, "create");
    CHECK(fsgc_server_add_graph(srv, 3) == FSGC_OK, "add");
    // occupy the lane so the next three queries form one batch
    fsgc_matching_order slow = order(5, 50), good = order(2, 51), badmo = order(6, 52);
    uint64_t t0, t1, t2, t3;
    CHECK(fsgc_server_submit(srv, 3, &slow, &t0) == FSGC_OK, "submit");
    CHECK(fsgc_server_submit(srv, 3, &good, &t1) == FSGC_OK, "submit");
    CHECK(fsgc_server_submit(srv, 3, &badmo, &t2) == FSGC_OK, "submit");
    CHECK(fsgc_server_submit(srv, 3, &good, &t3) == FSGC_OK, "submit");
    fsgc_result r;
    CHECK(fsgc_server_wait(srv, t0, 10, &r, nullptr) == FSGC_OK && r.count == 3005, "slow");
    CHECK(fsgc_server_wait(srv, t1, 10, &r, nullptr) == FSGC_OK && r.count == 3002, "good");
    CHECK(fsgc_server_wait(srv, t2, 10, &r, nullptr) == FSGC_EINVAL, "bad query did not fail");
    CHECK(fsgc_server_wait(srv, t3, 10, &r, nullptr) == FSGC_OK && r.count == 3002, "good after bad");
    fsgc_server_stats st;
    fsgc_server_stats_get(srv, &st);
    const uint64_t hits = st.cache_hits;
    uint64_t t4, t5;
    CHECK(fsgc_server_submit(srv, 3, &good, &t4) == FSGC_OK, "submit");
    CHECK(fsgc_server_poll(srv, t4, &r, nullptr) == FSGC_OK && r.count == 3002, "cache hit not immediate");
    CHECK(fsgc_server_submit(srv, 3, &badmo, &t5) == FSGC_OK, "submit");
    CHECK(fsgc_server_wait(srv, t5, 10, &r, nullptr) == FSGC_EINVAL, "failure was cached");
    fsgc_server_stats_get(srv, &st);
    CHECK(st.cache_hits == hits + 1, "cache hits %llu vs %llu", (unsigned long long)st.cache_hits,
          (unsigned long long)hits);
    CHECK(fsgc_server_poll(srv, t4, &r, nullptr) == FSGC_ENOTFOUND, "ticket not forgotten");
    // 4. destroy finishes what was submitted
    for (int i = 0; i < 5; i++) {
      fsgc_matching_order mo = order(3, 60 + i);
      uint64_t t;
      CHECK(fsgc_server_submit(srv, 3, &mo, &t) == FSGC_OK, "submit");
    }
    fsgc_server_destroy(srv);
  }

  // 5. a budget of one query: idle lanes holding arenas give them back so the
  //    head of the queue is admitted, one query at a time
  {
    fsgc_server* srv = nullptr;
    CHECK(fsgc_server_create(ctx, 5 * MiB, 4, 2, &srv) == FSGC_OK, "create");
    for (int g = 1; g <= 5; g++) fsgc_server_add_graph(srv, g);
    std::vector<uint64_t> ts;
    for (int i = 0; i < 40; i++) {
      fsgc_matching_order mo = order(1 + i % 3, 70 + i);
      uint64_t t;
      CHECK(fsgc_server_submit(srv, 1 + (i * 7) % 5, &mo, &t) == FSGC_OK, "submit");
      ts.push_back(t);
    }
    for (size_t i = 0; i < ts.size(); i++) {
      fsgc_result r;
      CHECK(fsgc_server_wait(srv, ts[i], 30, &r, nullptr) == FSGC_OK, "query %zu", i);
      CHECK(r.count == (uint64_t)(1 + (i * 7) % 5) * 1000 + 1 + i % 3, "count %zu", i);
    }
    fsgc_server_destroy(srv);
  }
  // 6. a count that fails inside a batch fails alone: the queries after it
  //    run one at a time and keep their own results
  {
    fsgc_server* srv = nullptr;
    CHECK(fsgc_server_create(ctx, 64 * MiB, 1, 8, &srv) == FSGC_OK, "create");
    CHECK(fsgc_server_add_graph(srv, 4) == FSGC_OK, "add");
    fsgc_matching_order slow = order(5, 80), a = order(2, 81), boom = order(3, 82), b = order(1, 83), c = order(4, 84);
    boom.startdeg = 99;
    uint64_t t0, t1, t2, t3, t4;
    CHECK(fsgc_server_submit(srv, 4, &slow, &t0) == FSGC_OK, "submit");
    CHECK(fsgc_server_submit(srv, 4, &a, &t1) == FSGC_OK, "submit");
    CHECK(fsgc_server_submit(srv, 4, &boom, &t2) == FSGC_OK, "submit");
    CHECK(fsgc_server_submit(srv, 4, &b, &t3) == FSGC_OK, "submit");
    CHECK(fsgc_server_submit(srv, 4, &c, &t4) == FSGC_OK, "submit");
    fsgc_result r;
    CHECK(fsgc_server_wait(srv, t0, 10, &r, nullptr) == FSGC_OK && r.count == 4005, "slow");
    CHECK(fsgc_server_wait(srv, t1, 10, &r, nullptr) == FSGC_OK && r.count == 4002, "before the failure");
    CHECK(fsgc_server_wait(srv, t2, 10, &r, nullptr) == FSGC_ECUDA, "the failing count");
    CHECK(fsgc_server_wait(srv, t3, 10, &r, nullptr) == FSGC_OK && r.count == 4001, "after the failure");
    CHECK(fsgc_server_wait(srv, t4, 10, &r, nullptr) == FSGC_OK && r.count == 4004, "after the failure");
    fsgc_server_destroy(srv);
  }

  // 7. registered graphs count against the budget: two 40 MiB graphs do not
  //    fit a 64 MiB budget, and a query needing 30 MiB waits for room beside
  //    the one that does
  {
    fsgc_server* srv = nullptr;
    CHECK(fsgc_server_create(ctx, 64 * MiB, 2, 4, &srv) == FSGC_OK, "create");
    CHECK(fsgc_server_add_graph(srv, 90) == FSGC_OK, "first 40 MiB graph");
    CHECK(fsgc_server_add_graph(srv, 91) == FSGC_EBUSY, "second 40 MiB graph accepted");
    CHECK(fsgc_server_add_graph(srv, 20) == FSGC_OK, "small graph");
    fsgc_matching_order mo = order(2, 90);
    uint64_t t;
    CHECK(fsgc_server_submit(srv, 20, &mo, &t) == FSGC_OK, "submit");
    fsgc_result r;
    CHECK(fsgc_server_wait(srv, t, 10, &r, nullptr) == FSGC_OK && r.count == 20002, "count beside a resident graph");
    fsgc_server_stats st;
    fsgc_server_stats_get(srv, &st);
    CHECK(st.in_use_bytes >= 40 * MiB, "resident bytes not reported");
    fsgc_server_destroy(srv);
  }

  size_t peak = 0;
  int peak_busy = 0;
  sim_ctx_peaks(ctx, &peak, &peak_busy);
  sim_ctx_destroy(ctx);
  printf("PASS serving loop over fake lanes (arena peak %zu bytes)\n", peak);
  return 0;
}
