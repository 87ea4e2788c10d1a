// Drop-in `fringeCount <graph.egr> <motif.mo>` (src/fringeCount.cu:2265-2331 of
// the reference).  Keeps the reference's tooling lines: `runtime: %.6f s`
// (the count itself, after the graph is resident, as the reference times
// occurrences()) and `%lld occurrences`.
#include <chrono>
#include <cstdio>
#include <cstdlib>

#include "fsgc.h"

int main(int argc, char* argv[]) {
  printf("GPU Fringe Counting (fsgc, GB300-native)\n\n");
  if (argc != 3) {
    printf("USAGE: %s input_graph motif_matching_order\n", argv[0]);
    return -1;
  }
  fsgc_ctx* ctx = nullptr;
  int st = fsgc_ctx_create(0, &ctx);
  if (st != FSGC_OK) {
    fprintf(stderr, "ERROR: no usable CUDA device (%d)\n\n", st);
    return -1;
  }
  int gid = 0;
  st = fsgc_graph_load_egr(ctx, argv[1], &gid);
  if (st != FSGC_OK) {
    fprintf(stderr, "ERROR: %s\n\n", fsgc_ctx_last_error(ctx));
    fsgc_ctx_destroy(ctx);
    return -1;
  }
  fsgc_graph_info info;
  fsgc_graph_info_get(ctx, gid, &info);
  printf("input: %s\n", argv[1]);
  printf("nodes: %d\n", info.n);
  printf("edges: %lld (%lld)\n\n", (long long)(info.m / 2), (long long)info.m);
  fsgc_matching_order mo;
  FILE* f = fopen(argv[2], "rb");
  const size_t size = f ? fread(&mo, 1, sizeof(mo), f) : 0;
  if (f) fclose(f);
  if (size != sizeof(mo)) {
    fprintf(stderr, "ERROR: could not read matching order from file\n");
    fsgc_ctx_destroy(ctx);
    return -1;
  }
  const auto t0 = std::chrono::steady_clock::now();
  fsgc_result r;
  st = fsgc_count(ctx, gid, &mo, &r);
  const double runtime = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (st != FSGC_OK) {
    fprintf(stderr, "ERROR: %s\n\n", fsgc_ctx_last_error(ctx));
    fsgc_ctx_destroy(ctx);
    return -1;
  }
  static const char* names[] = {"?", "vertex core", "edge core", "wedge core", "triangle core", "general core"};
  printf("%s\n", names[(r.core_type >= 1 && r.core_type <= 5) ? r.core_type : 0]);
  if (r.core_type >= 3) printf("automorphisms: %llu\n", (unsigned long long)r.automorphisms);
  printf("runtime: %.6f s\n", runtime);
  printf("%lld occurrences\n\n", (long long)r.count);
  fsgc_ctx_destroy(ctx);
  return 0;
}
