// graphgen -- TEST INFRASTRUCTURE ONLY.
//
// Writes a seeded RMAT graph as an ECLgraph .egr file (the reference's binary
// CSR layout, src/ECLgraph.h:58-85: int32 n, int32 m, int32 nindex[n+1],
// int32 nlist[m]) without loading the product library, so that the reference's
// own kernels (oracle/ref_runner) can be timed on the same graph as the product
// in a process that never maps libfsgc.
//
// The graph is the product generator's (fsgc_gen_rmat): every edge descends
// `scale` levels and picks a quadrant with one uniform draw per level; draws are
// a splitmix64 hash of (seed, stream 1, 64 * edge + level); self loops are
// dropped, duplicates merged, the result symmetrised with sorted lists.  A CPU
// test requires the two to agree byte for byte.
//
//   graphgen rmat <scale> <edge_factor> <a> <b> <c> <seed> <out.egr>
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <string_view>
#include <vector>
#include <omp.h>
#include <parallel/algorithm>

namespace {

uint64_t mix64(uint64_t x) {
  x += 0x9e3779b97f4a7c15ULL;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
  return x ^ (x >> 31);
}
uint64_t draw(uint64_t seed, uint64_t stream, uint64_t i) { return mix64(mix64(seed ^ mix64(stream)) + i); }
double unit(uint64_t r) { return (double)(r >> 11) * (1.0 / 9007199254740992.0); }

int write_egr(const char* path, int n, const std::vector<int64_t>& idx, const std::vector<int32_t>& adj) {
  if (adj.size() > 2147483647ULL) {
    fprintf(stderr, "graphgen: %zu entries do not fit the int32 .egr layout\n", adj.size());
    return 1;
  }
  FILE* f = fopen(path, "wb");
  if (!f) {
    fprintf(stderr, "graphgen: cannot write %s\n", path);
    return 1;
  }
  const int32_t hn = n, hm = (int32_t)adj.size();
  std::vector<int32_t> i32(idx.begin(), idx.end());
  bool ok = fwrite(&hn, 4, 1, f) == 1 && fwrite(&hm, 4, 1, f) == 1 &&
            fwrite(i32.data(), 4, i32.size(), f) == i32.size() &&
            (adj.empty() || fwrite(adj.data(), 4, adj.size(), f) == adj.size());
  ok = fclose(f) == 0 && ok;
  return ok ? 0 : 1;
}

int rmat(int scale, int ef, double a, double b, double c, uint64_t seed, const char* path) {
  if (scale < 1 || scale > 30 || ef < 1 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0) {
    fprintf(stderr, "graphgen: bad RMAT parameters\n");
    return 1;
  }
  const int n = 1 << scale;
  const int64_t E = (int64_t)ef << scale;
  const double ab = a + b, abc = a + b + c;
  std::vector<uint64_t> und((size_t)E);
#pragma omp parallel for schedule(static)
  for (long long e = 0; e < (long long)E; e++) {
    uint64_t u = 0, v = 0;
    for (int l = 0; l < scale; l++) {
      const double r = unit(draw(seed, 1, (uint64_t)e * 64 + (uint64_t)l));
      const uint64_t bit = 1ULL << (scale - 1 - l);
      if (r >= ab) u |= bit;
      if ((r >= a && r < ab) || r >= abc) v |= bit;
    }
    // undirected pair as (low << 32 | high); loops marked for removal
    und[e] = (u == v) ? ~0ULL : ((std::min(u, v) << 32) | std::max(u, v));
  }
  __gnu_parallel::sort(und.begin(), und.end());
  und.erase(std::unique(und.begin(), und.end()), und.end());
  if (!und.empty() && und.back() == ~0ULL) und.pop_back();
  // both directions, sorted by (source, target)
  std::vector<uint64_t> dir(2 * und.size());
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < (long long)und.size(); i++) {
    const uint64_t lo = und[i] >> 32, hi = und[i] & 0xffffffffULL;
    dir[2 * i] = (lo << 32) | hi;
    dir[2 * i + 1] = (hi << 32) | lo;
  }
  std::vector<uint64_t>().swap(und);
  __gnu_parallel::sort(dir.begin(), dir.end());
  std::vector<int64_t> idx((size_t)n + 1, 0);
  std::vector<int32_t> adj(dir.size());
  for (size_t i = 0; i < dir.size(); i++) {
    idx[(dir[i] >> 32) + 1]++;
    adj[i] = (int32_t)(dir[i] & 0xffffffffULL);
  }
  for (int v = 0; v < n; v++) idx[v + 1] += idx[v];
  return write_egr(path, n, idx, adj);
}

}  // namespace

int main(int argc, char** argv) {
  if (argc == 9 && std::string_view(argv[1]) == "rmat")
    return rmat(atoi(argv[2]), atoi(argv[3]), atof(argv[4]), atof(argv[5]), atof(argv[6]),
                strtoull(argv[7], nullptr, 10), argv[8]);
  fprintf(stderr, "usage: %s rmat <scale> <edge_factor> <a> <b> <c> <seed> <out.egr>\n", argv[0]);
  return 2;
}
