// Host-side graph handling: ECLgraph binary files, input validation, and seeded
// synthetic generators (RMAT, Erdos-Renyi G(n,m), Chung-Lu).
//
// The ECLgraph layout follows the reference's reader (src/ECLgraph.h:58-85):
// int32 node count, int32 edge count (directed entries), int32 nindex[n+1],
// int32 nlist[m], optionally int32 eweight[m] (ignored, as fringeCount ignores it).
// Graphs of 2^31 or more directed entries do not fit those int32 fields; they
// are written in an extension of the layout: int32 n, int32 -1 (an edge count
// the reference's reader refuses, so such a file is never misread as a
// classic one), int64 m, int64 nindex[n+1], int32 nlist[m].
//
// Generators are counter-based (every random draw is a hash of seed and draw
// index), so they produce identical graphs on any machine and thread count.

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <omp.h>
#include <cuda_runtime.h>

#include "fsgc.h"

namespace {

inline uint64_t mix64(uint64_t x) {  // splitmix64 finaliser
  x += 0x9e3779b97f4a7c15ULL;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
  return x ^ (x >> 31);
}
inline uint64_t draw(uint64_t seed, uint64_t stream, uint64_t i) { return mix64(mix64(seed ^ mix64(stream)) + i); }
inline double unit(uint64_t r) { return (double)(r >> 11) * (1.0 / 9007199254740992.0); }

// Parallel LSD radix sort of 64-bit keys on the low `bits` bits.
void radix_sort(std::vector<uint64_t>& a, int bits) {
  const size_t n = a.size();
  std::vector<uint64_t> b(n);
  const int R = 16, B = 1 << R;
  const int T = omp_get_max_threads();
  std::vector<size_t> hist((size_t)T * B);
  for (int shift = 0; shift < bits; shift += R) {
    std::fill(hist.begin(), hist.end(), 0);
#pragma omp parallel num_threads(T)
    {
      const int t = omp_get_thread_num();
      const size_t lo = n * t / T, hi = n * (t + 1) / T;
      size_t* h = &hist[(size_t)t * B];
      for (size_t i = lo; i < hi; i++) h[(a[i] >> shift) & (B - 1)]++;
    }
    size_t run = 0;
    for (int d = 0; d < B; d++)
      for (int t = 0; t < T; t++) {
        const size_t c = hist[(size_t)t * B + d];
        hist[(size_t)t * B + d] = run;
        run += c;
      }
#pragma omp parallel num_threads(T)
    {
      const int t = omp_get_thread_num();
      const size_t lo = n * t / T, hi = n * (t + 1) / T;
      size_t* h = &hist[(size_t)t * B];
      for (size_t i = lo; i < hi; i++) b[h[(a[i] >> shift) & (B - 1)]++] = a[i];
    }
    a.swap(b);
  }
}

int id_bits(int n) {
  int b = 1;
  while ((1LL << b) < (long long)n) b++;
  return b;
}

// Undirected pairs (u,v) -> symmetric CSR with sorted, unique lists, no loops.
int build_csr(int n, std::vector<uint64_t>& keys, int ib, fsgc_host_csr* out) {
  // keys hold (min << ib) | max with loops already removed
  radix_sort(keys, 2 * ib);
  keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
  const size_t und = keys.size();
  std::vector<uint64_t> dir(2 * und);
  const uint64_t mask = (1ULL << ib) - 1;
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < (long long)und; i++) {
    const uint64_t u = keys[i] >> ib, v = keys[i] & mask;
    dir[2 * i] = (u << ib) | v;
    dir[2 * i + 1] = (v << ib) | u;
  }
  std::vector<uint64_t>().swap(keys);
  radix_sort(dir, 2 * ib);
  out->n = n;
  out->m = (int64_t)dir.size();
  out->nindex = (int64_t*)malloc(sizeof(int64_t) * ((size_t)n + 1));
  out->nlist = (int32_t*)malloc(sizeof(int32_t) * (dir.size() ? dir.size() : 1));
  if (!out->nindex || !out->nlist) {
    free(out->nindex);
    free(out->nlist);
    out->nindex = nullptr;
    out->nlist = nullptr;
    return FSGC_ENOMEM;
  }
  std::vector<int64_t> deg((size_t)n + 1, 0);
  for (size_t i = 0; i < dir.size(); i++) deg[dir[i] >> ib]++;
  out->nindex[0] = 0;
  for (int v = 0; v < n; v++) out->nindex[v + 1] = out->nindex[v] + deg[v];
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < (long long)dir.size(); i++) out->nlist[i] = (int32_t)(dir[i] & mask);
  return FSGC_OK;
}

}  // namespace

extern "C" {

void fsgc_host_csr_free(fsgc_host_csr* g) {
  if (!g) return;
  if (g->nindex) { cudaHostUnregister(g->nindex); cudaGetLastError(); free(g->nindex); }
  if (g->nlist) { cudaHostUnregister(g->nlist); cudaGetLastError(); free(g->nlist); }
  g->nindex = nullptr;
  g->nlist = nullptr;
  g->n = 0;
  g->m = 0;
}

int fsgc_host_csr_pin(fsgc_host_csr* g) {
  if (!g || !g->nindex || !g->nlist) return FSGC_EINVAL;
  if (cudaHostRegister(g->nindex, sizeof(int64_t) * ((size_t)g->n + 1), cudaHostRegisterDefault) != cudaSuccess) {
    cudaGetLastError();
    return FSGC_ECUDA;
  }
  if (g->m > 0 && cudaHostRegister(g->nlist, sizeof(int32_t) * (size_t)g->m, cudaHostRegisterDefault) != cudaSuccess) {
    cudaGetLastError();
    return FSGC_ECUDA;
  }
  return FSGC_OK;
}

int fsgc_egr_read(const char* path, fsgc_host_csr* out) {
  if (!path || !out) return FSGC_EINVAL;
  memset(out, 0, sizeof(*out));
  FILE* f = fopen(path, "rb");
  if (!f) return FSGC_EIO;
  int32_t n = 0, m32 = 0;
  if (fread(&n, 4, 1, f) != 1 || fread(&m32, 4, 1, f) != 1 || n < 1 || m32 < -1) {
    fclose(f);
    return FSGC_EIO;
  }
  if (m32 == -1) {  // the int64 extension
    int64_t m = 0;
    if (fread(&m, 8, 1, f) != 1 || m < 0) {
      fclose(f);
      return FSGC_EIO;
    }
    out->nindex = (int64_t*)malloc(sizeof(int64_t) * ((size_t)n + 1));
    out->nlist = (int32_t*)malloc(sizeof(int32_t) * (m ? (size_t)m : 1));
    if (!out->nlist || !out->nindex) {
      fclose(f);
      fsgc_host_csr_free(out);
      return FSGC_ENOMEM;
    }
    if (fread(out->nindex, 8, (size_t)n + 1, f) != (size_t)n + 1 ||
        (m > 0 && fread(out->nlist, 4, (size_t)m, f) != (size_t)m)) {
      fclose(f);
      fsgc_host_csr_free(out);
      return FSGC_EIO;
    }
    fclose(f);
    out->n = n;
    out->m = m;
    return FSGC_OK;
  }
  const int32_t m = m32;
  std::vector<int32_t> idx((size_t)n + 1);
  out->nlist = (int32_t*)malloc(sizeof(int32_t) * (m ? (size_t)m : 1));
  out->nindex = (int64_t*)malloc(sizeof(int64_t) * ((size_t)n + 1));
  if (!out->nlist || !out->nindex) {
    fclose(f);
    fsgc_host_csr_free(out);
    return FSGC_ENOMEM;
  }
  if (fread(idx.data(), 4, (size_t)n + 1, f) != (size_t)n + 1 ||
      (m > 0 && fread(out->nlist, 4, (size_t)m, f) != (size_t)m)) {
    fclose(f);
    fsgc_host_csr_free(out);
    return FSGC_EIO;
  }
  fclose(f);
  for (int v = 0; v <= n; v++) out->nindex[v] = idx[v];
  out->n = n;
  out->m = m;
  return FSGC_OK;
}

int fsgc_egr_write64(const char* path, const fsgc_host_csr* g) {
  if (!path || !g || !g->nindex || g->n < 1 || g->m < 0 || (g->m > 0 && !g->nlist)) return FSGC_EINVAL;
  FILE* f = fopen(path, "wb");
  if (!f) return FSGC_EIO;
  const int32_t n = g->n, mark = -1;
  const int64_t m = g->m;
  bool ok = fwrite(&n, 4, 1, f) == 1 && fwrite(&mark, 4, 1, f) == 1 && fwrite(&m, 8, 1, f) == 1 &&
            fwrite(g->nindex, 8, (size_t)n + 1, f) == (size_t)n + 1 &&
            (m == 0 || fwrite(g->nlist, 4, (size_t)m, f) == (size_t)m);
  ok = (fclose(f) == 0) && ok;
  return ok ? FSGC_OK : FSGC_EIO;
}

int fsgc_egr_write(const char* path, const fsgc_host_csr* g) {
  if (!path || !g || !g->nindex || (g->m > 0 && !g->nlist)) return FSGC_EINVAL;
  if (g->m > 2147483647LL) return fsgc_egr_write64(path, g);
  FILE* f = fopen(path, "wb");
  if (!f) return FSGC_EIO;
  const int32_t n = g->n, m = (int32_t)g->m;
  std::vector<int32_t> idx((size_t)n + 1);
  for (int v = 0; v <= n; v++) idx[v] = (int32_t)g->nindex[v];
  bool ok = fwrite(&n, 4, 1, f) == 1 && fwrite(&m, 4, 1, f) == 1 &&
            fwrite(idx.data(), 4, (size_t)n + 1, f) == (size_t)n + 1 &&
            (m == 0 || fwrite(g->nlist, 4, (size_t)m, f) == (size_t)m);
  ok = (fclose(f) == 0) && ok;
  return ok ? FSGC_OK : FSGC_EIO;
}

int fsgc_csr_validate(const fsgc_host_csr* g, char* errbuf, int errlen) {
  auto fail = [&](const char* msg, long long a, long long b) {
    if (errbuf && errlen > 0) snprintf(errbuf, (size_t)errlen, msg, a, b);
    return FSGC_EINVAL;
  };
  if (!g || !g->nindex || g->n < 1) return fail("empty graph %lld %lld", 0, 0);
  if (g->nindex[0] != 0 || g->nindex[g->n] != g->m) return fail("offsets do not span the list (%lld, %lld)", g->nindex[0], g->m);
  for (int v = 0; v < g->n; v++) {
    if (g->nindex[v + 1] < g->nindex[v]) return fail("offsets decrease at vertex %lld %lld", v, 0);
    for (int64_t j = g->nindex[v]; j < g->nindex[v + 1]; j++) {
      const int32_t w = g->nlist[j];
      if (w < 0 || w >= g->n) return fail("vertex %lld has out-of-range neighbour %lld", v, w);
      if (w == v) return fail("self loop on vertex %lld %lld", v, 0);
      if (j > g->nindex[v] && g->nlist[j - 1] >= w) return fail("list of vertex %lld unsorted or duplicate at %lld", v, j);
      // symmetric: v must appear in N(w)
      const int32_t* b = g->nlist + g->nindex[w];
      const int32_t* e = g->nlist + g->nindex[w + 1];
      if (!std::binary_search(b, e, (int32_t)v)) return fail("edge %lld-%lld is not symmetric", v, w);
    }
  }
  return FSGC_OK;
}

int fsgc_csr_from_edges(int n, int64_t nedges, const int32_t* pairs, fsgc_host_csr* out) {
  if (!out || n < 1 || nedges < 0 || (nedges > 0 && !pairs)) return FSGC_EINVAL;
  memset(out, 0, sizeof(*out));
  const int ib = id_bits(n);
  std::vector<uint64_t> keys;
  keys.reserve((size_t)nedges);
  for (int64_t e = 0; e < nedges; e++) {
    const int32_t a = pairs[2 * e], b = pairs[2 * e + 1];
    if (a < 0 || b < 0 || a >= n || b >= n) return FSGC_EINVAL;
    if (a == b) continue;
    const uint64_t u = (uint64_t)std::min(a, b), v = (uint64_t)std::max(a, b);
    keys.push_back((u << ib) | v);
  }
  return build_csr(n, keys, ib, out);
}

// RMAT: each edge descends `scale` levels of the adjacency matrix, picking the
// quadrant (a | b / c | d) with one uniform draw per level.
int fsgc_gen_rmat(int scale, int edge_factor, double a, double b, double c, uint64_t seed, fsgc_host_csr* out) {
  if (!out || scale < 1 || scale > 30 || edge_factor < 1 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0)
    return FSGC_EINVAL;
  memset(out, 0, sizeof(*out));
  const int n = 1 << scale;
  const int64_t E = (int64_t)edge_factor << scale;
  const int ib = id_bits(n);
  std::vector<uint64_t> keys((size_t)E);
  const double ab = a + b, abc = a + b + c;
#pragma omp parallel for schedule(static)
  for (long long e = 0; e < (long long)E; e++) {
    uint64_t u = 0, v = 0;
    for (int l = 0; l < scale; l++) {
      const double r = unit(draw(seed, 1, (uint64_t)e * 64 + (uint64_t)l));
      const uint64_t bit = 1ULL << (scale - 1 - l);
      if (r >= ab) u |= bit;                   // c or d: lower half
      if ((r >= a && r < ab) || r >= abc) v |= bit;  // b or d: right half
    }
    keys[e] = (u == v) ? ~0ULL : ((std::min(u, v) << ib) | std::max(u, v));
  }
  keys.erase(std::remove(keys.begin(), keys.end(), ~0ULL), keys.end());
  return build_csr(n, keys, ib, out);
}

// G(n, m): candidate pairs are drawn in a fixed order; the first m distinct
// loop-free pairs (by draw index) are kept.
int fsgc_gen_er(int n, int64_t undirected_edges, uint64_t seed, fsgc_host_csr* out) {
  if (!out || n < 2 || undirected_edges < 0 || undirected_edges > (int64_t)n * (n - 1) / 2) return FSGC_EINVAL;
  memset(out, 0, sizeof(*out));
  const int ib = id_bits(n);
  std::vector<uint64_t> kept;
  int64_t drawn = 0;
  while ((int64_t)kept.size() < undirected_edges) {
    const int64_t need = undirected_edges - (int64_t)kept.size();
    const int64_t batch = need + need / 4 + 1024;
    // (key, draw index) packed: keys use 2*ib bits, draw index the rest
    std::vector<std::pair<uint64_t, int64_t>> cand((size_t)batch);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)batch; i++) {
      const uint64_t r1 = draw(seed, 2, (uint64_t)(drawn + i) * 2), r2 = draw(seed, 2, (uint64_t)(drawn + i) * 2 + 1);
      const uint64_t x = r1 % (uint64_t)n, y = r2 % (uint64_t)n;
      cand[i] = {x == y ? ~0ULL : ((std::min(x, y) << ib) | std::max(x, y)), drawn + i};
    }
    drawn += batch;
    for (uint64_t k : kept) cand.push_back({k, -1});  // already kept: earliest
    std::sort(cand.begin(), cand.end());
    std::vector<std::pair<int64_t, uint64_t>> firsts;
    for (size_t i = 0; i < cand.size(); i++) {
      if (cand[i].first == ~0ULL) break;
      if (i > 0 && cand[i].first == cand[i - 1].first) continue;
      firsts.push_back({cand[i].second, cand[i].first});
    }
    std::sort(firsts.begin(), firsts.end());
    kept.clear();
    for (size_t i = 0; i < firsts.size() && (int64_t)kept.size() < undirected_edges; i++) kept.push_back(firsts[i].second);
  }
  return build_csr(n, kept, ib, out);
}

// Chung-Lu: vertex i has weight (i + 1)^(-1/(exponent-1)); n*avg/2 edges are
// drawn with both endpoints proportional to weight, then deduplicated.
int fsgc_gen_chung_lu(int n, double avg_degree, double exponent, uint64_t seed, fsgc_host_csr* out) {
  if (!out || n < 2 || avg_degree <= 0 || exponent <= 1.0) return FSGC_EINVAL;
  memset(out, 0, sizeof(*out));
  const int ib = id_bits(n);
  std::vector<double> cdf((size_t)n);
  const double g = -1.0 / (exponent - 1.0);
  double run = 0;
  for (int i = 0; i < n; i++) {
    run += std::pow((double)(i + 1), g);
    cdf[i] = run;
  }
  const int64_t E = (int64_t)std::llround((double)n * avg_degree / 2.0);
  std::vector<uint64_t> keys((size_t)E);
#pragma omp parallel for schedule(static)
  for (long long e = 0; e < (long long)E; e++) {
    const double r1 = unit(draw(seed, 3, (uint64_t)e * 2)) * run, r2 = unit(draw(seed, 3, (uint64_t)e * 2 + 1)) * run;
    const uint64_t x = (uint64_t)(std::upper_bound(cdf.begin(), cdf.end(), r1) - cdf.begin());
    const uint64_t y = (uint64_t)(std::upper_bound(cdf.begin(), cdf.end(), r2) - cdf.begin());
    const uint64_t xx = std::min<uint64_t>(x, n - 1), yy = std::min<uint64_t>(y, n - 1);
    keys[e] = (xx == yy) ? ~0ULL : ((std::min(xx, yy) << ib) | std::max(xx, yy));
  }
  keys.erase(std::remove(keys.begin(), keys.end(), ~0ULL), keys.end());
  return build_csr(n, keys, ib, out);
}

}  // extern "C"
