// Graph loader on the GPU: degrees, the degree-ordered orientation of every
// undirected edge, and per-edge triangle supports.
//
// The reference relabels vertices by degree with CUB radix sorts inside the
// triangle-core count (relabelByDegree, src/fringeCount.cu:1221-1288) and builds
// a fresh degree-pruned worklist with one global atomic per edge for every count
// (init_wl_*, :617-663, 1167-1218, 1653-1751, 2054-2103).  Here a graph is
// prepared once when it becomes resident: the orientation (lower (deg, id)
// endpoint -> higher) bounds out-degrees by O(sqrt m), and one pass over the
// oriented edges computes |N(x) & N(y)| for every edge, which the edge,
// triangle and wedge cores all consume.  No relabel is needed: kernels compare
// (deg, id) pairs directly, which is the order the reference's relabel induces.
#include <algorithm>
#include <cstdio>

#include "fsgc_internal.h"

namespace fsgc {

namespace {

constexpr int kTPB = 256;

__device__ __forceinline__ bool above(int w, int dw, int v, int dv) {  // (dw, w) > (dv, v)
  return (dw > dv) || (dw == dv && w > v);
}

__global__ void degree_kernel(int n, const long long* __restrict__ off, int* __restrict__ deg,
                              int* __restrict__ maxdeg) {
  int local = 0;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const int d = (int)(off[v + 1] - off[v]);
    deg[v] = d;
    local = max(local, d);
  }
  local = __reduce_max_sync(0xffffffffu, local);
  if ((threadIdx.x & 31) == 0) atomicMax(maxdeg, local);
}

// warp per vertex: number of neighbours above it in degree order
__global__ void outdeg_kernel(GView g, long long* __restrict__ odeg) {
  const int lane = threadIdx.x & 31;
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int v = wid; v < g.n; v += nw) {
    const int dv = g.deg[v];
    const long long b = g.off[v], e = g.off[v + 1];
    int c = 0;
    for (long long j = b + lane; j < e; j += 32) {
      const int w = g.adj[j];
      c += above(w, g.deg[w], v, dv);
    }
    c = __reduce_add_sync(0xffffffffu, c);
    if (lane == 0) odeg[v] = c;
  }
}

__global__ void orient_fill_kernel(GView g, int* __restrict__ oadj, int* __restrict__ osrc) {
  const int lane = threadIdx.x & 31;
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  const unsigned lt = (1u << lane) - 1u;
  for (int v = wid; v < g.n; v += nw) {
    const int dv = g.deg[v];
    const long long b = g.off[v], e = g.off[v + 1];
    long long o = g.ooff[v];
    for (long long j0 = b; j0 < e; j0 += 32) {
      const long long j = j0 + lane;
      int w = -1;
      bool p = false;
      if (j < e) {
        w = g.adj[j];
        p = above(w, g.deg[w], v, dv);
      }
      const unsigned bal = __ballot_sync(0xffffffffu, p);
      if (p) {
        const long long pos = o + __popc(bal & lt);
        oadj[pos] = w;
        osrc[pos] = v;
      }
      o += __popc(bal);
    }
  }
}

// ---- exclusive scan of n int64 values into out[0..n] (out[n] = total)
constexpr int kScanTile = 2048;  // 256 threads x 8

__device__ __forceinline__ long long block_excl_scan(long long x, long long* s_warp, long long& total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  long long inc = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) s_warp[w] = inc;
  __syncthreads();
  if (w == 0) {
    long long t = (lane < (int)(blockDim.x >> 5)) ? s_warp[lane] : 0;
    long long ti = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, ti, o);
      if (lane >= o) ti += y;
    }
    if (lane < (int)(blockDim.x >> 5)) s_warp[lane] = ti - t;
    if (lane == 31) s_warp[32] = ti;
  }
  __syncthreads();
  const long long r = s_warp[w] + inc - x;
  total = s_warp[32];
  __syncthreads();
  return r;
}

__global__ void scan_tiles_kernel(const long long* __restrict__ in, long long n, long long* __restrict__ tile_sum) {
  __shared__ long long s_warp[33];
  const long long base = (long long)blockIdx.x * kScanTile + threadIdx.x * 8;
  long long x = 0;
#pragma unroll
  for (int i = 0; i < 8; i++) x += (base + i < n) ? in[base + i] : 0;
  long long tot;
  block_excl_scan(x, s_warp, tot);
  if (threadIdx.x == 0) tile_sum[blockIdx.x] = tot;
}

__global__ void scan_sums_kernel(long long* __restrict__ sums, long long nt) {  // one block, in place
  __shared__ long long s_warp[33];
  long long carry = 0;
  for (long long b = 0; b < nt; b += blockDim.x) {
    const long long i = b + threadIdx.x;
    const long long x = (i < nt) ? sums[i] : 0;
    long long tot;
    const long long ex = block_excl_scan(x, s_warp, tot);
    if (i < nt) sums[i] = carry + ex;
    carry += tot;
  }
}

__global__ void scan_apply_kernel(const long long* __restrict__ in, long long n, const long long* __restrict__ tile_off,
                                  long long* __restrict__ out) {
  __shared__ long long s_warp[33];
  const long long base = (long long)blockIdx.x * kScanTile + threadIdx.x * 8;
  long long v[8];
  long long x = 0;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    v[i] = (base + i < n) ? in[base + i] : 0;
    x += v[i];
  }
  long long tot;
  long long run = block_excl_scan(x, s_warp, tot) + tile_off[blockIdx.x];
#pragma unroll
  for (int i = 0; i < 8; i++) {
    if (base + i < n) out[base + i] = run;
    run += v[i];
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) out[n] = run;
}

// ---- triangle supports: thread per oriented edge (a -> b); the common
// out-neighbours c of a and b close the triangles a < b < c, each found once.
__device__ __forceinline__ void tri_found(unsigned* __restrict__ osup, long long sa, long long sb) {
  atomicAdd(osup + sa, 1u);
  atomicAdd(osup + sb, 1u);
}

__global__ void triangle_support_kernel(GView g, unsigned* __restrict__ osup, u64* __restrict__ tri_total) {
  const long long me = g.m / 2;
  u64 tot = 0;
  for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < me; j += (long long)gridDim.x * blockDim.x) {
    const int a = g.osrc[j], b = g.oadj[j];
    const long long ab = g.ooff[a], bb = g.ooff[b];
    const int la = (int)(g.ooff[a + 1] - ab), lb = (int)(g.ooff[b + 1] - bb);
    if (lb == 0) continue;
    const int* A = g.oadj + ab;
    const int* B = g.oadj + bb;
    unsigned cnt = 0;
    if ((long long)la * 16 < lb) {
      for (int i = 0; i < la; i++) {
        const int p = bsearch_pos(B, lb, A[i]);
        if (p >= 0) { cnt++; tri_found(osup, ab + i, bb + p); }
      }
    } else if ((long long)lb * 16 < la) {
      for (int k = 0; k < lb; k++) {
        const int p = bsearch_pos(A, la, B[k]);
        if (p >= 0) { cnt++; tri_found(osup, ab + p, bb + k); }
      }
    } else {
      int i = 0, k = 0;
      while (i < la && k < lb) {
        const int x = __ldg(A + i), y = __ldg(B + k);
        if (x < y) i++;
        else if (y < x) k++;
        else { cnt++; tri_found(osup, ab + i, bb + k); i++; k++; }
      }
    }
    if (cnt) atomicAdd(osup + j, cnt);
    tot += cnt;
  }
  block_sum_to(tot, tri_total);
}

// largest out-degree and largest out-degree * ceil(deg / 32) (bitmap rows)
__global__ void outdeg_stats_kernel(GView g, unsigned long long* __restrict__ stats) {
  unsigned long long k1 = 0, k2 = 0;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < g.n; v += gridDim.x * blockDim.x) {
    const unsigned long long k = (unsigned long long)(g.ooff[v + 1] - g.ooff[v]);
    k1 = max(k1, k);
    k2 = max(k2, k * (unsigned long long)((g.deg[v] + 31) >> 5));
  }
  for (int o = 16; o > 0; o >>= 1) {
    k1 = max(k1, __shfl_down_sync(0xffffffffu, k1, o));
    k2 = max(k2, __shfl_down_sync(0xffffffffu, k2, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(stats, k1);
    atomicMax(stats + 1, k2);
  }
}

__global__ void vertex_triangle_kernel(GView g, u64* __restrict__ vtri2) {
  const long long me = g.m / 2;
  for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < me; j += (long long)gridDim.x * blockDim.x) {
    const unsigned s = g.osup[j];
    if (s) {
      atomicAdd(vtri2 + g.osrc[j], (u64)s);
      atomicAdd(vtri2 + g.oadj[j], (u64)s);
    }
  }
}

// The support of each oriented edge, written to both of its list entries.
__global__ void entry_support_kernel(GView g, unsigned* __restrict__ esup) {
  const long long me = g.m / 2;
  for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < me; j += (long long)gridDim.x * blockDim.x) {
    const int a = g.osrc[j], b = g.oadj[j];
    const unsigned s = g.osup[j];
    const long long oa = g.off[a], ob = g.off[b];
    const int pa = bsearch_pos(g.adj + oa, (int)(g.off[a + 1] - oa), b);
    const int pb = bsearch_pos(g.adj + ob, (int)(g.off[b + 1] - ob), a);
    if (pa >= 0) esup[oa + pa] = s;
    if (pb >= 0) esup[ob + pb] = s;  // absent only in a non-symmetric input
  }
}

int g_sms = 0;

}  // namespace

int sm_count() {
  if (g_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_sms <= 0) g_sms = 1;
  }
  return g_sms;
}

static int grid_for(long long work, int tpb, int per_sm) {
  const long long want = (work + tpb - 1) / tpb;
  const long long cap = (long long)sm_count() * per_sm;
  return (int)std::max(1LL, std::min(want, cap));
}

#define FSGC_TRY(x)                               \
  do {                                            \
    cudaError_t e__ = (x);                        \
    if (e__ != cudaSuccess) return FSGC_ECUDA;    \
  } while (0)

// Degrees and the maximum degree into caller-provided device memory.
int launch_degrees(int n, const long long* off, int* deg, int* maxdeg, cudaStream_t s) {
  degree_kernel<<<grid_for(n, kTPB, 8), kTPB, 0, s>>>(n, off, deg, maxdeg);
  return cudaGetLastError() == cudaSuccess ? FSGC_OK : FSGC_ECUDA;
}

// Degrees and the maximum degree; run when a graph becomes resident.
int graph_degrees(DevGraph& g, cudaStream_t s, uint64_t* launches, u64* d_u64) {
  int* d_max = reinterpret_cast<int*>(d_u64);
  FSGC_TRY(cudaMemsetAsync(d_max, 0, sizeof(int), s));
  degree_kernel<<<grid_for(g.n, kTPB, 8), kTPB, 0, s>>>(g.n, g.off, g.deg, d_max);
  *launches += 1;
  int maxd = 0;
  FSGC_TRY(cudaMemcpyAsync(&maxd, d_max, sizeof(int), cudaMemcpyDeviceToHost, s));
  FSGC_TRY(cudaStreamSynchronize(s));
  FSGC_TRY(cudaGetLastError());
  g.maxdeg = maxd;
  return FSGC_OK;
}

int prepare_graph(DevGraph& g, cudaStream_t s, uint64_t* launches, u64* d_u64) {
  if (g.prepared) return FSGC_OK;
  const int n = g.n;
  const long long me = g.m / 2;
  const int maxd = g.maxdeg;
  // oriented CSR
  long long* odeg = nullptr;
  const long long ntiles = ((long long)n + kScanTile - 1) / kScanTile;
  long long* tiles = nullptr;
  FSGC_TRY(cudaMallocAsync((void**)&odeg, sizeof(long long) * ((size_t)n + 1), s));
  FSGC_TRY(cudaMallocAsync((void**)&tiles, sizeof(long long) * (size_t)std::max(1LL, ntiles), s));
  FSGC_TRY(cudaMallocAsync((void**)&g.ooff, sizeof(long long) * ((size_t)n + 1), s));
  FSGC_TRY(cudaMallocAsync((void**)&g.oadj, sizeof(int) * (size_t)std::max(1LL, me), s));
  FSGC_TRY(cudaMallocAsync((void**)&g.osrc, sizeof(int) * (size_t)std::max(1LL, me), s));
  FSGC_TRY(cudaMallocAsync((void**)&g.osup, sizeof(unsigned) * (size_t)std::max(1LL, me), s));
  GView v = g.view();
  const int wgrid = grid_for((long long)n * 32, kTPB, 16);
  outdeg_kernel<<<wgrid, kTPB, 0, s>>>(v, odeg);
  scan_tiles_kernel<<<(int)ntiles, kTPB, 0, s>>>(odeg, n, tiles);
  scan_sums_kernel<<<1, 1024, 0, s>>>(tiles, ntiles);
  scan_apply_kernel<<<(int)ntiles, kTPB, 0, s>>>(odeg, n, tiles, g.ooff);
  v = g.view();
  orient_fill_kernel<<<wgrid, kTPB, 0, s>>>(v, g.oadj, g.osrc);
  *launches += 5;
  // supports and triangle total
  FSGC_TRY(cudaMemsetAsync(g.osup, 0, sizeof(unsigned) * (size_t)std::max(1LL, me), s));
  u64* d_tri = d_u64 + 1;
  FSGC_TRY(cudaMemsetAsync(d_tri, 0, sizeof(u64), s));
  if (me > 0) {
    triangle_support_kernel<<<grid_for(me, kTPB, 8), kTPB, 0, s>>>(v, g.osup, d_tri);
    *launches += 1;
  }
  u64* d_stats = d_u64 + 2;
  FSGC_TRY(cudaMemsetAsync(d_stats, 0, 2 * sizeof(u64), s));
  outdeg_stats_kernel<<<grid_for(n, kTPB, 8), kTPB, 0, s>>>(v, d_stats);
  *launches += 1;
  u64 stats[3] = {0, 0, 0};
  FSGC_TRY(cudaMemcpyAsync(stats, d_tri, 3 * sizeof(u64), cudaMemcpyDeviceToHost, s));
  FSGC_TRY(cudaFreeAsync(odeg, s));
  FSGC_TRY(cudaFreeAsync(tiles, s));
  FSGC_TRY(cudaStreamSynchronize(s));
  FSGC_TRY(cudaGetLastError());
  g.triangles = (long long)stats[0];
  g.max_outdeg = (long long)stats[1];
  g.max_bitmap_words = (long long)stats[2];
  // the reference relabels (and so orders triangle roles by degree) only for
  // n > 10000, n <= m/10 and maximum degree > 16
  g.tri_relabel = (n > 10000) && !((long long)n > g.m / 10) && (maxd > 16);
  g.bytes += sizeof(long long) * ((size_t)n + 1) + (sizeof(int) * 2 + sizeof(unsigned)) * (size_t)std::max(1LL, me);
  g.prepared = true;
  return FSGC_OK;
}

int ensure_entry_supports(DevGraph& g, cudaStream_t s, uint64_t* launches) {
  if (g.esup) return FSGC_OK;
  FSGC_TRY(cudaMallocAsync((void**)&g.esup, sizeof(unsigned) * (size_t)std::max(1LL, g.m), s));
  FSGC_TRY(cudaMemsetAsync(g.esup, 0, sizeof(unsigned) * (size_t)std::max(1LL, g.m), s));
  const long long me = g.m / 2;
  if (me > 0) {
    entry_support_kernel<<<grid_for(me, kTPB, 8), kTPB, 0, s>>>(g.view(), g.esup);
    *launches += 1;
  }
  g.bytes += sizeof(unsigned) * (size_t)std::max(1LL, g.m);
  FSGC_TRY(cudaGetLastError());
  return FSGC_OK;
}

int ensure_vertex_triangles(DevGraph& g, cudaStream_t s, uint64_t* launches) {
  if (g.vtri2) return FSGC_OK;
  FSGC_TRY(cudaMallocAsync((void**)&g.vtri2, sizeof(u64) * (size_t)std::max(1, g.n), s));
  FSGC_TRY(cudaMemsetAsync(g.vtri2, 0, sizeof(u64) * (size_t)std::max(1, g.n), s));
  const long long me = g.m / 2;
  if (me > 0) {
    vertex_triangle_kernel<<<grid_for(me, kTPB, 8), kTPB, 0, s>>>(g.view(), g.vtri2);
    *launches += 1;
  }
  g.bytes += sizeof(u64) * (size_t)std::max(1, g.n);
  FSGC_TRY(cudaGetLastError());
  return FSGC_OK;
}

}  // namespace fsgc
