// Edge-list ingestion on the device: an arbitrary list of undirected pairs
// becomes the cleaned, symmetric CSR the counting kernels take (self loops
// dropped, duplicates merged, both directions, lists sorted ascending) -- the
// reference's documented input preconditions (src/fringeCount.cu:50-56), which
// its own loader only assumes (src/ECLgraph.h:58-85).  The host-side
// equivalent is fsgc_csr_from_edges.
//
// Pairs become 64-bit keys (low id << 32 | high id; loops the largest key),
// radix-sorted and made unique; the undirected keys expand to both directions,
// sorted again; offsets come from a binary search per vertex and the lists
// from the keys' low words.  Sorting uses CUB's device radix sort (this runs
// once per graph, off the counting path).
#include <cub/cub.cuh>

#include "fsgc_internal.h"

namespace fsgc {
namespace {

constexpr unsigned long long kLoopKey = ~0ULL;

__global__ void edge_keys_kernel(const int* __restrict__ pairs, long long E, int n, unsigned long long* __restrict__ keys,
                                 int* __restrict__ bad) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += (long long)gridDim.x * blockDim.x) {
    const int a = pairs[2 * e], b = pairs[2 * e + 1];
    unsigned long long k = kLoopKey;
    if (a < 0 || b < 0 || a >= n || b >= n) {
      atomicOr(bad, 1);
    } else if (a != b) {
      const unsigned long long lo = (unsigned)min(a, b), hi = (unsigned)max(a, b);
      k = (lo << 32) | hi;
    }
    keys[e] = k;
  }
}

__global__ void directed_keys_kernel(const unsigned long long* __restrict__ und, long long U,
                                     unsigned long long* __restrict__ dir) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < U; i += (long long)gridDim.x * blockDim.x) {
    const unsigned long long k = und[i];
    dir[2 * i] = k;
    dir[2 * i + 1] = (k << 32) | (k >> 32);
  }
}

// off[v] = first position of source v among the sorted directed keys
__global__ void csr_offsets_kernel(const unsigned long long* __restrict__ dir, long long M, int n,
                                   long long* __restrict__ off) {
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v <= n; v += (long long)gridDim.x * blockDim.x) {
    const unsigned long long x = (unsigned long long)v << 32;
    long long lo = 0, hi = M;
    while (lo < hi) {
      const long long mid = (lo + hi) >> 1;
      if (dir[mid] < x) lo = mid + 1;
      else hi = mid;
    }
    off[v] = lo;
  }
}

__global__ void csr_lists_kernel(const unsigned long long* __restrict__ dir, long long M, int* __restrict__ adj) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < M; i += (long long)gridDim.x * blockDim.x)
    adj[i] = (int)(dir[i] & 0xffffffffULL);
}

int grid_of(long long work) { return (int)std::max(1LL, std::min((work + 255) / 256, (long long)sm_count() * 16)); }

// Sorts keys[0..count) in place through `alt` (same size), growing `temp` as needed.
cudaError_t sort_keys(unsigned long long*& keys, unsigned long long*& alt, long long count, void*& temp,
                      size_t& temp_bytes, cudaStream_t s) {
  cub::DoubleBuffer<unsigned long long> db(keys, alt);
  size_t need = 0;
  cudaError_t e = cub::DeviceRadixSort::SortKeys(nullptr, need, db, count, 0, 64, s);
  if (e != cudaSuccess) return e;
  if (need > temp_bytes) {
    cudaFreeAsync(temp, s);
    temp = nullptr;
    temp_bytes = 0;
    e = cudaMallocAsync(&temp, need, s);
    if (e != cudaSuccess) return e;
    temp_bytes = need;
  }
  e = cub::DeviceRadixSort::SortKeys(temp, need, db, count, 0, 64, s);
  keys = db.Current();
  alt = db.Alternate();
  return e;
}

}  // namespace

int csr_from_device_edges(int n, long long E, const int* d_pairs, cudaStream_t s, long long** off_out, int** adj_out,
                          long long* m_out, u64* d_small) {
  *off_out = nullptr;
  *adj_out = nullptr;
  *m_out = 0;
  unsigned long long *a = nullptr, *b = nullptr;
  void* temp = nullptr;
  size_t temp_bytes = 0;
  long long* off = nullptr;
  int* adj = nullptr;
  int* bad = reinterpret_cast<int*>(d_small + 11);
  long long* nsel = reinterpret_cast<long long*>(d_small + 12);
  int status = FSGC_OK;
  cudaError_t e = cudaSuccess;
  auto fail = [&](int st) {
    cudaFreeAsync(a, s);
    cudaFreeAsync(b, s);
    cudaFreeAsync(temp, s);
    cudaFreeAsync(off, s);
    cudaFreeAsync(adj, s);
    cudaStreamSynchronize(s);
    cudaGetLastError();
    return st;
  };
  const size_t ebytes = sizeof(unsigned long long) * (size_t)std::max(1LL, E);
  if (cudaMallocAsync((void**)&a, ebytes, s) != cudaSuccess || cudaMallocAsync((void**)&b, ebytes, s) != cudaSuccess)
    return fail(FSGC_ENOMEM);
  cudaMemsetAsync(bad, 0, sizeof(int), s);
  long long U = 0;
  if (E > 0) {
    edge_keys_kernel<<<grid_of(E), 256, 0, s>>>(d_pairs, E, n, a, bad);
    e = sort_keys(a, b, E, temp, temp_bytes, s);
    if (e != cudaSuccess) return fail(e == cudaErrorMemoryAllocation ? FSGC_ENOMEM : FSGC_ECUDA);
    size_t need = 0;
    cub::DeviceSelect::Unique(nullptr, need, a, b, nsel, E, s);
    if (need > temp_bytes) {
      cudaFreeAsync(temp, s);
      temp = nullptr;
      if (cudaMallocAsync(&temp, need, s) != cudaSuccess) return fail(FSGC_ENOMEM);
      temp_bytes = need;
    }
    if (cub::DeviceSelect::Unique(temp, need, a, b, nsel, E, s) != cudaSuccess) return fail(FSGC_ECUDA);
    long long sel = 0;
    unsigned long long last = 0;
    int h_bad = 0;
    cudaMemcpyAsync(&sel, nsel, sizeof(long long), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return fail(FSGC_ECUDA);
    if (h_bad) return fail(FSGC_EINVAL);
    if (sel > 0) {
      cudaMemcpyAsync(&last, b + sel - 1, sizeof(last), cudaMemcpyDeviceToHost, s);
      if (cudaStreamSynchronize(s) != cudaSuccess) return fail(FSGC_ECUDA);
    }
    U = (sel > 0 && last == kLoopKey) ? sel - 1 : sel;  // loops sort last
    std::swap(a, b);  // a: the unique undirected keys
  }
  const long long M = 2 * U;
  // directed keys need 2U slots in both buffers
  cudaFreeAsync(b, s);
  b = nullptr;
  unsigned long long* d = nullptr;
  if (cudaMallocAsync((void**)&d, sizeof(unsigned long long) * (size_t)std::max(1LL, M), s) != cudaSuccess ||
      cudaMallocAsync((void**)&b, sizeof(unsigned long long) * (size_t)std::max(1LL, M), s) != cudaSuccess) {
    cudaFreeAsync(d, s);
    return fail(FSGC_ENOMEM);
  }
  if (U > 0) directed_keys_kernel<<<grid_of(U), 256, 0, s>>>(a, U, d);
  cudaFreeAsync(a, s);
  a = d;
  if (M > 0) {
    e = sort_keys(a, b, M, temp, temp_bytes, s);
    if (e != cudaSuccess) return fail(e == cudaErrorMemoryAllocation ? FSGC_ENOMEM : FSGC_ECUDA);
  }
  // the lists are padded by 16 bytes, as every resident graph's
  if (cudaMallocAsync((void**)&off, sizeof(long long) * ((size_t)n + 1), s) != cudaSuccess ||
      cudaMallocAsync((void**)&adj, sizeof(int) * (size_t)std::max(1LL, M) + 16, s) != cudaSuccess)
    return fail(FSGC_ENOMEM);
  csr_offsets_kernel<<<grid_of((long long)n + 1), 256, 0, s>>>(a, M, n, off);
  if (M > 0) csr_lists_kernel<<<grid_of(M), 256, 0, s>>>(a, M, adj);
  cudaFreeAsync(a, s);
  cudaFreeAsync(b, s);
  cudaFreeAsync(temp, s);
  a = b = nullptr;
  temp = nullptr;
  if (cudaStreamSynchronize(s) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
    status = FSGC_ECUDA;
    return fail(status);
  }
  *off_out = off;
  *adj_out = adj;
  *m_out = M;
  return FSGC_OK;
}

}  // namespace fsgc
