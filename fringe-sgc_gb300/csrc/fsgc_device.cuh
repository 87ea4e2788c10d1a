// Device-side building blocks shared by the counting kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

typedef unsigned long long u64;

namespace fsgc {

constexpr int kWarp = 32;
constexpr int kMaxDiv = 64;  // divisors 2..63 have precomputed magic numbers

// ----------------------------------------------------------------------------
// u64 division by a small constant d (2 <= d < 64) without the hardware-less
// 64-bit divide: the unsigned "round-up" method of Granlund and Montgomery,
// "Division by Invariant Integers using Multiplication" (PLDI 1994), Fig. 4.1:
//   l  = ceil(log2 d),  m' = floor(2^64 * (2^l - d) / d) + 1,
//   t1 = mulhi(m', x),  q = (t1 + ((x - t1) >> 1)) >> (l - 1).
// Exact for every 64-bit x.  The (m', l) table is built on the host at context
// creation (see fsgc_div_magic_init) and kept in constant memory.
struct DivMagic {
  u64 m;
  int l;
};

__host__ __device__ inline u64 mulhi64(u64 a, u64 b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (u64)(((unsigned __int128)a * b) >> 64);
#endif
}

__host__ __device__ inline u64 div_magic(u64 x, DivMagic mg) {
  const u64 t1 = mulhi64(mg.m, x);
  return (t1 + ((x - t1) >> 1)) >> (mg.l - 1);
}

// Host computation of the table (also used by the host-side self check).
inline DivMagic make_div_magic(unsigned d) {
  int l = 0;
  while ((1ULL << l) < d) l++;
  const unsigned __int128 num = ((unsigned __int128)1 << 64) * (((unsigned __int128)1 << l) - d);
  DivMagic r;
  r.m = (u64)(num / d) + 1;
  r.l = l;
  return r;
}

// ----------------------------------------------------------------------------
// Binomial coefficient with the reference's wrapping u64 arithmetic
// (src/fringeCount.cu:189-197): k = min(k, n-k); 0 if k < 0; 1 if k == 0;
// otherwise r = n, then r = r*(n+1-i)/i for i = 2..k, each product taken mod
// 2^64 before the truncating division.  `tab` holds the division magics.
__host__ __device__ inline u64 nck_ref(int n, int k, const DivMagic* tab) {
  k = (k < n - k) ? k : n - k;
  if (k < 0) return 0;
  if (k == 0) return 1;
  u64 r = (u64)n;
  for (int i = 2; i <= k; i++) {
    r = r * (u64)(n + 1 - i);
    r = (i < kMaxDiv) ? div_magic(r, tab[i]) : r / (u64)i;
  }
  return r;
}

// ----------------------------------------------------------------------------
// Sorted-list helpers.  Lists are ascending int32 runs in global memory.

// true if x occurs in a[0..len)
__device__ __forceinline__ bool bsearch_has(const int* __restrict__ a, int len, int x) {
  int lo = 0, hi = len;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    const int v = __ldg(a + mid);
    if (v < x) lo = mid + 1;
    else hi = mid;
  }
  return lo < len && __ldg(a + lo) == x;
}

// index of x in a[0..len), or -1
__device__ __forceinline__ int bsearch_pos(const int* __restrict__ a, int len, int x) {
  int lo = 0, hi = len;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    const int v = __ldg(a + mid);
    if (v < x) lo = mid + 1;
    else hi = mid;
  }
  return (lo < len && __ldg(a + lo) == x) ? lo : -1;
}

// number of elements < x in a[0..len)
__device__ __forceinline__ int lower_bound_dev(const int* __restrict__ a, int len, int x) {
  int lo = 0, hi = len;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(a + mid) < x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// ----------------------------------------------------------------------------
// Reductions: warp shuffle -> one shared-memory atomic per warp -> one global
// atomic per block into the task's result slot (mod 2^64 addition).
__device__ __forceinline__ u64 warp_sum_u64(u64 v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ int warp_sum_int(int v) { return __reduce_add_sync(0xffffffffu, v); }

// Every thread of the block must call this (it contains __syncthreads).
__device__ __forceinline__ void block_sum_to(u64 v, u64* __restrict__ slot) {
  __shared__ u64 s_acc;
  if (threadIdx.x == 0) s_acc = 0;
  __syncthreads();
  v = warp_sum_u64(v);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(&s_acc, v);
  __syncthreads();
  if (threadIdx.x == 0 && s_acc) atomicAdd(slot, s_acc);
}

}  // namespace fsgc
