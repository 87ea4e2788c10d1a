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

// C(n, k) for k = 0 or 1, equal to nck_ref(n, k) (and to the exact C(n, k))
// for every n: 1 if n >= 0 when k = 0; n if n >= 1 when k = 1; 0 otherwise.
__host__ __device__ inline u64 nck01(int n, int k) {
  return k == 0 ? (n >= 0 ? 1ULL : 0ULL) : (n >= 1 ? (u64)n : 0ULL);
}

// wedge() (src/fringeCount.cu:1381-1406): endpoints x (larger id) and y of a
// wedge; c = common neighbours of x and y other than the centre.  `nk(n, k)`
// gives the binomials in the count's arithmetic A.
template <class A, class Nck>
__host__ __device__ inline A wedge_formula_with(int dx, int dy, bool adj, int f_x, int f_xy, int f_y, int c, Nck nk) {
  const int a_xy = c - f_xy;
  if (a_xy < 0) return A(0);
  const int corr = adj ? 2 : 1;
  const int a_x = dx - (corr + c), a_y = dy - (corr + c);
  const int bound = (f_x < a_xy) ? f_x : a_xy;
  A sum = A(0);
  for (int j = 0; j <= bound; j++) {
    const int k = f_x - j;
    A term = nk(a_x, k) * nk(a_xy + a_y - j, f_y);
    if (f_x != f_y) term += nk(a_y, k) * nk(a_xy + a_x - j, f_y);
    sum += term * nk(a_xy, j);
  }
  return sum * nk(c, f_xy);
}

// ----------------------------------------------------------------------------
// Sorted-list helpers.  Lists are ascending int32 runs in global memory (the
// read-only loads below take global addresses only).

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

// number of elements < x in a[0..len) with plain loads: for lists that may sit
// in shared memory (the __ldg searches above take global addresses only)
__device__ __forceinline__ int lower_bound_any(const int* a, int len, int x) {
  int lo = 0, hi = len;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (a[mid] < x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// ----------------------------------------------------------------------------
// Bulk copies from global to shared memory (cp.async.bulk, the Blackwell copy
// engine without a tensor map), completed on an mbarrier.  Source and
// destination must be 16-byte aligned and the size a multiple of 16; the
// copies used here read this GPU's own memory and are never multicast.
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this thread's earlier shared-memory accesses before later copies.
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// One thread: arm the barrier for `bytes` and start the copy.
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// Waits for the barrier's phase `parity` to complete, polling at most `limit`
// times; false when it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity, int limit) {
  for (int i = 0; i < limit; i++) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// ----------------------------------------------------------------------------
// Exact counts: unsigned 128-bit values that saturate at 2^128 - 1 (every bit
// set) instead of wrapping.  A product with a zero factor is zero; any other
// operation with a saturated operand, or whose true result is >= 2^128 - 1,
// gives the saturated value.  Used where the reference's u64 arithmetic wraps.
struct X128 {
  u64 lo, hi;
  __host__ __device__ X128() : lo(0), hi(0) {}
  __host__ __device__ X128(u64 x) : lo(x), hi(0) {}
  __host__ __device__ X128(u64 l, u64 h) : lo(l), hi(h) {}
  __host__ __device__ static X128 saturated() { return X128(~0ULL, ~0ULL); }
  __host__ __device__ bool is_saturated() const { return (lo & hi) == ~0ULL; }
  __host__ __device__ bool is_zero() const { return (lo | hi) == 0; }
};

__host__ __device__ inline X128 operator+(X128 a, X128 b) {
  if (a.is_saturated() || b.is_saturated()) return X128::saturated();
  X128 r;
  r.lo = a.lo + b.lo;
  const u64 c = r.lo < a.lo;
  const u64 h = a.hi + b.hi;
  r.hi = h + c;
  if (h < a.hi || r.hi < h || r.is_saturated()) return X128::saturated();
  return r;
}

__host__ __device__ inline X128 operator*(X128 a, X128 b) {
  if (a.is_zero() || b.is_zero()) return X128();
  if (a.is_saturated() || b.is_saturated() || (a.hi && b.hi)) return X128::saturated();
  // at most one high word is non-zero: a*b = lo*lo + 2^64 (a.hi*b.lo + a.lo*b.hi)
  const u64 cross_a = a.hi ? a.hi : b.hi, cross_b = a.hi ? b.lo : a.lo;
  if (mulhi64(cross_a, cross_b)) return X128::saturated();
  const u64 cross = cross_a * cross_b;
  X128 r;
  r.lo = a.lo * b.lo;
  const u64 h = mulhi64(a.lo, b.lo);
  r.hi = h + cross;
  if (r.hi < h || r.is_saturated()) return X128::saturated();
  return r;
}

__host__ __device__ inline X128& operator+=(X128& a, X128 b) { return a = a + b; }
__host__ __device__ inline X128& operator*=(X128& a, X128 b) { return a = a * b; }

// a / d and a % d for 1 <= d < 2^32 (a not saturated), by 32-bit limbs.
__host__ __device__ inline X128 x_divmod_small(X128 a, unsigned d, unsigned* rem) {
  X128 q;
  q.hi = a.hi / d;
  u64 r = a.hi % d;
  const u64 t1 = (r << 32) | (a.lo >> 32);
  const u64 q1 = t1 / d;
  r = t1 % d;
  const u64 t0 = (r << 32) | (a.lo & 0xffffffffULL);
  q.lo = (q1 << 32) | (t0 / d);
  *rem = (unsigned)(t0 % d);
  return q;
}

// Exact binomial C(n, k) (0 when k < 0 or n < k), saturating.  The step
// r = r*(n+1-i)/i is taken as (r/i)*(n+1-i) + ((r%i)*(n+1-i))/i, exact because
// i divides r*(n+1-i), so no intermediate exceeds the final C(n, i).
__host__ __device__ inline X128 nck_x(int n, int k) {
  if (k < 0 || n < k) return X128();
  if (k > n - k) k = n - k;
  if (k == 0) return X128(1);
  X128 r((u64)n);
  for (int i = 2; i <= k; i++) {
    unsigned rem;
    const X128 q = x_divmod_small(r, (unsigned)i, &rem);
    const u64 f = (u64)(n + 1 - i);
    r = q * X128(f) + X128(((u64)rem * f) / (u64)i);
    if (r.is_saturated()) return r;
  }
  return r;
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

// Exact sums: slot[0..1] = low and high words of a 128-bit total, slot[2] is
// set to 1 once the total saturates.  Saturating adds within the warp, one
// shared partial per warp summed by thread 0, then a 128-bit atomic add into
// the slot: the low word's carry goes into the high word, and a carry out of
// the high word saturates.  Every thread of the block must call this.
__device__ __forceinline__ void block_sum_to(X128 v, u64* __restrict__ slot) {
  __shared__ u64 s_part[32][2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const X128 w(__shfl_down_sync(0xffffffffu, v.lo, o), __shfl_down_sync(0xffffffffu, v.hi, o));
    v = v + w;
  }
  if (lane == 0) { s_part[warp][0] = v.lo; s_part[warp][1] = v.hi; }
  __syncthreads();
  if (threadIdx.x == 0) {
    X128 t;
    for (int i = 0; i < (int)((blockDim.x + 31) >> 5); i++) t = t + X128(s_part[i][0], s_part[i][1]);
    if (t.is_saturated()) {
      atomicExch(slot + 2, 1ULL);
    } else if (!t.is_zero()) {
      const u64 old_lo = atomicAdd(slot, t.lo);
      const u64 carry = (old_lo + t.lo < old_lo) ? 1ULL : 0ULL;
      if (t.hi == ~0ULL && carry) {
        atomicExch(slot + 2, 1ULL);
      } else {
        const u64 add_hi = t.hi + carry;
        if (add_hi) {
          const u64 old_hi = atomicAdd(slot + 1, add_hi);
          if (old_hi + add_hi < old_hi) atomicExch(slot + 2, 1ULL);
        }
      }
    }
  }
  __syncthreads();  // s_part is free again for a later call
}

}  // namespace fsgc
