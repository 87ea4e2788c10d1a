// Counting kernels: one family per core shape of the matching order.
//
// Every kernel evaluates, per core match, the reference's closed-form fringe
// count with the reference's u64 arithmetic (nck_ref) and the reference's
// vertex roles, and adds it into a u64 result slot through a warp -> block ->
// slot reduction.  The per-match formulas are fixed by the reference; what
// changes is how the matches and their Venn sizes are found:
//   vertex core   one pass over the degrees;
//   edge core     one pass over oriented edges, common-neighbour counts taken
//                 from the loader's per-edge triangle supports;
//   triangle core one block per lowest vertex a builds bitmap rows
//                 N(a) & N(b_i) over the positions of N(a): the triangles are
//                 the set bits, pairwise overlaps come from the supports and
//                 the triple overlap is a popcount of two rows (the 4-clique
//                 modes, and graphs whose out-lists would not fit in shared
//                 memory, enumerate triangles on the oriented graph and take
//                 the triple overlap by a warp-cooperative intersection);
//   wedge core    (centre without fringes) aggregated per endpoint pair: the
//                 reference evaluates the same formula once per centre, and
//                 the formula does not depend on the centre, so each pair is
//                 evaluated once and multiplied by its number of centres;
//                 (centre with fringes) one warp per centre-endpoint edge;
//   general core  warp-cooperative depth-first matching of 4-6 core vertices,
//                 a Venn histogram per match and a per-lane placement sum.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include <vector>

#include "fsgc_internal.h"

namespace fsgc {

__constant__ DivMagic c_div[kMaxDiv];

void upload_div_magic() {
  DivMagic t[kMaxDiv];
  t[0] = DivMagic{0, 1};
  t[1] = DivMagic{0, 1};
  for (int d = 2; d < kMaxDiv; d++) t[d] = make_div_magic((unsigned)d);
  cudaMemcpyToSymbol(c_div, t, sizeof(t));
}

namespace {

constexpr int kTPB = 256;
enum { IU = 1, IV = 2, IW = 4, IUV = 3, IUW = 5, IVW = 6, IUVW = 7 };

__device__ __forceinline__ u64 nck(int n, int k) { return nck_ref(n, k, c_div); }

// Arithmetic of a count: u64 with the reference's wrapping binomials (A = u64),
// or exact saturating 128-bit values (A = X128).
template <class A> __device__ __forceinline__ A nck_a(int n, int k);
template <> __device__ __forceinline__ u64 nck_a<u64>(int n, int k) { return nck(n, k); }
template <> __device__ __forceinline__ X128 nck_a<X128>(int n, int k) { return nck_x(n, k); }
__device__ __forceinline__ bool a_is_zero(u64 x) { return x == 0; }
__device__ __forceinline__ bool a_is_zero(const X128& x) { return x.is_zero(); }

// Adds one match's value: into the thread's running sum for an ordinary graph,
// into the result slot of the match's member graph for a packed graph.
__device__ __forceinline__ void credit(const GView& g, u64& acc, u64 x, int vertex) {
  if (g.comp == nullptr) acc += x;
  else if (x) atomicAdd(g.comp_slots + g.comp[vertex], x);
}
// exact counts run on ordinary graphs only
__device__ __forceinline__ void credit(const GView&, X128& acc, X128 x, int) { acc += x; }
__device__ __forceinline__ int relabel_of(const GView& g, int relabel, int vertex) {
  return g.comp ? (int)g.comp_relabel[g.comp[vertex]] : relabel;
}

// ------------------------------------------------------------- shared formulas
// Edge-core formula (src/fringeCount.cu:2030-2049) for an edge (u, v), where
// u is the endpoint with the larger vertex id and c_uv = |N(u) & N(v)|.
template <class A>
__device__ A edge_formula(int du, int dv, int c_uv, int f_u, int f_uv, int f_v) {
  const int a_uv = c_uv - f_uv;
  if (a_uv < 0) return 0;
  const int c_u = du - 1 - c_uv, c_v = dv - 1 - c_uv;
  const int bound = min(f_u, a_uv);
  A acc = 0;
  for (int j = 0; j <= bound; j++) {
    const int k = f_u - j;
    A term = nck_a<A>(c_u, k) * nck_a<A>(a_uv + c_v - j, f_v);
    if (f_u != f_v) term += nck_a<A>(c_v, k) * nck_a<A>(a_uv + c_u - j, f_v);
    acc += term * nck_a<A>(a_uv, j);
  }
  return acc * nck_a<A>(c_uv, f_uv);
}

// Binomials for wedge_formula_with: the count's arithmetic in general, and
// the two-case form when every k is 0 or 1 (nck01, equal for those k).
template <class A>
struct NckA {
  __device__ A operator()(int n, int k) const { return nck_a<A>(n, k); }
};
template <class A>
struct Nck01 {
  __device__ A operator()(int n, int k) const { return A(nck01(n, k)); }
};

// wedge() (src/fringeCount.cu:1381-1406) for endpoints x (larger id) and y.
template <class A>
__device__ __forceinline__ A wedge_formula(int dx, int dy, bool adj, int f_x, int f_xy, int f_y, int c) {
  if ((unsigned)(f_x | f_xy | f_y) <= 1u) return wedge_formula_with<A>(dx, dy, adj, f_x, f_xy, f_y, c, Nck01<A>());
  return wedge_formula_with<A>(dx, dy, adj, f_x, f_xy, f_y, c, NckA<A>());
}

// fc3 (src/fringeCount.cu:233-327): placements of the seven anchor-set types of
// a 3-vertex core into its seven exclusive Venn regions.  Same summation
// indices and the same nck factors per term as the reference.
template <class A>
__device__ A fc3(const int* fr, const int* venn) {
  const int fuvw = fr[IUVW], fuv = fr[IUV], fuw = fr[IUW], fvw = fr[IVW];
  const int fu = fr[IU], fv = fr[IV], fw = fr[IW];
  int x_uvw = venn[IUVW];
  const int x_uv = venn[IUV], x_uw = venn[IUW], x_vw = venn[IVW];
  const int x_u = venn[IU], x_v = venn[IV], x_w = venn[IW];
  if (x_uvw < fuvw) return 0;
  const A base = nck_a<A>(x_uvw, fuvw);
  x_uvw -= fuvw;
  A total = 0;
  for (int i = min(x_uvw, fuv); i >= 0; i--) {
    if (x_uv < fuv - i) break;
    const A t1 = base * nck_a<A>(x_uvw, i) * nck_a<A>(x_uv, fuv - i);
    const int r1 = x_uvw - i, r_uv = x_uv - (fuv - i);
    for (int j = min(r1, fuw); j >= 0; j--) {
      if (x_uw < fuw - j) break;
      const A t2 = t1 * nck_a<A>(r1, j) * nck_a<A>(x_uw, fuw - j);
      const int r2 = r1 - j, r_uw = x_uw - (fuw - j);
      for (int k = min(r2, fvw); k >= 0; k--) {
        if (x_vw < fvw - k) break;
        const A t3 = t2 * nck_a<A>(r2, k) * nck_a<A>(x_vw, fvw - k);
        const int r3 = r2 - k, r_vw = x_vw - (fvw - k);
        for (int a = min(r3, fu); a >= 0; a--) {
          const A ta = t3 * nck_a<A>(r3, a);
          const int pool_v = (r3 - a) + r_vw;
          for (int b = min(r_uv, fu - a); b >= 0; b--) {
            const A tb = ta * nck_a<A>(r_uv, b);
            const int r_uv2 = r_uv - b;
            for (int c = min(r_uw, fu - a - b); c >= 0; c--) {
              if (x_u < fu - a - b - c) break;
              const A tc = tb * nck_a<A>(r_uw, c) * nck_a<A>(x_u, fu - a - b - c);
              const int r_uw2 = r_uw - c;
              for (int d = min(pool_v, fv); d >= 0; d--) {
                if (r_uv2 + x_v < fv - d) break;
                const A td = tc * nck_a<A>(pool_v, d) * nck_a<A>(r_uv2 + x_v, fv - d);
                const int pool_w = (pool_v - d) + r_uw2 + x_w;
                if (pool_w >= fw) total += td * nck_a<A>(pool_w, fw);
              }
            }
          }
        }
      }
    }
  }
  return total;
}

struct Rot3 {
  int fr[6][8];
  int count;
};

// ------------------------------------------------------------- vertex core
template <class A>
__global__ void star_kernel(GView g, int t, u64* __restrict__ slot) {
  A acc = A(0);
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < g.n; v += gridDim.x * blockDim.x) {
    const int d = g.deg[v];
    if (d >= t) credit(g, acc, nck_a<A>(d, t), v);
  }
  block_sum_to(acc, slot);
}

// ------------------------------------------------------------- edge core
struct EdgeParams {
  int f_u, f_uv, f_v, lim1, lim2;
};


template <class A>
__global__ void edge_kernel(GView g, EdgeParams p, u64* __restrict__ slot) {
  const long long me = g.m / 2;
  A acc = A(0);
  for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < me; j += (long long)gridDim.x * blockDim.x) {
    const int a = g.osrc[j], b = g.oadj[j];
    const int u = max(a, b), v = min(a, b);  // the reference orients by id, v < u
    const int du = g.deg[u], dv = g.deg[v];
    if (!(du > p.lim1 && dv > p.lim1 && du + dv > p.lim2)) continue;  // init_wl_edge pruning
    credit(g, acc, edge_formula<A>(du, dv, (int)g.osup[j], p.f_u, p.f_uv, p.f_v), a);
  }
  block_sum_to(acc, slot);
}

// triangle with `tails` fringes on one vertex: sum over triangles of the three
// vertex terms = sum over vertices of (triangles at v) * C(deg v - 2, tails)
template <class A>
__global__ void tailed_triangle_kernel(GView g, const u64* __restrict__ vtri2, int tails, u64* __restrict__ slot) {
  A acc = A(0);
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < g.n; v += gridDim.x * blockDim.x) {
    const u64 t2 = vtri2[v];
    if (t2) credit(g, acc, A(t2 >> 1) * nck_a<A>(g.deg[v] - 2, tails), v);
  }
  block_sum_to(acc, slot);
}

// packed graphs: per-member sum of a per-vertex value (6 x triangles from vtri2)
__global__ void packed_vertex_sum_kernel(GView g, const u64* __restrict__ vals, u64* __restrict__ slot) {
  u64 acc = 0;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < g.n; v += gridDim.x * blockDim.x)
    credit(g, acc, vals[v], v);
  block_sum_to(acc, slot);
}

// Vertex- and edge-pass patterns counted together: one pass over the vertices
// (stars, tailed triangles) or the oriented edges (edge-core formulas) adds
// every pattern of the set into its own slot; each term is the single-pattern
// kernel's.  Ordinary graphs and u64 counts only.
constexpr int kPassFuse = 8;
struct VertexSet {
  int np;
  int tailed[kPassFuse];  // 0: star, sum C(deg v, t); 1: tailed triangle, triangles(v) * C(deg v - 2, t)
  int t[kPassFuse];
  u64* slot[kPassFuse];
};

__global__ void vertex_set_kernel(GView g, const u64* __restrict__ vtri2, VertexSet p) {
  u64 acc[kPassFuse];
#pragma unroll
  for (int q = 0; q < kPassFuse; q++) acc[q] = 0;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < g.n; v += gridDim.x * blockDim.x) {
    const int d = g.deg[v];
    const u64 t2 = vtri2 ? vtri2[v] : 0;
#pragma unroll
    for (int q = 0; q < kPassFuse; q++) {
      if (q >= p.np) break;
      if (p.tailed[q]) {
        if (t2) acc[q] += (t2 >> 1) * nck(d - 2, p.t[q]);
      } else if (d >= p.t[q]) {
        acc[q] += nck(d, p.t[q]);
      }
    }
  }
#pragma unroll
  for (int q = 0; q < kPassFuse; q++)
    if (q < p.np) block_sum_to(acc[q], p.slot[q]);
}

struct EdgeSet {
  int np;
  EdgeParams e[kPassFuse];
  u64* slot[kPassFuse];
};

__global__ void edge_set_kernel(GView g, EdgeSet p) {
  const long long me = g.m / 2;
  u64 acc[kPassFuse];
#pragma unroll
  for (int q = 0; q < kPassFuse; q++) acc[q] = 0;
  for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < me; j += (long long)gridDim.x * blockDim.x) {
    const int a = g.osrc[j], b = g.oadj[j];
    const int u = max(a, b), v = min(a, b);  // the reference orients by id, v < u
    const int du = g.deg[u], dv = g.deg[v];
    const int sup = (int)g.osup[j];
#pragma unroll
    for (int q = 0; q < kPassFuse; q++) {
      if (q >= p.np) break;
      const EdgeParams& e = p.e[q];
      if (du > e.lim1 && dv > e.lim1 && du + dv > e.lim2)  // init_wl_edge pruning
        acc[q] += edge_formula<u64>(du, dv, sup, e.f_u, e.f_uv, e.f_v);
    }
  }
#pragma unroll
  for (int q = 0; q < kPassFuse; q++)
    if (q < p.np) block_sum_to(acc[q], p.slot[q]);
}

// ------------------------------------------------------------- triangle core
struct TriParams {
  int sum1, sum2, sum3;
  int mode;   // 0 general, 1 4-clique, 2 tailed 4-clique
  int tails;
  int relabel;  // roles by (deg, id) order (1) or by id (0)
  int kmax;     // largest out-degree (bitmap kernel)
  int stage;    // bitmap kernel: longest N(a) staged in shared memory (ints, multiple of 32)
  int walk_ratio;  // bitmap kernel: walk N(b) when deg b <= walk_ratio * deg a
  Rot3 rot;
};

// Merge step over two sorted out-lists: advance (i,k) to the next common element.
__device__ __forceinline__ bool next_common(const int* A, int la, const int* B, int lb, int& i, int& k) {
  while (i < la && k < lb) {
    const int x = __ldg(A + i), y = __ldg(B + k);
    if (x < y) i++;
    else if (y < x) k++;
    else return true;
  }
  return false;
}

// warp-cooperative |L0 & L1 & L2| for three sorted lists, iterating the shortest
__device__ int warp_triple(const int* L0, int l0, const int* L1, int l1, const int* L2, int l2) {
  const int lane = threadIdx.x & 31;
  // put the shortest list first
  if (l1 < l0) { const int* t = L0; L0 = L1; L1 = t; int tl = l0; l0 = l1; l1 = tl; }
  if (l2 < l0) { const int* t = L0; L0 = L2; L2 = t; int tl = l0; l0 = l2; l2 = tl; }
  int c = 0;
  for (int i = lane; i < l0; i += 32) {
    const int x = __ldg(L0 + i);
    if (bsearch_has(L1, l1, x) && bsearch_has(L2, l2, x)) c++;
  }
  return __reduce_add_sync(0xffffffffu, c);
}

__device__ __forceinline__ long long tri_key(int x, int d, int relabel) {
  // larger key = later in the reference's vertex order (its new ids ascend
  // with descending (deg, id) after the relabel, with the id otherwise)
  return relabel ? -(((long long)d << 32) | (unsigned)x) : (long long)x;
}

// One lane per oriented edge (a -> b); triangles a < b < c are found by merging
// the out-lists.  Found triangles are served one at a time by the whole warp.
template <class Ar>  // (A and B name out-lists below)
__global__ void triangle_core_kernel(GView g, TriParams p, u64* __restrict__ slot) {
  const int lane = threadIdx.x & 31;
  const long long me = g.m / 2;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  Ar acc = Ar(0);
  for (long long base = ((long long)blockIdx.x * blockDim.x + threadIdx.x - lane); base < me; base += nwarps * 32) {
    const long long j = base + lane;
    bool live = j < me;
    int a = 0, b = 0, la = 0, lb = 0, i = 0, k = 0;
    const int *A = nullptr, *B = nullptr;
    long long aoff = 0, boff = 0;
    if (live) {
      a = g.osrc[j];
      b = g.oadj[j];
      aoff = g.ooff[a];
      boff = g.ooff[b];
      la = (int)(g.ooff[a + 1] - aoff);
      lb = (int)(g.ooff[b + 1] - boff);
      A = g.oadj + aoff;
      B = g.oadj + boff;
    }
    while (__any_sync(0xffffffffu, live)) {
      bool found = false;
      int c = 0;
      if (live) {
        found = next_common(A, la, B, lb, i, k);
        if (!found) live = false;
        else c = A[i];
      }
      if (p.mode != 0) {
        // 4-cliques a < b < c < d: d in out(a) & out(b) & out(c)
        if (found) {
          const long long coff = g.ooff[c];
          const int lc = (int)(g.ooff[c + 1] - coff);
          const int* C = g.oadj + coff;
          for (int t = 0; t < lc; t++) {
            const int d = __ldg(C + t);
            if (bsearch_has(A, la, d) && bsearch_has(B, lb, d)) {
              if (p.mode == 1) credit(g, acc, Ar(1), a);
              else credit(g, acc, nck_a<Ar>(g.deg[a] - 3, p.tails) + nck_a<Ar>(g.deg[b] - 3, p.tails) +
                                  nck_a<Ar>(g.deg[c] - 3, p.tails) + nck_a<Ar>(g.deg[d] - 3, p.tails), a);
            }
          }
        }
      } else {
        // roles: u latest, w earliest in the reference's vertex order
        int x[3], dx[3];
        unsigned sx[3];  // support of the edge opposite... indexed by vertex pair below
        int venn[8];
        bool take = false;
        if (found) {
          x[0] = a; x[1] = b; x[2] = c;
          dx[0] = g.deg[a]; dx[1] = g.deg[b]; dx[2] = g.deg[c];
          // supports of edges ab, ac, bc
          const unsigned s_ab = g.osup[j], s_ac = g.osup[aoff + i], s_bc = g.osup[boff + k];
          // sort the three vertices by key descending: u, v, w
          const int rl = relabel_of(g, p.relabel, a);
          long long kx[3] = {tri_key(a, dx[0], rl), tri_key(b, dx[1], rl), tri_key(c, dx[2], rl)};
          int ord[3] = {0, 1, 2};
          if (kx[ord[0]] < kx[ord[1]]) { int t = ord[0]; ord[0] = ord[1]; ord[1] = t; }
          if (kx[ord[1]] < kx[ord[2]]) { int t = ord[1]; ord[1] = ord[2]; ord[2] = t; }
          if (kx[ord[0]] < kx[ord[1]]) { int t = ord[0]; ord[0] = ord[1]; ord[1] = t; }
          // pair support lookup
          auto sup = [&](int p0, int p1) -> unsigned {
            const int lo = min(p0, p1), hi = max(p0, p1);
            return (lo == 0) ? (hi == 1 ? s_ab : s_ac) : s_bc;
          };
          const int iu = ord[0], iv = ord[1], iw = ord[2];
          const int du = dx[iu], dv = dx[iv], dw = dx[iw];
          // the reference's pruning (init_wl_triangle, common3_triangle)
          const int th1 = max(p.sum1, p.sum2 - du);
          const int th2 = max(max(p.sum1, p.sum3 - du - dv), max(p.sum2 - du, p.sum2 - dv));
          take = (du >= p.sum1) && (dv >= th1) && (dw >= th2);
          venn[IUV] = (int)sup(iu, iv);
          venn[IUW] = (int)sup(iu, iw);
          venn[IVW] = (int)sup(iv, iw);
          venn[IU] = du; venn[IV] = dv; venn[IW] = dw;
          sx[0] = x[iu]; sx[1] = x[iv]; sx[2] = x[iw];
        }
        // triple overlaps, one triangle at a time across the warp
        unsigned bal = __ballot_sync(0xffffffffu, take);
        int c123 = 0;
        while (bal) {
          const int who = __ffs(bal) - 1;
          bal &= bal - 1;
          const int q0 = __shfl_sync(0xffffffffu, (int)sx[0], who);
          const int q1 = __shfl_sync(0xffffffffu, (int)sx[1], who);
          const int q2 = __shfl_sync(0xffffffffu, (int)sx[2], who);
          const long long o0 = g.off[q0], o1 = g.off[q1], o2 = g.off[q2];
          const int r = warp_triple(g.adj + o0, (int)(g.off[q0 + 1] - o0), g.adj + o1, (int)(g.off[q1 + 1] - o1),
                                    g.adj + o2, (int)(g.off[q2 + 1] - o2));
          if (lane == who) c123 = r;
        }
        if (take) {
          // com3 (src/fringeCount.cu:934-964): exclusive regions without the
          // triangle's own vertices
          const int p12 = venn[IUV], t13 = venn[IUW], t23 = venn[IVW];
          const int c12 = p12 - (c123 + 1), c13 = t13 - (c123 + 1), c23 = t23 - (c123 + 1);
          const int du = venn[IU], dv = venn[IV], dw = venn[IW];
          venn[0] = 0;
          venn[IU] = du - (c12 + c13 + (c123 + 2));
          venn[IV] = dv - (c12 + c23 + (c123 + 2));
          venn[IW] = dw - (c13 + c23 + (c123 + 2));
          venn[IUV] = c12; venn[IUW] = c13; venn[IVW] = c23; venn[IUVW] = c123;
          Ar t = Ar(0);
          for (int r = 0; r < p.rot.count; r++) t += fc3<Ar>(p.rot.fr[r], venn);
          credit(g, acc, t, a);
        }
      }
      if (found) { i++; k++; }
    }
  }
  block_sum_to(acc, slot);
}

// Triangle core, general placements: one block per vertex a, handling every
// triangle whose lowest (deg, id) vertex is a.  For each out-neighbour b_i of a
// the block builds the bitmap M_i of N(a) & N(b_i) over the positions of N(a).
// Then a pair (b_i, b_j) is a triangle iff bit pos(b_j) of M_i is set,
// |N(a) & N(b_i)| = popc(M_i), and the triple overlap |N(a) & N(b_i) & N(b_j)|
// = popc(M_i & M_j) -- a few word operations per triangle instead of an
// intersection of full neighbour lists.
//
// N(a) is staged in shared memory by a bulk copy when it fits p.stage ints.  A
// row then takes the cheaper of two ways: walk N(b_i) from global memory
// (coalesced) and look each entry up in the staged N(a), building the row in
// a per-warp shared buffer, when deg b_i <= p.walk_ratio * deg a; otherwise
// test each entry of N(a) by a binary search of N(b_i) (one ballot per 32).
constexpr int kTriThreads = 256;
constexpr int kBulkWaitPolls = 1 << 22;  // bounded wait for a bulk copy

// Triangle-core patterns of one pass: the bitmaps, roles and Venn sizes of a
// triangle do not depend on the pattern, only the pruning thresholds and the
// placement formulas do.  p.sum1 (the vertex gate) is the set's smallest.
// Every launch today carries one pattern (see enqueue_count_set).
constexpr int kTriFuse = 4;
struct TriSet {
  int np;
  int sum1[kTriFuse], sum2[kTriFuse], sum3[kTriFuse];
  Rot3 rot[kTriFuse];
  u64* slot[kTriFuse];
};

template <int NP, class A>
__global__ void __launch_bounds__(kTriThreads, 3) triangle_bitmap_kernel(GView g, TriParams p, TriSet ts,
                                                                      int* __restrict__ queue,
                                                                      unsigned* __restrict__ bits_all,
                                                                      long long bits_per_block,
                                                                      unsigned long long* __restrict__ err) {
  extern __shared__ __align__(16) int s_dyn[];
  __shared__ int s_a;
  __shared__ __align__(8) unsigned long long s_bar;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  unsigned* bits = bits_all + (size_t)blockIdx.x * (size_t)bits_per_block;
  const int kmax = p.kmax, stage = p.stage;
  int* s_na = s_dyn;                              // staged N(a): stage + 4 ints (16-byte aligned)
  unsigned* s_row = reinterpret_cast<unsigned*>(s_dyn + stage + 4);  // per warp: stage / 32 words
  int* outl = s_dyn + stage + 4 + (stage >> 5) * (kTriThreads >> 5);  // out-neighbours of a
  int* pos = outl + kmax;                         // their positions in N(a)
  int* rowpop = outl + 2 * kmax;                  // |N(a) & N(b_i)|
  unsigned parity = 0;
  if (threadIdx.x == 0 && stage > 0) mbar_init(&s_bar, 1);
  __syncthreads();
  A acc[NP];
#pragma unroll
  for (int q = 0; q < NP; q++) acc[q] = A(0);
  for (;;) {
    if (threadIdx.x == 0) s_a = atomicAdd(queue, 1);
    __syncthreads();
    const int a = s_a;
    if (a >= g.n) break;
    const long long ob = g.ooff[a];
    const int k = (int)(g.ooff[a + 1] - ob);
    const int da = g.deg[a];
    if (k >= 2 && da >= p.sum1) {
      const int W = (da + 31) >> 5;
      const long long abeg = g.off[a];
      const bool staged = da <= stage;
      const int* Na = g.adj + abeg;
      if (staged) {
        // the copy starts at the 16-byte boundary at or below N(a) (the list
        // array is padded by 16 bytes, so the rounded-up end stays inside it)
        const long long cbeg = abeg & ~3LL;
        const int shift = (int)(abeg - cbeg);
        if (threadIdx.x == 0) {
          fence_proxy_async_smem();
          const unsigned bytes = (unsigned)(((shift + da) * 4 + 15) & ~15);
          bulk_copy_g2s(s_na, g.adj + cbeg, bytes, &s_bar);
        }
        const bool done = mbar_wait_bounded(&s_bar, parity, kBulkWaitPolls);
        parity ^= 1u;
        if (__syncthreads_or(!done)) {
          // the copy did not complete: report it, give the copy one more
          // bounded wait and leave (the count is void)
          if (threadIdx.x == 0) atomicOr(err, 1ULL);
          mbar_wait_bounded(&s_bar, parity ^ 1u, kBulkWaitPolls);
          return;
        }
        Na = s_na + shift;
      }
      for (int i = threadIdx.x; i < k; i += blockDim.x) {
        const int b = g.oadj[ob + i];
        outl[i] = b;
        pos[i] = lower_bound_any(Na, da, b);  // Na may be the shared-memory stage
        rowpop[i] = (int)g.osup[ob + i];  // |N(a) & N(b_i)| is the edge's support
      }
      // bitmaps: row i = N(a) & N(b_i), skipped when the edge closes no triangle
      unsigned* wrow = s_row + warp * (stage >> 5);
      for (int i = warp; i < k; i += nwarp) {
        if (g.osup[ob + i] == 0) continue;
        const int b = g.oadj[ob + i];
        const int* Nb = g.adj + g.off[b];
        const int db = g.deg[b];
        unsigned* row = bits + (size_t)i * W;
        if (staged && (long long)db <= (long long)p.walk_ratio * da) {
          for (int w = lane; w < W; w += 32) wrow[w] = 0u;
          __syncwarp();
          // only N(b) entries inside [min N(a), max N(a)] can match
          const int t0 = lower_bound_dev(Nb, db, Na[0]);
          const int t1 = lower_bound_dev(Nb, db, Na[da - 1] + 1);
          for (int t = t0 + lane; t < t1; t += 32) {
            const int y = __ldg(Nb + t);
            int lo = 0, hi = da;  // y's position in the staged N(a)
            while (lo < hi) {
              const int mid = (lo + hi) >> 1;
              if (Na[mid] < y) lo = mid + 1;
              else hi = mid;
            }
            if (lo < da && Na[lo] == y) atomicOr(&wrow[lo >> 5], 1u << (lo & 31));
          }
          __syncwarp();
          for (int w = lane; w < W; w += 32) row[w] = wrow[w];
          __syncwarp();
        } else {
          for (int w = 0; w < W; w++) {
            const int x = w * 32 + lane;
            const bool hit = (x < da) && bsearch_has(Nb, db, Na[x]);
            const unsigned word = __ballot_sync(0xffffffffu, hit);
            if (lane == 0) row[w] = word;
          }
        }
      }
      __syncthreads();
      // pairs (i, j), i < j: warp per row, lanes over j
      for (int i = warp; i < k - 1; i += nwarp) {
        if (rowpop[i] == 0) continue;
        const unsigned* Mi = bits + (size_t)i * W;
        const int bi = outl[i], di = g.deg[bi];
        for (int j = i + 1 + lane; j < k; j += 32) {
          const int pj = pos[j];
          if (!((Mi[pj >> 5] >> (pj & 31)) & 1u)) continue;
          const int bj = outl[j], dj = g.deg[bj];
          const unsigned* Mj = bits + (size_t)j * W;
          int c123 = 0;
          for (int w = 0; w < W; w++) c123 += __popc(Mi[w] & Mj[w]);
          // support of edge (b_i, b_j): slot in the out-list of the lower one
          const bool i_low = (di < dj) || (di == dj && bi < bj);
          const int lo = i_low ? bi : bj, hi = i_low ? bj : bi;
          const long long lb = g.ooff[lo];
          const int sl = bsearch_pos(g.oadj + lb, (int)(g.ooff[lo + 1] - lb), hi);
          const int s_ij = (int)g.osup[lb + sl];
          // roles u (latest), v, w (earliest) in the reference's vertex order
          const int xv[3] = {a, bi, bj};
          const int dx[3] = {da, di, dj};
          long long kx[3];
          const int rl = relabel_of(g, p.relabel, a);
          for (int t = 0; t < 3; t++) kx[t] = tri_key(xv[t], dx[t], rl);
          int ord[3] = {0, 1, 2};
          if (kx[ord[0]] < kx[ord[1]]) { int t = ord[0]; ord[0] = ord[1]; ord[1] = t; }
          if (kx[ord[1]] < kx[ord[2]]) { int t = ord[1]; ord[1] = ord[2]; ord[2] = t; }
          if (kx[ord[0]] < kx[ord[1]]) { int t = ord[0]; ord[0] = ord[1]; ord[1] = t; }
          // pairwise overlaps by vertex slot: 0 = a, 1 = b_i, 2 = b_j
          const int sup01 = rowpop[i], sup02 = rowpop[j], sup12 = s_ij;
          auto sup = [&](int x, int y) {
            const int s = x + y;  // 1 -> (0,1), 2 -> (0,2), 3 -> (1,2)
            return s == 1 ? sup01 : (s == 2 ? sup02 : sup12);
          };
          const int iu = ord[0], iv = ord[1], iw = ord[2];
          const int du = dx[iu], dv = dx[iv], dw = dx[iw];
          const int p12 = sup(iu, iv), t13 = sup(iu, iw), t23 = sup(iv, iw);
          const int c12 = p12 - (c123 + 1), c13 = t13 - (c123 + 1), c23 = t23 - (c123 + 1);
          int venn[8];
          venn[0] = 0;
          venn[IU] = du - (c12 + c13 + (c123 + 2));
          venn[IV] = dv - (c12 + c23 + (c123 + 2));
          venn[IW] = dw - (c13 + c23 + (c123 + 2));
          venn[IUV] = c12; venn[IUW] = c13; venn[IVW] = c23; venn[IUVW] = c123;
#pragma unroll
          for (int q = 0; q < NP; q++) {
            if (q >= ts.np) break;
            // the reference's pruning (init_wl_triangle, common3_triangle)
            const int th1 = max(ts.sum1[q], ts.sum2[q] - du);
            const int th2 = max(max(ts.sum1[q], ts.sum3[q] - du - dv), max(ts.sum2[q] - du, ts.sum2[q] - dv));
            if (!((du >= ts.sum1[q]) && (dv >= th1) && (dw >= th2))) continue;
            A t = A(0);
            for (int r = 0; r < ts.rot[q].count; r++) t += fc3<A>(ts.rot[q].fr[r], venn);
            credit(g, acc[q], t, a);
          }
        }
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < NP; q++)
    if (q < ts.np) block_sum_to(acc[q], ts.slot[q]);
}

// ------------------------------------------------------------- wedge core
struct WedgeParams {
  int f_v, f_vw, f_w;  // fringes of the larger-id endpoint, both, the other
  int lim, minsum;     // min(min_v, min_w) and min_v + min_w
};

// Centre without fringes (wedgecore_specialized, src/fringeCount.cu:1409-1477).
// The reference evaluates wedge() once per (centre u, endpoints v > w); the
// value depends only on the endpoints and their centre count C = |N(v) & N(w)|,
// so here each endpoint pair is evaluated once and weighted by C: one block per
// endpoint v (from a queue) counts, for every w < v, the centres u in N(v) with
// w in N(u), with the counts kept in shared memory.  The ids w < v are swept in chunks of CH ids; per chunk every
// centre u in N(v) contributes the segment of N(u) inside the chunk (a cursor
// per centre walks each sorted list once; segment ends are found by galloping
// from the cursor).  The segment lengths are prefix-summed and every warp takes
// a contiguous range of the chunk's elements, following segment boundaries as
// it goes.  Counts go to shared-memory counters; the counters are then scanned,
// the non-zero ones compacted per warp so that every lane evaluates one pair,
// and cleared.  Chunks no centre reaches are skipped.
//
// SMALL (deg v <= kWDvMax): two 16-bit counters per word (a centre count never
// exceeds deg v < 2^16) and the per-centre cursors in shared memory.
// BIG (hub endpoints): 32-bit counters, cursors in a per-block global array.
constexpr int kWDvMax = 2048;
constexpr int kWThreads = 1024;
constexpr int kWGran = 32768;  // ids between the chunk boundaries in the boundary table

// SMALL packs counters of 16, 8 or 4 bits into 32-bit words, the narrowest
// that holds the owner's degree (a count C(v, w) never exceeds deg v), so one
// chunk covers 65,536, 131,072 or 262,144 ids; BIG uses 32-bit counters.
template <bool BIG>
struct WedgeCfg {
  static constexpr int CH = BIG ? 32768 : 65536;   // ids per chunk at 16-bit (BIG: 32-bit) counters
  static constexpr int WORDS = BIG ? CH : CH / 2;  // counter words
  static constexpr int TW = WORDS / 32;            // touched-bitmap words (= kWThreads)
  static constexpr int CH_MAX = BIG ? CH : 4 * CH; // widest chunk (4-bit counters)
};

// One bit, the lowest of the counter, for every non-zero `bits`-wide counter of
// `word` (bits = 4, 8, 16 or 32): each counter's bits are OR-folded into its
// lowest bit.
__device__ __forceinline__ unsigned nonzero_counter_bits(unsigned word, int bits) {
  if (bits == 32) return word != 0u ? 1u : 0u;
  unsigned t = word;
  for (int s = bits >> 1; s > 0; s >>= 1) t |= t >> s;
  return t & (bits == 16 ? 0x00010001u : (bits == 8 ? 0x01010101u : 0x11111111u));
}

// Position of the n-th (from 0) set bit of mask, which has more than n set
// bits: a halving search on the population counts of the low halves.
__device__ __forceinline__ int nth_set_bit(unsigned mask, int n) {
  int pos = 0;
  for (int w = 16; w >= 1; w >>= 1) {
    const int c = __popc(mask & ((1u << w) - 1u));
    if (n >= c) {
      n -= c;
      mask >>= w;
      pos += w;
    }
  }
  return pos;
}

// counter width for an owner of degree dv (SMALL kernel)
__device__ __forceinline__ int wedge_counter_bits(int dv) { return dv <= 15 ? 4 : (dv <= 255 ? 8 : 16); }
static_assert(WedgeCfg<false>::TW == kWThreads && WedgeCfg<true>::TW == kWThreads, "one bitmap word per thread");

// One non-zero counter handed from the counter words to the evaluation: its
// offset o in the chunk and its centre count C.  SMALL: o < 2^18 and
// C <= kWDvMax pack into 32 bits; BIG: 32-bit counts take 64.
template <bool BIG>
struct WedgePair {
  using T = unsigned;
  __device__ static T pack(int o, unsigned c) { return ((unsigned)o << 12) | c; }
  __device__ static int off(T x) { return (int)(x >> 12); }
  __device__ static unsigned count(T x) { return x & 0xfffu; }
};
template <>
struct WedgePair<true> {
  using T = unsigned long long;
  __device__ static T pack(int o, unsigned c) { return ((unsigned long long)o << 32) | c; }
  __device__ static int off(T x) { return (int)(x >> 32); }
  __device__ static unsigned count(T x) { return (unsigned)x; }
};
static_assert(kWDvMax < 4096 && WedgeCfg<false>::CH_MAX <= (1 << 20), "SMALL pairs pack into 32 bits");
constexpr int kPairBuf = 128;  // pairs staged per warp and pass

template <bool BIG>
struct WedgeSmem {
  unsigned cnt[WedgeCfg<BIG>::WORDS];
  unsigned touched[WedgeCfg<BIG>::TW];  // counter words that became non-zero
  int tpre[WedgeCfg<BIG>::TW + 1];      // prefix of touched popcounts
  unsigned adjbits[WedgeCfg<BIG>::CH_MAX / 32];
  long long cur[BIG ? 1 : kWDvMax];
  long long lim[BIG ? 1 : kWDvMax];
  typename WedgePair<BIG>::T pairs[kWThreads / 32][kPairBuf];
  int pre[BIG ? 1 : kWDvMax + 1];
  int warp_tmp[33];
  int v;
  int lo;
  int grab;  // next touched word to evaluate
};
// dynamic shared memory of one block, with 1 KB left for the reductions' static arrays
static_assert(sizeof(WedgeSmem<false>) + 1024 <= 232448 && sizeof(WedgeSmem<true>) + 1024 <= 232448,
              "wedge kernel shared memory");

// Per high-degree vertex u: offsets in N(u) of the first neighbour >= k *
// kWGran, for every k.  A chunk that ends on such a boundary finds the end of
// u's segment with one load instead of a search.
struct ChunkTable {
  const int* id;   // n entries: row of u, or -1
  const int* pos;  // rows of K offsets
  int K;
};

// first index i in [from, to) with a[i] >= x, searching outward from `from`
__device__ __forceinline__ long long gallop_lb(const int* __restrict__ a, long long from, long long to, int x) {
  if (from >= to || __ldg(a + from) >= x) return from;
  long long p = from, step = 1;  // invariant: a[p] < x
  while (p + step < to && __ldg(a + p + step) < x) {
    p += step;
    step <<= 1;
  }
  long long l = p + 1, r = min(p + step, to);  // answer in [l, r]
  while (l < r) {
    const long long m = (l + r) >> 1;
    if (__ldg(a + m) < x) l = m + 1;
    else r = m;
  }
  return l;
}

// block-wide exclusive scan of x[0..n) in place (x[n] = total); every thread calls
template <bool BIG>
__device__ void block_scan_inplace(int* x, int n, WedgeSmem<BIG>& S) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = blockDim.x >> 5;
  int carry = 0;
  for (int base = 0; base < n; base += 2 * blockDim.x) {
    const int i0 = base + 2 * tid, i1 = i0 + 1;
    const int x0 = (i0 < n) ? x[i0] : 0, x1 = (i1 < n) ? x[i1] : 0;
    const int sum = x0 + x1;
    int inc = sum;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += y;
    }
    if (lane == 31) S.warp_tmp[warp] = inc;
    __syncthreads();
    if (warp == 0) {
      const int wv = (lane < nwarp) ? S.warp_tmp[lane] : 0;
      int wi = wv;
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, wi, o);
        if (lane >= o) wi += y;
      }
      if (lane < nwarp) S.warp_tmp[lane] = wi - wv;
      if (lane == 31) S.warp_tmp[32] = wi;
    }
    __syncthreads();
    const int ex = carry + S.warp_tmp[warp] + inc - sum;
    if (i0 < n) x[i0] = ex;
    if (i1 < n) x[i1] = ex + x0;
    carry += S.warp_tmp[32];
    __syncthreads();
  }
  if (tid == 0) x[n] = carry;
}

// Patterns of this core shape counted together: the centre counts C(v, w)
// do not depend on the pattern, so one counting pass serves every pattern of
// the set and each pair is evaluated once per pattern.  lim is the smallest
// endpoint degree any of them takes.
constexpr int kWedgeFuse = 4;
struct WedgeSet {
  int np;
  int lim;
  int small_max;  // endpoints up to this degree go to the SMALL kernel (<= kWDvMax)
  WedgeParams w[kWedgeFuse];
  u64* slot[kWedgeFuse];
};

template <bool BIG, int NP, class A>
__device__ __forceinline__ void eval_pair(const GView& g, const WedgeSet& ws, WedgeSmem<BIG>& S, int o, unsigned C,
                                          int dw, int v, int dv, A* acc) {
  const bool vw = (S.adjbits[o >> 5] >> (o & 31)) & 1u;
#pragma unroll
  for (int q = 0; q < NP; q++) {
    if (q >= ws.np) break;
    const WedgeParams& p = ws.w[q];
    if (dv >= p.lim && dw >= max(p.lim, p.minsum - dv))
      credit(g, acc[q], A((u64)C) * wedge_formula<A>(dv, dw, vw, p.f_v, p.f_vw, p.f_w, (int)C - 1), v);
  }
}

template <bool BIG, int NP, class A>
__global__ void __launch_bounds__(kWThreads, 1) wedge_chunk_kernel(GView g, WedgeSet ws, int* __restrict__ queue,
                                                                   long long* __restrict__ gcur, int* __restrict__ gpre,
                                                                   long long gstride, ChunkTable tab) {
  constexpr int WORDS = WedgeCfg<BIG>::WORDS;
  constexpr int TW = WedgeCfg<BIG>::TW;
  extern __shared__ unsigned char s_raw[];
  WedgeSmem<BIG>& S = *reinterpret_cast<WedgeSmem<BIG>*>(s_raw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = blockDim.x >> 5;
  long long* cur = BIG ? gcur + (size_t)blockIdx.x * 2 * gstride : S.cur;
  long long* lim = BIG ? cur + gstride : S.lim;
  int* pre = BIG ? gpre + (size_t)blockIdx.x * (gstride + 1) : S.pre;
  for (int i = tid; i < WORDS; i += blockDim.x) S.cnt[i] = 0;
  for (int i = tid; i < TW; i += blockDim.x) S.touched[i] = 0;
  for (int i = tid; i < WedgeCfg<BIG>::CH_MAX / 32; i += blockDim.x) S.adjbits[i] = 0;
  A acc[NP];
#pragma unroll
  for (int q = 0; q < NP; q++) acc[q] = A(0);
  for (;;) {
    if (tid == 0) {
      S.v = atomicAdd(queue, 1);
      S.lo = 0;
    }
    __syncthreads();
    const int v = S.v;
    if (v >= g.n) break;
    const int dv = g.deg[v];
    if (dv < ws.lim || (BIG ? dv <= ws.small_max : dv > ws.small_max)) {
      __syncthreads();
      continue;
    }
    // counter layout: `bits` per counter, 2^lper counters per word, CH ids per chunk
    const int bits = BIG ? 32 : wedge_counter_bits(dv);
    const int lper = BIG ? 0 : (bits == 16 ? 1 : (bits == 8 ? 2 : 3));
    const int CH = WORDS << lper;
    const long long vb = g.off[v];
    const int* Nv = g.adj + vb;
    for (int t = tid; t < dv; t += blockDim.x) {
      const int u = __ldg(Nv + t);
      cur[t] = g.off[u];
      lim[t] = g.off[u + 1];
    }
    int cv = 0;  // cursor into N(v) for the adjacency marks
    __syncthreads();
    while (S.lo < v) {
      const int lo = S.lo;  // a multiple of CH
      const int hi = min(lo + CH, v);
      const bool aligned = (hi % kWGran) == 0;
      // segment of each centre's list inside [lo, hi): table lookup for
      // high-degree centres at aligned chunk ends, a gallop from the cursor otherwise
      for (int t = tid; t < dv; t += blockDim.x) {
        const long long c = cur[t];
        long long e = -1;
        if (aligned && tab.id) {
          const int u = __ldg(Nv + t);
          const int row = __ldg(tab.id + u);
          if (row >= 0) e = g.off[u] + __ldg(tab.pos + (size_t)row * tab.K + hi / kWGran);
        }
        if (e < 0) e = gallop_lb(g.adj, c, lim[t], hi);
        pre[t] = (int)(e - c);
      }
      const int cs = cv + lower_bound_dev(Nv + cv, dv - cv, lo);
      const int cend = cs + lower_bound_dev(Nv + cs, dv - cs, hi);
      for (int i = cs + tid; i < cend; i += blockDim.x) {
        const int o = __ldg(Nv + i) - lo;
        atomicOr(&S.adjbits[o >> 5], 1u << (o & 31));
      }
      __syncthreads();
      block_scan_inplace<BIG>(pre, dv, S);
      __syncthreads();
      // count: warp-contiguous ranges of the chunk's elements
      {
        const int L = pre[dv];
        const int ws = (int)(((long long)L * warp) / nwarp), we = (int)(((long long)L * (warp + 1)) / nwarp);
        if (ws < we) {
          int a = 0, b = dv;  // last segment with pre <= ws
          while (b - a > 1) {
            const int mid = (a + b) >> 1;
            if (pre[mid] <= ws) a = mid;
            else b = mid;
          }
          for (int e0 = ws; e0 < we; e0 += 32) {
            const int e = e0 + lane;
            int al = a;
            if (e < we) {
              while (pre[al + 1] <= e) al++;
              const int o = __ldg(g.adj + cur[al] + (e - pre[al])) - lo;
              const int wd = o >> lper;
              const unsigned old = atomicAdd(&S.cnt[wd], BIG ? 1u : (1u << ((o & ((1 << lper) - 1)) * bits)));
              if (old == 0) atomicOr(&S.touched[wd >> 5], 1u << (wd & 31));
            }
            a = __shfl_sync(0xffffffffu, al, 31);
          }
        }
      }
      __syncthreads();
      // evaluate: the chunk's touched counter words are numbered by a prefix
      // over the touched-bitmap words; a warp takes 32 words at a time, one
      // per lane, prefix-sums their non-zero counters, writes
      // them as (offset, centre count) pairs into its shared-memory buffer and
      // then evaluates one pair per lane per step, so the lanes evaluate in
      // lockstep and adjacent lanes take adjacent endpoints.
      {
        const int nw = (hi - lo + (1 << lper) - 1) >> lper;
        const int ntw = (nw + 31) >> 5;
        const int c0 = (tid < ntw) ? __popc(S.touched[tid]) : 0;
        int inc = c0;
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(0xffffffffu, inc, o);
          if (lane >= o) inc += y;
        }
        if (lane == 31) S.warp_tmp[warp] = inc;
        __syncthreads();
        if (warp == 0) {
          const int wv = (lane < nwarp) ? S.warp_tmp[lane] : 0;
          int wi = wv;
          for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += y;
          }
          if (lane < nwarp) S.warp_tmp[lane] = wi - wv;
          if (lane == 31) S.warp_tmp[32] = wi;
        }
        __syncthreads();
        S.tpre[tid] = S.warp_tmp[warp] + inc - c0;
        const int T = S.warp_tmp[32];
        if (tid == 0) S.grab = 0;
        __syncthreads();
        const int lbits = BIG ? 5 : (lper == 1 ? 4 : (lper == 2 ? 3 : 2));  // log2(bits)
        const unsigned cmask = BIG ? 0xffffffffu : ((1u << bits) - 1);
        using PT = WedgePair<BIG>;
        typename PT::T* buf = S.pairs[warp];
        // warps take the touched words 32 at a time from a shared counter, so
        // a warp whose words hold more pairs takes fewer of them
        for (;;) {
          int W = 0;
          if (lane == 0) W = atomicAdd(&S.grab, 32);
          W = __shfl_sync(0xffffffffu, W, 0);
          if (W >= T) break;
          const int W1 = min(W + 32, T);
          const int idx = W + lane;
          int wd = 0, c = 0;
          unsigned word = 0, nz = 0;
          if (idx < W1) {
            int a = 0, b = ntw;  // bitmap word holding touched word `idx`: last with tpre <= idx
            while (b - a > 1) {
              const int mid = (a + b) >> 1;
              if (S.tpre[mid] <= idx) a = mid;
              else b = mid;
            }
            wd = (a << 5) + nth_set_bit(S.touched[a], idx - S.tpre[a]);
            word = S.cnt[wd];
            nz = nonzero_counter_bits(word, bits);
            c = __popc(nz);
          }
          int incl = c;
          for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
          }
          const int excl = incl - c;
          const int P = __shfl_sync(0xffffffffu, incl, 31);
          // pairs excl .. excl + c - 1 are this lane's; a pass stages the
          // pairs [base, base + kPairBuf) and evaluates them
          for (int base = 0; base < P; base += kPairBuf) {
            unsigned mk = nz;
            for (int t = 0; t < c; t++) {
              const int kbit = __ffs(mk) - 1;  // low bit of the counter
              mk &= mk - 1;
              const int pos = excl + t - base;
              if (pos >= 0 && pos < kPairBuf) buf[pos] = PT::pack((wd << lper) + (kbit >> lbits), (word >> kbit) & cmask);
            }
            __syncwarp();
            const int np = min(kPairBuf, P - base);
            for (int i = lane; i < np; i += 32) {
              const typename PT::T x = buf[i];
              const int o = PT::off(x);
              eval_pair<BIG, NP, A>(g, ws, S, o, PT::count(x), __ldg(g.deg + lo + o), v, dv, acc);
            }
            __syncwarp();
          }
        }
      }
      // advance the cursors and find the next id any centre still reaches
      int nxt = 0x7fffffff;
      for (int t = tid; t < dv; t += blockDim.x) {
        const long long c = cur[t] + (pre[t + 1] - pre[t]);
        cur[t] = c;
        if (c < lim[t]) nxt = min(nxt, __ldg(g.adj + c));
      }
      nxt = __reduce_min_sync(0xffffffffu, nxt);
      if (tid == 0) S.lo = v;
      __syncthreads();  // touched, adjbits, pre and S.lo are free again
      for (int i = tid; i < TW; i += blockDim.x) {
        for (unsigned mk = S.touched[i]; mk; mk &= mk - 1) S.cnt[(i << 5) + __ffs(mk) - 1] = 0;
        S.touched[i] = 0;
      }
      for (int i = cs + tid; i < cend; i += blockDim.x) S.adjbits[(__ldg(Nv + i) - lo) >> 5] = 0;
      cv = cend;
      if (lane == 0 && nxt < v) atomicMin(&S.lo, max(hi, (nxt / CH) * CH));
      __syncthreads();
    }
  }
#pragma unroll
  for (int q = 0; q < NP; q++)
    if (q < ws.np) block_sum_to(acc[q], ws.slot[q]);
}

// boundary table: pass 1 gives each vertex of degree >= min_deg a row
__global__ void chunk_table_rows_kernel(GView g, int min_deg, int* __restrict__ id, int* __restrict__ rows,
                                        int* __restrict__ nrows) {
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < g.n; u += gridDim.x * blockDim.x) {
    int r = -1;
    if (g.deg[u] >= min_deg) {
      r = atomicAdd(nrows, 1);
      rows[r] = u;
    }
    id[u] = r;
  }
}

// pass 2: row r, column k = first position in N(rows[r]) with neighbour >= k * kWGran
__global__ void chunk_table_fill_kernel(GView g, const int* __restrict__ rows, int nrows, int K, int* __restrict__ pos) {
  const long long total = (long long)nrows * K;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i / K), k = (int)(i % K);
    const int u = rows[r];
    const long long b = g.off[u];
    const long long x = (long long)k * kWGran;
    pos[i] = (x > 0x7fffffffLL) ? (int)(g.off[u + 1] - b) : lower_bound_dev(g.adj + b, (int)(g.off[u + 1] - b), (int)x);
  }
}

struct GWedgeParams {
  int min_u, lim, sum1, sum2, sum3;
  Rot3 rot;
};

// Centre with fringes (general_wedge_core, src/fringeCount.cu:1480-1650): one
// warp per centre u, looping over endpoints v in N(u); lanes take w in N(u),
// w < v; open wedges use rotations 0 (and 3), triangles (counted once, with
// u < w < v) use all rotations.
template <class A>
__global__ void wedge_general_kernel(GView g, GWedgeParams p, const unsigned* __restrict__ esup,
                                     u64* __restrict__ slot) {
  const int lane = threadIdx.x & 31;
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  A acc = A(0);
  // one warp per list entry (u, v): a hub centre's pairs spread over as many
  // warps as it has neighbours
  for (long long j = wid; j < g.m; j += nw) {
    int lo = 0, hi = g.n;  // u = the last vertex with off[u] <= j
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (g.off[mid] <= j) lo = mid;
      else hi = mid;
    }
    const int u = lo;
    const int du = g.deg[u];
    if (du < p.sum1) continue;
    const long long ub = g.off[u];
    const int* Nu = g.adj + ub;
    const int th1u = max(p.sum1, p.sum2 - du);
    {
      const int v = __ldg(g.adj + j);
      const int dv = g.deg[v];
      if (dv < th1u) continue;  // init_wl_wedge
      const int* Nv = g.adj + g.off[v];
      const int p12 = (int)__ldg(esup + j);  // |N(u) & N(v)|
      const bool cond = (du >= p.min_u) && (dv >= p.lim);
      const int thres1 = max(p.lim, p.sum2 - dv);
      const int thres2 = max(max(p.sum1, p.sum3 - du - dv), max(p.sum2 - du, p.sum2 - dv));
      for (int t0 = 0; t0 < du; t0 += 32) {
        const int t = t0 + lane;
        bool active = false, tri = false;
        int w = 0, dw = 0;
        if (t < du) {
          w = __ldg(Nu + t);
          if (w < v) {
            dw = g.deg[w];
            if (dw >= thres2) {
              tri = bsearch_has(Nv, dv, w);
              active = tri ? (u < w) : (cond && dw >= thres1);
            }
          }
        }
        if (!__any_sync(0xffffffffu, t < du && w < v)) break;
        unsigned bal = __ballot_sync(0xffffffffu, active);
        // |N(u) & N(w)| is the support of the entry (u, w); |N(v) & N(w)|
        // and the triple overlap walk the shorter of N(v), N(w)
        const int t13 = active ? (int)__ldg(esup + ub + t) : 0;
        int t23 = 0, t123 = 0;
        while (bal) {
          const int who = __ffs(bal) - 1;
          bal &= bal - 1;
          const int ww = __shfl_sync(0xffffffffu, w, who);
          const int dww = __shfl_sync(0xffffffffu, dw, who);
          const int* Nw = g.adj + g.off[ww];
          const int* S = (dww <= dv) ? Nw : Nv;
          const int* L = (dww <= dv) ? Nv : Nw;
          const int ls = min(dww, dv), ll = max(dww, dv);
          int a23 = 0, a123 = 0;
          for (int q = lane; q < ls; q += 32) {
            const int x = __ldg(S + q);
            if (bsearch_has(L, ll, x)) {
              a23++;
              a123 += bsearch_has(Nu, du, x);
            }
          }
          a23 = __reduce_add_sync(0xffffffffu, a23);
          a123 = __reduce_add_sync(0xffffffffu, a123);
          if (lane == who) { t23 = a23; t123 = a123; }
        }
        if (active) {
          // common3_wedge (src/fringeCount.cu:1480-1510) + corrections
          int venn[8];
          const int c123 = t123, c12 = p12 - c123, c13 = t13 - c123, c23 = t23 - c123;
          venn[0] = 0;
          venn[IU] = du - (p12 + c13);
          venn[IV] = dv - (p12 + c23);
          venn[IW] = dw - (c13 + c23 + c123);
          venn[IUV] = c12; venn[IUW] = c13; venn[IVW] = c23; venn[IUVW] = c123;
          A t = A(0);
          if (tri) {
            venn[IUV]--; venn[IUW]--; venn[IVW]--;
            for (int r = 0; r < p.rot.count; r++) t += fc3<A>(p.rot.fr[r], venn);
          } else {
            venn[IU] -= 2; venn[IVW]--;
            t += fc3<A>(p.rot.fr[0], venn);
            if (p.rot.count > 3) t += fc3<A>(p.rot.fr[3], venn);
          }
          credit(g, acc, t, u);
        }
      }
    }
  }
  block_sum_to(acc, slot);
}

// ------------------------------------------------------------- general core
constexpr int kMaxSlots = 665;  // 3^6 - 2^6: (anchor set, region) pairs for 6 anchors

struct GenParams {
  int k;           // core vertices
  int anchors;     // bitmask of anchoring core vertices
  int nonanchors;  // the other core vertices
  int startdeg;
  uint8_t destdeg[5];
  uint8_t list[5];
  int nslots;
  int lane_venn_max;  // a lane builds its own match's Venn row up to this many list entries
  int grab;           // list entries a warp takes from the queue at a time (1..32)
  uint8_t slot_idx[kMaxSlots];  // region bitmap of each placement step
  uint8_t slot_set[kMaxSlots];  // anchor set index of each step
  uint8_t slot_top[kMaxSlots];  // 1 if the step takes all remaining fringes
  uint8_t fcnt[63];
  uint8_t anch[63];
  int nsets;
  int exact;  // 1: exact placement sum; 0: the reference's functionX
};

// Placement sum over the precomputed step list (exact count of placements):
// step s puts a fringes of its anchor set into region slot_idx[s]; the last
// step of each set takes all its remaining fringes.  Each complete placement
// adds the product of nck(remaining region size, fringes placed).  D bounds
// the number of steps (the host picks the smallest D >= nslots); per step the
// walk keeps the fringes placed, those left and the partial product.
template <int D, class A>
__device__ A placement_sum(const GenParams& p, int* venn) {
  int8_t a_[D];
  uint8_t rem_[D];
  A pre_[D];
  const int S = p.nslots;
  A sum = A(0);
  int s = 0;
  rem_[0] = p.fcnt[p.slot_set[0]];
  pre_[0] = A(1);
  a_[0] = (int8_t)(p.slot_top[0] ? rem_[0] : min(venn[p.slot_idx[0]], (int)rem_[0]));
  while (s >= 0) {
    if (a_[s] < 0) {  // this step is exhausted: back up
      s--;
      if (s >= 0) {
        venn[p.slot_idx[s]] += a_[s];
        a_[s] = p.slot_top[s] ? -1 : a_[s] - 1;
      }
      continue;
    }
    const int idx = p.slot_idx[s];
    const A w = pre_[s] * nck_a<A>(venn[idx], a_[s]);
    if (a_is_zero(w) || s == S - 1) {
      sum += w;
      a_[s] = p.slot_top[s] ? -1 : a_[s] - 1;
      continue;
    }
    venn[idx] -= a_[s];
    const int ns = s + 1;
    pre_[ns] = w;
    rem_[ns] = (uint8_t)(p.slot_top[s] ? (int)p.fcnt[p.slot_set[ns]] : rem_[s] - a_[s]);
    a_[ns] = (int8_t)(p.slot_top[ns] ? rem_[ns] : min(venn[p.slot_idx[ns]], (int)rem_[ns]));
    s = ns;
  }
  return sum;
}

// functionX with the reference's own control flow (src/fringeCount.cu:408-486),
// the default: a flat depth-first walk that saves (a, prod, venn[region],
// fr[set]) per level and, when it backs up, restores only the level it returns
// to.  A region changed by the step it abandons keeps that change, so later
// alternatives can see it reduced; for anchor sets with two or more fringes
// the sum then differs from placement_sum (the exact count), and the
// reference's counts are these sums.  Level s is step s of the host's step
// list, so the region and anchor set of a level come from the table instead of
// the saved state, and D (>= nslots, chosen on the host) bounds the depth:
// 14 bytes of state per level instead of the reference's 21 x 665.
template <int D>
__device__ u64 placement_sum_reference(const GenParams& p, int* venn) {
  int8_t savea[D];
  uint8_t savefr[D];
  int savevenn[D];
  u64 saveprod[D];
  uint8_t fr[64];
  for (int i = 0; i < 64; i++) fr[i] = 0;
  for (int i = 0; i < p.nsets; i++) fr[p.anch[i]] = p.fcnt[i];
  u64 sum = 0, prod = 1;
  int level = 0;
  int a = min(venn[p.slot_idx[0]], (int)fr[p.anch[p.slot_set[0]]]);
  for (;;) {
    const int idx = p.slot_idx[level];
    const int anch = p.anch[p.slot_set[level]];
    const bool top = p.slot_top[level] != 0;
    savea[level] = (int8_t)a; saveprod[level] = prod;
    savevenn[level] = venn[idx]; savefr[level] = fr[anch];
    if (a < 0) {
      prod = 0;
    } else if (top) {
      prod *= nck(venn[idx], fr[anch]);
      venn[idx] -= fr[anch];
      fr[anch] = 0;
      if (p.slot_set[level] == 0) { sum += prod; prod = 0; }
    } else {
      prod *= nck(venn[idx], a);
      venn[idx] -= a;
      fr[anch] = (uint8_t)(fr[anch] - a);
    }
    if (prod == 0) {
      level--;
      if (level < 0) break;
      a = savea[level] - 1;
      prod = saveprod[level];
      venn[p.slot_idx[level]] = savevenn[level];
      fr[p.anch[p.slot_set[level]]] = savefr[level];
    } else {
      level++;
      const int nidx = p.slot_idx[level];
      a = p.slot_top[level] ? 0 : min(venn[nidx], (int)fr[p.anch[p.slot_set[level]]]);
    }
  }
  return sum;
}

constexpr int kGenWarps = 4;  // warps per block in the general-core kernel

struct GenWarp {
  int stack[6];
  int venn[32][65];  // one Venn row per lane (the lane that owns the match); padded against bank conflicts
};

// Exclusive Venn regions of one core match: row[S] = number of vertices whose
// set of adjacent anchor core vertices is exactly S, minus the core vertices
// themselves (commonX, src/fringeCount.cu:345-405, computes the same sizes by
// inclusion-exclusion over every anchor's full list).  Here the anchor with the
// longest list, M, is never walked: every vertex adjacent to M and to another
// anchor is counted from the first other anchor (in core order) it touches,
// and row[{M}] = deg M - those.  Each walked entry needs one membership test
// per other anchor.  `vert(i)` gives the match's vertex at core position i.
// Warp-cooperative (LANES = 32, atomics into row) or by one lane (LANES = 1).
template <int LANES, class VertOf>
__device__ void venn_exclusive(const GView& g, const GenParams& p, VertOf vert, int* row) {
  const int lane = (LANES == 1) ? 0 : (threadIdx.x & 31);
  for (int i = lane; i < 64; i += LANES) row[i] = 0;
  if (LANES > 1) __syncwarp();
  int big = -1, bigdeg = -1;
  for (int i = 0; i < p.k; i++)
    if (p.anchors & (1 << i)) {
      const int d = g.deg[vert(i)];
      if (d >= bigdeg) { big = i; bigdeg = d; }
    }
  for (int i = 0; i < p.k; i++) {
    if (!(p.anchors & (1 << i)) || i == big) continue;
    const int vi = vert(i);
    const long long b = g.off[vi];
    const int d = (int)(g.off[vi + 1] - b);
    for (int t = lane; t < d; t += LANES) {
      const int x = __ldg(g.adj + b + t);
      int bmp = 1 << i;
      bool first = true;
      for (int q = 0; q < p.k && first; q++) {
        if (q == i || !(p.anchors & (1 << q))) continue;
        const int vq = vert(q);
        const long long qb = g.off[vq];
        if (bsearch_has(g.adj + qb, (int)(g.off[vq + 1] - qb), x)) {
          if (q < i && q != big) first = false;  // counted from anchor q
          else bmp |= 1 << q;
        }
      }
      if (first) {
        if (LANES > 1) atomicAdd(row + bmp, 1);
        else row[bmp]++;
      }
    }
  }
  if (LANES > 1) __syncwarp();
  if (lane == 0) {
    int shared_with_big = 0;
    for (int s = 1; s < 64; s++)
      if ((s & (1 << big)) && s != (1 << big)) shared_with_big += row[s];
    row[1 << big] = bigdeg - shared_with_big;
  }
  if (LANES > 1) __syncwarp();
  // core vertices themselves are not fringe candidates
  for (int c = lane; c < p.k; c += LANES) {
    const int x = vert(c);
    int bmp = 0;
    for (int q = 0; q < p.k; q++) {
      if (!(p.anchors & (1 << q))) continue;
      const int vq = vert(q);
      const long long qb = g.off[vq];
      if (bsearch_has(g.adj + qb, (int)(g.off[vq + 1] - qb), x)) bmp |= 1 << q;
    }
    if (bmp) {
      if (LANES > 1) atomicSub(row + bmp, 1);
      else row[bmp]--;
    }
  }
  if (LANES > 1) __syncwarp();
}

// Entries a Venn row walks: the anchors' lists except the longest.
template <class VertOf>
__device__ __forceinline__ int venn_walk_len(const GView& g, const GenParams& p, VertOf vert) {
  int sum = 0, big = 0;
  for (int i = 0; i < p.k; i++)
    if (p.anchors & (1 << i)) {
      const int d = g.deg[vert(i)];
      sum += d;
      big = max(big, d);
    }
  return sum - big;
}

template <int D, class A>
__device__ __forceinline__ A placement_of(const GenParams& p, int* row) {
  if constexpr (std::is_same<A, u64>::value)
    return p.exact ? placement_sum<D, u64>(p, row) : placement_sum_reference<D>(p, row);
  else
    return placement_sum<D, A>(p, row);  // exact counts: exact placements
}

template <int L, int D, class A>
__device__ A gen_level(const GView& g, const GenParams& p, GenWarp& w) {
  // choose stack[L+1] among the neighbours of the first core vertex it must touch
  const int lane = threadIdx.x & 31;
  const int list = p.list[L];
  const int first = __ffs(list) - 1;
  const int src = w.stack[first];
  const long long sb = g.off[src];
  const int sd = (int)(g.off[src + 1] - sb);
  const bool last = (L + 1 == p.k - 1);
  A acc = A(0);
  for (int t0 = 0; t0 < sd; t0 += 32) {
    const int t = t0 + lane;
    bool ok = false;
    int x = -1;
    if (t < sd) {
      x = __ldg(g.adj + sb + t);
      ok = g.deg[x] >= p.destdeg[L];
      for (int q = 0; q <= L && ok; q++) {
        if (list & (1 << q)) {
          if (q != first) {
            const int vq = w.stack[q];
            const long long qb = g.off[vq];
            ok = bsearch_has(g.adj + qb, (int)(g.off[vq + 1] - qb), x);
          }
        } else {
          ok = (w.stack[q] != x);
        }
      }
    }
    if (last) {
      // Venn rows: a lane builds its own when its lists are short, the warp
      // builds the long ones together, one match at a time
      auto vert = [&](int i) { return i == L + 1 ? x : w.stack[i]; };
      const bool alone = ok && venn_walk_len(g, p, vert) <= p.lane_venn_max;
      if (alone) venn_exclusive<1>(g, p, vert, w.venn[lane]);
      unsigned rows = __ballot_sync(0xffffffffu, ok && !alone);
      while (rows) {
        const int who = __ffs(rows) - 1;
        rows &= rows - 1;
        const int xx = __shfl_sync(0xffffffffu, x, who);
        auto vw = [&](int i) { return i == L + 1 ? xx : w.stack[i]; };
        venn_exclusive<32>(g, p, vw, w.venn[who]);
      }
      __syncwarp();
      if (ok) credit(g, acc, placement_of<D, A>(p, w.venn[lane]), w.stack[0]);
      __syncwarp();
    } else {
      unsigned bal = __ballot_sync(0xffffffffu, ok);
      while (bal) {
        const int who = __ffs(bal) - 1;
        bal &= bal - 1;
        const int xx = __shfl_sync(0xffffffffu, x, who);
        if (lane == 0) w.stack[L + 1] = xx;
        __syncwarp();
        if constexpr (L < 4) acc += gen_level<L + 1, D, A>(g, p, w);
        __syncwarp();
      }
    }
  }
  return acc;
}

// One warp per directed edge (u, v) at a time, u = core vertex A and v = core
// vertex B (the reference's worklist of general_core_level0,
// src/fringeCount.cu:567-663, with its degree pruning): warps take p.grab
// (1..32) consecutive list entries from a queue, find their owners in
// parallel and then walk each entry's matches.  Work is spread per edge, so a
// hub's edges go to many warps; on small graphs a warp takes one edge at a
// time, so that every warp of the GPU has work.
template <int D, class A>
__global__ void __launch_bounds__(kGenWarps * 32) general_core_kernel(GView g, const __grid_constant__ GenParams p,
                                                                       unsigned long long* __restrict__ queue,
                                                                       u64* __restrict__ slot) {
  __shared__ GenWarp sw[kGenWarps];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  GenWarp& w = sw[warp];
  A acc = A(0);
  const unsigned long long m = (unsigned long long)g.m;
  for (;;) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(queue, (unsigned long long)p.grab);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= m) break;
    const long long j = (long long)base + lane;
    bool ok = lane < p.grab && j < (long long)m;
    int u = 0, v = 0;
    if (ok) {
      int lo = 0, hi = g.n;  // owner: the last vertex with off[u] <= j
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (g.off[mid] <= j) lo = mid;
        else hi = mid;
      }
      u = lo;
      v = __ldg(g.adj + j);
      ok = g.deg[u] >= p.startdeg && g.deg[v] >= p.destdeg[0];  // init_wl_general
    }
    unsigned bal = __ballot_sync(0xffffffffu, ok);
    while (bal) {
      const int who = __ffs(bal) - 1;
      bal &= bal - 1;
      const int uu = __shfl_sync(0xffffffffu, u, who), vv = __shfl_sync(0xffffffffu, v, who);
      if (lane == 0) { w.stack[0] = uu; w.stack[1] = vv; }
      __syncwarp();
      acc += gen_level<1, D, A>(g, p, w);
      __syncwarp();
    }
  }
  block_sum_to(acc, slot);
}

// ------------------------------------------------------------- host helpers
void rotations3(const int f[8], bool wedge, Rot3& r) {
  auto rot = [](const int* q, int* o) {
    o[0] = 0; o[IUVW] = q[IUVW]; o[IUV] = q[IVW]; o[IUW] = q[IUV]; o[IVW] = q[IUW];
    o[IU] = q[IV]; o[IV] = q[IW]; o[IW] = q[IU];
  };
  auto rot2 = [](const int* q, int* o) {
    o[0] = 0; o[IUVW] = q[IUVW]; o[IUV] = q[IUW]; o[IUW] = q[IVW]; o[IVW] = q[IUV];
    o[IU] = q[IW]; o[IV] = q[IU]; o[IW] = q[IV];
  };
  for (int i = 0; i < 8; i++) r.fr[0][i] = (i == 0) ? 0 : f[i];
  r.count = 1;
  // triangleRotations (src/fringeCount.cu:1291-1317) / wedgeRotations (:1754-1780)
  const bool any = wedge || f[IU] != f[IV] || f[IU] != f[IW] || f[IUV] != f[IUW] || f[IUV] != f[IVW];
  if (!any) return;
  rot(r.fr[0], r.fr[1]);
  rot2(r.fr[0], r.fr[2]);
  r.count = 3;
  const bool fl = wedge ? (f[IV] != f[IW] || f[IUV] != f[IUW])
                        : ((f[IV] != f[IW] || f[IUV] != f[IUW]) && (f[IU] != f[IW] || f[IUV] != f[IVW]) &&
                           (f[IU] != f[IV] || f[IUW] != f[IVW]));
  if (!fl) return;
  int* q = r.fr[3];
  q[0] = 0; q[IUVW] = f[IUVW]; q[IUV] = f[IUW]; q[IUW] = f[IUV]; q[IVW] = f[IVW];
  q[IU] = f[IU]; q[IV] = f[IW]; q[IW] = f[IV];
  rot(r.fr[3], r.fr[4]);
  rot2(r.fr[3], r.fr[5]);
  r.count = 6;
}

int grid_for(long long work, int tpb, int per_sm) {
  const long long want = (work + tpb - 1) / tpb;
  const long long cap = (long long)sm_count() * per_sm;
  return (int)std::max(1LL, std::min(want, cap));
}

// Builds the wedge core's chunk-boundary table once per graph (vertices of
// degree >= 512, fewer when the table would pass 512 MiB).
int ensure_chunk_table(DevGraph& G, cudaStream_t s, uint64_t* launches, u64* d_small) {
  if (G.ctab_K > 0) return FSGC_OK;
  const int K = (int)(((long long)G.n + kWGran - 1) / kWGran) + 1;
  int min_deg = 512;
  GView gv = G.view();
  int* nrows_d = reinterpret_cast<int*>(d_small);
  if (cudaMalloc((void**)&G.ctab_id, sizeof(int) * (size_t)std::max(1, G.n)) != cudaSuccess ||
      cudaMalloc((void**)&G.ctab_rows, sizeof(int) * (size_t)std::max(1, G.n)) != cudaSuccess) {
    cudaGetLastError();
    return FSGC_ENOMEM;
  }
  int nrows = 0;
  for (;;) {
    cudaMemsetAsync(nrows_d, 0, sizeof(int), s);
    chunk_table_rows_kernel<<<grid_for(G.n, 256, 8), 256, 0, s>>>(gv, min_deg, G.ctab_id, G.ctab_rows, nrows_d);
    *launches += 1;
    if (cudaMemcpyAsync(&nrows, nrows_d, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return FSGC_ECUDA;
    if ((size_t)nrows * K * sizeof(int) <= ((size_t)512 << 20)) break;
    min_deg *= 2;
  }
  if (cudaMalloc((void**)&G.ctab_pos, sizeof(int) * std::max<size_t>(1, (size_t)nrows * K)) != cudaSuccess) {
    cudaGetLastError();
    return FSGC_ENOMEM;
  }
  if (nrows > 0) {
    chunk_table_fill_kernel<<<grid_for((long long)nrows * K, 256, 8), 256, 0, s>>>(gv, G.ctab_rows, nrows, K, G.ctab_pos);
    *launches += 1;
  }
  G.ctab_K = K;
  G.bytes += sizeof(int) * ((size_t)2 * G.n + (size_t)nrows * K);
  return cudaGetLastError() == cudaSuccess ? FSGC_OK : FSGC_ECUDA;
}

// Stream-ordered, so that growing one stream's arena neither waits for nor
// stalls work queued on other streams.
int ensure_plain_scratch(Scratch& sc, size_t need, cudaStream_t s) {
  if (sc.bytes >= need) return FSGC_OK;
  if (sc.ptr) {
    cudaFreeAsync(sc.ptr, s);
    sc.ptr = nullptr;
    sc.bytes = 0;
  }
  if (cudaMallocAsync(&sc.ptr, need, s) != cudaSuccess) {
    cudaGetLastError();
    sc.ptr = nullptr;
    return FSGC_ENOMEM;
  }
  sc.bytes = need;
  sc.gen++;
  return FSGC_OK;
}

// Triangle bitmap kernel geometry: rows of ceil(deg/32) words per out-neighbour
// of the block's vertex, one arena of max_bitmap_words per block, at most 8 GiB;
// three resident blocks per SM (the kernel is built for 80 registers a thread).
void triangle_bitmap_geometry(const DevGraph& G, long long* per_block, int* blocks) {
  *per_block = std::max(1LL, G.max_bitmap_words);
  const size_t budget = (size_t)8 << 30;
  *blocks = (int)std::max<size_t>(
      1, std::min<size_t>((size_t)sm_count() * 3, budget / (sizeof(unsigned) * (size_t)*per_block)));
}

bool triangle_uses_bitmaps(const fsgc_matching_order&, const DevGraph& G, int mode) {
  const size_t smem = (size_t)3 * sizeof(int) * (size_t)std::max(1LL, G.max_outdeg);
  return mode == 0 && smem <= (size_t)96 * 1024 && G.m / 2 > 0;
}

// Bitmap kernel shared memory: the out-neighbour arrays (3 ints each), then as
// long an N(a) stage as fits a 72 KB block (three blocks per SM): 4 bytes per
// staged entry plus one row bit per warp, up to stage_max entries.  Returns the
// stage length (a multiple of 32, or 0) and the block's dynamic shared memory.
// The bitmap rows stay in the global arena: keeping the rows of small vertices
// in a full 72 KB block made the 4-clique pattern of the RMAT-22 benchmark 58%
// slower, most likely because the larger shared-memory carve-out leaves the
// kernel's list reads a small L1.
int triangle_stage(int kmax, int stage_max, size_t* smem) {
  const long long fixed = 3LL * 4 * std::max(1, kmax);
  const long long budget = 72LL * 1024 - fixed - 16;
  long long stage = budget > 0 ? budget / (4 + (kTriThreads / 32) * 4 / 32) : 0;
  stage = std::min<long long>(stage, std::min(8192, std::max(0, stage_max))) & ~31LL;
  if (stage < 64) stage = 0;
  *smem = (size_t)(4 * (stage + 4) + 4 * (stage / 32) * (kTriThreads / 32) + fixed);
  return (int)stage;
}

}  // namespace

// What a count of `mo` on `G` needs beyond the resident graph.  The shape
// tests repeat enqueue_count's dispatch.
namespace {
struct Needs {
  bool chunk_table = false;  // wedge core with a fringe-free centre
  bool vertex_triangles = false;
  bool entry_supports = false;  // general wedge core
  size_t scratch = 0;        // arena bytes (hub cursors, triangle bitmaps)
};

Needs needs_of(const fsgc_matching_order& mo, const DevGraph& G, const fsgc_tuning& t) {
  Needs nd;
  if (mo.nodes < 2 || mo.nodes > FSGC_MAX_CORE) return nd;
  if (mo.nodes == 2) {
    int f[4] = {0, 0, 0, 0};
    for (int i = 0; i < mo.anchorsets; i++) f[mo.anch[i] & 3] = mo.fcnt[i];
    const int f_u = std::min(f[1], f[2]), f_uv = f[3], f_v = std::max(f[1], f[2]);
    if (f_uv == 1 && (f_u == 0 || f_v == 0)) nd.vertex_triangles = !(f_u == 0 && f_v == 0) || G.ngraphs > 0;
    return nd;
  }
  if (mo.nodes > 3) return nd;
  int f[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int i = 0; i < mo.anchorsets; i++) f[mo.anch[i] & 7] = mo.fcnt[i];
  if (__builtin_popcount(mo.list[1]) == 1) {
    if (mo.list[1] == 2) {
      std::swap(f[IU], f[IV]);
      std::swap(f[IUW], f[IVW]);
    }
    if (f[IUVW] == 0 && f[IUV] == 0 && f[IUW] == 0 && f[IU] == 0) {
      nd.chunk_table = true;
      if (G.maxdeg > std::min(kWDvMax, std::max(16, t.wedge_small_max_degree))) {
        const long long gs = G.maxdeg;
        nd.scratch = (size_t)sm_count() * ((size_t)2 * gs * sizeof(long long) + (size_t)(gs + 1) * sizeof(int));
      }
    } else {
      nd.entry_supports = true;
    }
    return nd;
  }
  const bool clique = (f[IUVW] == 1) && (f[IUV] + f[IUW] + f[IVW] == 0) &&
                      ((f[IU] == 0) + (f[IV] == 0) + (f[IW] == 0) >= 2);
  if (triangle_uses_bitmaps(mo, G, clique ? 1 : 0)) {
    long long per_block;
    int blocks;
    triangle_bitmap_geometry(G, &per_block, &blocks);
    nd.scratch = sizeof(unsigned) * (size_t)per_block * (size_t)blocks;
  }
  return nd;
}
}  // namespace

size_t count_scratch_bytes(const fsgc_matching_order& mo, const DevGraph& G, const fsgc_tuning& t) {
  return needs_of(mo, G, t).scratch;
}

int check_tuning(const fsgc_tuning& t) {
  const bool ok = t.wedge_small_max_degree >= 16 && t.wedge_small_max_degree <= kWDvMax && t.triangle_walk_ratio >= 0 &&
                  t.triangle_walk_ratio <= (1 << 20) && t.triangle_stage_max >= 0 && t.triangle_stage_max <= 8192 &&
                  t.triangle_stage_max % 32 == 0 && t.general_lane_venn_max >= 0 &&
                  t.general_lane_venn_max <= (1 << 20) && t.general_blocks_per_sm >= 1 && t.general_blocks_per_sm <= 16;
  return ok ? FSGC_OK : FSGC_EINVAL;
}

int prepare_for_count(const fsgc_matching_order& mo, DevGraph& G, cudaStream_t s, uint64_t* launches,
                      DevWork& work) {
  if (mo.nodes < 2) return FSGC_OK;
  int st = prepare_graph(G, s, launches, work.small);
  if (st != FSGC_OK) return st;
  const Needs nd = needs_of(mo, G, work.tune);
  if (nd.chunk_table) {
    st = ensure_chunk_table(G, s, launches, work.small + 9);
    if (st != FSGC_OK) return st;
  }
  if (nd.vertex_triangles) {
    st = ensure_vertex_triangles(G, s, launches);
    if (st != FSGC_OK) return st;
  }
  if (nd.entry_supports) {
    st = ensure_entry_supports(G, s, launches);
    if (st != FSGC_OK) return st;
  }
  return cudaStreamSynchronize(s) == cudaSuccess ? FSGC_OK : FSGC_ECUDA;
}

int prepare_all(DevGraph& G, cudaStream_t s, uint64_t* launches, DevWork& work) {
  int st = prepare_graph(G, s, launches, work.small);
  if (st == FSGC_OK && G.ngraphs == 0) st = ensure_chunk_table(G, s, launches, work.small + 9);
  if (st == FSGC_OK) st = ensure_vertex_triangles(G, s, launches);
  if (st == FSGC_OK && G.ngraphs == 0) st = ensure_entry_supports(G, s, launches);
  if (st != FSGC_OK) return st;
  return cudaStreamSynchronize(s) == cudaSuccess ? FSGC_OK : FSGC_ECUDA;
}

namespace {
// Both pair kernels of the fringe-free-centre wedge core for a set of
// patterns: endpoints of degree <= kWDvMax, then hub endpoints (cursors and
// segment offsets in the work arena).
template <int NP, class A>
int launch_wedge_set(DevGraph& G, const GView& gv, const WedgeSet& ws0, cudaStream_t s, uint64_t* launches,
                     DevWork& work) {
  int* q1 = reinterpret_cast<int*>(work.small + 7);
  int* q2 = reinterpret_cast<int*>(work.small + 8);
  int st = ensure_chunk_table(G, s, launches, work.small + 9);
  if (st != FSGC_OK) return st;
  const ChunkTable tab{G.ctab_id, G.ctab_pos, G.ctab_K};
  cudaMemsetAsync(q1, 0, 2 * sizeof(u64), s);
  const int blocks = sm_count();
  WedgeSet ws = ws0;
  ws.small_max = std::min(kWDvMax, std::max(16, work.tune.wedge_small_max_degree));
  {
    const size_t smem = sizeof(WedgeSmem<false>);
    cudaFuncSetAttribute(wedge_chunk_kernel<false, NP, A>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    wedge_chunk_kernel<false, NP, A><<<blocks, kWThreads, smem, s>>>(gv, ws, q1, nullptr, nullptr, 0, tab);
    *launches += 1;
  }
  if (G.maxdeg > ws.small_max) {
    // hub endpoints: cursors (2 x int64) and segment offsets (int32) per block
    const long long gs = G.maxdeg;
    const size_t need = (size_t)blocks * ((size_t)2 * gs * sizeof(long long) + (size_t)(gs + 1) * sizeof(int));
    st = ensure_plain_scratch(work.tri, std::max(need, work.tri.bytes), s);
    if (st != FSGC_OK) return st;
    long long* gcur = reinterpret_cast<long long*>(work.tri.ptr);
    int* gpre = reinterpret_cast<int*>(gcur + (size_t)blocks * 2 * gs);
    const size_t smem = sizeof(WedgeSmem<true>);
    cudaFuncSetAttribute(wedge_chunk_kernel<true, NP, A>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    wedge_chunk_kernel<true, NP, A><<<blocks, kWThreads, smem, s>>>(gv, ws, q2, gcur, gpre, gs, tab);
    *launches += 1;
  }
  return cudaGetLastError() == cudaSuccess ? FSGC_OK : FSGC_ECUDA;
}

// The triangle bitmap kernel for a set of patterns (tp: shared fields, with
// tp.sum1 the set's smallest vertex gate).
template <int NP, class A>
int launch_triangle_set(DevGraph& G, const GView& gv, TriParams tp, const TriSet& ts, cudaStream_t s,
                        uint64_t* launches, DevWork& work) {
  size_t smem = 0;
  tp.kmax = (int)G.max_outdeg;
  tp.stage = triangle_stage(tp.kmax, work.tune.triangle_stage_max, &smem);
  tp.walk_ratio = std::max(0, work.tune.triangle_walk_ratio);
  long long per_block;
  int blocks;
  triangle_bitmap_geometry(G, &per_block, &blocks);
  const size_t need = sizeof(unsigned) * (size_t)per_block * (size_t)blocks;
  int st = ensure_plain_scratch(work.tri, need, s);
  if (st != FSGC_OK) return st;
  int* queue = reinterpret_cast<int*>(work.small + 6);
  cudaMemsetAsync(queue, 0, sizeof(int), s);
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(triangle_bitmap_kernel<NP, A>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  triangle_bitmap_kernel<NP, A><<<blocks, kTriThreads, smem, s>>>(
      gv, tp, ts, queue, reinterpret_cast<unsigned*>(work.tri.ptr), per_block,
      reinterpret_cast<unsigned long long*>(work.small + kErrWord));
  *launches += 1;
  // the kernel's error bits (a bulk copy that never completed) for the caller
  if (work.h_err) cudaMemcpyAsync(work.h_err, work.small + kErrWord, sizeof(u64), cudaMemcpyDeviceToHost, s);
  return cudaGetLastError() == cudaSuccess ? FSGC_OK : FSGC_ECUDA;
}

template <class A>
int enqueue_count_a(CountJob& job, cudaStream_t s, uint64_t* launches, DevWork& work) {
  const fsgc_matching_order& mo = *job.mo;
  DevGraph& G = *job.g;
  job.host_only = false;
  job.host_value = 0;
  job.per_member_div = 1;
  if (mo.nodes < 1 || mo.nodes > FSGC_MAX_CORE || mo.anchorsets > 63) return FSGC_EINVAL;
  const int TPB = kTPB;
  const bool packed = G.ngraphs > 0;

  // ---- vertex core (vertexCore, src/fringeCount.cu:2172-2191)
  if (mo.nodes == 1) {
    job.core_type = FSGC_CORE_VERTEX;
    // single vertex: n; single edge: m/2 (per member graph for packed graphs, on the host)
    if (mo.anchorsets == 0) { job.host_only = true; job.host_value = (u64)G.n; return FSGC_OK; }
    if (mo.fcnt[0] == 1) { job.host_only = true; job.host_value = (u64)(G.m / 2); return FSGC_OK; }
    GView gv0 = G.view();
    gv0.comp_slots = job.d_comp_slots;
    star_kernel<A><<<grid_for(G.n, TPB, 8), TPB, 0, s>>>(gv0, mo.fcnt[0], job.d_slot);
    *launches += 1;
    return cudaGetLastError() == cudaSuccess ? FSGC_OK : FSGC_ECUDA;
  }

  int st = prepare_graph(G, s, launches, work.small);
  if (st != FSGC_OK) return st;
  GView gv = G.view();
  gv.comp_slots = job.d_comp_slots;
  const long long me = G.m / 2;

  // ---- edge core (edgeCore, src/fringeCount.cu:2106-2144)
  if (mo.nodes == 2) {
    job.core_type = FSGC_CORE_EDGE;
    int f[4] = {0, 0, 0, 0};
    for (int i = 0; i < mo.anchorsets; i++) f[mo.anch[i] & 3] = mo.fcnt[i];
    const int f_u = std::min(f[1], f[2]), f_uv = f[3], f_v = std::max(f[1], f[2]);
    if (f_uv == 1 && (f_u == 0 || f_v == 0)) {
      if (f_u == 0 && f_v == 0) {  // triangle
        if (!packed) {
          job.host_only = true;
          job.host_value = (u64)G.triangles;
          return FSGC_OK;
        }
        // per member: sum of 2 x (triangles at v) over its vertices = 6 x triangles
        st = ensure_vertex_triangles(G, s, launches);
        if (st != FSGC_OK) return st;
        packed_vertex_sum_kernel<<<grid_for(G.n, TPB, 8), TPB, 0, s>>>(gv, G.vtri2, job.d_slot);
        *launches += 1;
        job.per_member_div = 6;
        return cudaGetLastError() == cudaSuccess ? FSGC_OK : FSGC_ECUDA;
      }
      st = ensure_vertex_triangles(G, s, launches);
      if (st != FSGC_OK) return st;
      tailed_triangle_kernel<A><<<grid_for(G.n, TPB, 8), TPB, 0, s>>>(gv, G.vtri2, f_v, job.d_slot);
      *launches += 1;
      return cudaGetLastError() == cudaSuccess ? FSGC_OK : FSGC_ECUDA;
    }
    EdgeParams ep{f_u, f_uv, f_v, f_u + f_uv, f_u + f_uv + f_v};
    if (me > 0) {
      edge_kernel<A><<<grid_for(me, TPB, 8), TPB, 0, s>>>(gv, ep, job.d_slot);
      *launches += 1;
    }
    return cudaGetLastError() == cudaSuccess ? FSGC_OK : FSGC_ECUDA;
  }

  int f[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (mo.nodes == 3)
    for (int i = 0; i < mo.anchorsets; i++) f[mo.anch[i] & 7] = mo.fcnt[i];

  // ---- wedge core (wedgeCore, src/fringeCount.cu:1783-1825)
  if (mo.nodes == 3 && __builtin_popcount(mo.list[1]) == 1) {
    job.core_type = FSGC_CORE_WEDGE;
    if (mo.list[1] == 2) {  // centre is B: swap roles of A and B
      std::swap(f[IU], f[IV]);
      std::swap(f[IUW], f[IVW]);
    }
    const int min_u = f[IUVW] + f[IUV] + f[IUW] + f[IU] + 2;
    const int min_v = f[IUVW] + f[IUV] + f[IVW] + f[IV] + 1;
    const int min_w = f[IUVW] + f[IUW] + f[IVW] + f[IW] + 1;
    const int sum3 = min_u + min_v + min_w;
    const int sum2 = sum3 - std::max(std::max(min_u, min_v), min_w);
    const int sum1 = std::min(std::min(min_u, min_v), min_w);
    const int lim = std::min(min_v, min_w);
    if (f[IUVW] == 0 && f[IUV] == 0 && f[IUW] == 0 && f[IU] == 0) {
      WedgeSet ws;
      memset(&ws, 0, sizeof(ws));
      ws.np = 1;
      ws.lim = lim;
      ws.w[0] = WedgeParams{f[IV], f[IVW], f[IW], lim, min_v + min_w};
      ws.slot[0] = job.d_slot;
      return launch_wedge_set<1, A>(G, gv, ws, s, launches, work);
    }
    GWedgeParams gp;
    gp.min_u = min_u; gp.lim = lim; gp.sum1 = sum1; gp.sum2 = sum2; gp.sum3 = sum3;
    rotations3(f, true, gp.rot);
    st = ensure_entry_supports(G, s, launches);
    if (st != FSGC_OK) return st;
    wedge_general_kernel<A><<<grid_for(G.m * 32, TPB, 8), TPB, 0, s>>>(gv, gp, G.esup, job.d_slot);
    *launches += 1;
    return cudaGetLastError() == cudaSuccess ? FSGC_OK : FSGC_ECUDA;
  }

  // ---- triangle core (triangleCore, src/fringeCount.cu:1320-1373)
  if (mo.nodes == 3) {
    job.core_type = FSGC_CORE_TRIANGLE;
    const int min_u = f[IUVW] + f[IUV] + f[IUW] + f[IU];
    const int min_v = f[IUVW] + f[IUV] + f[IVW] + f[IV];
    const int min_w = f[IUVW] + f[IUW] + f[IVW] + f[IW];
    TriParams tp;
    tp.sum3 = min_u + min_v + min_w + 6;
    tp.sum2 = tp.sum3 - (std::max(std::max(min_u, min_v), min_w) + 2);
    tp.sum1 = std::min(std::min(min_u, min_v), min_w) + 2;
    const bool clique = (f[IUVW] == 1) && (f[IUV] + f[IUW] + f[IVW] == 0) &&
                        ((f[IU] == 0) + (f[IV] == 0) + (f[IW] == 0) >= 2);
    tp.tails = f[IU] + f[IV] + f[IW];
    tp.mode = clique ? (tp.tails == 0 ? 1 : 2) : 0;
    tp.relabel = G.tri_relabel ? 1 : 0;
    tp.kmax = (int)G.max_outdeg;
    rotations3(f, false, tp.rot);
    if (me == 0) return FSGC_OK;
    if (triangle_uses_bitmaps(mo, G, tp.mode)) {
      TriSet ts;
      memset(&ts, 0, sizeof(ts));
      ts.np = 1;
      ts.sum1[0] = tp.sum1; ts.sum2[0] = tp.sum2; ts.sum3[0] = tp.sum3;
      ts.rot[0] = tp.rot;
      ts.slot[0] = job.d_slot;
      return launch_triangle_set<1, A>(G, gv, tp, ts, s, launches, work);
    } else {
      triangle_core_kernel<A><<<grid_for(me, TPB, 8), TPB, 0, s>>>(gv, tp, job.d_slot);
    }
    *launches += 1;
    return cudaGetLastError() == cudaSuccess ? FSGC_OK : FSGC_ECUDA;
  }

  // ---- general core (generalCore, src/fringeCount.cu:666-692)
  job.core_type = FSGC_CORE_GENERAL;
  if (mo.anchorsets == 0) return FSGC_EINVAL;
  GenParams* gp = new GenParams();
  memset(gp, 0, sizeof(GenParams));
  gp->k = mo.nodes;
  for (int i = 0; i < mo.anchorsets; i++) gp->anchors |= mo.anch[i];
  gp->nonanchors = gp->anchors ^ ((1 << mo.nodes) - 1);
  gp->startdeg = mo.startdeg;
  for (int i = 0; i < 5; i++) { gp->destdeg[i] = mo.destdeg[i]; gp->list[i] = mo.list[i]; }
  for (int i = 0; i < 63; i++) gp->fcnt[i] = mo.fcnt[i];
  for (int i = 0; i < 63; i++) gp->anch[i] = mo.anch[i];
  gp->nsets = mo.anchorsets;
  gp->exact = job.exact_placements;
  // placement steps: anchor sets from the last to the first; within a set the
  // regions containing it in increasing bitmap order, the all-anchor region last
  int ns = 0;
  for (int asi = mo.anchorsets - 1; asi >= 0; asi--) {
    const int anch = mo.anch[asi];
    int idx = anch;
    for (;;) {
      if (ns >= kMaxSlots) { delete gp; return FSGC_EUNSUPPORTED; }
      gp->slot_idx[ns] = (uint8_t)idx;
      gp->slot_set[ns] = (uint8_t)asi;
      gp->slot_top[ns] = (idx == gp->anchors) ? 1 : 0;
      ns++;
      if (idx == gp->anchors) break;
      idx = (((idx | gp->nonanchors) + 1) | anch) & ~gp->nonanchors;
    }
  }
  gp->nslots = ns;
  gp->lane_venn_max = std::max(0, work.tune.general_lane_venn_max);
  auto* queue = reinterpret_cast<unsigned long long*>(work.small + 5);
  cudaMemsetAsync(queue, 0, sizeof(unsigned long long), s);
  const int blocks = sm_count() * std::min(16, std::max(1, work.tune.general_blocks_per_sm));
  // one edge per grab until there are many more edges than warps
  gp->grab = (int)std::max(1LL, std::min(32LL, G.m / ((long long)blocks * kGenWarps * 64)));
  // the placement walk's state is sized by the step count
  if (ns <= 32) general_core_kernel<32, A><<<blocks, kGenWarps * 32, 0, s>>>(gv, *gp, queue, job.d_slot);
  else if (ns <= 64) general_core_kernel<64, A><<<blocks, kGenWarps * 32, 0, s>>>(gv, *gp, queue, job.d_slot);
  else if (ns <= 128) general_core_kernel<128, A><<<blocks, kGenWarps * 32, 0, s>>>(gv, *gp, queue, job.d_slot);
  else general_core_kernel<kMaxSlots, A><<<blocks, kGenWarps * 32, 0, s>>>(gv, *gp, queue, job.d_slot);
  *launches += 1;
  delete gp;
  return cudaGetLastError() == cudaSuccess ? FSGC_OK : FSGC_ECUDA;
}
}  // namespace

int enqueue_count(CountJob& job, cudaStream_t s, uint64_t* launches, DevWork& work) {
  return job.exact_count ? enqueue_count_a<X128>(job, s, launches, work) : enqueue_count_a<u64>(job, s, launches, work);
}

// Many patterns on one graph: patterns whose kernels share their match
// enumeration run as sets -- stars and tailed triangles in one vertex pass,
// edge-core formulas in one pass over the oriented edges, fringe-free-centre
// wedges over one set of centre counts, triangle cores over one set of
// bitmaps -- and every other pattern as a count of its own.  Each job's
// result goes to its own slot; the values equal the single-pattern kernels'.
int enqueue_count_set(std::vector<CountJob*>& jobs, cudaStream_t s, uint64_t* launches, DevWork& work) {
  if (jobs.empty()) return FSGC_OK;
  DevGraph& G = *jobs[0]->g;
  for (CountJob* j : jobs)
    if (j->g != &G || j->exact_count || G.ngraphs > 0) return FSGC_EINVAL;
  int st = prepare_graph(G, s, launches, work.small);
  if (st != FSGC_OK) return st;
  GView gv = G.view();
  std::vector<std::pair<CountJob*, std::pair<int, int>>> verts;  // (job, (tailed, t))
  std::vector<std::pair<CountJob*, EdgeParams>> edges;
  std::vector<std::pair<CountJob*, WedgeParams>> wedges;
  std::vector<std::pair<CountJob*, TriParams>> tris;
  std::vector<CountJob*> single;
  for (CountJob* jp : jobs) {
    CountJob& job = *jp;
    const fsgc_matching_order& mo = *job.mo;
    job.host_only = false;
    job.host_value = 0;
    job.per_member_div = 1;
    if (mo.nodes == 1 && mo.anchorsets > 0 && mo.fcnt[0] > 1) {
      job.core_type = FSGC_CORE_VERTEX;
      verts.push_back({jp, {0, (int)mo.fcnt[0]}});
      continue;
    }
    if (mo.nodes == 2) {
      int f[4] = {0, 0, 0, 0};
      for (int i = 0; i < mo.anchorsets; i++) f[mo.anch[i] & 3] = mo.fcnt[i];
      const int f_u = std::min(f[1], f[2]), f_uv = f[3], f_v = std::max(f[1], f[2]);
      job.core_type = FSGC_CORE_EDGE;
      if (f_uv == 1 && (f_u == 0 || f_v == 0)) {
        if (f_u == 0 && f_v == 0) { single.push_back(jp); continue; }  // the triangle total
        verts.push_back({jp, {1, f_v}});
      } else {
        edges.push_back({jp, EdgeParams{f_u, f_uv, f_v, f_u + f_uv, f_u + f_uv + f_v}});
      }
      continue;
    }
    if (mo.nodes == 3) {
      int f[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      for (int i = 0; i < mo.anchorsets; i++) f[mo.anch[i] & 7] = mo.fcnt[i];
      if (__builtin_popcount(mo.list[1]) == 1) {
        if (mo.list[1] == 2) {
          std::swap(f[IU], f[IV]);
          std::swap(f[IUW], f[IVW]);
        }
        if (f[IUVW] == 0 && f[IUV] == 0 && f[IUW] == 0 && f[IU] == 0) {
          const int min_v = f[IUVW] + f[IUV] + f[IVW] + f[IV] + 1;
          const int min_w = f[IUVW] + f[IUW] + f[IVW] + f[IW] + 1;
          job.core_type = FSGC_CORE_WEDGE;
          wedges.push_back({jp, WedgeParams{f[IV], f[IVW], f[IW], std::min(min_v, min_w), min_v + min_w}});
          continue;
        }
      } else {
        const int min_u = f[IUVW] + f[IUV] + f[IUW] + f[IU];
        const int min_v = f[IUVW] + f[IUV] + f[IVW] + f[IV];
        const int min_w = f[IUVW] + f[IUW] + f[IVW] + f[IW];
        const bool clique = (f[IUVW] == 1) && (f[IUV] + f[IUW] + f[IVW] == 0) &&
                            ((f[IU] == 0) + (f[IV] == 0) + (f[IW] == 0) >= 2);
        if (!clique && triangle_uses_bitmaps(mo, G, 0)) {
          TriParams tp;
          memset(&tp, 0, sizeof(tp));
          tp.sum3 = min_u + min_v + min_w + 6;
          tp.sum2 = tp.sum3 - (std::max(std::max(min_u, min_v), min_w) + 2);
          tp.sum1 = std::min(std::min(min_u, min_v), min_w) + 2;
          tp.relabel = G.tri_relabel ? 1 : 0;
          rotations3(f, false, tp.rot);
          job.core_type = FSGC_CORE_TRIANGLE;
          tris.push_back({jp, tp});
          continue;
        }
      }
    }
    single.push_back(jp);
  }
  const int TPB = kTPB;
  for (size_t b = 0; b < verts.size(); b += kPassFuse) {
    VertexSet vs;
    memset(&vs, 0, sizeof(vs));
    bool tailed = false;
    for (size_t i = b; i < std::min(verts.size(), b + kPassFuse); i++) {
      const int q = vs.np++;
      vs.tailed[q] = verts[i].second.first;
      vs.t[q] = verts[i].second.second;
      vs.slot[q] = verts[i].first->d_slot;
      tailed |= vs.tailed[q] != 0;
    }
    if (tailed) {
      st = ensure_vertex_triangles(G, s, launches);
      if (st != FSGC_OK) return st;
    }
    vertex_set_kernel<<<grid_for(G.n, TPB, 8), TPB, 0, s>>>(gv, tailed ? G.vtri2 : nullptr, vs);
    *launches += 1;
  }
  for (size_t b = 0; b < edges.size(); b += kPassFuse) {
    EdgeSet es;
    memset(&es, 0, sizeof(es));
    for (size_t i = b; i < std::min(edges.size(), b + kPassFuse); i++) {
      const int q = es.np++;
      es.e[q] = edges[i].second;
      es.slot[q] = edges[i].first->d_slot;
    }
    if (G.m / 2 > 0) {
      edge_set_kernel<<<grid_for(G.m / 2, TPB, 8), TPB, 0, s>>>(gv, es);
      *launches += 1;
    }
  }
  for (size_t b = 0; b < wedges.size(); b += kWedgeFuse) {
    WedgeSet ws;
    memset(&ws, 0, sizeof(ws));
    ws.lim = 1 << 30;
    for (size_t i = b; i < std::min(wedges.size(), b + kWedgeFuse); i++) {
      const int q = ws.np++;
      ws.w[q] = wedges[i].second;
      ws.slot[q] = wedges[i].first->d_slot;
      ws.lim = std::min(ws.lim, ws.w[q].lim);
    }
    st = ws.np == 1 ? launch_wedge_set<1, u64>(G, gv, ws, s, launches, work)
                    : launch_wedge_set<kWedgeFuse, u64>(G, gv, ws, s, launches, work);
    if (st != FSGC_OK) return st;
  }
  // Triangle-core patterns get one bitmap pass each.  A pass over four
  // patterns shares the row build, but its kernel carries four inlined copies
  // of fc3 and spills: six fringe-heavy triangle patterns on RMAT-20 took 31 s
  // in passes of four and two against 20 s one by one.
  for (const auto& t : tris) {
    TriSet ts;
    memset(&ts, 0, sizeof(ts));
    const TriParams& tp = t.second;
    ts.np = 1;
    ts.sum1[0] = tp.sum1; ts.sum2[0] = tp.sum2; ts.sum3[0] = tp.sum3;
    ts.rot[0] = tp.rot;
    ts.slot[0] = t.first->d_slot;
    st = launch_triangle_set<1, u64>(G, gv, tp, ts, s, launches, work);
    if (st != FSGC_OK) return st;
  }
  for (CountJob* jp : single) {
    st = enqueue_count(*jp, s, launches, work);
    if (st != FSGC_OK) return st;
  }
  return FSGC_OK;
}

// Launchers for callers that bring their own device memory (noalloc.cu): the
// wedge-core pair kernels on a view whose deg[] the caller filled.
namespace {
WedgeSet single_wedge(int f_v, int f_vw, int f_w, int lim, int minsum, u64* slot) {
  WedgeSet ws;
  memset(&ws, 0, sizeof(ws));
  ws.np = 1;
  ws.lim = lim;
  ws.small_max = kWDvMax;
  ws.w[0] = WedgeParams{f_v, f_vw, f_w, lim, minsum};
  ws.slot[0] = slot;
  return ws;
}
}  // namespace

int launch_wedge_small(const GView& gv, int f_v, int f_vw, int f_w, int lim, int minsum, int* queue, u64* slot,
                       cudaStream_t s) {
  const WedgeSet ws = single_wedge(f_v, f_vw, f_w, lim, minsum, slot);
  const size_t smem = sizeof(WedgeSmem<false>);
  cudaFuncSetAttribute(wedge_chunk_kernel<false, 1, u64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  wedge_chunk_kernel<false, 1, u64><<<sm_count(), kWThreads, smem, s>>>(gv, ws, queue, nullptr, nullptr, 0,
                                                                   ChunkTable{nullptr, nullptr, 0});
  return cudaGetLastError() == cudaSuccess ? FSGC_OK : FSGC_ECUDA;
}

int launch_wedge_big(const GView& gv, int f_v, int f_vw, int f_w, int lim, int minsum, int* queue, long long* gcur,
                     int* gpre, long long gstride, int blocks, u64* slot, cudaStream_t s) {
  const WedgeSet ws = single_wedge(f_v, f_vw, f_w, lim, minsum, slot);
  const size_t smem = sizeof(WedgeSmem<true>);
  cudaFuncSetAttribute(wedge_chunk_kernel<true, 1, u64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  wedge_chunk_kernel<true, 1, u64><<<blocks, kWThreads, smem, s>>>(gv, ws, queue, gcur, gpre, gstride,
                                                              ChunkTable{nullptr, nullptr, 0});
  return cudaGetLastError() == cudaSuccess ? FSGC_OK : FSGC_ECUDA;
}

int wedge_small_max_degree() { return kWDvMax; }

}  // namespace fsgc
