// fsgc oracle -- TEST INFRASTRUCTURE ONLY.
//
// A CPU restatement of Fringe-SGC's counting path (src/fringeCount.cu of the
// reference) and an independent brute-force subgraph enumerator.  Only the test
// suite, the smoke check and the CPU-baseline legs of bench.py load this
// library; the product (libfsgc) never links, loads or calls it.
//
// Parity status: the restatement is pinned against the brute-force enumerator
// and closed-form counts on graphs where the reference's u64 binomials do not
// wrap.  The pattern decomposition is pinned byte-for-byte against the
// reference's own fringePreprocess (built from its sources by oracle/Makefile).
//
// Every routine follows the reference one match at a time, with the same vertex
// roles, the same pruning thresholds and the same binomial factorisation, so the
// u64 totals agree bit for bit even where the reference's nCk wraps.  Summation
// order is free: the reference only ever adds and multiplies mod 2^64 after nCk.
//
// Graph input: n vertices, int64 offsets idx[n+1], int32 sorted neighbour lists
// adj[idx[n]] (symmetric, no self loops, no duplicates -- the reference's
// documented preconditions, src/fringeCount.cu:50-56).

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include <vector>
#include <omp.h>

typedef unsigned long long u64;
typedef unsigned __int128 u128;

namespace {

struct MO {  // src/fringes.h:50-58 (139 packed bytes)
  uint8_t nodes, anchorsets, startdeg, destdeg[5], list[5], anch[63], fcnt[63];
};
static_assert(sizeof(MO) == 139, "matching order layout");

struct Graph {
  int n;
  long long m;
  const long long* idx;
  const int* adj;
  int deg(int v) const { return (int)(idx[v + 1] - idx[v]); }
  const int* beg(int v) const { return adj + idx[v]; }
  const int* end(int v) const { return adj + idx[v + 1]; }
};

// Vertex bits of a 3-vertex core (src/fringeCount.cu:61-67).
enum { IU = 1, IV = 2, IW = 4, IUV = 3, IUW = 5, IVW = 6, IUVW = 7 };

// Binomial coefficient with the reference's u64 arithmetic: r = r*(n+1-i)/i,
// wrapping multiply then truncating divide (src/fringeCount.cu:189-197).
static inline u64 nck(int n, int k) {
  k = std::min(k, n - k);
  if (k < 0) return 0;
  if (k == 0) return 1;
  u64 r = (u64)n;
  for (int i = 2; i <= k; i++) r = r * (u64)(n + 1 - i) / (u64)i;
  return r;
}

// Exact counting: a 128-bit value with a saturation flag (the true value is
// 2^128 - 1 or more).  Zero times anything is zero.  The binomial is computed
// in 128 bits from the multiplicative formula, with every intermediate checked.
struct Xo {
  u128 v = 0;
  bool sat = false;
  Xo() {}
  Xo(u64 x) : v(x) {}
  static Xo saturated() { Xo r; r.sat = true; return r; }
};
static const u128 kU128Max = ~(u128)0;
static inline Xo operator+(Xo a, Xo b) {
  if (a.sat || b.sat) return Xo::saturated();
  Xo r;
  r.v = a.v + b.v;
  if (r.v < a.v || r.v == kU128Max) return Xo::saturated();
  return r;
}
static inline Xo operator*(Xo a, Xo b) {
  if ((!a.sat && a.v == 0) || (!b.sat && b.v == 0)) return Xo();
  if (a.sat || b.sat || a.v > (kU128Max - 1) / b.v) return Xo::saturated();
  Xo r;
  r.v = a.v * b.v;
  if (r.v == kU128Max) return Xo::saturated();
  return r;
}
static inline Xo& operator+=(Xo& a, Xo b) { return a = a + b; }
#pragma omp declare reduction(+ : Xo : omp_out = omp_out + omp_in) initializer(omp_priv = Xo())

static inline Xo nck_exact(int n, int k) {
  if (k < 0 || n < k) return Xo();
  k = std::min(k, n - k);
  u128 r = 1;
  for (int i = 1; i <= k; i++) {
    // r = C(n, i-1); C(n, i) = r * (n+1-i) / i, exact
    const u128 f = (u128)(n + 1 - i);
    const u128 q = r / (u128)i, m = r % (u128)i;
    if (q > (kU128Max - 1) / f) return Xo::saturated();
    const u128 hi = q * f, lo = m * f / (u128)i;
    if (hi > kU128Max - 1 - lo) return Xo::saturated();
    r = hi + lo;
  }
  Xo x;
  x.v = r;
  return x;
}

template <class T> static inline T nck_t(int n, int k);
template <> inline u64 nck_t<u64>(int n, int k) { return nck(n, k); }
template <> inline Xo nck_t<Xo>(int n, int k) { return nck_exact(n, k); }
static inline bool is_zero(u64 x) { return x == 0; }
static inline bool is_zero(const Xo& x) { return !x.sat && x.v == 0; }

static inline bool has(const Graph& g, int v, int x) {  // x in N(v)
  return std::binary_search(g.beg(v), g.end(v), x);
}

static int common2(const Graph& g, int a, int b) {  // |N(a) & N(b)| by merge
  const int *p = g.beg(a), *pe = g.end(a), *q = g.beg(b), *qe = g.end(b);
  int c = 0;
  while (p < pe && q < qe) {
    if (*p < *q) p++;
    else if (*q < *p) q++;
    else { c++; p++; q++; }
  }
  return c;
}

// ---------------------------------------------------------------- 3-core formula
// fc3: ways to place the fringes of the 7 anchor-set types into the 7 exclusive
// Venn regions of a 3-vertex core (src/fringeCount.cu:233-327).  The loop nest
// below visits the same (i,j,k,a,b,c,d) tuples and forms each term from the same
// nCk factors as the reference; terms the reference skips with `break` are zero.
template <class T>
static T fc3(const int fr[8], const int venn[8]) {
  const int fuvw = fr[IUVW], fuv = fr[IUV], fuw = fr[IUW], fvw = fr[IVW];
  const int fu = fr[IU], fv = fr[IV], fw = fr[IW];
  int x_uvw = venn[IUVW], x_uv = venn[IUV], x_uw = venn[IUW], x_vw = venn[IVW];
  const int x_u = venn[IU], x_v = venn[IV], x_w = venn[IW];
  if (x_uvw < fuvw) return 0;
  const T base = nck_t<T>(x_uvw, fuvw);
  x_uvw -= fuvw;
  T total = 0;
  // i of the uv-fringes go into the shared uvw region, the rest into uv
  for (int i = std::min(x_uvw, fuv); i >= 0; i--) {
    if (x_uv < fuv - i) break;
    const T t1 = base * nck_t<T>(x_uvw, i) * nck_t<T>(x_uv, fuv - i);
    const int r_uvw1 = x_uvw - i, r_uv = x_uv - (fuv - i);
    for (int j = std::min(r_uvw1, fuw); j >= 0; j--) {
      if (x_uw < fuw - j) break;
      const T t2 = t1 * nck_t<T>(r_uvw1, j) * nck_t<T>(x_uw, fuw - j);
      const int r_uvw2 = r_uvw1 - j, r_uw = x_uw - (fuw - j);
      for (int k = std::min(r_uvw2, fvw); k >= 0; k--) {
        if (x_vw < fvw - k) break;
        const T t3 = t2 * nck_t<T>(r_uvw2, k) * nck_t<T>(x_vw, fvw - k);
        const int r_uvw3 = r_uvw2 - k, r_vw = x_vw - (fvw - k);
        // u-fringes: a from uvw, b from uv, c from uw, rest from u
        for (int a = std::min(r_uvw3, fu); a >= 0; a--) {
          const T ta = t3 * nck_t<T>(r_uvw3, a);
          const int r_uvw4 = r_uvw3 - a;
          const int pool_v = r_uvw4 + r_vw;  // regions still open to v (uvw + vw)
          for (int b = std::min(r_uv, fu - a); b >= 0; b--) {
            const T tb = ta * nck_t<T>(r_uv, b);
            const int r_uv2 = r_uv - b;
            for (int c = std::min(r_uw, fu - a - b); c >= 0; c--) {
              if (x_u < fu - a - b - c) break;
              const T tc = tb * nck_t<T>(r_uw, c) * nck_t<T>(x_u, fu - a - b - c);
              const int r_uw2 = r_uw - c;
              // v-fringes: d from (uvw + vw), rest from (uv + v)
              for (int d = std::min(pool_v, fv); d >= 0; d--) {
                if (r_uv2 + x_v < fv - d) break;
                const T td = tc * nck_t<T>(pool_v, d) * nck_t<T>(r_uv2 + x_v, fv - d);
                // w-fringes: everything still open to w
                const int pool_w = (pool_v - d) + r_uw2 + x_w;
                if (pool_w >= fw) total += td * nck_t<T>(pool_w, fw);
              }
            }
          }
        }
      }
    }
  }
  return total;
}

// Rotations and flips of the 3-core anchor counts, listed as the reference lists
// them (triangle: src/fringeCount.cu:1291-1317, wedge: 1754-1780).
static void rotate(const int q[8], int out[8]) {  // u<-v, v<-w, w<-u
  out[IUVW] = q[IUVW]; out[IUV] = q[IVW]; out[IUW] = q[IUV]; out[IVW] = q[IUW];
  out[IU] = q[IV]; out[IV] = q[IW]; out[IW] = q[IU]; out[0] = 0;
}
static void rotate2(const int q[8], int out[8]) {
  out[IUVW] = q[IUVW]; out[IUV] = q[IUW]; out[IUW] = q[IVW]; out[IVW] = q[IUV];
  out[IU] = q[IW]; out[IV] = q[IU]; out[IW] = q[IV]; out[0] = 0;
}
static void flip(const int f[8], int out[8]) {  // v<->w
  out[IUVW] = f[IUVW]; out[IUV] = f[IUW]; out[IUW] = f[IUV]; out[IVW] = f[IVW];
  out[IU] = f[IU]; out[IV] = f[IW]; out[IW] = f[IV]; out[0] = 0;
}
static int rotations3(const int f[8], int fr[6][8], bool wedge) {
  int p = 0;
  for (int i = 0; i < 8; i++) fr[0][i] = (i == 0) ? 0 : f[i];
  p = 1;
  const bool rot = wedge || (f[IU] != f[IV]) || (f[IU] != f[IW]) || (f[IUV] != f[IUW]) || (f[IUV] != f[IVW]);
  if (!rot) return p;
  rotate(fr[0], fr[1]);
  rotate2(fr[0], fr[2]);
  p = 3;
  bool fl;
  if (wedge) {
    fl = (f[IV] != f[IW]) || (f[IUV] != f[IUW]);
  } else {
    fl = ((f[IV] != f[IW]) || (f[IUV] != f[IUW])) && ((f[IU] != f[IW]) || (f[IUV] != f[IVW])) &&
         ((f[IU] != f[IV]) || (f[IUW] != f[IVW]));
  }
  if (fl) {
    flip(f, fr[3]);
    rotate(fr[3], fr[4]);
    rotate2(fr[3], fr[5]);
    p = 6;
  }
  return p;
}

// Sampling for the CPU baseline: the reference's work items -- vertices for
// the vertex core, worklist entries (u, v) for the other cores -- are processed
// only when a hash of the item falls in residue `phase` modulo `stride`.
// stride 1 processes everything.
struct Sample {
  int stride = 1, phase = 0;
  static u64 mix(u64 x) {
    x += 0x9e3779b97f4a7c15ULL;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
    return x ^ (x >> 31);
  }
  bool take(int v) const { return stride <= 1 || (int)(mix((u64)(unsigned)v) % (u64)stride) == phase; }
  bool take(int u, int v) const {
    return stride <= 1 || (int)(mix(((u64)(unsigned)u << 32) | (unsigned)v) % (u64)stride) == phase;
  }
};

// ---------------------------------------------------------------- vertex core
// src/fringeCount.cu:2152-2191
template <class T>
static T vertex_core(const MO& mo, const Graph& g, const Sample& s) {
  if (mo.anchorsets == 0) return (T)g.n;
  if (mo.fcnt[0] == 1) return (T)(g.m / 2);
  const int t = mo.fcnt[0];
  T tot = 0;
#pragma omp parallel for reduction(+ : tot) schedule(dynamic, 4096)
  for (int v = 0; v < g.n; v++)
    if (s.take(v) && g.deg(v) >= t) tot += nck_t<T>(g.deg(v), t);
  return tot;
}

// ---------------------------------------------------------------- edge core
// Worklist: undirected edges (u,v) with v < u by vertex id, pruned by degree
// (init_wl_edge, src/fringeCount.cu:2054-2103); kernels triangle /
// tailed_triangle / general_edge_core (1864-2051); dispatch edgeCore 2106-2144.
template <class T>
static T edge_formula(int du, int dv, int c_uv, int f_u, int f_uv, int f_v) {
  const int a_uv = c_uv - f_uv;
  if (a_uv < 0) return 0;
  const int c_u = du - 1 - c_uv, c_v = dv - 1 - c_uv;
  const int bound = std::min(f_u, a_uv);
  T acc = 0;
  for (int j = 0; j <= bound; j++) {
    const int k = f_u - j;
    T term = nck_t<T>(c_u, k) * nck_t<T>(a_uv + c_v - j, f_v);
    if (f_u != f_v) term += nck_t<T>(c_v, k) * nck_t<T>(a_uv + c_u - j, f_v);
    acc += term * nck_t<T>(a_uv, j);
  }
  return acc * nck_t<T>(c_uv, f_uv);
}

template <class T>
static T edge_core(const MO& mo, const Graph& g, const Sample& s) {
  int f[4] = {0, 0, 0, 0};
  for (int i = 0; i < mo.anchorsets; i++) f[mo.anch[i] & 3] = mo.fcnt[i];
  const int f_u = std::min(f[1], f[2]), f_uv = f[3], f_v = std::max(f[1], f[2]);
  const bool special = (f_uv == 1) && (f_u == 0 || f_v == 0);
  const int lim1 = special ? 1 : f_u + f_uv;
  const int lim2 = special ? 1 : f_u + f_uv + f_v;
  T tot = 0;
#pragma omp parallel for reduction(+ : tot) schedule(dynamic, 64)
  for (int u = 0; u < g.n; u++) {
    const int du = g.deg(u);
    if (du <= lim1) continue;
    const T cu = special ? nck_t<T>(du - 2, f_v) : 0;
    for (const int* p = g.beg(u); p < g.end(u) && *p < u; p++) {
      const int v = *p, dv = g.deg(v);
      if (!(dv > lim1 && du + dv > lim2)) continue;
      if (!s.take(u, v)) continue;
      if (special) {
        // triangles w < v < u
        const T c12 = cu + nck_t<T>(dv - 2, f_v);
        const int *a = g.beg(u), *ae = g.end(u), *b = g.beg(v), *be = g.end(v);
        while (a < ae && b < be && *a < v && *b < v) {
          if (*a < *b) a++;
          else if (*b < *a) b++;
          else {
            if (f_u == 0 && f_v == 0) tot += 1;
            else tot += c12 + nck_t<T>(g.deg(*a) - 2, f_v);
            a++; b++;
          }
        }
      } else {
        tot += edge_formula<T>(du, dv, common2(g, u, v), f_u, f_uv, f_v);
      }
    }
  }
  return tot;
}

// ---------------------------------------------------------------- wedge core
// src/fringeCount.cu:1381-1825.
template <class T>
static T wedge_formula(int du, int dv, bool adj, int f_u, int f_uv, int f_v, int c_uv) {
  // wedge(): endpoints "u","v" of a wedge whose centre is not counted in c_uv
  const int a_uv = c_uv - f_uv;
  if (a_uv < 0) return 0;
  const int corr = adj ? 2 : 1;
  const int a_u = du - (corr + c_uv), a_v = dv - (corr + c_uv);
  const int bound = std::min(f_u, a_uv);
  T sum = 0;
  for (int j = 0; j <= bound; j++) {
    const int k = f_u - j;
    T term = nck_t<T>(a_u, k) * nck_t<T>(a_uv + a_v - j, f_v);
    if (f_u != f_v) term += nck_t<T>(a_v, k) * nck_t<T>(a_uv + a_u - j, f_v);
    sum += term * nck_t<T>(a_uv, j);
  }
  return sum * nck_t<T>(c_uv, f_uv);
}

// Exclusive Venn sizes of N(u),N(v),N(w) for a wedge or triangle centred at u,
// before the caller's corrections (common3_wedge, src/fringeCount.cu:1480-1510).
static void venn3_wedge(const Graph& g, int u, int v, int w, int p12, int venn[8]) {
  int t13 = 0, t23 = 0, t123 = 0;
  for (const int* p = g.beg(w); p < g.end(w); p++) {
    const bool b13 = has(g, u, *p), b23 = has(g, v, *p);
    t13 += b13; t23 += b23; t123 += (b13 && b23);
  }
  const int c123 = t123, c12 = p12 - c123, c13 = t13 - c123, c23 = t23 - c123;
  venn[0] = 0;
  venn[IU] = g.deg(u) - (p12 + c13);
  venn[IV] = g.deg(v) - (p12 + c23);
  venn[IW] = g.deg(w) - (c13 + c23 + c123);
  venn[IUV] = c12; venn[IUW] = c13; venn[IVW] = c23; venn[IUVW] = c123;
}

template <class T>
static T wedge_core(const MO& mo, const Graph& g, const Sample& s) {
  int f[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int i = 0; i < mo.anchorsets; i++) f[mo.anch[i] & 7] = mo.fcnt[i];
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
  T tot = 0;
  if (f[IUVW] == 0 && f[IUV] == 0 && f[IUW] == 0 && f[IU] == 0) {
    // centre has no fringes: init_wl_specialized_wedge + wedgecore_specialized
    const int fv = f[IV], fvw = f[IVW], fw = f[IW];
#pragma omp parallel for reduction(+ : tot) schedule(dynamic, 16)
    for (int u = 0; u < g.n; u++) {
      if (g.deg(u) < 2) continue;
      for (const int* pv = g.beg(u); pv < g.end(u); pv++) {
        const int v = *pv, dv = g.deg(v);
        if (dv < lim || !s.take(u, v)) continue;
        const int thres = std::max(lim, min_v + min_w - dv);
        for (const int* pw = g.beg(u); pw < g.end(u) && *pw < v; pw++) {
          const int w = *pw, dw = g.deg(w);
          if (dw < thres) continue;
          const int c = common2(g, v, w) - 1;
          tot += wedge_formula<T>(dv, dw, has(g, w, v), fv, fvw, fw, c);
        }
      }
    }
    return tot;
  }
  int fr[6][8];
  const int rot = rotations3(f, fr, true);
#pragma omp parallel for reduction(+ : tot) schedule(dynamic, 16)
  for (int u = 0; u < g.n; u++) {
    const int du = g.deg(u);
    if (du < sum1) continue;
    const int th1u = std::max(sum1, sum2 - du);
    for (const int* pv = g.beg(u); pv < g.end(u); pv++) {
      const int v = *pv, dv = g.deg(v);
      if (dv < th1u || !s.take(u, v)) continue;  // init_wl_wedge
      const int p12 = common2(g, u, v);
      const bool cond = (du >= min_u) && (dv >= lim);
      const int thres1 = std::max(lim, sum2 - dv);
      const int thres2 = std::max(std::max(sum1, sum3 - du - dv), std::max(sum2 - du, sum2 - dv));
      for (const int* pw = g.beg(u); pw < g.end(u) && *pw < v; pw++) {
        const int w = *pw, dw = g.deg(w);
        if (dw < thres2) continue;
        const bool tri = has(g, v, w);
        int venn[8];
        if (tri) {
          if (!(u < w)) continue;
          venn3_wedge(g, u, v, w, p12, venn);
          venn[IUV]--; venn[IUW]--; venn[IVW]--;
          for (int r = 0; r < rot; r++) tot += fc3<T>(fr[r], venn);
        } else {
          if (!(cond && dw >= thres1)) continue;
          venn3_wedge(g, u, v, w, p12, venn);
          venn[IU] -= 2; venn[IVW]--;
          tot += fc3<T>(fr[0], venn);
          if (rot > 3) tot += fc3<T>(fr[3], venn);
        }
      }
    }
  }
  return tot;
}

// ---------------------------------------------------------------- triangle core
// src/fringeCount.cu:700-1373.  Vertex roles follow the reference's vertex
// order: after its degree relabel (new id = rank of (degree, id) descending,
// src/fringeCount.cu:1065-1085, 1247) when the relabel gates fire
// (1237, 1342-1344), else the input ids.  key(x) reproduces "new id" order:
// a smaller key is a smaller relabelled id.
struct TriOrder {
  bool relabel;
  const Graph* g;
  long long key(int x) const {
    if (!relabel) return x;
    return -(((long long)g->deg(x) << 32) + x);
  }
};

static bool triangle_relabel_gate(const Graph& g) {
  if (g.n <= 10000) return false;
  if ((long long)g.n > g.m / 10) return false;
  int maxd = 0;
  for (int v = 0; v < g.n; v++) maxd = std::max(maxd, g.deg(v));
  return maxd > 16;
}

template <class T>
static T triangle_core(const MO& mo, const Graph& g, const Sample& s) {
  int f[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int i = 0; i < mo.anchorsets; i++) f[mo.anch[i] & 7] = mo.fcnt[i];
  const int min_u = f[IUVW] + f[IUV] + f[IUW] + f[IU];
  const int min_v = f[IUVW] + f[IUV] + f[IVW] + f[IV];
  const int min_w = f[IUVW] + f[IUW] + f[IVW] + f[IW];
  const int sum3 = min_u + min_v + min_w + 6;
  const int sum2 = sum3 - (std::max(std::max(min_u, min_v), min_w) + 2);
  const int sum1 = std::min(std::min(min_u, min_v), min_w) + 2;
  int fr[6][8];
  const int rot = rotations3(f, fr, false);
  TriOrder ord{triangle_relabel_gate(g), &g};
  const bool clique = (f[IUVW] == 1) && (f[IUV] + f[IUW] + f[IVW] == 0) &&
                      ((f[IU] == 0) + (f[IV] == 0) + (f[IW] == 0) >= 2);
  const int tails = f[IU] + f[IV] + f[IW];
  T tot = 0;
#pragma omp parallel for reduction(+ : tot) schedule(dynamic, 16)
  for (int u = 0; u < g.n; u++) {
    const int du = g.deg(u);
    if (du < sum1) continue;
    const int th1 = std::max(sum1, sum2 - du);
    const long long ku = ord.key(u);
    for (const int* pv = g.beg(u); pv < g.end(u); pv++) {
      const int v = *pv, dv = g.deg(v);
      const long long kv = ord.key(v);
      if (!(kv < ku) || dv < th1) continue;  // init_wl_triangle: v before u
      if (!s.take(u, v)) continue;
      // w in N(u) & N(v) with w before v
      std::vector<int> ws;
      for (const int* pw = g.beg(u); pw < g.end(u); pw++)
        if (ord.key(*pw) < kv && has(g, v, *pw)) ws.push_back(*pw);
      if (clique) {
        const T c12 = nck_t<T>(du - 3, tails) + nck_t<T>(dv - 3, tails);
        for (int w : ws) {
          const int dw = g.deg(w);
          if (dw < 3) continue;
          const long long kw = ord.key(w);
          const T c123 = c12 + nck_t<T>(dw - 3, tails);
          for (const int* pq = g.beg(w); pq < g.end(w); pq++) {
            const int q = *pq;
            if (ord.key(q) < kw && has(g, u, q) && has(g, v, q))
              tot += (tails == 0) ? 1 : c123 + nck_t<T>(g.deg(q) - 3, tails);
          }
        }
        continue;
      }
      const int p12 = common2(g, u, v);
      const int thres2 = std::max(std::max(sum1, sum3 - du - dv), std::max(sum2 - du, sum2 - dv));
      for (int w : ws) {
        const int dw = g.deg(w);
        if (dw < thres2) continue;
        int t13 = 0, t23 = 0, t123 = 0;  // com3, src/fringeCount.cu:934-964
        for (const int* pq = g.beg(w); pq < g.end(w); pq++) {
          const bool b13 = has(g, u, *pq), b23 = has(g, v, *pq);
          t13 += b13; t23 += b23; t123 += (b13 && b23);
        }
        int venn[8];
        const int c123 = t123, c12 = p12 - (c123 + 1), c13 = t13 - (c123 + 1), c23 = t23 - (c123 + 1);
        venn[0] = 0;
        venn[IU] = du - (c12 + c13 + (c123 + 2));
        venn[IV] = dv - (c12 + c23 + (c123 + 2));
        venn[IW] = dw - (c13 + c23 + (c123 + 2));
        venn[IUV] = c12; venn[IUW] = c13; venn[IVW] = c23; venn[IUVW] = c123;
        for (int r = 0; r < rot; r++) tot += fc3<T>(fr[r], venn);
      }
    }
  }
  return tot;
}

// ---------------------------------------------------------------- general core
// src/fringeCount.cu:345-692.  Ordered core matches are enumerated by the
// matching order (mo.list / mo.destdeg); for each, the exclusive Venn region
// sizes of the anchor vertices' neighbourhoods (commonX) feed a sum over all
// placements of the fringes (functionX).
struct GenCtx {
  const MO* mo;
  const Graph* g;
  int k;            // core vertices
  int anchors;      // bitmask of core vertices that anchor fringes
  int nonanchors;
  int stack[6];
  int venn[64];
};

// commonX: histogram with prefix bitmaps, inclusion-exclusion correction, then
// removal of the core vertices themselves (src/fringeCount.cu:345-405).
static void venn_general(GenCtx& c) {
  const Graph& g = *c.g;
  for (int i = 0; i < 64; i++) c.venn[i] = 0;
  for (int i = c.k - 1; i >= 0; i--) {
    if (c.nonanchors & (1 << i)) continue;
    const int vi = c.stack[i];
    for (const int* p = g.beg(vi); p < g.end(vi); p++) {
      int bmp = 1 << i;
      for (int t = 0; t < i; t++) {
        if (c.nonanchors & (1 << t)) continue;
        if (has(g, c.stack[t], *p)) bmp |= 1 << t;
      }
      c.venn[bmp]++;
    }
  }
  const int top = 1 << c.k;
  for (int i = c.k - 2; i >= 0; i--) {
    const int hi = 2 << i;
    for (int j = 1 << i; j < hi; j++) {
      int sum = 0;
      for (int pos = j + hi; pos < top; pos += hi) sum += c.venn[pos];
      c.venn[j] -= sum;
    }
  }
  for (int l = 0; l < c.k; l++) {
    const int x = c.stack[l];
    int bmp = 0;
    for (int t = 0; t < c.k; t++) {
      if (c.nonanchors & (1 << t)) continue;
      if (has(g, c.stack[t], x)) bmp |= 1 << t;
    }
    c.venn[bmp]--;
  }
}

// functionX (src/fringeCount.cu:408-486): anchor sets are placed from the last to
// the first; each set's fringes are spread over the regions that contain the
// set, visited in increasing bitmap order, with the remainder going to the
// region of all anchors.  Each placement contributes the product of
// nCk(remaining region size, fringes put there).
template <class T>
static T place(GenCtx& c, int asi, int idx, int remaining);
template <class T>
static T place_set(GenCtx& c, int asi) {
  const int anch = c.mo->anch[asi];
  return place<T>(c, asi, anch, c.mo->fcnt[asi]);
}
template <class T>
static T place(GenCtx& c, int asi, int idx, int remaining) {
  const int top = c.anchors;
  const int anch = c.mo->anch[asi];
  if (idx == top) {
    const T w = nck_t<T>(c.venn[top], remaining);
    if (is_zero(w)) return T(0);
    if (asi == 0) return w;
    c.venn[top] -= remaining;
    const T r = w * place_set<T>(c, asi - 1);
    c.venn[top] += remaining;
    return r;
  }
  const int next = (((idx | c.nonanchors) + 1) | anch) & ~c.nonanchors;
  T s = T(0);
  for (int a = std::min(c.venn[idx], remaining); a >= 0; a--) {
    const T w = nck_t<T>(c.venn[idx], a);
    if (is_zero(w)) continue;
    c.venn[idx] -= a;
    s += w * place<T>(c, asi, next, remaining - a);
    c.venn[idx] += a;
  }
  return s;
}

// functionX with the reference's own control flow (src/fringeCount.cu:408-486):
// a flat depth-first walk that saves (a, prod, region, venn[region], fr[set])
// per level and, when it backs up, restores only the level it returns to.  A
// region changed by the step it abandons keeps that change, so later
// alternatives can see a reduced region size; for anchor sets with two or
// more fringes this gives different sums than placement() above (the exact
// count), and this is what the reference computes.
static u64 place_reference(GenCtx& c, int* fr) {
  const MO& mo = *c.mo;
  const int top = c.anchors, non = c.nonanchors;
  static thread_local int savea[665], saveidx[665], savevenn[665];
  static thread_local u64 saveprod[665];
  static thread_local int savefr[665];
  int asi = mo.anchorsets - 1;
  u64 sum = 0, prod = 1;
  int level = 0;
  int anch = mo.anch[asi];
  int idx = anch;
  int a = std::min(c.venn[idx], fr[anch]);
  for (;;) {
    savea[level] = a; saveprod[level] = prod; saveidx[level] = idx;
    savevenn[level] = c.venn[idx]; savefr[level] = fr[anch];
    if (a < 0) {
      prod = 0;
    } else if (idx == top) {
      prod *= nck(c.venn[idx], fr[anch]);
      c.venn[idx] -= fr[anch];
      fr[anch] = 0;
      if (asi == 0) { sum += prod; prod = 0; }
    } else {
      prod *= nck(c.venn[idx], a);
      c.venn[idx] -= a;
      fr[anch] -= a;
    }
    if (prod == 0) {
      level--;
      if (level < 0) break;
      a = savea[level] - 1;
      prod = saveprod[level];
      idx = saveidx[level];
      if (idx == top) { asi++; anch = mo.anch[asi]; }
      c.venn[idx] = savevenn[level];
      fr[anch] = savefr[level];
    } else {
      level++;
      if (idx == top) { asi--; anch = mo.anch[asi]; idx = anch; }
      else idx = (((idx | non) + 1) | anch) & ~non;
      a = (idx == top) ? 0 : std::min(c.venn[idx], fr[anch]);
    }
  }
  fr[mo.anch[mo.anchorsets - 1]] = savefr[0];
  return sum;
}

static int g_exact_placements = 0;  // 1: exact placement sum, 0: the reference's functionX

// T = Xo (exact counts) always sums the exact placements.
template <class T>
static T gen_dfs(GenCtx& c, int level) {
  // choose stack[level+1]
  const MO& mo = *c.mo;
  const Graph& g = *c.g;
  const int list = mo.list[level];
  const int first = __builtin_ctz(list);
  const int src = c.stack[first];
  T sum = T(0);
  for (const int* p = g.beg(src); p < g.end(src); p++) {
    const int x = *p;
    if (g.deg(x) < mo.destdeg[level]) continue;
    bool ok = true;
    for (int t = 0; t <= level && ok; t++) {
      if (list & (1 << t)) {
        if (t != first && !has(g, c.stack[t], x)) ok = false;
      } else if (c.stack[t] == x) {
        ok = false;
      }
    }
    if (!ok) continue;
    c.stack[level + 1] = x;
    if (level + 1 == c.k - 1) {
      venn_general(c);
      if (g_exact_placements || !std::is_same<T, u64>::value) {
        sum += place_set<T>(c, mo.anchorsets - 1);
      } else {
        int fr[64] = {0};
        for (int i = 0; i < mo.anchorsets; i++) fr[mo.anch[i]] = mo.fcnt[i];
        sum += place_reference(c, fr);
      }
    } else {
      sum += gen_dfs<T>(c, level + 1);
    }
  }
  return sum;
}

template <class T>
static T general_core(const MO& mo, const Graph& g, const Sample& s) {
  int anchors = 0;
  for (int i = 0; i < mo.anchorsets; i++) anchors |= mo.anch[i];
  const int k = mo.nodes;
  T tot = T(0);
#pragma omp parallel for reduction(+ : tot) schedule(dynamic, 4)
  for (int u = 0; u < g.n; u++) {
    if (g.deg(u) < mo.startdeg) continue;
    GenCtx c;
    c.mo = &mo; c.g = &g; c.k = k; c.anchors = anchors;
    c.nonanchors = anchors ^ ((1 << k) - 1);
    for (const int* p = g.beg(u); p < g.end(u); p++) {
      const int v = *p;
      if (g.deg(v) < mo.destdeg[0] || !s.take(u, v)) continue;  // init_wl_general
      c.stack[0] = u;
      c.stack[1] = v;
      tot += gen_dfs<T>(c, 1);
    }
  }
  return tot;
}

// ---------------------------------------------------------------- dispatch
// Pattern graph of a matching order: core vertices 0..k-1 with the mo.list
// adjacency, then each anchor set's fringes (matchingOrder2ECLgraph,
// src/fringeCount.cu:121-186).
static void pattern_graph(const MO& mo, std::vector<long long>& idx, std::vector<int>& adj) {
  int n = mo.nodes;
  for (int i = 0; i < mo.anchorsets; i++) n += mo.fcnt[i];
  std::vector<std::vector<int>> nb(n);
  for (int i = 0; i < mo.nodes - 1; i++)
    for (int j = 0; j <= i; j++)
      if (mo.list[i] & (1 << j)) { nb[i + 1].push_back(j); nb[j].push_back(i + 1); }
  int v = mo.nodes;
  for (int i = 0; i < mo.anchorsets; i++)
    for (int t = 0; t < mo.fcnt[i]; t++, v++)
      for (int j = 0; j < 6; j++)
        if (mo.anch[i] & (1 << j)) { nb[j].push_back(v); nb[v].push_back(j); }
  idx.assign(n + 1, 0);
  adj.clear();
  for (int x = 0; x < n; x++) {
    std::sort(nb[x].begin(), nb[x].end());
    adj.insert(adj.end(), nb[x].begin(), nb[x].end());
    idx[x + 1] = (long long)adj.size();
  }
}

template <class T>
static T count_core(const MO& mo, const Graph& g, const Sample& s, int* core_type) {
  if (mo.nodes == 1) { *core_type = 1; return vertex_core<T>(mo, g, s); }
  if (mo.nodes == 2) { *core_type = 2; return edge_core<T>(mo, g, s); }
  if (mo.nodes == 3) {
    if (__builtin_popcount(mo.list[1]) == 1) { *core_type = 3; return wedge_core<T>(mo, g, s); }
    *core_type = 4;
    return triangle_core<T>(mo, g, s);
  }
  *core_type = 5;
  return general_core<T>(mo, g, s);
}

}  // namespace

extern "C" {

// Count the occurrences of the pattern described by the 139-byte matching
// order in graph (n, idx, adj) the way src/fringeCount.cu:2199-2262 does:
// cores of 3 or more vertices are divided by the pattern's count in itself.
// out[0] = final count, out[1] = raw total before the division,
// out[2] = automorphism divisor, out[3] = core type (1 vertex .. 5 general).
// stride/phase select a sample of top-level work items (stride 1 = all); the
// automorphism divisor is always computed in full.
int oracle_count(int n, const long long* idx, const int* adj, const unsigned char* mo_bytes, int stride,
                 int phase, int threads, unsigned long long* out) {
  MO mo;
  memcpy(&mo, mo_bytes, sizeof(MO));
  if (mo.nodes < 1 || mo.nodes > 6 || mo.anchorsets > 63) return -1;
  if (threads > 0) omp_set_num_threads(threads);
  Graph g{n, idx[n], idx, adj};
  Sample s;
  s.stride = stride < 1 ? 1 : stride;
  s.phase = phase;
  u64 aut = 1;
  int ct = 0;
  if (mo.nodes >= 3) {
    std::vector<long long> pidx;
    std::vector<int> padj;
    pattern_graph(mo, pidx, padj);
    const int pn = (int)pidx.size() - 1;
    if (pn > n || pidx[pn] > g.m) {
      out[0] = 0; out[1] = 0; out[2] = 0;
      out[3] = (mo.nodes == 3) ? ((__builtin_popcount(mo.list[1]) == 1) ? 3 : 4) : 5;
      return 0;
    }
    Graph pg{pn, pidx[pn], pidx.data(), padj.data()};
    aut = count_core<u64>(mo, pg, Sample(), &ct);
    // the reference keeps the divisor in an int and asserts it is positive
    // (src/fringeCount.cu:2213, 2230-2232)
    const int aut_int = (int)(unsigned int)(aut & 0xffffffffULL);
    if (aut_int <= 0) return -2;
    aut = (u64)aut_int;
  }
  const u64 raw = count_core<u64>(mo, g, s, &ct);
  out[0] = raw / aut;
  out[1] = raw;
  out[2] = aut;
  out[3] = (u64)ct;
  return 0;
}

// Exact count (128-bit, saturating) of the same pattern: the same per-match
// formulas in exact arithmetic, general cores with the exact placement sum.
// out[0..1] count (lo, hi) = raw / divisor, out[2..3] raw total, out[4] divisor
// (exact placements, as the divisor of the exact count), out[5] core type,
// out[6] flags: 1 = pattern larger than the graph (count 0), 2 = saturated.
int oracle_count_exact(int n, const long long* idx, const int* adj, const unsigned char* mo_bytes, int threads,
                       unsigned long long* out) {
  MO mo;
  memcpy(&mo, mo_bytes, sizeof(MO));
  if (mo.nodes < 1 || mo.nodes > 6 || mo.anchorsets > 63) return -1;
  if (threads > 0) omp_set_num_threads(threads);
  Graph g{n, idx[n], idx, adj};
  for (int i = 0; i < 7; i++) out[i] = 0;
  u64 aut = 1;
  int ct = 0;
  if (mo.nodes >= 3) {
    std::vector<long long> pidx;
    std::vector<int> padj;
    pattern_graph(mo, pidx, padj);
    const int pn = (int)pidx.size() - 1;
    if (pn > n || pidx[pn] > g.m) {
      out[5] = (mo.nodes == 3) ? ((__builtin_popcount(mo.list[1]) == 1) ? 3 : 4) : 5;
      out[6] = 1;
      return 0;
    }
    Graph pg{pn, pidx[pn], pidx.data(), padj.data()};
    const Xo a = count_core<Xo>(mo, pg, Sample(), &ct);
    if (a.sat || a.v == 0 || a.v > 0xffffffffULL) return -2;
    aut = (u64)a.v;
  }
  const Xo raw = count_core<Xo>(mo, g, Sample(), &ct);
  out[5] = (u64)ct;
  out[4] = aut;
  if (raw.sat) {
    out[6] = 2;
    return 0;
  }
  const u128 q = raw.v / aut;
  out[0] = (u64)q; out[1] = (u64)(q >> 64);
  out[2] = (u64)raw.v; out[3] = (u64)(raw.v >> 64);
  return 0;
}

// Exact binomial, for unit tests: out[0..1] = C(n, k) (lo, hi), out[2] = saturated.
void oracle_nck_exact(int n, int k, unsigned long long* out) {
  const Xo x = nck_exact(n, k);
  out[0] = (u64)x.v; out[1] = (u64)(x.v >> 64); out[2] = x.sat ? 1 : 0;
}

// General-core placement sums: 0 (default) follows the reference's functionX
// exactly, 1 computes the exact number of fringe placements.
void oracle_set_exact_placements(int on) { g_exact_placements = on ? 1 : 0; }

// Per-call building blocks exposed for unit tests.
unsigned long long oracle_nck(int n, int k) { return nck(n, k); }
unsigned long long oracle_fc3(const int* fr8, const int* venn8) { return fc3<u64>(fr8, venn8); }
int oracle_rotations(const int* f8, int wedge, int* fr48) {
  int fr[6][8];
  const int p = rotations3(f8, fr, wedge != 0);
  memcpy(fr48, fr, sizeof(fr));
  return p;
}

// ---------------------------------------------------------------- brute force
// Independent check: number of injective maps of the pattern into the graph that
// send every pattern edge to a graph edge, divided by the number of such maps of
// the pattern into itself.  Exact (128-bit) for small graphs.
namespace {
struct Brute {
  int pn;
  std::vector<std::vector<int>> padj;  // pattern adjacency
  std::vector<int> order;              // pattern vertices in search order
  std::vector<int> parent;             // an earlier pattern neighbour, or -1
  const Graph* g;
  std::vector<int> map;
  std::vector<char> used;
  bool adj(int a, int b) const { return has(*g, a, b); }
  u128 rec(int i) {
    if (i == pn) return 1;
    const int p = order[i];
    u128 s = 0;
    auto try_vertex = [&](int x) {
      if (used[x]) return;
      for (int q : padj[p]) {
        const int mq = map[q];
        if (mq >= 0 && !adj(mq, x)) return;
      }
      used[x] = 1; map[p] = x;
      s += rec(i + 1);
      used[x] = 0; map[p] = -1;
    };
    if (parent[i] >= 0) {
      const int px = map[parent[i]];
      for (const int* it = g->beg(px); it < g->end(px); it++) try_vertex(*it);
    } else {
      for (int x = 0; x < g->n; x++) try_vertex(x);
    }
    return s;
  }
};

static u128 brute_embeddings(int pn, const int* pedges, int npe, const Graph& g) {
  Brute b;
  b.pn = pn;
  b.padj.assign(pn, {});
  for (int e = 0; e < npe; e++) {
    const int a = pedges[2 * e], c = pedges[2 * e + 1];
    if (a == c) continue;
    if (std::find(b.padj[a].begin(), b.padj[a].end(), c) == b.padj[a].end()) {
      b.padj[a].push_back(c);
      b.padj[c].push_back(a);
    }
  }
  // BFS order from the highest-degree vertex so each later vertex has a parent
  std::vector<char> seen(pn, 0);
  int start = 0;
  for (int v = 0; v < pn; v++) if (b.padj[v].size() > b.padj[start].size()) start = v;
  b.order.push_back(start);
  b.parent.push_back(-1);
  seen[start] = 1;
  for (size_t h = 0; h < b.order.size(); h++) {
    const int x = b.order[h];
    for (int y : b.padj[x]) if (!seen[y]) { seen[y] = 1; b.order.push_back(y); b.parent.push_back(x); }
  }
  for (int v = 0; v < pn; v++) if (!seen[v]) { b.order.push_back(v); b.parent.push_back(-1); }
  b.g = &g;
  b.map.assign(pn, -1);
  b.used.assign(g.n, 0);
  return b.rec(0);
}
}  // namespace

// out[0..1] = count (low, high 64 bits), out[2..3] = |Aut(P)| (low, high).
int oracle_bruteforce(int n, const long long* idx, const int* adj, int pn, const int* pedges, int npe,
                      unsigned long long* out) {
  Graph g{n, idx[n], idx, adj};
  std::vector<long long> pidx;
  std::vector<int> padjv;
  {
    std::vector<std::vector<int>> nb(pn);
    for (int e = 0; e < npe; e++) {
      const int a = pedges[2 * e], c = pedges[2 * e + 1];
      if (a == c) continue;
      nb[a].push_back(c); nb[c].push_back(a);
    }
    pidx.assign(pn + 1, 0);
    for (int v = 0; v < pn; v++) {
      std::sort(nb[v].begin(), nb[v].end());
      nb[v].erase(std::unique(nb[v].begin(), nb[v].end()), nb[v].end());
      padjv.insert(padjv.end(), nb[v].begin(), nb[v].end());
      pidx[v + 1] = (long long)padjv.size();
    }
  }
  Graph pg{pn, pidx[pn], pidx.data(), padjv.data()};
  const u128 aut = brute_embeddings(pn, pedges, npe, pg);
  const u128 emb = brute_embeddings(pn, pedges, npe, g);
  if (aut == 0) return -1;
  const u128 c = emb / aut;
  out[0] = (u64)c; out[1] = (u64)(c >> 64);
  out[2] = (u64)aut; out[3] = (u64)(aut >> 64);
  return 0;
}

}  // extern "C"
