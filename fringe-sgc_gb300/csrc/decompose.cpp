// Pattern decomposition: split a small pattern into a connected core of at most
// six vertices plus fringe vertices, and emit the 139-byte matching order that
// the counting path consumes.
//
// This is the in-process replacement of the reference's fringePreprocess CLI
// (src/fringePreprocess.cpp:287-365).  The greedy core choice (determineCore,
// :260-284), the core-connection step (connectCore, :189-257) and the matching
// order with its tie-breaks (genCoreMatchingOrder, :49-128) must pick the same
// vertices as the reference, because the counting kernels' vertex roles and
// pruning thresholds come from those bytes.  Bytes of the struct that the
// reference leaves unwritten are zero here.

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <vector>

#include "fsgc.h"

namespace {

enum { UNDECIDED = 0, CORE = 1, FRINGE = 2 };

struct Pattern {
  int n = 0;
  std::vector<std::vector<int>> adj;  // sorted, duplicate-free
};

void set_err(char* errbuf, int errlen, const char* fmt, ...) {
  if (!errbuf || errlen <= 0) return;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(errbuf, (size_t)errlen, fmt, ap);
  va_end(ap);
}

void add_edge(Pattern& p, int a, int b) {
  auto ins = [](std::vector<int>& v, int x) {
    auto it = std::lower_bound(v.begin(), v.end(), x);
    if (it == v.end() || *it != x) v.insert(it, x);
  };
  ins(p.adj[a], b);
  ins(p.adj[b], a);
}

bool connected(const Pattern& p) {
  std::vector<char> seen(p.n, 0);
  std::vector<int> q{0};
  seen[0] = 1;
  for (size_t h = 0; h < q.size(); h++)
    for (int y : p.adj[q[h]])
      if (!seen[y]) { seen[y] = 1; q.push_back(y); }
  return (int)q.size() == p.n;
}

// Promote fringe vertices until the core induces a connected subgraph: grow the
// component of the highest-numbered core vertex; from it, search outward through
// non-core vertices and promote the vertex from which the first unreached core
// vertex is seen.
void connect_core(const Pattern& p, std::vector<char>& state, FILE* log) {
  const int n = p.n;
  std::vector<char> reached(n), visited(n);
  for (;;) {
    int c = -1;
    for (int u = 0; u < n; u++) {
      reached[u] = (state[u] != CORE);
      if (state[u] == CORE) c = u;
    }
    // component of c inside the core
    std::deque<int> q{c};
    while (!q.empty()) {
      const int u = q.front();
      q.pop_front();
      if (reached[u]) continue;
      reached[u] = 1;
      for (int v : p.adj[u])
        if (!reached[v]) q.push_back(v);
    }
    bool all = true;
    for (int u = 0; u < n; u++) all = all && reached[u];
    if (all) return;
    q.clear();
    for (int u = 0; u < n; u++) {
      visited[u] = (state[u] == CORE && reached[u]);
      if (visited[u]) q.push_back(u);
    }
    bool promoted = false;
    while (!q.empty() && !promoted) {
      const int u = q.front();
      q.pop_front();
      for (int v : p.adj[u]) {
        if (visited[v]) continue;
        visited[v] = 1;
        if (!reached[v]) {
          if (log) fprintf(log, "including %d in core vertices\n", u);
          state[u] = CORE;
          promoted = true;
          break;
        }
        q.push_back(v);
      }
    }
    if (!promoted) return;  // cannot happen for a connected pattern
  }
}

// Greedy split: for x = 1, 2, ..., every still-undecided vertex of degree x
// (scanned from the highest number down) becomes a fringe and its neighbours
// become core.
void determine_core(const Pattern& p, std::vector<char>& state, FILE* log) {
  state.assign(p.n, UNDECIDED);
  for (int x = 1; x < p.n; x++)
    for (int u = p.n - 1; u >= 0; u--)
      if (state[u] == UNDECIDED && (int)p.adj[u].size() == x) {
        state[u] = FRINGE;
        for (int v : p.adj[u]) state[v] = CORE;
      }
  connect_core(p, state, log);
}

// Core vertices in matching order: next is the unvisited core vertex with the
// most edges to visited vertices, then the highest degree, then the smallest
// first neighbour.  list[i] marks the earlier core vertices that core vertex
// i+1 must be adjacent to; anchor sets are the bitmaps of each fringe's core
// neighbours, listed in increasing bitmap order with their fringe counts.
void matching_order(int src, const Pattern& p, const std::vector<char>& state, fsgc_matching_order* mo) {
  memset(mo, 0, sizeof(*mo));
  const int n = p.n;
  std::vector<int> map(n, 0);
  std::vector<char> visited(n, 0);
  visited[src] = 1;
  mo->startdeg = (uint8_t)p.adj[src].size();
  auto adjacent = [&](int a, int b) { return std::binary_search(p.adj[a].begin(), p.adj[a].end(), b); };
  int top = 0;
  while (top < n - 1) {
    int dst = -1, con = -1;
    for (int v = 0; v < n; v++) {
      if (visited[v] || state[v] != CORE) continue;
      int cnt = 0;
      for (int u = 0; u < n; u++)
        if (visited[u] && adjacent(v, u)) cnt++;
      bool better = con < cnt;
      if (!better && con == cnt) {
        const size_t dd = p.adj[dst].size(), dv = p.adj[v].size();
        better = (dd < dv) || (dd == dv && p.adj[dst].front() > p.adj[v].front());
      }
      if (better) { dst = v; con = cnt; }
    }
    if (dst < 0) break;
    map[dst] = top + 1;
    mo->destdeg[top] = (uint8_t)p.adj[dst].size();
    uint8_t bits = 0;
    for (int v = 0; v < n; v++)
      if (visited[v] && adjacent(dst, v)) bits |= (uint8_t)(1 << map[v]);
    mo->list[top] = bits;
    visited[dst] = 1;
    top++;
  }
  mo->nodes = (uint8_t)(top + 1);
  int per_set[64] = {0};
  for (int v = 0; v < n; v++) {
    if (state[v] != FRINGE) continue;
    int bmp = 0;
    for (int x : p.adj[v]) bmp |= 1 << map[x];
    per_set[bmp]++;
  }
  int k = 0;
  for (int b = 1; b < 64; b++)
    if (per_set[b] > 0) {
      mo->anch[k] = (uint8_t)b;
      mo->fcnt[k] = (uint8_t)per_set[b];
      k++;
    }
  mo->anchorsets = (uint8_t)k;
}

int decompose(const Pattern& p, fsgc_matching_order* out, char* errbuf, int errlen, FILE* log) {
  if (!connected(p)) {
    set_err(errbuf, errlen, "motif is disconnected");
    return FSGC_EINVAL;
  }
  std::vector<char> state;
  determine_core(p, state, log);
  int cores = 0;
  for (int u = 0; u < p.n; u++) cores += (state[u] == CORE);
  if (log) fprintf(log, "%d core nodes\n\n", cores);
  if (cores > FSGC_MAX_CORE) {
    set_err(errbuf, errlen, "only motifs with up to %d core nodes supported", FSGC_MAX_CORE);
    return FSGC_EUNSUPPORTED;
  }
  int src = -1, best = -1;
  for (int u = 0; u < p.n; u++)
    if (state[u] == CORE && (int)p.adj[u].size() > best) {
      best = (int)p.adj[u].size();
      src = u;
    }
  matching_order(src, p, state, out);
  return FSGC_OK;
}

// The reference's 31 predefined motifs (src/patterns.h:57-354), as vertex count
// plus undirected edge list with the reference's vertex numbering (A=0, B=1, ...).
struct Predef {
  int n;
  const char* edges;
  const char* name;
};
const Predef kPredef[31] = {
    {16, "0 1 0 2 0 3 0 4 0 5 0 6 0 14 0 15 1 2 1 5 1 6 1 7 1 11 1 12 1 13 1 14 1 15 2 8 2 9 2 10 2 11 2 12 2 13 2 14 2 15 3 4",
     "16-vertex three-hub pattern"},
    {2, "0 1", "single edge"},
    {3, "0 1 0 2", "wedge"},
    {3, "0 1 0 2 1 2", "triangle"},
    {4, "0 1 0 2 0 3", "3-star"},
    {4, "0 1 0 3 1 2", "4-path"},
    {4, "0 1 0 2 0 3 1 2", "tailed triangle"},
    {4, "0 2 0 3 1 2 1 3", "4-cycle"},
    {4, "0 1 0 2 0 3 1 2 1 3", "diamond"},
    {4, "0 1 0 2 0 3 1 2 1 3 2 3", "4-clique"},
    {5, "0 1 0 2 0 3 0 4", "4-star"},
    {5, "0 1 0 3 0 4 1 2", "spider 2+1"},
    {5, "0 1 0 2 0 3 0 4 1 2", "2-tailed triangle"},
    {5, "0 2 0 4 1 2 1 3", "5-path"},
    {5, "0 1 0 2 0 4 1 2 1 3", "1+1-tailed triangle"},
    {5, "0 2 0 3 0 4 1 2 1 3", "tailed 4-cycle"},
    {5, "0 1 0 2 0 3 0 4 1 2 1 3", "tailed diamond"},
    {5, "0 2 0 3 0 4 1 2 1 3 1 4", "K2,3"},
    {5, "0 1 0 2 0 3 0 4 1 2 1 3 1 4", "book of three triangles"},
    {5, "0 1 0 4 1 2 1 3 2 3", "triangle with long tail"},
    {5, "0 1 0 2 0 4 1 2 1 3 2 3", "tailed diamond (triangle core)"},
    {5, "0 1 0 2 0 3 0 4 1 2 1 3 2 3", "tailed 4-clique"},
    {5, "0 1 0 2 0 3 0 4 1 4 2 3", "hourglass"},
    {5, "0 3 0 4 1 2 1 4 2 3", "5-cycle"},
    {5, "0 1 0 3 0 4 1 2 1 4 2 3", "house"},
    {5, "0 1 0 2 0 3 0 4 1 2 1 4 2 3", "triangle with two wedge fringes"},
    {5, "0 2 0 3 0 4 1 2 1 3 1 4 2 3", "5-vertex pattern 254"},
    {5, "0 1 0 2 0 3 0 4 1 2 1 3 1 4 2 3", "5-vertex pattern 255"},
    {5, "0 1 0 2 0 3 0 4 1 3 1 4 2 3 2 4", "4-cycle with centre"},
    {5, "0 1 0 2 0 3 0 4 1 2 1 3 1 4 2 3 2 4", "5-clique minus an edge"},
    {5, "0 1 0 2 0 3 0 4 1 2 1 3 1 4 2 3 2 4 3 4", "5-clique"},
};

}  // namespace

extern "C" {

int fsgc_preprocess(int n, const int* edges, int nedges, fsgc_matching_order* out, char* errbuf, int errlen) {
  if (!out) {
    set_err(errbuf, errlen, "null output");
    return FSGC_EINVAL;
  }
  if (n < 2 || n > FSGC_MAX_PATTERN) {
    set_err(errbuf, errlen, "number_of_nodes must be between 2 and %d", FSGC_MAX_PATTERN);
    return FSGC_EINVAL;
  }
  if (nedges < 0 || (nedges > 0 && !edges)) {
    set_err(errbuf, errlen, "bad edge list");
    return FSGC_EINVAL;
  }
  Pattern p;
  p.n = n;
  p.adj.assign(n, {});
  for (int e = 0; e < nedges; e++) {
    const int s = edges[2 * e], d = edges[2 * e + 1];
    if (s < 0 || s >= n) {
      set_err(errbuf, errlen, "edge source must be between 0 and %d", n - 1);
      return FSGC_EINVAL;
    }
    if (d < 0 || d >= n) {
      set_err(errbuf, errlen, "edge destination must be between 0 and %d", n - 1);
      return FSGC_EINVAL;
    }
    if (s == d) {  // the reference aborts on an assertion for self loops
      set_err(errbuf, errlen, "self loop on vertex %d", s);
      return FSGC_EINVAL;
    }
    add_edge(p, s, d);
  }
  return decompose(p, out, errbuf, errlen, nullptr);
}

int fsgc_predefined_pattern(int number, int* n, int* edges, int max_edges, int* nedges) {
  if (number < 0 || number > 30 || !n || !nedges) return FSGC_EINVAL;
  const Predef& d = kPredef[number];
  *n = d.n;
  int cnt = 0, a, b, off = 0, used = 0;
  const char* s = d.edges;
  while (sscanf(s + off, "%d %d%n", &a, &b, &used) == 2) {
    if (edges && cnt < max_edges) {
      edges[2 * cnt] = a;
      edges[2 * cnt + 1] = b;
    }
    cnt++;
    off += used;
  }
  *nedges = cnt;
  return (edges && cnt > max_edges) ? FSGC_EINVAL : FSGC_OK;
}

const char* fsgc_predefined_name(int number) {
  if (number < 0 || number > 30) return nullptr;
  return kPredef[number].name;
}

int fsgc_preprocess_predefined(int number, fsgc_matching_order* out, char* errbuf, int errlen) {
  int n = 0, ne = 0, e[2 * 64];
  if (fsgc_predefined_pattern(number, &n, e, 64, &ne) != FSGC_OK) {
    set_err(errbuf, errlen, "unknown pattern");
    return FSGC_EINVAL;
  }
  return fsgc_preprocess(n, e, ne, out, errbuf, errlen);
}

// Verbose variant used by the fringePreprocess CLI: same result, with the
// reference's progress lines written to `log`.
int fsgc_preprocess_log(int n, const int* edges, int nedges, fsgc_matching_order* out, char* errbuf, int errlen,
                        FILE* log) {
  fsgc_matching_order tmp;
  int st = fsgc_preprocess(n, edges, nedges, &tmp, errbuf, errlen);  // validation
  if (st != FSGC_OK && st != FSGC_EUNSUPPORTED) return st;
  Pattern p;
  p.n = n;
  p.adj.assign(n, {});
  for (int e = 0; e < nedges; e++) add_edge(p, edges[2 * e], edges[2 * e + 1]);
  return decompose(p, out, errbuf, errlen, log);
}

}  // extern "C"
