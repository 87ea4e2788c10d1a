// ref_runner -- TEST INFRASTRUCTURE ONLY.
//
// Runs the reference's own counting kernels on the GPU.  oracle/Makefile
// compiles the reference's src/fringeCount.cu (where it lies, unmodified) into
// _ref/fringeCount.cubin; this program loads that cubin with the CUDA driver
// API and performs the host-side steps of the reference's occurrences()
// (src/fringeCount.cu:2199-2262) around the reference's kernels: worklist
// builders, core kernels, the automorphism self-count on the pattern graph,
// the u64 division.  The one host step done differently is the triangle
// core's degree relabel (relabelByDegree, :1221-1288, CUB sorts on the device):
// it is done here on the host with the same total order, (degree, id)
// descending, which yields the same relabelled graph.
//
//   ref_runner <fringeCount.cubin> <graph.egr> <motif.mo> [<motif.mo> ...]
// prints one line per matching order:
//   core=<type> aut=<divisor> raw=<u64 total> count=<u64 count> ms=<time of occurrences()>
// Each count starts from the original graph and zeroed device globals, as a
// fresh fringeCount process would.
#include <cuda.h>

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

typedef unsigned long long ull;

namespace {

struct MO {  // src/fringes.h:50-58
  uint8_t nodes, anchorsets, startdeg, destdeg[5], list[5], anch[63], fcnt[63];
};
static_assert(sizeof(MO) == 139, "MatchingOrder layout");

struct DevGraph {  // the reference's ECLgraph passed by value (src/ECLgraph.h:45-51)
  int nodes;
  int edges;
  CUdeviceptr nindex;
  CUdeviceptr nlist;
  CUdeviceptr eweight;
};
static_assert(sizeof(DevGraph) == 32, "ECLgraph layout");

struct HostGraph {
  int n = 0, m = 0;
  std::vector<int> idx, adj;
};

void die(const char* what, CUresult r) {
  const char* s = nullptr;
  cuGetErrorString(r, &s);
  fprintf(stderr, "ref_runner: %s failed: %s\n", what, s ? s : "?");
  exit(2);
}
#define CKD(x, what)                      \
  do {                                    \
    CUresult r__ = (x);                   \
    if (r__ != CUDA_SUCCESS) die(what, r__); \
  } while (0)

const int TPB = 512;
enum { IU = 1, IV = 2, IW = 4, IUV = 3, IUW = 5, IVW = 6, IUVW = 7 };

struct Ref {
  CUmodule mod;
  int sms = 0, mtpsm = 0;
  CUdeviceptr total = 0, wlsize = 0, wlpos = 0, maxdeg = 0, d_fr = 0;
  std::vector<std::pair<std::string, CUfunction>> fns;

  CUfunction fn(const char* name) {
    // kernels are static functions; match the mangled name's "<len><name>"
    const std::string key = std::to_string(strlen(name)) + name;
    for (auto& p : fns)
      if (p.first.find(key) != std::string::npos) return p.second;
    fprintf(stderr, "ref_runner: kernel %s not found\n", name);
    exit(2);
  }
  CUdeviceptr global(const char* name, size_t want) {
    const std::string cands[2] = {"_ZL" + std::to_string(strlen(name)) + name, name};
    for (auto& c : cands) {
      CUdeviceptr p;
      size_t bytes;
      if (cuModuleGetGlobal(&p, &bytes, mod, c.c_str()) == CUDA_SUCCESS && bytes == want) return p;
    }
    fprintf(stderr, "ref_runner: global %s not found\n", name);
    exit(2);
  }
  void launch(CUfunction f, unsigned grid, unsigned block, void** args) {
    if (grid == 0) return;
    CKD(cuLaunchKernel(f, grid, 1, 1, block, 1, 1, 0, 0, args, nullptr), "cuLaunchKernel");
  }
  ull get_total() {
    ull v;
    CKD(cuCtxSynchronize(), "kernel");
    CKD(cuMemcpyDtoH(&v, total, 8), "read total");
    return v;
  }
  int get_int(CUdeviceptr p) {
    int v;
    CKD(cuCtxSynchronize(), "kernel");
    CKD(cuMemcpyDtoH(&v, p, 4), "read int");
    return v;
  }
  void set_u64(CUdeviceptr p, ull v) { CKD(cuMemcpyHtoD(p, &v, 8), "write"); }
  void set_int(CUdeviceptr p, int v) { CKD(cuMemcpyHtoD(p, &v, 4), "write"); }
};

DevGraph upload(const HostGraph& h) {
  DevGraph d;
  d.nodes = h.n;
  d.edges = h.m;
  CKD(cuMemAlloc(&d.nindex, sizeof(int) * (h.n + 1)), "alloc");
  CKD(cuMemAlloc(&d.nlist, sizeof(int) * std::max(1, h.m)), "alloc");
  CKD(cuMemcpyHtoD(d.nindex, h.idx.data(), sizeof(int) * (h.n + 1)), "upload");
  if (h.m) CKD(cuMemcpyHtoD(d.nlist, h.adj.data(), sizeof(int) * h.m), "upload");
  d.eweight = 0;
  return d;
}
void release(DevGraph& d) {
  cuMemFree(d.nindex);
  cuMemFree(d.nlist);
}

// Pattern graph of a matching order, as matchingOrder2ECLgraph builds it
// (src/fringeCount.cu:121-186).
HostGraph pattern_graph(const MO& mo) {
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
  HostGraph h;
  h.n = n;
  h.idx.assign(n + 1, 0);
  for (int x = 0; x < n; x++) {
    std::sort(nb[x].begin(), nb[x].end());
    h.adj.insert(h.adj.end(), nb[x].begin(), nb[x].end());
    h.idx[x + 1] = (int)h.adj.size();
  }
  h.m = (int)h.adj.size();
  return h;
}

// Same total order as the reference's relabel: new id = rank of (deg, id) descending.
HostGraph relabel(const HostGraph& g) {
  std::vector<int> order(g.n);
  for (int i = 0; i < g.n; i++) order[i] = i;
  auto deg = [&](int v) { return g.idx[v + 1] - g.idx[v]; };
  std::sort(order.begin(), order.end(), [&](int a, int b) {
    return deg(a) != deg(b) ? deg(a) > deg(b) : a > b;
  });
  std::vector<int> nid(g.n);
  for (int r = 0; r < g.n; r++) nid[order[r]] = r;
  HostGraph h;
  h.n = g.n;
  h.m = g.m;
  h.idx.assign(g.n + 1, 0);
  h.adj.resize(g.m);
  for (int r = 0; r < g.n; r++) h.idx[r + 1] = h.idx[r] + deg(order[r]);
  for (int r = 0; r < g.n; r++) {
    const int old = order[r];
    int* out = &h.adj[h.idx[r]];
    for (int j = g.idx[old]; j < g.idx[old + 1]; j++) *out++ = nid[g.adj[j]];
    std::sort(&h.adj[h.idx[r]], &h.adj[h.idx[r + 1]]);
  }
  return h;
}

int rotations(const int f[8], int fr[6][8], bool wedge) {
  auto rot = [](const int* q, int* o) {
    o[IUVW] = q[IUVW]; o[IUV] = q[IVW]; o[IUW] = q[IUV]; o[IVW] = q[IUW]; o[IU] = q[IV]; o[IV] = q[IW]; o[IW] = q[IU];
  };
  auto rot2 = [](const int* q, int* o) {
    o[IUVW] = q[IUVW]; o[IUV] = q[IUW]; o[IUW] = q[IVW]; o[IVW] = q[IUV]; o[IU] = q[IW]; o[IV] = q[IU]; o[IW] = q[IV];
  };
  memset(fr, 0, sizeof(int) * 48);
  for (int i = 1; i < 8; i++) fr[0][i] = f[i];
  int p = 1;
  const bool any = wedge || f[IU] != f[IV] || f[IU] != f[IW] || f[IUV] != f[IUW] || f[IUV] != f[IVW];
  if (!any) return p;
  rot(fr[0], fr[1]);
  rot2(fr[0], fr[2]);
  p = 3;
  const bool fl = wedge ? (f[IV] != f[IW] || f[IUV] != f[IUW])
                        : ((f[IV] != f[IW] || f[IUV] != f[IUW]) && (f[IU] != f[IW] || f[IUV] != f[IVW]) &&
                           (f[IU] != f[IV] || f[IUW] != f[IVW]));
  if (!fl) return p;
  int* q = fr[3];
  q[IUVW] = f[IUVW]; q[IUV] = f[IUW]; q[IUW] = f[IUV]; q[IVW] = f[IVW]; q[IU] = f[IU]; q[IV] = f[IW]; q[IW] = f[IV];
  rot(fr[3], fr[4]);
  rot2(fr[3], fr[5]);
  return 6;
}

struct Runner {
  Ref& R;
  CUdeviceptr wl;
  HostGraph* host;  // host copy of the current data graph (for the relabel)

  unsigned pervertex(const DevGraph& g) { return (unsigned)((g.nodes + TPB - 1) / TPB); }

  ull vertex_core(const MO& mo, DevGraph g) {
    if (mo.anchorsets == 0) return (ull)g.nodes;
    if (mo.fcnt[0] == 1) return (ull)(g.edges / 2);
    R.set_u64(R.total, 0);
    int tails = mo.fcnt[0];
    void* a[] = {&g, &tails};
    R.launch(R.fn("k_stars"), pervertex(g), TPB, a);
    return R.get_total();
  }

  ull edge_core(const MO& mo, DevGraph g) {
    int f[4] = {0, 0, 0, 0};
    for (int i = 0; i < mo.anchorsets; i++) f[mo.anch[i] & 3] = mo.fcnt[i];
    int f_u = std::min(f[1], f[2]), f_uv = f[3], f_v = std::max(f[1], f[2]);
    const bool special = (f_uv == 1) && (f_u == 0 || f_v == 0);
    int l1 = special ? 1 : f_u + f_uv, l2 = special ? 1 : f_u + f_uv + f_v;
    void* a0[] = {&g, &wl, &l1, &l2};
    R.launch(R.fn("init_wl_edge"), pervertex(g), TPB, a0);
    const int wls = R.get_int(R.wlsize);
    const unsigned blocks = (unsigned)((wls + TPB - 1) / TPB);
    if (blocks == 0) return 0;
    R.set_u64(R.total, 0);
    if (special) {
      if (f_u == 0 && f_v == 0) {
        void* a[] = {&g, &wl};
        R.launch(R.fn("triangle"), blocks, TPB, a);
      } else {
        void* a[] = {&g, &wl, &f_v};
        R.launch(R.fn("tailed_triangle"), blocks, TPB, a);
      }
    } else {
      void* a[] = {&g, &wl, &f_u, &f_uv, &f_v};
      R.launch(R.fn("general_edge_core"), blocks, TPB, a);
    }
    return R.get_total();
  }

  ull wedge_core(const MO& mo, DevGraph g) {
    int f[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = 0; i < mo.anchorsets; i++) f[mo.anch[i] & 7] = mo.fcnt[i];
    if (mo.list[1] == 2) { std::swap(f[IU], f[IV]); std::swap(f[IUW], f[IVW]); }
    int min_u = f[IUVW] + f[IUV] + f[IUW] + f[IU] + 2;
    int min_v = f[IUVW] + f[IUV] + f[IVW] + f[IV] + 1;
    int min_w = f[IUVW] + f[IUW] + f[IVW] + f[IW] + 1;
    int sum3 = min_u + min_v + min_w;
    int sum2 = sum3 - std::max(std::max(min_u, min_v), min_w);
    int sum1 = std::min(std::min(min_u, min_v), min_w);
    int lim = std::min(min_v, min_w);
    if (f[IUVW] == 0 && f[IUV] == 0 && f[IUW] == 0 && f[IU] == 0) {
      void* a0[] = {&g, &wl, &lim};
      R.launch(R.fn("init_wl_specialized_wedge"), pervertex(g), TPB, a0);
      int fv = f[IV], fvw = f[IVW], fw = f[IW];
      void* a1[] = {&g, &wl, &fv, &fvw, &fw};
      R.launch(R.fn("wedgecore_specialized"), (unsigned)(R.sms * (R.mtpsm / TPB)), TPB, a1);
    } else {
      int fr[6][8];
      int rot = rotations(f, fr, true);
      CKD(cuMemcpyHtoD(R.d_fr, fr, sizeof(fr)), "d_fr");
      void* a0[] = {&g, &wl, &sum1, &sum2};
      R.launch(R.fn("init_wl_wedge"), pervertex(g), TPB, a0);
      void* a1[] = {&g, &wl, &min_u, &lim, &sum1, &sum2, &sum3, &rot};
      R.launch(R.fn("general_wedge_core"), (unsigned)(R.sms * ((R.mtpsm - 512) / TPB)), TPB, a1);
    }
    return R.get_total();
  }

  ull triangle_core(const MO& mo, DevGraph g, bool main_graph) {
    int f[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = 0; i < mo.anchorsets; i++) f[mo.anch[i] & 7] = mo.fcnt[i];
    int min_u = f[IUVW] + f[IUV] + f[IUW] + f[IU];
    int min_v = f[IUVW] + f[IUV] + f[IVW] + f[IV];
    int min_w = f[IUVW] + f[IUW] + f[IVW] + f[IW];
    int sum3 = min_u + min_v + min_w + 6;
    int sum2 = sum3 - (std::max(std::max(min_u, min_v), min_w) + 2);
    int sum1 = std::min(std::min(min_u, min_v), min_w) + 2;
    int fr[6][8];
    int rot = rotations(f, fr, false);
    CKD(cuMemcpyHtoD(R.d_fr, fr, sizeof(fr)), "d_fr");
    // the reference's relabel gates (src/fringeCount.cu:1342-1344, 1237)
    if (main_graph && g.nodes > 10000 && !(g.nodes > g.edges / 10)) {
      int maxd = 0;
      for (int v = 0; v < host->n; v++) maxd = std::max(maxd, host->idx[v + 1] - host->idx[v]);
      if (maxd > 16) {
        HostGraph h = relabel(*host);
        CKD(cuMemcpyHtoD(g.nindex, h.idx.data(), sizeof(int) * (h.n + 1)), "relabel upload");
        if (h.m) CKD(cuMemcpyHtoD(g.nlist, h.adj.data(), sizeof(int) * h.m), "relabel upload");
      }
    }
    void* a0[] = {&g, &wl, &sum1, &sum2};
    R.launch(R.fn("init_wl_triangle"), pervertex(g), TPB, a0);
    const unsigned blocks = (unsigned)(R.sms * (R.mtpsm / TPB));
    if (f[IUVW] == 1 && f[IUV] + f[IUW] + f[IVW] == 0 && ((f[IU] == 0) + (f[IV] == 0) + (f[IW] == 0) >= 2)) {
      int tails = f[IU] + f[IV] + f[IW];
      if (tails == 0) {
        void* a[] = {&g, &wl};
        R.launch(R.fn("clique"), blocks, TPB, a);
      } else {
        void* a[] = {&g, &wl, &tails};
        R.launch(R.fn("tailed_clique_triangle"), blocks, TPB, a);
      }
    } else {
      void* a[] = {&g, &wl, &rot, &sum1, &sum2, &sum3};
      R.launch(R.fn("general_triangle_core"), blocks, TPB, a);
    }
    return R.get_total();
  }

  ull general_core(const MO& mo, DevGraph g) {
    int l1 = mo.startdeg, l2 = mo.destdeg[0];
    void* a0[] = {&g, &wl, &l1, &l2};
    R.launch(R.fn("init_wl_general"), pervertex(g), TPB, a0);
    int anchors = 0;
    for (int i = 0; i < mo.anchorsets; i++) anchors |= mo.anch[i];
    unsigned char nonanchors = (unsigned char)(anchors ^ ((1 << mo.nodes) - 1));
    const unsigned blocks = (unsigned)(R.sms * (R.mtpsm / TPB));
    CUdeviceptr venn, fr;
    CKD(cuMemAlloc(&venn, sizeof(int) * (size_t)blocks * TPB * 64), "alloc");
    CKD(cuMemAlloc(&fr, (size_t)blocks * TPB * 64), "alloc");
    MO m2 = mo;
    void* a[] = {&m2, &g, &wl, &nonanchors, &venn, &fr};
    R.launch(R.fn("general_core_level0"), blocks, TPB, a);
    const ull t = R.get_total();
    cuMemFree(venn);
    cuMemFree(fr);
    return t;
  }

  // occurrences() (src/fringeCount.cu:2199-2262)
  ull occurrences(const MO& mo, DevGraph g, bool doauto, int* core, ull* aut_out, ull* raw_out) {
    if (mo.nodes == 1) { *core = 1; return *raw_out = vertex_core(mo, g); }
    if (mo.nodes == 2) { *core = 2; return *raw_out = edge_core(mo, g); }
    ull aut = 1;
    if (doauto) {
      HostGraph pg = pattern_graph(mo);
      if (pg.n > g.nodes || pg.m > g.edges) { *core = 0; *aut_out = 0; *raw_out = 0; return 0; }
      DevGraph dpg = upload(pg);
      int c2;
      ull a2, r2;
      const int aut_int = (int)occurrences(mo, dpg, false, &c2, &a2, &r2);  // int automorphisms (:2230)
      R.set_u64(R.total, 0);
      R.set_int(R.wlsize, 0);
      R.set_int(R.wlpos, 0);
      R.set_int(R.maxdeg, 0);
      release(dpg);
      // assert(automorphisms > 0) (:2232)
      if (aut_int <= 0) { fprintf(stderr, "ref_runner: automorphisms %d not positive\n", aut_int); exit(2); }
      aut = (ull)aut_int;
    }
    *aut_out = aut;
    ull raw;
    if (mo.nodes == 3) {
      if (__builtin_popcount(mo.list[1]) == 1) { *core = 3; raw = wedge_core(mo, g); }
      else { *core = 4; raw = triangle_core(mo, g, doauto); }
    } else {
      *core = 5;
      raw = general_core(mo, g);
    }
    *raw_out = raw;
    return raw / aut;
  }
};

HostGraph read_egr(const char* path) {
  FILE* f = fopen(path, "rb");
  if (!f) { fprintf(stderr, "ref_runner: cannot open %s\n", path); exit(2); }
  HostGraph h;
  if (fread(&h.n, 4, 1, f) != 1 || fread(&h.m, 4, 1, f) != 1) { fprintf(stderr, "bad egr\n"); exit(2); }
  h.idx.resize(h.n + 1);
  h.adj.resize(h.m);
  if (fread(h.idx.data(), 4, h.n + 1, f) != (size_t)h.n + 1 ||
      (h.m && fread(h.adj.data(), 4, h.m, f) != (size_t)h.m)) { fprintf(stderr, "bad egr\n"); exit(2); }
  fclose(f);
  return h;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 4) {
    fprintf(stderr, "usage: %s fringeCount.cubin graph.egr motif.mo [motif.mo ...]\n", argv[0]);
    return 2;
  }
  CKD(cuInit(0), "cuInit");
  CUdevice dev;
  CKD(cuDeviceGet(&dev, 0), "cuDeviceGet");
  CUcontext ctx;
  CKD(cuDevicePrimaryCtxRetain(&ctx, dev), "context");
  CKD(cuCtxSetCurrent(ctx), "context");
  Ref R;
  CKD(cuModuleLoad(&R.mod, argv[1]), "cuModuleLoad");
  cuDeviceGetAttribute(&R.sms, CU_DEVICE_ATTRIBUTE_MULTIPROCESSOR_COUNT, dev);
  cuDeviceGetAttribute(&R.mtpsm, CU_DEVICE_ATTRIBUTE_MAX_THREADS_PER_MULTIPROCESSOR, dev);
  unsigned nf = 0;
  CKD(cuModuleGetFunctionCount(&nf, R.mod), "function count");
  std::vector<CUfunction> fs(nf);
  CKD(cuModuleEnumerateFunctions(fs.data(), nf, R.mod), "enumerate functions");
  for (CUfunction f : fs) {
    const char* name = nullptr;
    if (cuFuncGetName(&name, f) == CUDA_SUCCESS && name) R.fns.push_back({name, f});
  }
  R.total = R.global("total", 8);
  R.wlsize = R.global("wlsize", 4);
  R.wlpos = R.global("wlpos", 4);
  R.maxdeg = R.global("maxdeg", 4);
  R.d_fr = R.global("d_fr", 6 * 8 * 4);
  HostGraph h = read_egr(argv[2]);
  DevGraph g = upload(h);
  Runner run{R, 0, &h};
  CKD(cuMemAlloc(&run.wl, std::max(sizeof(int) * 2 * (size_t)std::max(1, h.m), sizeof(int) * (size_t)h.n)), "worklist");
  for (int a = 3; a < argc; a++) {
    MO mo;
    FILE* f = fopen(argv[a], "rb");
    if (!f || fread(&mo, 1, sizeof(mo), f) != sizeof(mo)) { fprintf(stderr, "bad .mo %s\n", argv[a]); return 2; }
    fclose(f);
    CKD(cuMemcpyHtoD(g.nindex, h.idx.data(), sizeof(int) * (h.n + 1)), "upload");
    if (h.m) CKD(cuMemcpyHtoD(g.nlist, h.adj.data(), sizeof(int) * h.m), "upload");
    R.set_u64(R.total, 0);
    R.set_int(R.wlsize, 0);
    R.set_int(R.wlpos, 0);
    R.set_int(R.maxdeg, 0);
    CKD(cuCtxSynchronize(), "setup");
    int core = 0;
    ull aut = 1, raw = 0;
    const auto t0 = std::chrono::steady_clock::now();
    const ull count = run.occurrences(mo, g, true, &core, &aut, &raw);
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    printf("core=%d aut=%llu raw=%llu count=%llu ms=%.3f\n", core, aut, raw, count, ms);
    fflush(stdout);
  }
  cuMemFree(run.wl);
  release(g);
  return 0;
}
