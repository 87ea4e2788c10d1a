// Allocation-free count entry point.
//
// Some callers cannot call cudaMalloc at the time they want a count: code that
// runs while a host framework forbids allocation (an inference or real-time
// loop whose memory was reserved up front, a plugin living inside another
// library's memory pool, a caller that must not grow its footprint after
// start-up).  They own the graph in device memory and only need the number.
// fsgc_count_wedge_noalloc serves the wedge core whose centre carries no
// fringes (the reference's wedgecore_specialized path): every intermediate --
// the degree array, the pattern graph that gives the divisor, the work queues,
// the per-centre cursors of hub endpoints -- lives in one file-scope device
// array of fixed size, so the call allocates nothing.
//
// Limits and sharing: the array is kNoAllocScratchBytes long and every GPU that
// loads this library keeps it until the process exits.  A graph needs 4 bytes
// per vertex plus, when some vertex has more than 2048 neighbours, 20 bytes
// per unit of the maximum degree for each block of the hub-endpoint pass;
// larger graphs are rejected with FSGC_EUNSUPPORTED.  All calls share the
// array and it keeps the last call's contents: each call clears the counters
// and queues it uses.  Calls that overlap on the GPU (two host threads, or two
// streams, at once) race on it and must be serialised by the caller.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "fsgc_internal.h"

namespace {

constexpr size_t kNoAllocScratchBytes = (size_t)64 << 20;  // 64 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// byte offsets inside the scratch array
constexpr size_t kSlotsOff = 0;       // 32 u64: totals, queues, maximum degrees
constexpr size_t kPatternOff = 256;   // pattern graph: offsets, lists, degrees
constexpr size_t kPatternBytes = 8192;
constexpr size_t kDegOff = kPatternOff + kPatternBytes;
enum { S_RAW = 0, S_PRAW = 1, S_MAXDEG = 2, S_Q_SMALL = 3, S_Q_BIG = 4, S_Q_PSMALL = 5, S_PMAXDEG = 6 };

std::mutex g_setup_mu;
void* g_scratch_dev[64] = {nullptr};

int set_err(char* errbuf, int errlen, int code, const char* msg) {
  if (errbuf && errlen > 0) snprintf(errbuf, (size_t)errlen, "%s", msg);
  return code;
}

// Once per device, with that device current: the device address of the
// scratch array (the host-side symbol is only a stand-in for it) and the
// binomial division table in constant memory.
int setup_device(int dev, unsigned char** base) {
  if (dev < 0 || dev >= 64) return FSGC_EINVAL;
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_dev[dev]) {
    void* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || ptr == nullptr) {
      cudaGetLastError();
      return FSGC_ECUDA;
    }
    fsgc::upload_div_magic();
    if (cudaGetLastError() != cudaSuccess) return FSGC_ECUDA;
    g_scratch_dev[dev] = ptr;
  }
  *base = static_cast<unsigned char*>(g_scratch_dev[dev]);
  return FSGC_OK;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

extern "C" {

int fsgc_count_wedge_noalloc(int n, int64_t m, const int64_t* d_nindex, const int32_t* d_nlist,
                             const fsgc_matching_order* mo, void* stream, fsgc_result* out, char* errbuf,
                             int errlen) {
  if (!mo || !out || n < 1 || m < 0 || !d_nindex || (m > 0 && !d_nlist))
    return set_err(errbuf, errlen, FSGC_EINVAL, "bad arguments");
  memset(out, 0, sizeof(*out));
  if (!fsgc::matching_order_valid(*mo)) return set_err(errbuf, errlen, FSGC_EINVAL, "malformed matching order");
  // the wedge core with a fringe-free centre (src/fringeCount.cu:1783-1810)
  if (mo->nodes != 3 || __builtin_popcount(mo->list[1]) != 1 || mo->anchorsets < 1 || mo->anchorsets > 63)
    return set_err(errbuf, errlen, FSGC_EUNSUPPORTED, "only wedge-core patterns are supported");
  int f[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int pn = 3, pm = 2 * 2;
  for (int i = 0; i < mo->anchorsets; i++) {
    if (mo->anch[i] == 0 || mo->anch[i] > 7) return set_err(errbuf, errlen, FSGC_EINVAL, "malformed matching order");
    f[mo->anch[i]] = mo->fcnt[i];
    pn += mo->fcnt[i];
    pm += 2 * mo->fcnt[i] * __builtin_popcount(mo->anch[i]);
  }
  if (pn > FSGC_MAX_PATTERN) return set_err(errbuf, errlen, FSGC_EINVAL, "pattern larger than 32 vertices");
  if (mo->list[1] == 2) {  // centre is B
    std::swap(f[1], f[2]);
    std::swap(f[5], f[6]);
  }
  if (f[7] || f[3] || f[5] || f[1])
    return set_err(errbuf, errlen, FSGC_EUNSUPPORTED, "the wedge centre carries fringes");
  out->core_type = FSGC_CORE_WEDGE;
  // the reference returns 0 before any work when the pattern exceeds the graph
  if ((long long)pn > n || (long long)pm > m) {
    out->flags = FSGC_FLAG_PATTERN_TOO_LARGE;
    return FSGC_OK;
  }
  const int min_v = f[6] + f[2] + 1, min_w = f[6] + f[4] + 1;
  const int lim = std::min(min_v, min_w), minsum = min_v + min_w;
  const size_t deg_bytes = align256(sizeof(int) * (size_t)n);
  if (kDegOff + deg_bytes > kNoAllocScratchBytes)
    return set_err(errbuf, errlen, FSGC_EUNSUPPORTED, "graph exceeds the fixed scratch (too many vertices)");

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return set_err(errbuf, errlen, FSGC_ENODEV, "no CUDA device");
  unsigned char* base = nullptr;
  int st = setup_device(dev, &base);
  if (st != FSGC_OK) return set_err(errbuf, errlen, st, "scratch set-up failed");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  u64* slots = reinterpret_cast<u64*>(base + kSlotsOff);

  // pattern graph of the matching order (src/fringeCount.cu:121-186), built in
  // fixed host arrays (at most 32 vertices, each adjacent to at most 31)
  int nbr[FSGC_MAX_PATTERN][FSGC_MAX_PATTERN];
  int nbc[FSGC_MAX_PATTERN] = {0};
  auto link = [&](int a, int b) {
    nbr[a][nbc[a]++] = b;
    nbr[b][nbc[b]++] = a;
  };
  for (int i = 0; i < 2; i++)
    for (int j = 0; j <= i; j++)
      if (mo->list[i] & (1 << j)) link(i + 1, j);
  int vx = 3;
  for (int i = 0; i < mo->anchorsets; i++)
    for (int t = 0; t < mo->fcnt[i]; t++, vx++)
      for (int j = 0; j < 3; j++)
        if (mo->anch[i] & (1 << j)) link(j, vx);
  long long poff[FSGC_MAX_PATTERN + 1];
  int padj[FSGC_MAX_PATTERN * FSGC_MAX_PATTERN];
  poff[0] = 0;
  for (int x = 0; x < pn; x++) {
    std::sort(nbr[x], nbr[x] + nbc[x]);
    for (int k = 0; k < nbc[x]; k++) padj[poff[x] + k] = nbr[x][k];
    poff[x + 1] = poff[x] + nbc[x];
  }
  long long* d_poff = reinterpret_cast<long long*>(base + kPatternOff);
  int* d_padj = reinterpret_cast<int*>(base + kPatternOff + 512);
  int* d_pdeg = reinterpret_cast<int*>(base + kPatternOff + 512 + 4096 + 2048);
  int* deg = reinterpret_cast<int*>(base + kDegOff);

#define NA_TRY(x, msg)                                           \
  do {                                                           \
    if ((x) != cudaSuccess) {                                    \
      cudaGetLastError();                                        \
      return set_err(errbuf, errlen, FSGC_ECUDA, msg);           \
    }                                                            \
  } while (0)

  NA_TRY(cudaMemsetAsync(slots, 0, 32 * sizeof(u64), s), "clearing scratch");
  NA_TRY(cudaMemcpyAsync(d_poff, poff, sizeof(long long) * (pn + 1), cudaMemcpyHostToDevice, s), "pattern upload");
  NA_TRY(cudaMemcpyAsync(d_padj, padj, sizeof(int) * (size_t)poff[pn], cudaMemcpyHostToDevice, s), "pattern upload");
  // divisor: the pattern counted in itself with the same kernel
  if (fsgc::launch_degrees(pn, d_poff, d_pdeg, reinterpret_cast<int*>(slots + S_PMAXDEG), s) != FSGC_OK)
    return set_err(errbuf, errlen, FSGC_ECUDA, "degree pass failed");
  fsgc::GView pv;
  memset(&pv, 0, sizeof(pv));
  pv.n = pn; pv.m = poff[pn]; pv.off = d_poff; pv.adj = d_padj; pv.deg = d_pdeg;
  if (fsgc::launch_wedge_small(pv, f[2], f[6], f[4], lim, minsum, reinterpret_cast<int*>(slots + S_Q_PSMALL),
                               slots + S_PRAW, s) != FSGC_OK)
    return set_err(errbuf, errlen, FSGC_ECUDA, "pattern count failed");
  // degrees of the data graph, then its maximum to size the hub pass
  const long long* d_off = reinterpret_cast<const long long*>(d_nindex);
  if (fsgc::launch_degrees(n, d_off, deg, reinterpret_cast<int*>(slots + S_MAXDEG), s) != FSGC_OK)
    return set_err(errbuf, errlen, FSGC_ECUDA, "degree pass failed");
  int maxdeg = 0;
  NA_TRY(cudaMemcpyAsync(&maxdeg, slots + S_MAXDEG, sizeof(int), cudaMemcpyDeviceToHost, s), "reading degrees");
  NA_TRY(cudaStreamSynchronize(s), "degree pass");
  fsgc::GView gv;
  memset(&gv, 0, sizeof(gv));
  gv.n = n; gv.m = m; gv.off = d_off; gv.adj = d_nlist; gv.deg = deg;
  int big_blocks = 0;
  long long* gcur = nullptr;
  int* gpre = nullptr;
  if (maxdeg > fsgc::wedge_small_max_degree()) {
    // per block: two int64 cursors and one int32 offset per centre
    const size_t start = kDegOff + deg_bytes;
    const size_t per_block = align256((size_t)maxdeg * 2 * sizeof(long long)) + align256(((size_t)maxdeg + 1) * sizeof(int));
    const size_t room = kNoAllocScratchBytes - start;
    big_blocks = (int)std::min<size_t>((size_t)fsgc::sm_count(), room / per_block);
    if (big_blocks < 1)
      return set_err(errbuf, errlen, FSGC_EUNSUPPORTED, "graph exceeds the fixed scratch (maximum degree too large)");
    gcur = reinterpret_cast<long long*>(base + start);
    gpre = reinterpret_cast<int*>(base + start + (size_t)big_blocks * align256((size_t)maxdeg * 2 * sizeof(long long)));
  }
  if (fsgc::launch_wedge_small(gv, f[2], f[6], f[4], lim, minsum, reinterpret_cast<int*>(slots + S_Q_SMALL),
                               slots + S_RAW, s) != FSGC_OK)
    return set_err(errbuf, errlen, FSGC_ECUDA, "count failed");
  if (big_blocks > 0 &&
      fsgc::launch_wedge_big(gv, f[2], f[6], f[4], lim, minsum, reinterpret_cast<int*>(slots + S_Q_BIG), gcur, gpre,
                             (long long)maxdeg, big_blocks, slots + S_RAW, s) != FSGC_OK)
    return set_err(errbuf, errlen, FSGC_ECUDA, "count failed");
  u64 res[2] = {0, 0};
  NA_TRY(cudaMemcpyAsync(res, slots + S_RAW, 2 * sizeof(u64), cudaMemcpyDeviceToHost, s), "reading the count");
  NA_TRY(cudaStreamSynchronize(s), "count");
  uint64_t aut = 0;
  if (fsgc_divisor_from_self_count(res[1], &aut) != FSGC_OK)
    return set_err(errbuf, errlen, FSGC_EINVAL, "the pattern's count in itself is not a positive int: no divisor");
  out->raw_total = res[0];
  out->automorphisms = aut;
  out->count = res[0] / aut;
  return FSGC_OK;
#undef NA_TRY
}

}  // extern "C"
