// Internal types shared by the library's translation units.
#pragma once
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

#include "fsgc.h"
#include "fsgc_device.cuh"

namespace fsgc {

// Graph resident in HBM.  Full CSR (int64 offsets, int32 sorted lists) plus the
// loader's derived structures:
//  - degree order:  x < y  iff  (deg x, x) < (deg y, y); every undirected edge
//    is stored once, from its lower to its higher endpoint ("oriented" CSR);
//  - osrc: the lower endpoint of each oriented slot (edge-parallel kernels);
//  - osup: per oriented slot, |N(x) & N(y)| (triangles through the edge);
//  - vtri2: per vertex, twice its triangle count (lazily).
struct GView {
  int n;
  long long m;                       // directed entries
  const long long* __restrict__ off;  // n+1
  const int* __restrict__ adj;        // m
  const int* __restrict__ deg;        // n
  const long long* __restrict__ ooff; // n+1
  const int* __restrict__ oadj;       // m/2
  const int* __restrict__ osrc;       // m/2
  const unsigned* __restrict__ osup;  // m/2
  // packed graphs (many member graphs in one CSR): member of each vertex,
  // the triangle-core relabel gate of each member, and one result slot per
  // member that kernels add each match into; comp == nullptr for one graph
  const int* __restrict__ comp;
  const unsigned char* __restrict__ comp_relabel;
  u64* comp_slots;
};

struct DevGraph {
  int n = 0;
  long long m = 0;
  long long* off = nullptr;
  int* adj = nullptr;
  int* deg = nullptr;
  int maxdeg = 0;
  // orientation + supports (built by prepare_graph)
  bool prepared = false;
  long long* ooff = nullptr;
  int* oadj = nullptr;
  int* osrc = nullptr;
  unsigned* osup = nullptr;
  long long triangles = -1;
  long long max_outdeg = 0;        // largest oriented out-degree
  long long max_bitmap_words = 0;  // max over v of outdeg(v) * ceil(deg(v) / 32)
  u64* vtri2 = nullptr;  // lazily
  unsigned* esup = nullptr;  // lazily: per list entry (u, v), |N(u) & N(v)|
  // wedge core: offsets of chunk boundaries in the lists of high-degree vertices (lazily)
  int* ctab_id = nullptr;
  int* ctab_rows = nullptr;
  int* ctab_pos = nullptr;
  int ctab_K = 0;
  // the reference's degree-relabel gate for the triangle core
  // (src/fringeCount.cu:1237, 1342-1344): vertex roles follow (deg, id) order
  // when it fires, vertex ids otherwise
  bool tri_relabel = false;
  size_t bytes = 0;
  // packed graphs
  int ngraphs = 0;                 // 0 for an ordinary graph
  int* comp = nullptr;             // member of each vertex (device)
  unsigned char* comp_relabel = nullptr;  // per member (device)
  std::vector<int> member_n;       // per member: vertices, directed entries
  std::vector<long long> member_m;

  GView view() const {
    GView g;
    g.n = n; g.m = m; g.off = off; g.adj = adj; g.deg = deg;
    g.ooff = ooff; g.oadj = oadj; g.osrc = osrc; g.osup = osup;
    g.comp = comp; g.comp_relabel = comp_relabel; g.comp_slots = nullptr;
    return g;
  }
};

// Device scratch arena owned by a context; grows on demand, never shrinks.
struct Scratch {
  void* ptr = nullptr;
  size_t bytes = 0;
  int layout_n = -1, layout_rows = -1;
  uint64_t gen = 0;  // bumped whenever ptr changes (captured launch sequences hold the pointer)
};

// Per-context device work areas: a few u64 counters/queues (kernel work
// queues, loader results) and a growable scratch arena (triangle-core bitmaps,
// wedge-core hub cursors).
struct DevWork {
  u64* small = nullptr;  // 32 u64; small[kErrWord] collects kernel error bits
  Scratch tri;
  u64* h_err = nullptr;  // pinned host copy of small[kErrWord], refreshed after kernels that can set it
  fsgc_tuning tune = {2048, 16, 8192, 96, 8};
};
constexpr int kErrWord = 10;

// FSGC_ETIMEDOUT when a kernel of this work area gave up a bounded wait since
// the last call (its count is void), FSGC_OK otherwise; clears the bits.
// Call after the stream has been synchronised.
int take_kernel_error(DevWork& w, cudaStream_t s);

struct Launcher;  // forward

// Structural checks of a matching order shared by every entry point (api.cu).
bool matching_order_valid(const fsgc_matching_order& mo);

// Entry points implemented in prep.cu / count.cu.
int graph_degrees(DevGraph& g, cudaStream_t s, uint64_t* launches, u64* d_scratch_u64);
int prepare_graph(DevGraph& g, cudaStream_t s, uint64_t* launches, u64* d_scratch_u64);
int ensure_vertex_triangles(DevGraph& g, cudaStream_t s, uint64_t* launches);
int ensure_entry_supports(DevGraph& g, cudaStream_t s, uint64_t* launches);
void upload_div_magic();
int sm_count();

struct CountJob {
  const fsgc_matching_order* mo;
  DevGraph* g;
  u64* d_slot;        // result slot (zeroed by the caller)
  int core_type;      // out
  u64 host_value;     // used when the result needs no device work (n, m/2, T)
  bool host_only;
  int exact_placements;  // general core: exact placement sum instead of the reference's
  u64* d_comp_slots;     // packed graphs: per-member result slots (zeroed by the caller)
  int per_member_div;    // packed graphs: divide each member's total by this on the host (1 = none)
  bool exact_count = false;  // exact 128-bit sums: d_slot holds (lo, hi, saturated); ordinary graphs only
};

// Launchers over caller-provided device memory (used by noalloc.cu).
int launch_degrees(int n, const long long* off, int* deg, int* maxdeg, cudaStream_t s);
int launch_wedge_small(const GView& gv, int f_v, int f_vw, int f_w, int lim, int minsum, int* queue, u64* slot,
                       cudaStream_t s);
int launch_wedge_big(const GView& gv, int f_v, int f_vw, int f_w, int lim, int minsum, int* queue, long long* gcur,
                     int* gpre, long long gstride, int blocks, u64* slot, cudaStream_t s);
int wedge_small_max_degree();

// Enqueue the kernels that add the raw total of `mo` on `g` into *d_slot.
int enqueue_count(CountJob& job, cudaStream_t s, uint64_t* launches, DevWork& work);
// Many jobs on one ordinary graph (u64 counts): patterns whose kernels share
// their match enumeration are counted in shared passes (count.cu).
int enqueue_count_set(std::vector<CountJob*>& jobs, cudaStream_t s, uint64_t* launches, DevWork& work);
// Builds, on `s` and synchronously, every per-graph structure a count of `mo`
// would otherwise build on first use, so that counts enqueued afterwards on
// other streams only read the graph.
int prepare_for_count(const fsgc_matching_order& mo, DevGraph& g, cudaStream_t s, uint64_t* launches,
                      DevWork& work);
// Edge list (device pairs) -> cleaned CSR on the device (ingest.cu).  The
// arrays are the caller's to keep (stream-ordered allocations); the list
// array is padded by 16 bytes.  FSGC_EINVAL for an id outside [0, n).
int csr_from_device_edges(int n, long long E, const int* d_pairs, cudaStream_t s, long long** off_out, int** adj_out,
                          long long* m_out, u64* d_small);
// Builds every per-graph structure any count could need, synchronously.
int prepare_all(DevGraph& g, cudaStream_t s, uint64_t* launches, DevWork& work);
// Scratch-arena bytes a count of `mo` on the prepared graph `g` grows to.
size_t count_scratch_bytes(const fsgc_matching_order& mo, const DevGraph& g, const fsgc_tuning& t);
// FSGC_EINVAL unless every field of `t` is in its documented range.
int check_tuning(const fsgc_tuning& t);

}  // namespace fsgc
