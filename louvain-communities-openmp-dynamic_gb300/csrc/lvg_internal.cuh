// lvg_internal.cuh — device data layout and kernel launchers shared by the
// translation units of liblouvain_gb300.so.
#pragma once
#include <utility>
#include <vector>

#include "lvg_common.cuh"

namespace lvg {

// Device bytes are counted per owner (a graph with its workspace, a state, a
// device batch): a C-ABI call names the owner for the duration of the call
// (AcctScope) and every buffer allocated meanwhile adds to, and on release
// subtracts from, that owner's counter. One owner is used by one thread at a
// time (calls on one handle are not concurrent).
inline size_t *&acct_target() {
  static thread_local size_t *t = nullptr;
  return t;
}
struct AcctScope {
  size_t *prev;
  explicit AcctScope(size_t *t) : prev(acct_target()) { acct_target() = t; }
  ~AcctScope() { acct_target() = prev; }
  AcctScope(const AcctScope &) = delete;
  AcctScope &operator=(const AcctScope &) = delete;
};

// Device buffer that grows on demand (contents are not kept when it grows).
template <class T>
struct DBuf {
  T *p = nullptr;
  size_t n = 0;
  size_t *acct = nullptr;  // owner's byte counter (see AcctScope)
  DBuf() = default;
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  ~DBuf() { release(); }
  void ensure(size_t k) {
    if (p && k <= n) return;
    release();
    if (k == 0) k = 1;
    LVG_CUDA(cudaMalloc(&p, k * sizeof(T)));
    n = k;
    acct = acct_target();
    if (acct) *acct += n * sizeof(T);
  }
  void release() {
    if (p) {
      cudaFree(p);
      if (acct) *acct -= n * sizeof(T);
    }
    p = nullptr;
    n = 0;
    acct = nullptr;
  }
  void swap(DBuf &o) {
    std::swap(p, o.p);
    std::swap(n, o.n);
    std::swap(acct, o.acct);
  }
};

template <class T>
struct HBuf {  // pinned host buffer, grows on demand
  T *p = nullptr;
  size_t n = 0;
  HBuf() = default;
  HBuf(const HBuf &) = delete;
  HBuf &operator=(const HBuf &) = delete;
  ~HBuf() { if (p) cudaFreeHost(p); }
  void ensure(size_t k) {
    if (p && k <= n) return;
    if (p) cudaFreeHost(p);
    p = nullptr;
    LVG_CUDA(cudaMallocHost(&p, (k ? k : 1) * sizeof(T)));
    n = k;
  }
};


// Work plan of the chunked path for the largest vertices (degree bin 11) of a
// level: each hub's edge list is cut into chunks (the graph's
// lvg_tuning::hub_chunk edges, HUB_CHUNK by default) that different blocks
// aggregate at once; a second kernel merges a hub's chunks. Hubs are ordered
// by colour class; chunks by hub.
constexpr uint32_t HUB_CHUNK = 4096;
struct HubPlan {
  size_t hubs = 0, chunks = 0, part = 0;        // counts; part = partial-entry capacity
  size_t hub_begin[MAX_COLORS + 1] = {};        // hubs of colour k: [hub_begin[k], hub_begin[k+1])
  size_t chunk_begin[MAX_COLORS + 1] = {};      // chunks of colour k
  const uint32_t *hub_vertex = nullptr;         // [hubs] vertex id
  const uint32_t *hub_first = nullptr;          // [hubs+1] first chunk of each hub
  const uint4 *chunk = nullptr;                 // [chunks] (hub, first edge, end edge, hub vertex)
  const uint64_t *chunk_part = nullptr;         // [chunks] offset of the chunk's partial entries
  // Spill tables (hub_spill_kernel): hub h's table holds 2^hub_tlog[h] >= 2
  // deg slots at hub_toff[h] within its colour class's region; class k's
  // tables take class_slots[k] slots, at most spill_slots. Every table is a
  // whole number of pages of 2^SPILL_PAGE_LOG slots (a hub's degree is above
  // 8192), and page_hub[page_begin[k] + p] is the hub of class k's page p.
  const uint64_t *hub_toff = nullptr;           // [hubs]
  const uint8_t *hub_tlog = nullptr;            // [hubs]
  const uint32_t *page_hub = nullptr;
  size_t spill_slots = 0;
  size_t class_slots[MAX_COLORS] = {};
  size_t page_begin[MAX_COLORS + 1] = {};
};
constexpr int SPILL_PAGE_LOG = 15;

// A graph level in HBM: gapped CSR (row u = key/w[off[u] .. off[u]+deg[u])),
// the layout of the reference's DiGraphCsr (inc/Graph.hxx:384-640). Level 0 is
// the uploaded graph (ex = existence flags); aggregated levels have every
// vertex present (ex = nullptr), as the reference's DiGraphCsr::hasVertex.
struct Level {
  size_t span = 0, order = 0, edges = 0;
  uint64_t *off = nullptr;
  uint32_t *deg = nullptr;
  uint32_t *key = nullptr;
  float *w = nullptr;
  const uint8_t *ex = nullptr;
  // Graph unions (lvg_graph_create_union): the graph of each vertex, and each
  // graph's first vertex on this level ([graphs+1]); nullptr for one graph.
  const uint32_t *gid = nullptr;
  const uint32_t *gbase = nullptr;
  // Every edge weight is exactly 1 (set for the uploaded level when it is so;
  // aggregated levels never): the local-moving kernels then read no weights
  // and sum a group of equal keys by counting it. Sums of 1.0 are exact
  // integers in FP32 below 2^24 whatever the order, so the results are those
  // of the weighted path bit for bit.
  bool unit = false;
  // Vertices grouped by (colour class, degree bin), ascending id within a
  // group: group (k, b) is bins[bin_start[k*NUM_BINS+b] .. bin_start[k*NUM_BINS+b+1]).
  uint32_t *bins = nullptr;
  int colors = 1;
  BinLimits lim = default_bin_limits();  // the degree bins' limits the grouping used
  size_t bin_start[MAX_BUCKETS + 1] = {};
  uint64_t bin_maxdeg[NUM_BINS] = {};
  HubPlan hub;  // chunked work for degree bin 11
  size_t bucket_begin(int k, int b) const { return bin_start[k * NUM_BINS + b]; }
  size_t bucket_size(int k, int b) const { return bin_start[k * NUM_BINS + b + 1] - bin_start[k * NUM_BINS + b]; }
  size_t color_begin(int k) const { return bin_start[k * NUM_BINS]; }
  size_t color_end(int k) const { return bin_start[(k + 1) * NUM_BINS]; }
};

// Device counters block (one allocation; mirrored in pinned host memory).
struct Counters {
  unsigned long long el_fix;     // Σ best gains, 2^-16 fixed point
  unsigned long long vertices;   // processed vertices
  unsigned long long edges;      // scanned edges
  unsigned long long moves;      // moved vertices
  unsigned long long agg_edges;  // edges read by aggregation
  unsigned long long affected;   // residual affected flags
  unsigned int err;              // ERR_* bits
  unsigned int cn;               // community count
  double fp64[4];                // FP64 reductions (total weight, modularity terms)
  unsigned long long bin_vertices[NUM_BINS];  // processed vertices per degree bin
  unsigned long long bin_edges[NUM_BINS];     // scanned edges per degree bin
  unsigned long long bin_over[NUM_BINS];      // vertices redone with an HBM table per bin
  unsigned long long hub_chunk_over;          // hub chunks that wrote raw pairs
  unsigned int gactive;                       // graph unions: graphs still moving after an iteration
  unsigned int ds_long;                       // delta-screening sources with more than 32 insertions
  uint32_t ds_chunks;                         // delta-screening neighbour chunks of the high-degree vertices
  unsigned long long nonunit;                 // edge weights other than 1 (count_nonunit)
  unsigned int dev_iters;                     // iterations run by the device-side loop (iter_end_kernel)
  double dev_el;                              // its last iteration's el
  // Worklists of the first local-moving iteration filled by df_start_kernel
  // (one colour class): pre_flag set, the per-bin counts in pre_count; the
  // first compaction takes them instead of scanning the flags.
  unsigned int pre_flag;
  uint32_t pre_count[NUM_BINS];
  unsigned int qdiff[2];  // an uploaded prior differs from the host-call table caches' memberships
  unsigned long long ht_slots;                // hub-table slots read by hub_table_kernel
  unsigned long long ht_over;                 // hub tables that ran out of room (their hubs scan again)
};

// Resident hub tables (the uploaded level of a unit-weight graph, in the
// first pass of a dynamic method): for every vertex above degree 8192 (a hub)
// the communities of its neighbours with their neighbour counts, k_c of the
// reference's louvainScanCommunitiesW (inc/louvain.hxx:423) kept up to date
// by every move instead of recounted from the hub's edges. Hub h's table has
// 2^lg[h] slots at off[h] (linear probing, keys never removed: a count can
// drop to 0); bad[h] marks a table that ran out of room, whose hub then takes
// the chunked scan path. The counts are exact integers, so a hub's gains are
// those of a fresh scan whatever the order of the updates.
constexpr uint32_t NO_HUB = 0xFFFFFFFFu;
struct HubTabView {
  const uint32_t *slot = nullptr;  // [span] hub index of each vertex, NO_HUB for the others
  const uint64_t *off = nullptr;   // [hubs] first slot
  const uint8_t *lg = nullptr;     // [hubs] log2 of the slot count
  uint32_t *key = nullptr;         // community, EMPTY
  uint32_t *cnt = nullptr;         // neighbours in it
  uint8_t *bad = nullptr;          // [hubs]
  uint32_t *nbad = nullptr;        // hubs marked bad (never lowered while the tables live)
};

// Mark hub h's table bad: the count first, so that whoever sees the mark
// also sees a nonzero count.
__device__ __forceinline__ void ht_mark_bad(const HubTabView &t, uint32_t h) {
  atomicAdd(t.nbad, 1u);
  __threadfence();
  t.bad[h] = 1;
}

// Hub v's table after a neighbour moved from community `from` to `to` (a no-op
// when v is not a hub or its table is marked bad). `from` is present: it is
// the neighbour's community, counted when the table was built or when the
// neighbour moved in. A table without room for `to` is marked bad.
__device__ __forceinline__ void ht_move(const HubTabView &t, uint32_t v, uint32_t from, uint32_t to, Counters *ctr) {
  const uint32_t h = t.slot[v];
  if (h == NO_HUB || t.bad[h]) return;
  const uint64_t o = t.off[h];
  const int lg = t.lg[h];
  const uint32_t mask = (1u << lg) - 1u;
  bool found = false, placed = false;
  uint32_t s = hash_hi(from, lg);
  for (uint32_t p = 0; p <= mask; ++p) {
    const uint32_t k = ld_relaxed(t.key + o + s);
    if (k == from) { atomicSub(t.cnt + o + s, 1u); found = true; break; }
    if (k == EMPTY) break;
    s = (s + 1u) & mask;
  }
  s = hash_hi(to, lg);
  for (uint32_t p = 0; p <= mask; ++p) {
    uint32_t k = ld_relaxed(t.key + o + s);
    if (k == EMPTY) {
      k = atomicCAS(t.key + o + s, EMPTY, to);
      if (k == EMPTY) k = to;
    }
    if (k == to) { atomicAdd(t.cnt + o + s, 1u); placed = true; break; }
    s = (s + 1u) & mask;
  }
  if (!found || !placed) {
    ht_mark_bad(t, h);
    atomicAdd(&ctr->ht_over, 1ull);
  }
}

// Per-graph control of a graph-union run (lvg_static_union), on the device:
// the pass driver of inc/louvain.hxx:1180-1215 kept for each graph.
struct GraphCtl {
  double el;             // last iteration's Σ best gains / M (the reference's el)
  unsigned long long aff;  // residual affected flags at the end (affectedVertices)
  uint32_t it;           // iterations of the current pass
  uint32_t l, p;         // iterations and passes so far
  uint32_t cn;           // communities counted at the end of the last pass
  uint8_t done;          // finished: its result is final
  uint8_t fin;           // finishes at the end of the current pass
  uint8_t pad[6];
};

// Arguments of the local-moving kernels (inc/louvain.hxx:588-609).
struct MoveArgs {
  const uint64_t *off;
  const uint32_t *deg;
  const uint32_t *key;
  const float *w;
  const uint32_t *list;  // vertices of one degree bin
  uint32_t count;        // list length (an upper bound when count_ptr is set)
  const uint32_t *count_ptr;  // device-side list length (worklists), or nullptr
  uint32_t *vcom;        // membership (async: read/write; sync: snapshot, read only)
  tot_t *ctot;           // community totals (async: read/write; sync: snapshot)
  uint32_t *dec;         // sync: decided community per vertex (EMPTY = stay)
  uint8_t *vaff;         // affected flags
  uint8_t *mark;         // sync: neighbour marks of this iteration
  const uint8_t *fa;     // may the vertex move (delta-screening pass 0), or nullptr
  const tot_t *vtot;     // vertex weights
  float kr;              // R / (2M)
  int bin;               // degree bin of the list (statistics)
  Counters *ctr;
  uint32_t *gkeys;       // global fallback tables: [grid][2^glog2]
  float *gvals;
  int glog2;             // log2 of the global table capacity
  // chunked hub path (bin 11)
  HubPlan hub;
  uint32_t *chunk_cnt;   // [chunks] partial entries written by each chunk
  uint32_t *part_key;    // [part] partial (community, weight) entries
  float *part_val;
  float *hub_kd;         // [span] weight to the own community, summed over chunks
  uint8_t *hub_over = nullptr;  // [hubs] a chunk of the hub handed raw pairs on (reset by the merge)
  uint32_t *spill_keys = nullptr;  // the class's hub spill tables (nullptr: the merge merges the partials itself)
  float *spill_vals = nullptr;
  unsigned long long *hub_best = nullptr;  // [hubs] best (gain bits << 32 | ~community) of a spilled hub
  bool big_direct = false;  // degree 513-8192 vertices above the shared claim budget go straight to HBM
  int color;             // colour class of the launch
  // Graph unions (nullptr for one graph): graph of each vertex, per graph
  // R/(2M), the id of its vertex 0 on this level (never a move target, as
  // community 0 of a graph alone), Σ best gains, and whether it still moves.
  const uint32_t *gid = nullptr;
  const float *gkr = nullptr;
  const uint32_t *gzero = nullptr;
  unsigned long long *gfix = nullptr;
  const uint8_t *gact = nullptr;
  // resident blocks per SM of the degree 513-8192 kernels (0 = as many as fit)
  int big_cap = 0;
  // the level's weights are all 1 (Level::unit): the launchers pick the
  // kernels that do not read them
  bool unit = false;
  // resident hub tables (ht.key == nullptr: none; hubs take the chunked path)
  HubTabView ht;
};

// Arguments of the aggregation kernels (inc/louvain.hxx:897-912, 987-992).
struct AggArgs {
  const uint64_t *off;   // input level
  const uint32_t *deg;
  const uint32_t *key;
  const float *w;
  const uint32_t *vcom;  // renumbered membership of the input level
  const uint32_t *coff;  // community -> members CSR
  const uint32_t *cmem;
  const uint32_t *list;  // communities of one total-degree bin
  uint32_t count;
  const uint64_t *yoff;  // output row capacity offsets (scan of total degree)
  uint32_t *ydeg;        // output row degrees
  uint32_t *ykey;
  float *yw;
  uint32_t cn;           // number of communities (distinct keys per row <= cn)
  Counters *ctr;
  uint32_t *gkeys;
  float *gvals;
  int glog2;
};

// Aggregation of the communities above total degree 8192 in AGG_CHUNK-edge
// chunks (lvg_aggregate.cu): community slot j is community comm[j]; its
// global table holds 2^tlog[j] slots at toff[j] (toff[n] = all slots); mpre
// is the prefix of member degrees in member-list order.
constexpr uint32_t AGG_CHUNK = 16384;
struct AggChunks {
  const uint2 *chunk;     // [chunks] (community slot, chunk index)
  const uint32_t *comm;   // [n]
  const uint64_t *toff;   // [n+1]
  const int *tlog;        // [n]
  const uint64_t *mpre;   // [members+1]
  uint32_t *gkeys;        // [toff[n]] EMPTY-initialised
  float *gvals;           // [toff[n]] zero-initialised
  uint32_t n;
};

// ---------------------------------------------------------------- scans (lvg_scan.cu)
size_t scan_scratch_elems(size_t n);
// Exclusive scan; out may alias in. If total != nullptr the sum is written there.
void exclusive_scan_u32(const uint32_t *in, uint32_t *out, size_t n, uint32_t *total, uint32_t *scratch,
                        cudaStream_t s);
void exclusive_scan_u64(const uint64_t *in, uint64_t *out, size_t n, uint64_t *total, uint64_t *scratch,
                        cudaStream_t s);
// Stable multi-split of items [0,n) into `list` by (colour class of the id,
// degree bin), colour-major, ascending id within a group; items with
// ex[i] == 0 (ex != nullptr) are left out. Writes the colors*NUM_BINS+1 group
// starts and the per-bin max degree to the host arrays (synchronises). For a
// graph union (gid != nullptr) the class of item j is that of j - gbase[gid[j]],
// its id within its own graph.
constexpr int BIN_CHUNK = 2048;
size_t bin_scratch_elems(size_t n, int colors);
size_t bin_host_elems(int colors);
void bin_items_u32(const uint32_t *deg, const uint8_t *ex, size_t n, int colors, uint32_t *list, size_t *bin_start,
                   uint64_t *bin_maxdeg, uint32_t *scratch, uint32_t *host_pinned, cudaStream_t s,
                   const uint32_t *gid = nullptr, const uint32_t *gbase = nullptr,
                   const BinLimits &lim = default_bin_limits());
void bin_items_u64(const uint64_t *deg, const uint8_t *ex, size_t n, int colors, uint32_t *list,
                   size_t *bin_start, uint64_t *bin_maxdeg, uint32_t *scratch, uint32_t *host_pinned,
                   cudaStream_t s);

// ---------------------------------------------------------------- element kernels (lvg_kernels.cu)
int grid_for(size_t n, int block, int max_blocks_per_sm = 8);
void launch_degrees(const uint64_t *off, uint32_t *deg, size_t span, cudaStream_t s);
void launch_fill_u8(uint8_t *p, uint8_t v, size_t n, cudaStream_t s);
// n bytes of value v at p, stored by a kernel (not by the copy engines)
void launch_fill_bytes(void *p, uint8_t v, size_t n, cudaStream_t s);
// *el_fix = 0 and wl_count[0..n) = 0 in one launch
void launch_iter_begin(unsigned long long *el_fix, uint32_t *wl_count, int n, cudaStream_t s);
void launch_fill_f32(float *p, size_t n, float v, cudaStream_t s);
void launch_init_static(const Level &g, uint32_t *ucom, tot_t *utot, tot_t *ctot, cudaStream_t s);
void launch_total_weight(const float *w, size_t n, Counters *ctr, cudaStream_t s);  // -> ctr->fp64[0]
// ctr->nonunit += the count of w[0..n) other than 1.0f.
void launch_count_nonunit(const float *w, size_t n, Counters *ctr, cudaStream_t s);
// louvainVertexWeightsOmpW / louvainCommunityWeightsOmpW in FP64 (the C-ABI utilities).
void launch_vertex_weights_f64(const Level &g, double *vtot, cudaStream_t s);
void launch_community_weights_f64(const uint32_t *q, const double *vtot, size_t n, double *ctot, cudaStream_t s);
void launch_batch_weights(const uint32_t *src, const float *w, size_t n, float sign, const uint32_t *vcom,
                          tot_t *vtot, tot_t *ctot, cudaStream_t s);
struct BinBounds;
// Dynamic-frontier Louvain's start in one pass over the batch (the weight
// update and the marking of affected vertices; existing degree-0 vertices are
// left unmarked). With bb (one colour class, no graph union), every vertex it
// marks in degree bins 1..NUM_BINS-2 is appended to the class's worklists
// (ctr->pre_count, ctr->pre_flag) for the first iteration.
void launch_df_start(const uint32_t *ds, const uint32_t *dd, const float *dw, size_t nd, const uint32_t *is,
                     const uint32_t *id, const float *iw, size_t ni, const uint32_t *vcom, tot_t *vtot, tot_t *ctot,
                     const Level &g, uint8_t *vaff, const BinBounds *bb, uint32_t *wl, Counters *ctr,
                     cudaStream_t s);
void launch_df_mark(const uint32_t *ds, const uint32_t *dd, size_t nd, const uint32_t *is, const uint32_t *id,
                    size_t ni, const uint32_t *vcom, uint8_t *vaff, cudaStream_t s);
// seg: ni entries (sources left to the per-source pass, then those with more
// than 32 insertions); list: g.span entries; count: 2 entries; chunks: g.span
// entries and scan_scratch for exclusive_scan_u32 over them.
void launch_ds_mark(const Level &g, const uint32_t *ds, const uint32_t *dd, size_t nd, const uint32_t *is,
                    const uint32_t *id, const float *iw, size_t ni, const uint32_t *seg, size_t nseg,
                    const uint32_t *vcom, const tot_t *vtot, const tot_t *ctot, double M, double R,
                    uint8_t *vertices, uint8_t *neighbors, uint8_t *communities, uint32_t *gkeys, float *gvals,
                    uint32_t *gfirst, int glog2, Counters *ctr, uint32_t *list, uint32_t *count, uint32_t *chunks,
                    uint32_t *scan_scratch, cudaStream_t s);
void launch_clear_isolated(const uint32_t *list, size_t n, uint8_t *vaff, const uint8_t *fa, cudaStream_t s);
struct IsolatedLists {
  const uint32_t *list[MAX_COLORS];
  size_t n[MAX_COLORS];
  int k;
};
void launch_clear_isolated_multi(const IsolatedLists &L, uint8_t *vaff, const uint8_t *fa, cudaStream_t s);
// vaff[u] = 0 for the endpoints u (a, b) of degree 0 that exist.
void launch_clear_isolated_endpoints(const uint32_t *a, size_t na, const uint32_t *b, size_t nb,
                                     const uint32_t *deg, const uint8_t *ex, uint8_t *vaff, cudaStream_t s);
void launch_merge_marks(uint8_t *vaff, uint8_t *mark, size_t n, cudaStream_t s);
// Worklists of one colour class: the active vertices of degree bins
// 1..NUM_BINS-2 (positions bins[start[1] .. start[NUM_BINS-1])) are copied to
// wl at the same bin offsets; wl_count[b] receives each bin's count.
struct BinBounds {
  uint64_t start[NUM_BINS + 1];
};
// One colour class, no graph union: the same worklists from a sequential
// pass over the level's flags. An append outside its bin's slice sets
// ERR_WORKLIST in ctr->err (degrees changed without recomputing the bins).
void launch_compact_active_scan(const Level &g, const BinBounds &bb, const uint8_t *vaff, const uint8_t *fa,
                                uint32_t *wl, uint32_t *wl_count, Counters *ctr, cudaStream_t s);
// Graph unions: only vertices whose graph still moves (gact[gid[u]]).
void launch_compact_active(const uint32_t *bins, const BinBounds &bb, const uint8_t *vaff, const uint8_t *fa,
                           uint32_t *wl, uint32_t *wl_count, cudaStream_t s, const uint32_t *gid = nullptr,
                           const uint8_t *gact = nullptr);
// Deterministic mode: apply the decisions of one colour class (list of its vertices).
void launch_apply_moves(const uint32_t *list, size_t n, uint32_t *dec, uint32_t *vcom, tot_t *ctot,
                        const tot_t *vtot, cudaStream_t s);
void launch_community_flags(const Level &g, const uint32_t *vcom, uint32_t *cext, cudaStream_t s);
void launch_lookup(uint32_t *a, const uint32_t *map, size_t n, cudaStream_t s);  // a[u] = map[a[u]]
void launch_community_sizes(const Level &g, const uint32_t *vcom, uint32_t *csize, uint64_t *ctdeg,
                            cudaStream_t s);
void launch_community_scatter(const Level &g, const uint32_t *vcom, const uint32_t *coff, uint32_t *ccur,
                              uint32_t *cmem, cudaStream_t s);
void launch_level_init(size_t n, const tot_t *vtot, uint32_t *vcom, tot_t *ctot, uint8_t *vaff, cudaStream_t s);
// The next level's vertex weights from this level's community totals: for
// every live community c of the level (cext: exclusive scan of the community
// flags over the level's span, whose sum is *total: c is live when the next
// entry, or the sum after the last one, is larger), vtot_next[cext[c]] =
// ctot[c]. A super-vertex's weight (its row sum with the self-loop,
// louvainVertexWeightsOmpW on the aggregated graph) equals its community's
// total; it is taken from the exact FP64 total instead of re-summing the
// aggregated rows.
void launch_next_vertex_weights(const uint32_t *cext, size_t span, const uint32_t *total, const tot_t *ctot,
                                tot_t *vtot_next, cudaStream_t s);
void launch_count_flags(const uint8_t *f, size_t n, Counters *ctr, cudaStream_t s);
// The device-side iteration loop's test (louvainMoveOmpW, inc/louvain.hxx:588-609):
// el = the iteration's gain sum / M; another iteration while el > E, fewer
// than L have run and no error is flagged (ctr->dev_iters counts them). With
// by_graph (graph unions) each graph has run its own test and the loop goes on
// while any graph is still moving (ctr->gactive).
void launch_iter_end(Counters *ctr, double M, double E, int L, bool by_graph, cudaGraphConditionalHandle h,
                     cudaStream_t s);
// Set ERR_BAD_ID in ctr->err if any a[i] >= limit.
void launch_check_ids(const uint32_t *a, size_t n, uint32_t limit, Counters *ctr, cudaStream_t s);
// launch_check_ids on a prior membership q, and ctr->qdiff[k] = whether q
// differs from the cached membership c0 / c1 (nullptr: not compared).
void launch_check_prior(const uint32_t *q, size_t n, uint32_t limit, const uint32_t *c0, const uint32_t *c1,
                        Counters *ctr, cudaStream_t s);
void launch_modularity(const Level &g, const uint32_t *memb, double *ctot64, Counters *ctr, cudaStream_t s);
void launch_sq_sum(const double *x, size_t n, Counters *ctr, cudaStream_t s);  // -> ctr->fp64[2]

// ---------------------------------------------------------------- local moving (lvg_move.cu)
// Launch the move kernel of degree bin b over a.list[0..a.count).
void launch_move_bin(int b, bool sync, const MoveArgs &a, cudaStream_t s);

// ---------------------------------------------------------------- aggregation (lvg_aggregate.cu)
void launch_aggregate_bin(int b, const AggArgs &a, cudaStream_t s);
// out[i] = total degree of community list[i] (from the row offsets yoff).
void launch_comm_tdeg(const uint32_t *list, size_t n, const uint64_t *yoff, uint64_t *out, cudaStream_t s);
// dst[i] = deg[cmem[i]] for the member list.
void launch_member_degrees(const uint32_t *cmem, const uint32_t *deg, size_t n, uint64_t *dst, cudaStream_t s);
// The chunked communities: chunk merges into the global tables, then the rows.
void launch_aggregate_chunks(const AggArgs &a, const AggChunks &ch, size_t chunks, uint64_t slots, cudaStream_t s);

// Record a failure message for lvg_last_error() and return `code` (for entry
// points outside the driver and the C-ABI files).
int fail_noalloc(int code, const char *msg);

// ---------------------------------------------------------------- batch apply (lvg_update.cu)
// A row touched by a batch: its vertex and its ranges in the (source,
// target)-sorted, duplicate-free deletion and insertion lists.
struct UpdRow {
  uint32_t u, d0, d1, i0, i1;
};
// Row capacity of the gapped layout for a row of degree d.
__host__ __device__ inline uint32_t row_capacity(uint32_t d) { return d + (d >> 3) + 4; }
// Slots of the batch-apply counters.
constexpr int UPD_EDGES = 0;  // change of the edge count (two's complement)
constexpr int UPD_ORDER = 1;  // present vertices after the batch
constexpr int UPD_MAXG = 2;   // longest run of insertions sharing a source
constexpr int UPD_SLOTS = 3;
void launch_row_caps(const uint64_t *coff, size_t n, uint32_t *deg, uint32_t *cap, uint64_t *cap64, cudaStream_t s);
void launch_spread_rows(const uint64_t *coff, const uint32_t *ckey, const float *cw, size_t n, const uint64_t *off,
                        const uint32_t *cap, uint32_t *key, float *w, cudaStream_t s);
// Per touched row: new degree, first changed old index (0 when the row
// moves to the pool), kept deletions and insertions.
struct RowPlan {
  uint32_t n1, f0, dcarry, icarry;
};
void launch_row_plan(const uint64_t *off, const uint32_t *deg, const uint32_t *cap, const uint32_t *key,
                     const float *w, const UpdRow *rows, size_t nrows, const uint32_t *dd, const uint32_t *id,
                     const float *iw, size_t nd_all, uint32_t *pre, uint32_t *keep, RowPlan *plan, uint64_t *len,
                     uint64_t *src, uint64_t *grow, uint8_t *ex, unsigned long long *upd, double *wdelta,
                     cudaStream_t s);
void launch_merge_items(const uint64_t *off, const uint32_t *deg, const uint32_t *key, const float *w,
                        const UpdRow *rows, size_t nrows, const uint32_t *dd, const uint32_t *id, const float *iw,
                        size_t nd_all, const uint32_t *pre, const uint32_t *keep, const RowPlan *plan,
                        const uint64_t *src, uint64_t total, const uint64_t *spos, uint32_t *skey, float *sw,
                        cudaStream_t s);
void launch_copy_items(const uint64_t *off, const UpdRow *rows, size_t nrows, const RowPlan *plan,
                       const uint64_t *spos, uint64_t total, const uint64_t *grow, const uint64_t *gpos,
                       uint64_t pool, const uint32_t *skey, const float *sw, uint32_t *key, float *w,
                       cudaStream_t s);
void launch_finish_rows(uint64_t *off, uint32_t *deg, uint32_t *cap, uint32_t *key, float *w, const UpdRow *rows,
                        size_t nrows, const RowPlan *plan, const uint64_t *grow, const uint64_t *gpos,
                        uint64_t pool, cudaStream_t s);
void launch_count_present(const uint8_t *ex, size_t span, unsigned long long *upd, cudaStream_t s);
void launch_tidy_compact(const uint32_t *src, const uint32_t *dst, const float *w, size_t n, const uint32_t *keep,
                         const uint32_t *pos, const uint32_t *pos_base, uint32_t *osrc, uint32_t *odst, float *ow,
                         cudaStream_t s);
void launch_fresh_caps(const uint32_t *deg, size_t n, uint32_t *cap, uint64_t *cap64, cudaStream_t s);
// The device-side plan of a batch: packed keys, stable sort, first of each
// run, rows of the touched vertices.
void launch_pack_keys(const uint32_t *src, const uint32_t *dst, size_t n, int b, uint64_t *key, uint32_t *val,
                      cudaStream_t s);
void launch_first_flags(const uint64_t *key, size_t n, uint32_t *flag, cudaStream_t s);
void launch_unpack_keys(const uint64_t *key, const uint32_t *val, const uint32_t *flag, const uint32_t *pos,
                        size_t n, int b, const float *w, uint32_t *os, uint32_t *od, float *ow, cudaStream_t s);
void launch_plan_rows(const uint32_t *ds, const uint32_t *nd, const uint32_t *is, const uint32_t *ni, size_t cap,
                      uint32_t *touched, uint32_t *tpos, uint32_t *scan, size_t span, UpdRow *rows,
                      unsigned long long *upd, uint32_t *nrows, cudaStream_t s);

// ---------------------------------------------------------------- generators (lvg_gen.cu)
// Stable radix sorts of 64-bit keys over bits [0, end_bit) (cub); the result
// is in the second buffers when they return true.
bool sort_keys_u64(uint64_t *k0, uint64_t *k1, size_t n, int end_bit, DBuf<uint8_t> &tmp, cudaStream_t s);
bool sort_pairs_u64(uint64_t *k0, uint64_t *k1, uint32_t *v0, uint32_t *v1, size_t n, int end_bit,
                    DBuf<uint8_t> &tmp, cudaStream_t s);
// A synthetic graph: planted partition or R-MAT, as the host generators draw them.
struct GenSpec {
  enum Kind { PP, RMAT } kind = PP;
  size_t span = 0, draws = 0;
  uint32_t n = 0, block = 1;
  double p_in = 0;
  int scale = 0;
  double a = 0, ab = 0, abc = 0;
  std::vector<uint32_t> perm;  // R-MAT vertex permutation (empty: none)
  uint64_t seed = 0;
};
std::vector<uint32_t> rmat_permutation(int scale, uint64_t seed);
size_t generate_graph(const GenSpec &g, DBuf<uint64_t> &coff, DBuf<uint32_t> &ckey, DBuf<float> &cw,
                      DBuf<uint8_t> &ex, cudaStream_t s);
size_t graph_from_edges(const uint32_t *src, const uint32_t *dst, const float *w, size_t n, size_t span,
                        DBuf<uint64_t> &coff, DBuf<uint32_t> &ckey, DBuf<float> &cw, DBuf<uint8_t> &ex,
                        cudaStream_t s);
void generate_batch(const uint64_t *off, const uint32_t *deg, const uint32_t *key, const float *w, size_t nd,
                    size_t ni, uint32_t begin, uint32_t range, float weight, uint64_t seed, DBuf<uint32_t> &ds,
                    DBuf<uint32_t> &dd, DBuf<float> &dw, DBuf<uint32_t> &is, DBuf<uint32_t> &id,
                    DBuf<float> &iw, size_t &out_nd, size_t &out_ni, cudaStream_t s);
void launch_relayout_rows(const uint64_t *old_off, const uint32_t *deg, const uint32_t *old_key, const float *old_w,
                          size_t n, const uint64_t *off, const uint32_t *cap, uint32_t *key, float *w, cudaStream_t s);

// Chunked path of the largest vertices: per colour, one kernel aggregates
// the chunks, a second merges each hub's chunks and moves it. With resident
// tables (a.ht) the hubs of good tables are done by hub_table_kernel, on
// s_tab when given (else on s, before the pair).
void launch_move_hubs(bool sync, const MoveArgs &a, cudaStream_t s, cudaStream_t s_tab = nullptr);
// Resident hub tables. Building (from membership q, for the hubs of plan P of
// the uploaded level): each chunk of a hub's edges counts its communities in
// shared memory and adds them to the hub's scratch table (2^slg[h] >= 2 deg
// slots at soff[h]); ht_count gives each hub's distinct communities; ht_fill
// copies each scratch table into the hub's table of the final layout.
void launch_ht_slots(const uint32_t *hubs, size_t n, uint32_t *slot, cudaStream_t s);
void launch_ht_scratch(const Level &lv, const uint32_t *q, const uint32_t *slot, const uint64_t *soff,
                       const uint8_t *slg, uint32_t *skey, uint32_t *scnt, Counters *ctr, cudaStream_t s);
void launch_ht_count(size_t hubs, const uint64_t *soff, const uint8_t *slg, const uint32_t *skey, uint32_t *n,
                     cudaStream_t s);
void launch_ht_fill(size_t hubs, const uint64_t *soff, const uint8_t *slg, const uint32_t *skey,
                    const uint32_t *scnt, const HubTabView &t, cudaStream_t s);
// Deterministic mode: the table updates of a colour class's decided moves
// (dec[u] != EMPTY), before they are applied (vcom still holds the old
// communities).
void launch_ht_sync_moves(const Level &lv, const uint32_t *list, size_t n, const uint32_t *dec, const uint32_t *vcom,
                          const HubTabView &t, Counters *ctr, cudaStream_t s);
// A tidied batch's edges (src[i], dst[i]) on the tables of hubs src[i], with
// the membership q the tables describe: deletions (insert = false) lower the
// count of q[dst], insertions raise it.
void launch_ht_batch(const uint32_t *src, const uint32_t *dst, size_t n, bool insert, const uint32_t *q,
                     const HubTabView &t, Counters *ctr, cudaStream_t s);
// dst[i] = src[idx[i]]
void launch_gather_u32(const uint32_t *idx, size_t n, const uint32_t *src, uint32_t *dst, cudaStream_t s);

// Global-table capacity (log2) for a maximum degree.
inline int global_table_log2(uint64_t maxdeg) {
  int l = 1;
  while ((uint64_t(1) << l) < 2 * maxdeg) ++l;
  return l;
}
int global_table_blocks(size_t count);
// Worklists of consecutive degree bins of one colour class for one fused
// launch (bins lo..hi of 1..8, at most 6): list, device-side length, and the
// first block of each bin (block_begin[hi-lo+1] = the grid).
struct SmallBins {
  const uint32_t *list[6];
  const uint32_t *count_ptr[6];
  uint32_t block_begin[7];
};
// small_regs: registers a thread of the bins 1-6 launch (32 or 64, lvg_tuning.small_regs).
void launch_move_small(int lo, int hi, bool sync, const MoveArgs &a, const SmallBins &sb, cudaStream_t s,
                       int small_regs = 32);
int device_sms();
// Grid of the local-moving kernel of a large-degree bin (9, 10; 11 = the hub
// merge) for `count` vertices: the size of its per-block global fallback.
int move_grid_blocks(int bin, bool sync, bool unit, size_t count, int big_cap = 0);


// ---------------------------------------------------------------- graph unions (lvg_union.cu)
// Level-0 vertices of graph i: [vb[i], vb[i+1]); gid[x] = i for those.
void launch_fill_gid(const uint32_t *vb, size_t n, uint32_t *gid, cudaStream_t s);
// Union CSR assembly: widened degrees, then rows copied with ids shifted by the graph's base.
void launch_union_degrees(const uint32_t *deg, size_t span, uint64_t *dst, cudaStream_t s);
void launch_union_rows(const uint64_t *off, const uint32_t *deg, const uint32_t *key, const float *w, size_t span,
                       uint32_t vbase, const uint64_t *coff, uint32_t *ckey, float *cw, cudaStream_t s);
// After an iteration: per-graph el, iteration count, stop test; counts the
// graphs still moving into ctr->gactive.
void launch_iter_control(size_t n, GraphCtl *ctl, uint8_t *gact, unsigned long long *fix, const double *M, double E,
                         int L, Counters *ctr, cudaStream_t s);
// At the start of a pass: gact = graph not done; iteration counts reset.
void launch_pass_begin(size_t n, GraphCtl *ctl, uint8_t *gact, cudaStream_t s);
// After a pass's local moving: iterations/passes, and fin for m <= 1 or p >= P.
void launch_pass_end(size_t n, GraphCtl *ctl, int P, cudaStream_t s);
// Graphs with nothing to do (M = 0 or no passes) finish before the first pass.
void launch_pass_skip(size_t n, GraphCtl *ctl, const double *M, int P, cudaStream_t s);
// Community flags of the graphs that go on (not fin, not done).
void launch_union_flags(const uint8_t *ex, size_t span, const uint32_t *vcom, const uint32_t *gid,
                        const GraphCtl *ctl, uint32_t *cext, cudaStream_t s);
// Per graph: communities counted; fin when CN/GN >= tol (GN = existing
// vertices on the first pass, else the graph's vertices on the level), and
// then its flags cleared.
void launch_union_tolerance(size_t n, const uint32_t *gbase, uint32_t *cext, GraphCtl *ctl, const uint64_t *order,
                            bool first, double tol, cudaStream_t s);
// Copies of the level's Σtot and affected flags into each graph's result
// slice (the reference's arrays keep earlier levels' entries past the level's
// span).
void launch_union_snapshot(size_t span, const uint32_t *gid, const uint32_t *gbase, const uint32_t *vb0,
                           const GraphCtl *ctl, const tot_t *ctot, const uint8_t *vaff, tot_t *ct_res,
                           uint8_t *aff_res, cudaStream_t s);
// Final membership of the graphs finishing now: (vcom ? vcom[ucom[v]] : ucom[v]) - gbase[g]; then done.
void launch_union_finalize(size_t S, const uint32_t *gid0, const uint32_t *ucom, const uint32_t *vcom,
                           const uint32_t *gbase, GraphCtl *ctl, uint32_t *q, cudaStream_t s);
void launch_union_mark_done(size_t n, GraphCtl *ctl, cudaStream_t s);
// ucom[v] = map[ucom[v]] for vertices of graphs not done.
void launch_union_lookup(uint32_t *ucom, const uint32_t *map, size_t S, const uint32_t *gid0, const GraphCtl *ctl,
                         cudaStream_t s);
// Next level's bases: gbase_new[i] = cext[gbase[i]] (the total past the end).
void launch_union_bases(size_t n, const uint32_t *gbase, size_t span, const uint32_t *cext, const uint32_t *total,
                        uint32_t *gbase_new, cudaStream_t s);
// Aggregation mask of a level: existing vertices of graphs that go on.
void launch_union_aggex(const uint8_t *ex, size_t span, const uint32_t *gid, const GraphCtl *ctl, uint8_t *aggex,
                        cudaStream_t s);
// affectedVertices of each graph from its result flags.
void launch_union_affected(size_t n, const uint32_t *vb0, const uint8_t *aff_res, GraphCtl *ctl, cudaStream_t s);

}  // namespace lvg
