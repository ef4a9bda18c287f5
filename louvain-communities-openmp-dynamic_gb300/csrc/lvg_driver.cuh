// lvg_driver.cuh — the device graph handles (lvg_graph, lvg_state,
// lvg_device_batch), their workspaces, and the pass driver's entry points
// shared by the driver (lvg_driver.cu) and the C-ABI (lvg_api.cu).
#pragma once
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include <cuda_profiler_api.h>

#include "lvg_internal.cuh"

namespace lvg {

extern thread_local std::string g_err;  // the calling thread's last error (lvg_last_error)

struct HubPlanBuffers {
  DBuf<uint32_t> hub_vertex, hub_first, degs;
  DBuf<uint4> chunk;
  DBuf<uint64_t> chunk_part, hub_toff;
  DBuf<uint8_t> hub_tlog;
  DBuf<uint32_t> page_hub;
};

struct LevelBuffers {
  DBuf<uint64_t> off;
  DBuf<uint32_t> deg, key, bins;
  DBuf<float> w;
  HubPlanBuffers hubplan;
};

struct Workspace {
  size_t S = 0, X = 0;
  DBuf<uint8_t> vaff, mark, fv, fn, fc;
  DBuf<uint32_t> ucom, vcom, com_next, dec, cext, csize, ccur, cmem, cbins, wl, wl_count;
  DBuf<tot_t> utot, vtot, ctot;  // vertex weights (level 0 / current level) and community totals
  DBuf<uint64_t> scan64;
  DBuf<uint32_t> scan32, binscratch;
  LevelBuffers lv[2];
  DBuf<uint32_t> gkeys, gfirst;
  DBuf<float> gvals;
  DBuf<double> ctot64;
  DBuf<uint32_t> prior_q;
  DBuf<tot_t> prior_vt, prior_ct;
  DBuf<double> stage_a, stage_b;
  // chunked hub path
  DBuf<uint32_t> chunk_cnt, part_key;
  DBuf<float> part_val, hub_kd;
  DBuf<uint8_t> hub_over;
  DBuf<unsigned long long> hub_best;
  // hub spill tables of static Louvain's first sweep (one colour class's worth)
  DBuf<uint32_t> spill_keys;
  DBuf<float> spill_vals;
  bool spill_now = false;  // the iteration being enqueued spills overflowing hubs
  bool first_sweep = false;  // static Louvain's first iteration (every neighbour a singleton)
  // resident hub tables: build scratch, and the tables the first pass of the
  // run being enqueued keeps up to date (key == nullptr: none)
  DBuf<uint64_t> ht_soff;
  DBuf<uint8_t> ht_slg;
  DBuf<uint32_t> ht_skey, ht_scnt, ht_n;
  HubTabView ht_now;
  // chunked aggregation of the largest communities
  DBuf<uint64_t> mpre, agg_toff, agg_tdeg;
  DBuf<uint2> agg_chunk;
  DBuf<int> agg_tlog;
  DBuf<uint32_t> agg_gk;
  DBuf<float> agg_gv;

  void allocate(size_t S_, size_t X_, cudaStream_t st) {
    S = S_;
    X = X_;
    // vaff: whole 32-bit words (df_start_kernel sets flags by atomics on them)
    vaff.ensure((S + 3) / 4 * 4); mark.ensure(S); fv.ensure(S); fn.ensure(S); fc.ensure(S);
    ucom.ensure(S); vcom.ensure(S); com_next.ensure(S); dec.ensure(S); wl.ensure(S + 1);
    wl_count.ensure(size_t(MAX_COLORS) * NUM_BINS);
    cext.ensure(S + 1); csize.ensure(S + 1); ccur.ensure(S + 1); cmem.ensure(S + 1); cbins.ensure(S + 1);
    utot.ensure(S); vtot.ensure(S); ctot.ensure(S);
    scan64.ensure(scan_scratch_elems(S + 1));
    scan32.ensure(scan_scratch_elems(S + 1));
    binscratch.ensure(bin_scratch_elems(S + 1, MAX_COLORS));
    for (auto &l : lv) {
      l.off.ensure(S + 1);
      l.deg.ensure(S + 1);
      l.bins.ensure(S + 1);
      l.key.ensure(X);
      l.w.ensure(X);
    }
    LVG_CUDA(cudaMemsetAsync(mark.p, 0, S, st));
    LVG_CUDA(cudaMemsetAsync(dec.p, 0xFF, S * sizeof(uint32_t), st));
    // the aggregated levels' membership and weights: every entry a run reads
    // is written by it first, except that the lookups over the whole span
    // also map the entries past the level's live ids, so those must hold ids
    // below the span: zero here, and ids of an earlier run after it
    LVG_CUDA(cudaMemsetAsync(vcom.p, 0, S * sizeof(uint32_t), st));
    LVG_CUDA(cudaMemsetAsync(vtot.p, 0, S * sizeof(tot_t), st));
    hub_kd.ensure(S);
    LVG_CUDA(cudaMemsetAsync(hub_kd.p, 0, S * sizeof(float), st));
  }
};

struct EventPool {
  std::vector<cudaEvent_t> ev;
  size_t used = 0;
  ~EventPool() {
    for (auto e : ev) cudaEventDestroy(e);
  }
  cudaEvent_t record(cudaStream_t s) {
    if (used == ev.size()) {
      cudaEvent_t e;
      LVG_CUDA(cudaEventCreate(&e));
      ev.push_back(e);
    }
    cudaEvent_t e = ev[used++];
    LVG_CUDA(cudaEventRecord(e, s));
    return e;
  }
  void reset() { used = 0; }
};

inline float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0;
  LVG_CUDA(cudaEventElapsedTime(&ms, a, b));
  return ms;
}

struct DBatch {
  const uint32_t *ds = nullptr, *dd = nullptr, *is = nullptr, *id = nullptr;
  const float *dw = nullptr, *iw = nullptr;
  uint32_t *seg = nullptr;
  size_t nd = 0, ni = 0;
  size_t max_group = 0;  // longest run of insertions sharing a source
  // the graph version its batch apply produced (~0: not applied by this
  // library); its edges are then exactly the change from the version before
  uint64_t applied_version = ~0ull;
};

// Resident hub tables of a state (HubTabView): valid for graph version
// `version` and hub index generation `index` (~0: not valid).
struct HubTables {
  DBuf<uint64_t> off;
  DBuf<uint8_t> lg, bad;
  DBuf<uint32_t> key, cnt, nbad;
  size_t hubs = 0, slots = 0;
  uint64_t version = ~0ull, index = ~0ull;
  // the byte counter of the tables' owner (a state's tables are filled by
  // calls on its graph, and a state may outlive the graph); nullptr: the
  // calling handle's
  size_t *acct = nullptr;
  HubTabView view(const uint32_t *slot) const {
    HubTabView v;
    v.slot = slot;
    v.off = off.p;
    v.lg = lg.p;
    v.key = key.p;
    v.cnt = cnt.p;
    v.bad = bad.p;
    v.nbad = nbad.p;
    return v;
  }
};

// Everything an iteration's launches depend on; a captured iteration is
// replayed only while all of it is unchanged.
struct IterKey {
  const void *p[34];
  size_t n[4];
  int k[4];
  float kr;
  double E;  // the stop test's tolerance (graph unions, the device-side loop)
  double M;  // the device-side loop: half the total weight, and the iteration cap
  int L;
  bool operator==(const IterKey &o) const {
    return !std::memcmp(p, o.p, sizeof(p)) && !std::memcmp(n, o.n, sizeof(n)) && !std::memcmp(k, o.k, sizeof(k)) &&
           kr == o.kr && E == o.E && M == o.M && L == o.L;
  }
};

// A graph union (lvg_graph_create_union): graph i owns level-0 vertices
// [vb[i], vb[i+1]) and keeps its own M, order and pass driver.
struct UnionInfo {
  size_t n = 0;
  std::vector<uint64_t> vb;     // host copy of the level-0 bases
  std::vector<double> M;        // per graph: total edge weight / 2
  DBuf<uint32_t> gid0, vb0;     // level 0: graph of each vertex; bases [n+1]
  DBuf<uint64_t> order;         // existing vertices per graph
  DBuf<double> Md;
  // per call
  DBuf<float> kr;               // R / (2M) per graph
  DBuf<uint32_t> gid[2], gbase[2];  // aggregated levels (alternating)
  DBuf<unsigned long long> fix; // Σ best gains of the current iteration per graph
  DBuf<GraphCtl> ctl;
  HBuf<GraphCtl> hctl;
  DBuf<uint8_t> gact, aggex;
  DBuf<uint32_t> q;             // results (level-0 sized)
  DBuf<tot_t> ct;
  DBuf<uint8_t> aff;
};

// What the local-moving launches of a union run need besides the level.
struct UnionCall {
  size_t n;
  const float *kr;
  unsigned long long *fix;
  uint8_t *gact;
  GraphCtl *ctl;
  const double *M;
  double E;
  int L;
};

inline lvg_tuning default_tuning() {
  lvg_tuning t;
  t.frontier_colors = DEFAULT_COLORS_ASYNC;
  t.concurrent_bins = 1;
  t.fused_small = 0;
  t.hub_chunk = HUB_CHUNK;
  t.big_blocks_per_sm = 0;
  t.frontier_max_fraction = 1e-3;
  t.hub_tables = 1;
  for (auto &x : t.bin_max_degree) x = 0;
  t.level_graphs = 1;
  t.small_regs = 64;  // 32 spills ~450 B a thread (R-MAT s24 DF: 0.169 -> 0.166 ms with 64)
  return t;
}

// The local-moving degree bins a tuning asks for (0 entries: the bin's full
// reach). The tuning was checked (check_tuning): every limit is within its
// bin's reach and at least the previous bin's.
inline BinLimits bin_limits_of(const lvg_tuning &t) {
  BinLimits L = default_bin_limits();
  for (int b = 1; b <= 9; ++b)
    if (t.bin_max_degree[b]) L.hi[b] = t.bin_max_degree[b];
  return L;
}

struct RunInfo {
  int iterations = 0, passes = 0;
  float t = 0, tm = 0, ti = 0, tp = 0, tl = 0, ta = 0;
  uint64_t affected = 0;
};

}  // namespace lvg

using namespace lvg;

struct lvg_graph {
  size_t bytes = 0;  // device bytes held (graph, workspace, scratch)
  int device = 0;
  cudaStream_t stream = nullptr;
  Level base;
  uint64_t version = 0;  // bumped by every batch apply that changes an edge
  // the uploaded level's hubs (degree bin 11) in id order and each vertex's
  // index among them (NO_HUB), taken at graph version hub_index_version;
  // hub_index_gen changes only when the set of hubs does
  DBuf<uint32_t> hub_ids, hub_slot;
  std::vector<uint32_t> hub_ids_h, hub_deg_h;
  uint64_t hub_index_version = ~0ull, hub_index_gen = 0;
  HubTables ht_tune;  // the result tables of the autotuner's runs
  // Resident hub tables for the host-array entry points (lvg_naive_dynamic,
  // lvg_delta_screening, lvg_frontier), whose prior comes from host memory
  // on every call: two memberships (a device copy of each) with their
  // tables, taken when a call's uploaded prior equals one of them exactly,
  // the least recently used replaced otherwise; a batch apply carries the
  // current ones to the new graph version. hwork: a call's result tables.
  struct HostTables {
    DBuf<uint32_t> q;
    HubTables t;
    uint64_t stamp = 0;
  };
  HostTables htab[2];
  HubTables hwork;
  uint64_t htab_clock = 0;
  cudaEvent_t vt_ev[2] = {nullptr, nullptr};  // the host entry points' early vertex-weight update
  // Gapped CSR: row u holds deg[u] entries at off[u] with room for cap[u];
  // rows that outgrow their room move to the overflow pool, entries
  // [pool_begin, slots) of key/w. Unused entries hold (0, 0.0).
  DBuf<uint64_t> off;
  DBuf<uint32_t> deg, cap, key, bins;
  DBuf<float> w;
  DBuf<uint8_t> ex;
  size_t slots = 0, pool_begin = 0, pool_cursor = 0;
  bool rows_sorted = true;  // every row sorted by neighbour id (batch apply needs it)
  // batch apply: counters (UPD_*) and scratch
  DBuf<unsigned long long> upd;
  HBuf<unsigned long long> hupd;
  HBuf<uint32_t> hcnt;
  DBuf<UpdRow> u_rows;
  DBuf<uint64_t> u_len, u_src, u_grow, u_spos, u_srcpos, u_gpos, u_scan, u_k0, u_k1;
  DBuf<RowPlan> u_plan;
  DBuf<double> u_wdelta;
  DBuf<uint32_t> u_skey, u_pre, u_keep, u_pos, u_pscan, u_v0, u_v1, u_flag, u_touch, u_tpos, u_tscan;
  DBuf<uint32_t> u_cnt;
  DBuf<uint32_t> u_ds, u_dd, u_is, u_id;
  DBuf<float> u_sw, u_dw, u_iw;
  DBuf<uint8_t> u_tmp;
  HubPlanBuffers hubplan;  // chunked hub work of the uploaded level
  double total_weight = 0;
  std::unique_ptr<Workspace> ws;
  DBuf<Counters> ctr;
  HBuf<Counters> hctr;
  HBuf<uint32_t> hbins;
  EventPool events;
  // captured local-moving iteration of the uploaded level
  cudaGraphExec_t iter_exec = nullptr;
  IterKey iter_key{};
  unsigned long long iter_nodes = 0, iter_moves = 0;
  bool no_graphs = false;
  // the local-moving phase of the uploaded level as one graph: a conditional
  // while node around one iteration, the stop test on the device
  cudaGraphExec_t phase_exec = nullptr;
  IterKey phase_key{};
  bool no_phase_graphs = false;
  bool no_level_graphs = false;  // a level's phase graph could not be built: eager from then on
  // the uploaded level's key of the last call (graphs are captured when a
  // call repeats it)
  IterKey seen_key{};
  bool key_seen = false;
  // side streams for the degree-bin kernels of one colour class, which run
  // concurrently (fork/join with events): bins 1-4 (or the fused 1-6), 5-8
  // (7-8), 9, 10, and the hubs' resident tables
  cudaStream_t aux[5] = {};
  cudaEvent_t fork_ev = nullptr, join_ev[5] = {};
  // result copies that overlap the run (host-array entry points)
  cudaStream_t copy_stream = nullptr;
  ~lvg_graph() {
    if (copy_stream) cudaStreamDestroy(copy_stream);
    if (iter_exec) cudaGraphExecDestroy(iter_exec);
    if (phase_exec) cudaGraphExecDestroy(phase_exec);
    for (auto &a : aux)
      if (a) cudaStreamDestroy(a);
    if (fork_ev) cudaEventDestroy(fork_ev);
    for (auto &e : join_ev)
      if (e) cudaEventDestroy(e);
    for (auto &e : vt_ev)
      if (e) cudaEventDestroy(e);
  }
  bool profiling = false;
  lvg_stats stats = {};
  // batch buffers of the host-array entry points
  DBuf<uint32_t> b_ds, b_dd, b_is, b_id, b_seg;
  DBuf<float> b_dw, b_iw;
  std::unique_ptr<UnionInfo> uni;  // set for graph unions
  lvg_tuning tuning = default_tuning();
};

// A state or a device batch may outlive its graph (it keeps its own device
// id for its destruction and never touches the graph there).
struct lvg_state {
  size_t bytes = 0;
  lvg_graph *g = nullptr;
  int device = 0;
  DBuf<uint32_t> q;
  DBuf<tot_t> vt, ct;
  // the hub tables of membership q (a cache: built when a dynamic method
  // first runs from this state, kept up to date by the runs that write it)
  lvg::HubTables ht;
};

struct lvg_device_batch {
  size_t bytes = 0;
  lvg_graph *g = nullptr;
  int device = 0;
  DBuf<uint32_t> ds, dd, is, id, seg;
  DBuf<float> dw, iw;
  DBatch b;
  bool applied = false;  // replaced by its tidied batch by a batch apply
};


namespace lvg {

// A first-level state on the device: membership, vertex and community weights.
struct StateRef {
  uint32_t *q;
  tot_t *vt, *ct;
};

// Sizes of a tidied batch (deletions, insertions, touched rows, longest
// run of insertions from one source).
struct PlanCounts {
  size_t nd = 0, ni = 0, nrows = 0, max_group = 0;
};

// Records msg as the calling thread's last error and returns code.
int fail(int code, const std::string &msg);

// Runs f, turning exceptions into return codes and last-error messages.
template <class F>
int guarded(F &&f) {
  try {
    g_err.clear();
    return f();
  } catch (const Error &e) {
    return fail(e.code, e.what());
  } catch (const std::bad_alloc &) {
    return fail(LVG_ENOMEM, "host allocation failed");
  } catch (const std::exception &e) {
    return fail(LVG_ECUDA, e.what());
  }
}

void ensure_ws(lvg_graph *g);
// Wait for the graph's stream, counted in the call's statistics (host_syncs).
void host_sync(lvg_graph *g);
// Drop the captured local-moving graphs (their launch shapes and buffers are stale).
void drop_graphs(lvg_graph *g);
void read_counters(lvg_graph *g);
void compute_bins(lvg_graph *g, Level &lv, const uint32_t *deg, uint32_t *list, uint32_t *scratch, int colors);
void build_hub_plan(lvg_graph *g, Level &lv, HubPlanBuffers &hb);
Level aggregate(lvg_graph *g, const Level &lv, const uint32_t *com, size_t CN, int which, int colors,
                const uint32_t *ngid = nullptr, const uint32_t *ngbase = nullptr);
bool uses_hub_tables(const lvg_graph *g, int method);
// tprior/tout (optional): the hub tables of the prior and of the result
// state (the same object for a run in place).
void run(lvg_graph *g, int method, const DBatch &b, StateRef prior, StateRef out, const lvg_options &o,
         RunInfo &info, const std::function<void(cudaEvent_t)> *on_init = nullptr, HubTables *tprior = nullptr,
         HubTables *tout = nullptr, bool vt_ready = false);
void run_union(lvg_graph *g, const lvg_options &o, RunInfo &info);
void check_batch(const lvg_graph *g, const lvg_batch *b, bool need_sorted);
size_t max_group(const lvg_batch *b);
void upload_batch(lvg_graph *g, const lvg_batch *b, DBuf<uint32_t> &ds, DBuf<uint32_t> &dd, DBuf<float> &dw,
                  DBuf<uint32_t> &is, DBuf<uint32_t> &id, DBuf<float> &iw, DBuf<uint32_t> &seg, DBatch &out);
void fill_result(lvg_result *out, const RunInfo &info, size_t span);
void upload_prior(lvg_graph *g, const uint32_t *q, const double *qvtot, const double *qctot, uint32_t *dq,
                  tot_t *dvt, tot_t *dct,
                  const uint32_t *const *cq = nullptr);
int run_host(lvg_graph *g, int method, const lvg_batch *b, const uint32_t *q, const double *qvtot,
             const double *qctot, const lvg_options *o, lvg_result *out);
void init_graph(lvg_graph *g, size_t span, size_t order, size_t X, const uint64_t *coff, const uint32_t *ckey,
                const float *cw, bool has_exists);
PlanCounts tidy_apply(lvg_graph *g, const uint32_t *ds, const uint32_t *dd, const float *dw, size_t nd,
                      const uint32_t *is, const uint32_t *id, const float *iw, size_t ni, uint32_t *tds,
                      uint32_t *tdd, float *tdw, uint32_t *tis, uint32_t *tid, float *tiw);

}  // namespace lvg
