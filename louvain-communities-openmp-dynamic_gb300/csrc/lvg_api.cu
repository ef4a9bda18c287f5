// lvg_api.cu — C-ABI entry points, device graph handles and the pass driver.
//
// The pass driver follows louvainInvokeOmp (inc/louvain.hxx:1120-1221): per
// repetition it initialises membership and weights (fi), marks affected
// vertices (fm), then alternates local moving and aggregation until a pass
// converges in one iteration, maxPasses is reached, or the community count
// stops shrinking below aggregationTolerance. Everything runs on the graph's
// own CUDA stream; the host only reads back the per-iteration gain sum and the
// per-pass community count to take the reference's branch decisions.
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

thread_local std::string g_err;

struct HubPlanBuffers {
  DBuf<uint32_t> hub_vertex, hub_first, degs;
  DBuf<uint4> chunk;
  DBuf<uint64_t> chunk_part;
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
  DBuf<float> utot, vtot, ctot;
  DBuf<uint64_t> scan64;
  DBuf<uint32_t> scan32, binscratch;
  LevelBuffers lv[2];
  DBuf<uint32_t> gkeys, gfirst;
  DBuf<float> gvals;
  DBuf<double> ctot64;
  DBuf<uint32_t> prior_q;
  DBuf<float> prior_vt, prior_ct;
  DBuf<double> stage_a, stage_b;
  // chunked hub path
  DBuf<uint32_t> chunk_cnt, part_key;
  DBuf<float> part_val, hub_kd;
  // chunked aggregation of the largest communities
  DBuf<uint64_t> mpre, agg_toff, agg_tdeg;
  DBuf<uint2> agg_chunk;
  DBuf<int> agg_tlog;
  DBuf<uint32_t> agg_gk;
  DBuf<float> agg_gv;

  void allocate(size_t S_, size_t X_, cudaStream_t st) {
    S = S_;
    X = X_;
    vaff.ensure(S); mark.ensure(S); fv.ensure(S); fn.ensure(S); fc.ensure(S);
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

float elapsed(cudaEvent_t a, cudaEvent_t b) {
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
};

// Everything an iteration's launches depend on; a captured iteration is
// replayed only while all of it is unchanged.
struct IterKey {
  const void *p[22];
  size_t n[4];
  int k[4];
  float kr;
  double E;  // graph unions: the tolerance the per-graph stop test uses
  bool operator==(const IterKey &o) const {
    return !std::memcmp(p, o.p, sizeof(p)) && !std::memcmp(n, o.n, sizeof(n)) && !std::memcmp(k, o.k, sizeof(k)) &&
           kr == o.kr && E == o.E;
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
  DBuf<float> ct;
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
  return t;
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
  // side streams for the degree-bin kernels of one colour class, which run
  // concurrently (fork/join with events)
  cudaStream_t aux[4] = {};
  cudaEvent_t fork_ev = nullptr, join_ev[4] = {};
  // result copies that overlap the run (host-array entry points)
  cudaStream_t copy_stream = nullptr;
  ~lvg_graph() {
    if (copy_stream) cudaStreamDestroy(copy_stream);
    if (iter_exec) cudaGraphExecDestroy(iter_exec);
    for (auto &a : aux)
      if (a) cudaStreamDestroy(a);
    if (fork_ev) cudaEventDestroy(fork_ev);
    for (auto &e : join_ev)
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
  DBuf<float> vt, ct;
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
namespace {

int fail(int code, const std::string &msg) {
  g_err = msg;
  return code;
}

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

void ensure_ws(lvg_graph *g) {
  if (!g->ws) {
    g->ws = std::make_unique<Workspace>();
    g->ws->allocate(g->base.span, g->base.edges, g->stream);
  }
}

void read_counters(lvg_graph *g) {
  LVG_CUDA(cudaMemcpyAsync(g->hctr.p, g->ctr.p, sizeof(Counters), cudaMemcpyDeviceToHost, g->stream));
  LVG_CUDA(cudaStreamSynchronize(g->stream));
  if (g->hctr.p->err) {
    unsigned e = g->hctr.p->err;
    LVG_CUDA(cudaMemsetAsync(&g->ctr.p->err, 0, sizeof(unsigned), g->stream));
    if (e & ERR_BAD_ID) throw Error(LVG_EINVAL, "prior membership id >= span");
    throw Error(LVG_ETIMEOUT, "device hash table overflow guard tripped (err=" + std::to_string(e) + ")");
  }
}

void compute_bins(lvg_graph *g, Level &lv, const uint32_t *deg, uint32_t *list, uint32_t *scratch, int colors) {
  g->hbins.ensure(bin_host_elems(MAX_COLORS));
  lv.colors = colors;
  bin_items_u32(deg, lv.ex, lv.span, colors, list, lv.bin_start, lv.bin_maxdeg, scratch, g->hbins.p, g->stream,
                lv.gid, lv.gbase);
  lv.bins = list;
}

// Chunked work of degree bin 11 (see HubPlan): hubs in colour order, each
// hub's edges cut into chunks of the graph's hub_chunk edges, each with a
// partial region of the chunk's size. Built on the host from the hubs'
// degrees (synchronises).
void build_hub_plan(lvg_graph *g, Level &lv, HubPlanBuffers &hb) {
  cudaStream_t s = g->stream;
  HubPlan &P = lv.hub;
  P = HubPlan{};
  const int K = lv.colors;
  size_t H = 0;
  for (int k = 0; k < K; ++k) {
    P.hub_begin[k] = H;
    H += lv.bucket_size(k, NUM_BINS - 1);
  }
  P.hub_begin[K] = H;
  P.hubs = H;
  if (!H) return;
  hb.hub_vertex.ensure(H);
  hb.degs.ensure(H);
  for (int k = 0; k < K; ++k) {
    const size_t n = lv.bucket_size(k, NUM_BINS - 1);
    if (n)
      LVG_CUDA(cudaMemcpyAsync(hb.hub_vertex.p + P.hub_begin[k], lv.bins + lv.bucket_begin(k, NUM_BINS - 1),
                               n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
  }
  launch_gather_u32(hb.hub_vertex.p, H, lv.deg, hb.degs.p, s);
  std::vector<uint32_t> degs(H), verts(H), first(H + 1);
  LVG_CUDA(cudaMemcpyAsync(degs.data(), hb.degs.p, H * 4, cudaMemcpyDeviceToHost, s));
  LVG_CUDA(cudaMemcpyAsync(verts.data(), hb.hub_vertex.p, H * 4, cudaMemcpyDeviceToHost, s));
  LVG_CUDA(cudaStreamSynchronize(s));
  std::vector<uint4> chunks;
  std::vector<uint64_t> parts;
  uint64_t part = 0;
  for (int k = 0; k < K; ++k) {
    P.chunk_begin[k] = chunks.size();
    for (size_t h = P.hub_begin[k]; h < P.hub_begin[k + 1]; ++h) {
      first[h] = uint32_t(chunks.size());
      const uint32_t step = g->tuning.hub_chunk;
      for (uint32_t lo = 0; lo < degs[h]; lo += step) {
        chunks.push_back(make_uint4(uint32_t(h), lo, std::min<uint32_t>(degs[h], lo + step), verts[h]));
        parts.push_back(part + lo);
      }
      part += degs[h];
    }
  }
  P.chunk_begin[K] = chunks.size();
  first[H] = uint32_t(chunks.size());
  P.chunks = chunks.size();
  P.part = part;
  hb.hub_first.ensure(H + 1);
  hb.chunk.ensure(chunks.size());
  hb.chunk_part.ensure(chunks.size());
  LVG_CUDA(cudaMemcpyAsync(hb.hub_first.p, first.data(), (H + 1) * 4, cudaMemcpyHostToDevice, s));
  LVG_CUDA(cudaMemcpyAsync(hb.chunk.p, chunks.data(), chunks.size() * sizeof(uint4), cudaMemcpyHostToDevice, s));
  LVG_CUDA(cudaMemcpyAsync(hb.chunk_part.p, parts.data(), parts.size() * 8, cudaMemcpyHostToDevice, s));
  LVG_CUDA(cudaStreamSynchronize(s));
  P.hub_vertex = hb.hub_vertex.p;
  P.hub_first = hb.hub_first.p;
  P.chunk = hb.chunk.p;
  P.chunk_part = hb.chunk_part.p;
}

// Colour classes of a run: the options' count, else 16 (deterministic), else
// the graph's tuned count for the frontier methods on batches of at most
// frontier_max_fraction entries per edge, else 8.
int colors_for(const lvg_options &o, int method, const lvg_tuning &t, size_t batch_entries = 0,
               size_t edges = 0) {
  int k = o.colors;
  if (k <= 0) {
    const bool small = double(batch_entries) <= t.frontier_max_fraction * double(edges);
    if (o.deterministic) k = DEFAULT_COLORS_SYNC;
    else if ((method == LVG_METHOD_FRONTIER || method == LVG_METHOD_DELTA) && small) k = t.frontier_colors;
    else k = DEFAULT_COLORS_ASYNC;
  }
  return k < 1 ? 1 : (k > MAX_COLORS ? MAX_COLORS : k);
}

void ensure_global_tables(Workspace &W, size_t blocks, int log2cap, bool first_too) {
  size_t need = blocks * (size_t(1) << log2cap);
  W.gkeys.ensure(need);
  W.gvals.ensure(need);
  if (first_too) W.gfirst.ensure(need);
}

// ---------------------------------------------------------------- local moving

// Launch one local-moving iteration: every colour class in order; within a
// class the worklist compaction, then one kernel per degree bin (two for the
// chunked hubs); in deterministic mode the class's decisions are applied and
// its marks merged before the next class. The device gain sum is reset first.
// With bin_ev, events bracket each bin launch (profiling).
void ensure_aux(lvg_graph *g) {
  if (g->aux[0]) return;
  for (auto &a : g->aux) LVG_CUDA(cudaStreamCreateWithFlags(&a, cudaStreamNonBlocking));
  LVG_CUDA(cudaEventCreateWithFlags(&g->fork_ev, cudaEventDisableTiming));
  for (auto &e : g->join_ev) LVG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
}

// The stream of degree bin b within a colour class: the small bins on two
// side streams, bins 9 and 10 on two more, the hubs on the main stream.
int bin_stream(int b) { return b <= 4 ? 0 : b <= 8 ? 1 : b == 9 ? 2 : b == 10 ? 3 : -1; }

void enqueue_iteration(lvg_graph *g, const Level &lv, uint32_t *com, float *ctot, const float *tot,
                       const uint8_t *fa, float kr, bool sync, int fused, const int *glog2, const size_t *goff,
                       size_t need, std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> *bin_ev,
                       const UnionCall *uc) {
  auto set_union = [&](MoveArgs &a) {
    if (!uc) return;
    a.gid = lv.gid; a.gkr = uc->kr; a.gzero = lv.gbase; a.gfix = uc->fix; a.gact = uc->gact;
  };
  Workspace &W = *g->ws;
  cudaStream_t s = g->stream;
  const int K = lv.colors;
  // The bins of one class are independent (different vertices; the class's
  // reads of other vertices' communities race in asynchronous mode exactly as
  // the reference's threads do, and in deterministic mode nothing they read
  // changes before the class's moves are applied), so they run concurrently.
  // Per-bin profiling keeps them on one stream to time each launch.
  const bool conc = bin_ev == nullptr && g->tuning.concurrent_bins;
  if (conc) ensure_aux(g);
  auto stream_of = [&](int b) { const int i = bin_stream(b); return conc && i >= 0 ? g->aux[i] : s; };
  LVG_CUDA(cudaMemsetAsync(&g->ctr.p->el_fix, 0, sizeof(unsigned long long), s));
  LVG_CUDA(cudaMemsetAsync(W.wl_count.p, 0, size_t(K) * NUM_BINS * sizeof(uint32_t), s));
  for (int k = 0; k < K; ++k) {
    // this class's active vertices of bins 1..NUM_BINS-2 -> worklists
    BinBounds bb;
    for (int b = 0; b <= NUM_BINS; ++b) bb.start[b] = lv.bin_start[k * NUM_BINS + b];
    uint32_t *wlc = W.wl_count.p + size_t(k) * NUM_BINS;
    if (bb.start[NUM_BINS - 1] > bb.start[1])
      launch_compact_active(lv.bins, bb, W.vaff.p, fa, W.wl.p, wlc, s, uc ? lv.gid : nullptr, uc ? uc->gact : nullptr);
    if (conc) {  // fork
      LVG_CUDA(cudaEventRecord(g->fork_ev, s));
      for (auto a : g->aux) LVG_CUDA(cudaStreamWaitEvent(a, g->fork_ev, 0));
    }
    if (fused) {
      // bins 1-6 and 7-8 in one launch each; each bin gets blocks for its
      // bucket, at most `fused` per SM (few where the worklists are short)
      static const int tpb[NUM_BINS] = {0, 64, 32, 16, 8, 8, 8, 8, 8, 0, 0, 0};
      const size_t cap = size_t(device_sms()) * size_t(fused);
      for (const auto &grp : {std::pair<int, int>{1, 6}, std::pair<int, int>{7, 8}}) {
        SmallBins sb{};
        uint32_t nb = 0;
        for (int b = grp.first; b <= grp.second; ++b) {
          const int j = b - grp.first;
          const size_t cnt = lv.bucket_size(k, b);
          sb.list[j] = W.wl.p + lv.bucket_begin(k, b);
          sb.count_ptr[j] = wlc + b;
          sb.block_begin[j] = nb;
          nb += uint32_t(std::min(cap, (cnt + tpb[b] - 1) / tpb[b]));
        }
        sb.block_begin[grp.second - grp.first + 1] = nb;
        if (!nb) continue;
        MoveArgs a;
        a.off = lv.off; a.deg = lv.deg; a.key = lv.key; a.w = lv.w;
        a.vcom = com; a.ctot = ctot; a.dec = W.dec.p;
        a.vaff = W.vaff.p; a.mark = W.mark.p; a.fa = fa; a.vtot = tot;
        a.kr = kr; a.ctr = g->ctr.p; a.bin = grp.first;
        set_union(a);
        cudaEvent_t b0 = bin_ev ? g->events.record(s) : nullptr;
        launch_move_small(grp.first, grp.second, sync, a, sb, stream_of(grp.first));
        if (bin_ev) bin_ev->push_back({grp.first, {b0, g->events.record(s)}});
        ++g->stats.move_launches;
      }
    }
    for (int b = fused ? 9 : 1; b < NUM_BINS; ++b) {
      const size_t cnt = lv.bucket_size(k, b);
      if (!cnt) continue;
      MoveArgs a;
      a.off = lv.off; a.deg = lv.deg; a.key = lv.key; a.w = lv.w;
      a.list = (b == NUM_BINS - 1 ? lv.bins : W.wl.p) + lv.bucket_begin(k, b);
      a.count = uint32_t(cnt);
      a.count_ptr = b == NUM_BINS - 1 ? nullptr : wlc + b;
      a.vcom = com; a.ctot = ctot; a.dec = W.dec.p;
      a.vaff = W.vaff.p; a.mark = W.mark.p; a.fa = fa; a.vtot = tot;
      a.kr = kr; a.ctr = g->ctr.p; a.bin = b;
      a.gkeys = need ? W.gkeys.p + goff[b] : nullptr;
      a.gvals = need ? W.gvals.p + goff[b] : nullptr;
      a.glog2 = glog2[b];
      a.big_cap = g->tuning.big_blocks_per_sm;
      set_union(a);
      cudaEvent_t b0 = bin_ev ? g->events.record(s) : nullptr;
      if (b == NUM_BINS - 1) {
        a.hub = lv.hub;
        a.color = k;
        a.chunk_cnt = W.chunk_cnt.p;
        a.part_key = W.part_key.p;
        a.part_val = W.part_val.p;
        a.hub_kd = W.hub_kd.p;
        launch_move_hubs(sync, a, s);
      } else {
        launch_move_bin(b, sync, a, stream_of(b));
      }
      if (bin_ev) bin_ev->push_back({b, {b0, g->events.record(s)}});
      ++g->stats.move_launches;
    }
    if (conc) {  // join
      for (int i = 0; i < 4; ++i) {
        LVG_CUDA(cudaEventRecord(g->join_ev[i], g->aux[i]));
        LVG_CUDA(cudaStreamWaitEvent(s, g->join_ev[i], 0));
      }
    }
    if (sync) {
      launch_apply_moves(lv.bins + lv.color_begin(k), lv.color_end(k) - lv.color_begin(k), W.dec.p, com, ctot, tot, s);
      launch_merge_marks(W.vaff.p, W.mark.p, lv.span, s);
    }
  }
  if (uc) launch_iter_control(uc->n, uc->ctl, uc->gact, uc->fix, uc->M, uc->E, uc->L, g->ctr.p, s);
  LVG_CUDA(cudaMemcpyAsync(g->hctr.p, g->ctr.p, sizeof(Counters), cudaMemcpyDeviceToHost, s));
}

// Capture one iteration of the uploaded level into a CUDA graph (after an
// eager iteration, so every kernel's attributes are already set). A capture
// failure disables graphs for this handle; the eager path stays correct.
void capture_iteration(lvg_graph *g, const Level &lv, uint32_t *com, float *ctot, const float *tot,
                       const uint8_t *fa, float kr, bool sync, int fused, const int *glog2, const size_t *goff,
                       size_t need, const IterKey &key, const UnionCall *uc) {
  cudaStream_t s = g->stream;
  if (g->iter_exec) {
    cudaGraphExecDestroy(g->iter_exec);
    g->iter_exec = nullptr;
  }
  const unsigned long long l0 = launch_counter();
  const unsigned long long m0 = g->stats.move_launches;
  cudaGraph_t graph = nullptr;
  if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    g->no_graphs = true;
    return;
  }
  bool fine = true;
  try {
    enqueue_iteration(g, lv, com, ctot, tot, fa, kr, sync, fused, glog2, goff, need, nullptr, uc);
  } catch (const Error &) {
    fine = false;
  }
  const cudaError_t e = cudaStreamEndCapture(s, &graph);
  g->iter_nodes = launch_counter() - l0;
  g->iter_moves = g->stats.move_launches - m0;
  launch_counter() = l0;
  g->stats.move_launches = m0;
  if (!fine || e != cudaSuccess || !graph || cudaGraphInstantiate(&g->iter_exec, graph, 0) != cudaSuccess) {
    cudaGetLastError();
    if (graph) cudaGraphDestroy(graph);
    g->iter_exec = nullptr;
    g->no_graphs = true;
    return;
  }
  cudaGraphDestroy(graph);
  g->iter_key = key;
}

// louvainMoveOmpW (inc/louvain.hxx:588-609). Returns the iteration count, 0
// if the first iteration found nothing to gain. Each iteration sweeps the
// colour classes in order (enqueue_iteration). For the uploaded level the
// iteration is captured once into a CUDA graph and replayed, one graph
// launch per iteration instead of ~12 launches per colour class.
int move_phase(lvg_graph *g, const Level &lv, uint32_t *com, float *ctot, const float *tot, const uint8_t *fa,
               double M, float kr, int L, double E, bool sync, int fused, const UnionCall *uc = nullptr,
               const DBatch *endpoints = nullptr) {
  Workspace &W = *g->ws;
  cudaStream_t s = g->stream;
  const int K = lv.colors;
  // Existing degree-0 vertices are processed once and never re-marked. In
  // the dynamic-frontier first pass only batch endpoints can be such
  // vertices with their flag set (`endpoints`).
  if (endpoints) {
    launch_clear_isolated_endpoints(endpoints->ds, endpoints->nd, endpoints->is, endpoints->ni, lv.deg, lv.ex,
                                    W.vaff.p, s);
  } else {
    IsolatedLists iso{};
    iso.k = K;
    for (int k = 0; k < K; ++k) {
      iso.list[k] = lv.bins + lv.bucket_begin(k, 0);
      iso.n[k] = lv.bucket_size(k, 0);
    }
    launch_clear_isolated_multi(iso, W.vaff.p, fa, s);
  }
  // Global fallback regions of the large-degree bins (9-11): each launch's
  // blocks get 2^glog2[b] slots, enough for the bin's largest degree.
  int glog2[NUM_BINS] = {};
  size_t goff[NUM_BINS] = {};
  size_t need = 0;
  for (int b = 9; b < NUM_BINS; ++b) {
    size_t most = 0;
    for (int k = 0; k < K; ++k) most = std::max(most, lv.bucket_size(k, b));
    if (!most) continue;
    glog2[b] = global_table_log2(lv.bin_maxdeg[b]);
    goff[b] = need;  // each bin its own regions: the bins' kernels run concurrently
    need += size_t(move_grid_blocks(b, sync, most, g->tuning.big_blocks_per_sm)) << glog2[b];
  }
  if (need) {
    W.gkeys.ensure(need);
    W.gvals.ensure(need);
  }
  if (lv.hub.hubs) {
    W.chunk_cnt.ensure(lv.hub.chunks);
    W.part_key.ensure(lv.hub.part);
    W.part_val.ensure(lv.hub.part);
  }
  const bool base = lv.off == g->base.off;
  IterKey key{};
  if (base) {
    const void *ps[22] = {lv.off, lv.bins, com, ctot, tot, fa, W.vaff.p, W.mark.p, W.dec.p, W.wl.p, W.wl_count.p,
                          W.gkeys.p, W.gvals.p, W.chunk_cnt.p, W.part_key.p, W.part_val.p, W.hub_kd.p, g->ctr.p,
                          g->hctr.p, lv.hub.chunk, lv.hub.hub_vertex, lv.gid};
    std::memcpy(key.p, ps, sizeof(ps));
    key.n[0] = lv.span; key.n[1] = need; key.n[2] = lv.hub.chunks; key.n[3] = lv.bin_start[K * NUM_BINS];
    key.k[0] = K; key.k[1] = sync; key.k[2] = glog2[9] | glog2[10] << 8 | glog2[11] << 16; key.k[3] = fused;
    key.kr = kr;
    key.E = uc ? E : 0.0;
  }
  const bool graphs = base && !g->profiling && !g->no_graphs;
  int l = 0;
  double el = 0;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> bin_ev;
  while (l < L) {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    const bool replay = graphs && g->iter_exec && g->iter_key == key;
    if (replay) {
      LVG_CUDA(cudaGraphLaunch(g->iter_exec, s));
      launch_counter() += g->iter_nodes;
      g->stats.move_launches += g->iter_moves;
    } else {
      bin_ev.clear();
      if (g->profiling) e0 = g->events.record(s);
      enqueue_iteration(g, lv, com, ctot, tot, fa, kr, sync, fused, glog2, goff, need,
                        g->profiling ? &bin_ev : nullptr, uc);
      if (g->profiling) e1 = g->events.record(s);
    }
    LVG_CUDA(cudaStreamSynchronize(s));
    if (g->hctr.p->err) read_counters(g);  // raises the device error
    if (g->profiling) {
      g->stats.move_kernel_ms += elapsed(e0, e1);
      for (auto &be : bin_ev) g->stats.move_bin_ms[be.first] += elapsed(be.second.first, be.second.second);
    }
    if (graphs && !replay)
      capture_iteration(g, lv, com, ctot, tot, fa, kr, sync, fused, glog2, goff, need, key, uc);
    ++l;
    if (uc) {  // each graph ran its own stop test (iter_control_kernel)
      if (g->hctr.p->gactive == 0) break;
      continue;
    }
    el = double(g->hctr.p->el_fix) / GAIN_FIX / M;
    if (el <= E) break;
  }
  return (l > 1 || el != 0) ? l : 0;
}

// ---------------------------------------------------------------- aggregation

// Renumbered membership `com` of level `lv` with CN communities -> next level
// in buffer set `which` (louvainCommunityVerticesOmpW + louvainAggregateOmpW,
// inc/louvain.hxx:1197-1203). Also writes the new level's vertex weights.
Level aggregate(lvg_graph *g, const Level &lv, const uint32_t *com, size_t CN, int which, int colors,
                const uint32_t *ngid = nullptr, const uint32_t *ngbase = nullptr) {
  Workspace &W = *g->ws;
  cudaStream_t s = g->stream;
  LevelBuffers &nb = W.lv[which];
  Level nl;
  nl.span = nl.order = CN;
  nl.off = nb.off.p; nl.deg = nb.deg.p; nl.key = nb.key.p; nl.w = nb.w.p; nl.ex = nullptr;
  nl.gid = ngid; nl.gbase = ngbase;
  // Community -> members CSR and row capacities.
  LVG_CUDA(cudaMemsetAsync(W.csize.p, 0, (CN + 1) * sizeof(uint32_t), s));
  LVG_CUDA(cudaMemsetAsync(W.ccur.p, 0, (CN + 1) * sizeof(uint32_t), s));
  LVG_CUDA(cudaMemsetAsync(nl.off, 0, (CN + 1) * sizeof(uint64_t), s));
  launch_community_sizes(lv, com, W.csize.p, nl.off, s);
  size_t cb[NUM_BINS + 1];
  uint64_t cmax[NUM_BINS];
  g->hbins.ensure(bin_host_elems(MAX_COLORS));
  bin_items_u64(nl.off, nullptr, CN, 1, W.cbins.p, cb, cmax, W.binscratch.p, g->hbins.p, s);
  exclusive_scan_u32(W.csize.p, W.csize.p, CN, W.csize.p + CN, W.scan32.p, s);
  exclusive_scan_u64(nl.off, nl.off, CN, nl.off + CN, W.scan64.p, s);
  launch_community_scatter(lv, com, W.csize.p, W.ccur.p, W.cmem.p, s);
  // Empty communities never reach a kernel: zero their rows and weights first.
  LVG_CUDA(cudaMemsetAsync(nl.deg, 0, CN * sizeof(uint32_t), s));
  LVG_CUDA(cudaMemsetAsync(W.vtot.p, 0, CN * sizeof(float), s));
  // Global fallback regions of bins 9-10 (bin 11 is chunked below).
  int glog2[NUM_BINS] = {};
  size_t need = 0;
  for (int b = 9; b < NUM_BINS - 1; ++b) {
    const size_t cnt = cb[b + 1] - cb[b];
    if (!cnt) continue;
    glog2[b] = global_table_log2(std::min<uint64_t>(cmax[b], CN));
    need = std::max(need, size_t(global_table_blocks(cnt)) << glog2[b]);
  }
  if (need) {
    W.gkeys.ensure(need);
    W.gvals.ensure(need);
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (g->profiling) e0 = g->events.record(s);
  for (int b = 1; b < NUM_BINS - 1; ++b) {
    const size_t cnt = cb[b + 1] - cb[b];
    if (!cnt) continue;
    AggArgs a;
    a.off = lv.off; a.deg = lv.deg; a.key = lv.key; a.w = lv.w;
    a.vcom = com; a.coff = W.csize.p; a.cmem = W.cmem.p;
    a.list = W.cbins.p + cb[b];
    a.count = uint32_t(cnt);
    a.yoff = nl.off; a.ydeg = nl.deg; a.ykey = nl.key; a.yw = nl.w;
    a.vtot = W.vtot.p; a.ctr = g->ctr.p; a.cn = uint32_t(CN);
    a.gkeys = need ? W.gkeys.p : nullptr; a.gvals = need ? W.gvals.p : nullptr; a.glog2 = glog2[b];
    launch_aggregate_bin(b, a, s);
    ++g->stats.aggregate_launches;
  }
  // communities above total degree 8192: chunks of AGG_CHUNK edges over many
  // blocks, merged in per-community tables in HBM
  if (const size_t n11 = cb[NUM_BINS] - cb[NUM_BINS - 1]) {
    const uint32_t *list = W.cbins.p + cb[NUM_BINS - 1];
    uint32_t members = 0;
    LVG_CUDA(cudaMemcpyAsync(&members, W.csize.p + CN, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    W.agg_tdeg.ensure(n11);
    launch_comm_tdeg(list, n11, nl.off, W.agg_tdeg.p, s);
    std::vector<uint64_t> tdeg(n11);
    LVG_CUDA(cudaMemcpyAsync(tdeg.data(), W.agg_tdeg.p, n11 * 8, cudaMemcpyDeviceToHost, s));
    LVG_CUDA(cudaStreamSynchronize(s));
    W.mpre.ensure(size_t(members) + 1);
    launch_member_degrees(W.cmem.p, lv.deg, members, W.mpre.p, s);
    exclusive_scan_u64(W.mpre.p, W.mpre.p, members, W.mpre.p + members, W.scan64.p, s);
    std::vector<uint2> chunks;
    std::vector<uint64_t> toff(n11 + 1, 0);
    std::vector<int> tlog(n11);
    for (size_t j = 0; j < n11; ++j) {
      const uint64_t want = 2 * std::min<uint64_t>(tdeg[j], CN);
      int lg = 1;
      while ((uint64_t(1) << lg) < want) ++lg;
      tlog[j] = lg;
      toff[j + 1] = toff[j] + (uint64_t(1) << lg);
      for (uint64_t k = 0; k * AGG_CHUNK < tdeg[j]; ++k) chunks.push_back(make_uint2(uint32_t(j), uint32_t(k)));
    }
    const uint64_t slots = toff[n11];
    W.agg_chunk.ensure(chunks.size());
    W.agg_toff.ensure(n11 + 1);
    W.agg_tlog.ensure(n11);
    W.agg_gk.ensure(slots);
    W.agg_gv.ensure(slots);
    LVG_CUDA(cudaMemcpyAsync(W.agg_chunk.p, chunks.data(), chunks.size() * sizeof(uint2), cudaMemcpyHostToDevice, s));
    LVG_CUDA(cudaMemcpyAsync(W.agg_toff.p, toff.data(), (n11 + 1) * 8, cudaMemcpyHostToDevice, s));
    LVG_CUDA(cudaMemcpyAsync(W.agg_tlog.p, tlog.data(), n11 * sizeof(int), cudaMemcpyHostToDevice, s));
    LVG_CUDA(cudaMemsetAsync(W.agg_gk.p, 0xFF, slots * 4, s));
    LVG_CUDA(cudaMemsetAsync(W.agg_gv.p, 0, slots * 4, s));
    AggArgs a;
    a.off = lv.off; a.deg = lv.deg; a.key = lv.key; a.w = lv.w;
    a.vcom = com; a.coff = W.csize.p; a.cmem = W.cmem.p;
    a.list = list;
    a.count = uint32_t(n11);
    a.yoff = nl.off; a.ydeg = nl.deg; a.ykey = nl.key; a.yw = nl.w;
    a.vtot = W.vtot.p; a.ctr = g->ctr.p; a.cn = uint32_t(CN);
    a.gkeys = nullptr; a.gvals = nullptr; a.glog2 = 0;
    AggChunks ch{W.agg_chunk.p, list, W.agg_toff.p, W.agg_tlog.p, W.mpre.p, W.agg_gk.p, W.agg_gv.p, uint32_t(n11)};
    launch_aggregate_chunks(a, ch, chunks.size(), slots, s);
    g->stats.aggregate_launches += 2;
    LVG_CUDA(cudaStreamSynchronize(s));  // the host vectors above are freed next
  }
  if (g->profiling) {
    e1 = g->events.record(s);
  }
  compute_bins(g, nl, nl.deg, nb.bins.p, W.binscratch.p, colors);  // synchronises
  build_hub_plan(g, nl, nb.hubplan);
  if (g->profiling) g->stats.aggregate_kernel_ms += elapsed(e0, e1);
  return nl;
}

// ---------------------------------------------------------------- driver

struct StateRef {
  uint32_t *q;
  float *vt, *ct;
};

// One call of a method. prior: device FP32 prior state (dynamic methods);
// out: where the first level's membership/weights and final totals live.
// on_init (optional) is called once, in the last repetition, with an event
// recorded when the first level's vertex weights (out.vt) are final.
void run(lvg_graph *g, int method, const DBatch &b, StateRef prior, StateRef out, const lvg_options &o,
         RunInfo &info, const std::function<void(cudaEvent_t)> *on_init = nullptr) {
  if (g->uni) throw Error(LVG_EINVAL, "graph union: run it with lvg_static_union");
  ensure_ws(g);
  Workspace &W = *g->ws;
  cudaStream_t s = g->stream;
  const size_t S = g->base.span;
  const double M = g->total_weight / 2;
  const double R = o.resolution;
  const float kr = M > 0 ? float(R / (2.0 * M)) : 0.f;
  const int L = o.maxIterations, P = o.maxPasses;
  const bool sync = o.deterministic != 0;
  const int rep = std::max(1, o.repeat);
  const int K = colors_for(o, method, g->tuning, b.nd + b.ni, g->base.edges);
  if (g->base.colors != K) {
    compute_bins(g, g->base, g->deg.p, g->bins.p, W.binscratch.p, K);
    build_hub_plan(g, g->base, g->hubplan);
  }
  uint32_t *ucom = out.q;
  float *utot = out.vt, *ctot = out.ct;
  g->stats = lvg_stats{};
  const unsigned long long launches0 = launch_counter();
  LVG_CUDA(cudaMemsetAsync(g->ctr.p, 0, sizeof(Counters), s));
  int l = 0, p = 0;
  for (int r = 0; r < rep; ++r) {
    g->events.reset();
    // Reset buffers, as the reference does before each repetition.
    LVG_CUDA(cudaMemsetAsync(W.vaff.p, 0, S, s));
    LVG_CUDA(cudaMemsetAsync(W.vcom.p, 0, S * sizeof(uint32_t), s));
    LVG_CUDA(cudaMemsetAsync(W.vtot.p, 0, S * sizeof(float), s));
    cudaEvent_t e0 = g->events.record(s);
    // fi: initial membership and weights.
    if (method == LVG_METHOD_STATIC) {
      launch_init_static(g->base, ucom, utot, ctot, s);
    } else {
      if (prior.q != ucom) LVG_CUDA(cudaMemcpyAsync(ucom, prior.q, S * 4, cudaMemcpyDeviceToDevice, s));
      if (prior.vt != utot) LVG_CUDA(cudaMemcpyAsync(utot, prior.vt, S * 4, cudaMemcpyDeviceToDevice, s));
      if (prior.ct != ctot) LVG_CUDA(cudaMemcpyAsync(ctot, prior.ct, S * 4, cudaMemcpyDeviceToDevice, s));
      launch_batch_weights(b.ds, b.dw, b.nd, -1.f, ucom, utot, ctot, s);
      launch_batch_weights(b.is, b.iw, b.ni, +1.f, ucom, utot, ctot, s);
    }
    cudaEvent_t e1 = g->events.record(s);
    if (on_init && r == rep - 1) (*on_init)(e1);
    // fm: mark affected vertices.
    const uint8_t *fa = nullptr;
    if (method == LVG_METHOD_STATIC || method == LVG_METHOD_NAIVE) {
      LVG_CUDA(cudaMemsetAsync(W.vaff.p, 1, S, s));
    } else if (method == LVG_METHOD_FRONTIER) {
      launch_df_mark(b.ds, b.dd, b.nd, b.is, b.id, b.ni, ucom, W.vaff.p, s);
    } else {
      LVG_CUDA(cudaMemsetAsync(W.fv.p, 0, S, s));
      LVG_CUDA(cudaMemsetAsync(W.fn.p, 0, S, s));
      LVG_CUDA(cudaMemsetAsync(W.fc.p, 0, S, s));
      int dlog = 1;
      if (b.max_group * 2 > 2048) {
        dlog = global_table_log2(b.max_group);
        ensure_global_tables(W, size_t(global_table_blocks(b.ni)), dlog, true);
      }
      launch_ds_mark(g->base, b.ds, b.dd, b.nd, b.is, b.id, b.iw, b.ni, b.seg, b.ni, ucom, utot, ctot, M, R,
                     W.fv.p, W.fn.p, W.fc.p, W.gkeys.p, W.gvals.p, W.gfirst.p, dlog, g->ctr.p, W.wl.p,
                     W.wl_count.p, W.cext.p, W.scan32.p, s);
      LVG_CUDA(cudaMemcpyAsync(W.vaff.p, W.fv.p, S, cudaMemcpyDeviceToDevice, s));
      fa = W.fv.p;
    }
    cudaEvent_t e2 = g->events.record(s);
    cudaEvent_t ep1 = nullptr;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> tl_ev, ta_ev;
    double E = o.tolerance;
    Level lv = g->base;
    uint32_t *com = ucom;
    const float *tot = utot;
    int which = 0;
    for (l = 0, p = 0; M > 0 && P > 0;) {
      if (p == 1) ep1 = g->events.record(s);
      const bool first = p == 0;
      cudaEvent_t a0 = g->events.record(s);
      // the frontier methods' first pass: the small degree bins go in two
      // fused launches per class, with blocks per SM and bin for DF's short
      // worklists (2) or for delta-screening's whole communities (8: with
      // two, its first pass took 2.8x as long on a 4M-vertex graph of
      // average degree 87)
      const int fused = !first || !g->tuning.fused_small ? 0
                        : method == LVG_METHOD_FRONTIER  ? 2
                        : method == LVG_METHOD_DELTA     ? 8
                                                         : 0;
      const int m = move_phase(g, lv, com, ctot, tot, first ? fa : nullptr, M, kr, L, E, sync, fused, nullptr,
                               first && method == LVG_METHOD_FRONTIER ? &b : nullptr);
      tl_ev.push_back({a0, g->events.record(s)});
      l += std::max(m, 1);
      ++p;
      if (m <= 1 || p >= P) break;
      const size_t GN = first ? g->base.order : lv.span;
      LVG_CUDA(cudaMemsetAsync(W.cext.p, 0, (lv.span + 1) * sizeof(uint32_t), s));
      launch_community_flags(lv, com, W.cext.p, s);
      exclusive_scan_u32(W.cext.p, W.cext.p, lv.span, &g->ctr.p->cn, W.scan32.p, s);
      read_counters(g);
      const size_t CN = g->hctr.p->cn;
      if (double(CN) / double(GN) >= o.aggregationTolerance) break;
      launch_lookup(com, W.cext.p, S, s);
      if (!first) launch_lookup(ucom, W.vcom.p, S, s);
      cudaEvent_t g0 = g->events.record(s);
      lv = aggregate(g, lv, com, CN, which, K);
      ta_ev.push_back({g0, g->events.record(s)});
      which ^= 1;
      com = W.vcom.p;
      tot = W.vtot.p;
      launch_level_init(CN, W.vtot.p, W.vcom.p, ctot, W.vaff.p, s);
      E /= o.toleranceDrop;
    }
    if (p > 1) launch_lookup(ucom, W.vcom.p, S, s);
    cudaEvent_t eend = g->events.record(s);
    LVG_CUDA(cudaStreamSynchronize(s));
    info.ti += elapsed(e0, e1);
    info.tm += elapsed(e1, e2);
    info.tp += elapsed(e2, ep1 ? ep1 : eend);
    for (auto &pr : tl_ev) info.tl += elapsed(pr.first, pr.second);
    for (auto &pr : ta_ev) info.ta += elapsed(pr.first, pr.second);
    info.t += elapsed(e0, eend);
  }
  launch_count_flags(W.vaff.p, S, g->ctr.p, s);
  read_counters(g);
  info.affected = g->hctr.p->affected;
  info.iterations = l;
  info.passes = p;
  info.t /= rep; info.tm /= rep; info.ti /= rep; info.tp /= rep; info.tl /= rep; info.ta /= rep;
  g->stats.move_vertices = g->hctr.p->vertices;
  g->stats.move_edges = g->hctr.p->edges;
  g->stats.moves = g->hctr.p->moves;
  g->stats.aggregate_edges = g->hctr.p->agg_edges;
  for (int b = 0; b < NUM_BINS; ++b) {
    g->stats.move_bin_vertices[b] = g->hctr.p->bin_vertices[b];
    g->stats.move_bin_edges[b] = g->hctr.p->bin_edges[b];
    g->stats.move_bin_overflow[b] = g->hctr.p->bin_over[b];
  }
  g->stats.hub_chunk_overflow = g->hctr.p->hub_chunk_over;
  g->stats.kernel_launches = launch_counter() - launches0;
}

// Static Louvain on a graph union: one run over all graphs, each graph
// keeping the reference's pass driver for itself (louvainOmp,
// inc/louvain.hxx:1180-1215) through its GraphCtl entry: its own M and
// R/(2M), colour classes by its own vertex ids, its own iteration stop test,
// aggregation test and pass count. A graph that finishes leaves the union:
// its membership, Σtot and affected flags are final at that point and it
// takes no ids on the next level. The launches are those of one graph; what
// differs is that a class's worklists hold the vertices of every graph still
// moving.
void run_union(lvg_graph *g, const lvg_options &o, RunInfo &info) {
  ensure_ws(g);
  Workspace &W = *g->ws;
  UnionInfo &U = *g->uni;
  cudaStream_t s = g->stream;
  const size_t S = g->base.span, n = U.n;
  const double R = o.resolution;
  const int L = o.maxIterations, P = o.maxPasses;
  const bool sync = o.deterministic != 0;
  const int rep = std::max(1, o.repeat);
  const int K = colors_for(o, LVG_METHOD_STATIC, g->tuning);
  if (g->base.colors != K) {
    compute_bins(g, g->base, g->deg.p, g->bins.p, W.binscratch.p, K);
    build_hub_plan(g, g->base, g->hubplan);
  }
  {
    std::vector<float> kr(n);
    for (size_t i = 0; i < n; ++i) kr[i] = U.M[i] > 0 ? float(R / (2.0 * U.M[i])) : 0.f;
    U.kr.ensure(n);
    LVG_CUDA(cudaMemcpyAsync(U.kr.p, kr.data(), n * sizeof(float), cudaMemcpyHostToDevice, s));
    LVG_CUDA(cudaStreamSynchronize(s));
  }
  U.fix.ensure(n); U.ctl.ensure(n); U.hctl.ensure(n); U.gact.ensure(n);
  U.gid[0].ensure(S); U.gid[1].ensure(S); U.gbase[0].ensure(n + 1); U.gbase[1].ensure(n + 1);
  U.aggex.ensure(S); U.q.ensure(S); U.ct.ensure(S); U.aff.ensure(S);
  uint32_t *ucom = W.ucom.p;
  float *utot = W.utot.p, *ctot = W.ctot.p;
  g->stats = lvg_stats{};
  const unsigned long long launches0 = launch_counter();
  LVG_CUDA(cudaMemsetAsync(g->ctr.p, 0, sizeof(Counters), s));
  const UnionCall uc0{n, U.kr.p, U.fix.p, U.gact.p, U.ctl.p, U.Md.p, 0.0, L};
  for (int r = 0; r < rep; ++r) {
    g->events.reset();
    LVG_CUDA(cudaMemsetAsync(W.vaff.p, 0, S, s));
    LVG_CUDA(cudaMemsetAsync(W.vcom.p, 0, S * sizeof(uint32_t), s));
    LVG_CUDA(cudaMemsetAsync(W.vtot.p, 0, S * sizeof(float), s));
    LVG_CUDA(cudaMemsetAsync(U.ctl.p, 0, n * sizeof(GraphCtl), s));
    LVG_CUDA(cudaMemsetAsync(U.fix.p, 0, n * sizeof(unsigned long long), s));
    cudaEvent_t e0 = g->events.record(s);
    launch_init_static(g->base, ucom, utot, ctot, s);
    cudaEvent_t e1 = g->events.record(s);
    LVG_CUDA(cudaMemsetAsync(W.vaff.p, 1, S, s));
    cudaEvent_t e2 = g->events.record(s);
    // graphs with M = 0 (or no passes) end as initialised
    launch_pass_skip(n, U.ctl.p, U.Md.p, P, s);
    launch_union_snapshot(S, U.gid0.p, U.vb0.p, U.vb0.p, U.ctl.p, ctot, W.vaff.p, U.ct.p, U.aff.p, s);
    launch_union_finalize(S, U.gid0.p, ucom, nullptr, U.vb0.p, U.ctl.p, U.q.p, s);
    launch_union_mark_done(n, U.ctl.p, s);
    cudaEvent_t ep1 = nullptr;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> tl_ev, ta_ev;
    double E = o.tolerance;
    Level lv = g->base;
    uint32_t *com = ucom;
    const float *tot = utot;
    int which = 0;
    for (int p = 0;; ++p) {
      if (p == 1) ep1 = g->events.record(s);
      const bool first = p == 0;
      launch_pass_begin(n, U.ctl.p, U.gact.p, s);
      UnionCall uc = uc0;
      uc.E = E;
      cudaEvent_t a0 = g->events.record(s);
      move_phase(g, lv, com, ctot, tot, nullptr, 0.0, 0.f, L, E, sync, 0, &uc);
      tl_ev.push_back({a0, g->events.record(s)});
      launch_pass_end(n, U.ctl.p, P, s);
      launch_union_snapshot(lv.span, lv.gid, lv.gbase, U.vb0.p, U.ctl.p, ctot, W.vaff.p, U.ct.p, U.aff.p, s);
      // communities of the graphs that go on; the aggregation test per graph
      LVG_CUDA(cudaMemsetAsync(W.cext.p, 0, (lv.span + 1) * sizeof(uint32_t), s));
      launch_union_flags(lv.ex, lv.span, com, lv.gid, U.ctl.p, W.cext.p, s);
      launch_union_tolerance(n, lv.gbase, W.cext.p, U.ctl.p, U.order.p, first, o.aggregationTolerance, s);
      exclusive_scan_u32(W.cext.p, W.cext.p, lv.span, &g->ctr.p->cn, W.scan32.p, s);
      launch_union_finalize(S, U.gid0.p, ucom, first ? nullptr : com, lv.gbase, U.ctl.p, U.q.p, s);
      launch_union_aggex(lv.ex, lv.span, lv.gid, U.ctl.p, U.aggex.p, s);
      launch_union_mark_done(n, U.ctl.p, s);
      read_counters(g);
      const size_t CN = g->hctr.p->cn;
      if (CN == 0) break;  // every graph is done
      // next level: the remaining graphs' communities, renumbered in order
      uint32_t *ngid = U.gid[which].p, *ngbase = U.gbase[which].p;
      launch_union_bases(n, lv.gbase, lv.span, W.cext.p, &g->ctr.p->cn, ngbase, s);
      launch_fill_gid(ngbase, n, ngid, s);
      launch_lookup(com, W.cext.p, lv.span, s);
      if (!first) launch_union_lookup(ucom, W.vcom.p, S, U.gid0.p, U.ctl.p, s);
      Level am = lv;
      am.ex = U.aggex.p;
      cudaEvent_t g0 = g->events.record(s);
      lv = aggregate(g, am, com, CN, which, K, ngid, ngbase);
      ta_ev.push_back({g0, g->events.record(s)});
      which ^= 1;
      com = W.vcom.p;
      tot = W.vtot.p;
      launch_level_init(CN, W.vtot.p, W.vcom.p, ctot, W.vaff.p, s);
      E /= o.toleranceDrop;
    }
    cudaEvent_t eend = g->events.record(s);
    LVG_CUDA(cudaStreamSynchronize(s));
    info.ti += elapsed(e0, e1);
    info.tm += elapsed(e1, e2);
    info.tp += elapsed(e2, ep1 ? ep1 : eend);
    for (auto &pr : tl_ev) info.tl += elapsed(pr.first, pr.second);
    for (auto &pr : ta_ev) info.ta += elapsed(pr.first, pr.second);
    info.t += elapsed(e0, eend);
  }
  launch_union_affected(n, U.vb0.p, U.aff.p, U.ctl.p, s);
  LVG_CUDA(cudaMemcpyAsync(U.hctl.p, U.ctl.p, n * sizeof(GraphCtl), cudaMemcpyDeviceToHost, s));
  read_counters(g);
  info.t /= rep; info.tm /= rep; info.ti /= rep; info.tp /= rep; info.tl /= rep; info.ta /= rep;
  g->stats.move_vertices = g->hctr.p->vertices;
  g->stats.move_edges = g->hctr.p->edges;
  g->stats.moves = g->hctr.p->moves;
  g->stats.aggregate_edges = g->hctr.p->agg_edges;
  for (int b = 0; b < NUM_BINS; ++b) {
    g->stats.move_bin_vertices[b] = g->hctr.p->bin_vertices[b];
    g->stats.move_bin_edges[b] = g->hctr.p->bin_edges[b];
    g->stats.move_bin_overflow[b] = g->hctr.p->bin_over[b];
  }
  g->stats.hub_chunk_overflow = g->hctr.p->hub_chunk_over;
  g->stats.kernel_launches = launch_counter() - launches0;
}

// ---------------------------------------------------------------- host-side validation

void check_batch(const lvg_graph *g, const lvg_batch *b, bool need_sorted) {
  const size_t S = g->base.span;
  if (!b) return;
  if ((b->num_deletions && (!b->del_src || !b->del_dst || !b->del_w)) ||
      (b->num_insertions && (!b->ins_src || !b->ins_dst || !b->ins_w)))
    throw Error(LVG_EINVAL, "batch: null array with a non-zero count");
  for (size_t i = 0; i < b->num_deletions; ++i)
    if (b->del_src[i] >= S || b->del_dst[i] >= S) throw Error(LVG_EINVAL, "batch: deletion id >= span");
  for (size_t i = 0; i < b->num_insertions; ++i) {
    if (b->ins_src[i] >= S || b->ins_dst[i] >= S) throw Error(LVG_EINVAL, "batch: insertion id >= span");
    if (need_sorted && i && b->ins_src[i] < b->ins_src[i - 1])
      throw Error(LVG_EINVAL, "delta-screening needs insertions sorted by source vertex");
  }
}

size_t max_group(const lvg_batch *b) {
  size_t best = 0, run_len = 0;
  for (size_t i = 0; i < b->num_insertions; ++i) {
    run_len = (i && b->ins_src[i] == b->ins_src[i - 1]) ? run_len + 1 : 1;
    best = std::max(best, run_len);
  }
  return best;
}

void upload_batch(lvg_graph *g, const lvg_batch *b, DBuf<uint32_t> &ds, DBuf<uint32_t> &dd, DBuf<float> &dw,
                  DBuf<uint32_t> &is, DBuf<uint32_t> &id, DBuf<float> &iw, DBuf<uint32_t> &seg, DBatch &out) {
  cudaStream_t s = g->stream;
  out = DBatch{};
  if (!b) return;
  out.nd = b->num_deletions;
  out.ni = b->num_insertions;
  ds.ensure(out.nd); dd.ensure(out.nd); dw.ensure(out.nd);
  is.ensure(out.ni); id.ensure(out.ni); iw.ensure(out.ni); seg.ensure(out.ni + 1);
  if (out.nd) {
    LVG_CUDA(cudaMemcpyAsync(ds.p, b->del_src, out.nd * 4, cudaMemcpyHostToDevice, s));
    LVG_CUDA(cudaMemcpyAsync(dd.p, b->del_dst, out.nd * 4, cudaMemcpyHostToDevice, s));
    LVG_CUDA(cudaMemcpyAsync(dw.p, b->del_w, out.nd * 4, cudaMemcpyHostToDevice, s));
  }
  if (out.ni) {
    LVG_CUDA(cudaMemcpyAsync(is.p, b->ins_src, out.ni * 4, cudaMemcpyHostToDevice, s));
    LVG_CUDA(cudaMemcpyAsync(id.p, b->ins_dst, out.ni * 4, cudaMemcpyHostToDevice, s));
    LVG_CUDA(cudaMemcpyAsync(iw.p, b->ins_w, out.ni * 4, cudaMemcpyHostToDevice, s));
  }
  out.ds = ds.p; out.dd = dd.p; out.dw = dw.p;
  out.is = is.p; out.id = id.p; out.iw = iw.p; out.seg = seg.p;
  out.max_group = max_group(b);
}

void fill_result(lvg_result *out, const RunInfo &info, size_t span) {
  out->span = span;
  out->iterations = info.iterations;
  out->passes = info.passes;
  out->time = info.t;
  out->markingTime = info.tm;
  out->initializationTime = info.ti;
  out->firstPassTime = info.tp;
  out->localMoveTime = info.tl;
  out->aggregationTime = info.ta;
  out->affectedVertices = info.affected;
}

// Download the first-level membership/weights and final totals to the
// result's host arrays (allocating the ones left NULL).
// skip_vw: the vertex weights were copied out during the run.
void download_result(lvg_graph *g, lvg_result *out, StateRef st, bool skip_vw = false) {
  Workspace &W = *g->ws;
  cudaStream_t s = g->stream;
  const size_t S = g->base.span;
  if (!out->membership) { out->membership = (uint32_t *)std::malloc(S * 4 + 1); out->owned |= 1; }
  if (!out->vertexWeight) { out->vertexWeight = (double *)std::malloc(S * 8 + 1); out->owned |= 2; }
  if (!out->communityWeight) { out->communityWeight = (double *)std::malloc(S * 8 + 1); out->owned |= 4; }
  if (!out->membership || !out->vertexWeight || !out->communityWeight) throw std::bad_alloc();
  W.stage_a.ensure(S);
  W.stage_b.ensure(S);
  if (!skip_vw) launch_f32_to_f64(st.vt, W.stage_a.p, S, s);
  launch_f32_to_f64(st.ct, W.stage_b.p, S, s);
  LVG_CUDA(cudaMemcpyAsync(out->membership, st.q, S * 4, cudaMemcpyDeviceToHost, s));
  if (!skip_vw) LVG_CUDA(cudaMemcpyAsync(out->vertexWeight, W.stage_a.p, S * 8, cudaMemcpyDeviceToHost, s));
  LVG_CUDA(cudaMemcpyAsync(out->communityWeight, W.stage_b.p, S * 8, cudaMemcpyDeviceToHost, s));
  LVG_CUDA(cudaStreamSynchronize(s));
}

void upload_prior(lvg_graph *g, const uint32_t *q, const double *qvtot, const double *qctot, uint32_t *dq,
                  float *dvt, float *dct) {
  Workspace &W = *g->ws;
  cudaStream_t s = g->stream;
  const size_t S = g->base.span;
  if (!q || !qvtot || !qctot) throw Error(LVG_EINVAL, "prior state: null array");
  W.stage_a.ensure(S);
  W.stage_b.ensure(S);
  LVG_CUDA(cudaMemcpyAsync(dq, q, S * 4, cudaMemcpyHostToDevice, s));
  LVG_CUDA(cudaMemcpyAsync(W.stage_a.p, qvtot, S * 8, cudaMemcpyHostToDevice, s));
  LVG_CUDA(cudaMemcpyAsync(W.stage_b.p, qctot, S * 8, cudaMemcpyHostToDevice, s));
  launch_prior_to_f32(W.stage_a.p, dvt, S, s);
  launch_prior_to_f32(W.stage_b.p, dct, S, s);
  // every prior id must be < span (checked on the device; read back before any use)
  launch_check_ids(dq, S, uint32_t(S), g->ctr.p, s);
  read_counters(g);
}

int run_host(lvg_graph *g, int method, const lvg_batch *b, const uint32_t *q, const double *qvtot,
             const double *qctot, const lvg_options *o, lvg_result *out) {
  AcctScope acct_(g ? &g->bytes : nullptr);
  if (!g || !out) return fail(LVG_EINVAL, "null graph or result");
  return guarded([&] {
    LVG_CUDA(cudaSetDevice(g->device));
    // a copy left in flight by a call that failed
    if (g->copy_stream) LVG_CUDA(cudaStreamSynchronize(g->copy_stream));
    lvg_options opt;
    if (o) opt = *o; else lvg_options_default(&opt);
    const auto t0 = std::chrono::steady_clock::now();
    check_batch(g, b, method == LVG_METHOD_DELTA);
    ensure_ws(g);
    Workspace &W = *g->ws;
    DBatch db;
    upload_batch(g, method == LVG_METHOD_STATIC ? nullptr : b, g->b_ds, g->b_dd, g->b_dw, g->b_is, g->b_id,
                 g->b_iw, g->b_seg, db);
    StateRef prior{nullptr, nullptr, nullptr};
    if (method != LVG_METHOD_STATIC) {
      W.prior_q.ensure(W.S); W.prior_vt.ensure(W.S); W.prior_ct.ensure(W.S);
      upload_prior(g, q, qvtot, qctot, W.prior_q.p, W.prior_vt.p, W.prior_ct.p);
      prior = StateRef{W.prior_q.p, W.prior_vt.p, W.prior_ct.p};
    }
    LVG_CUDA(cudaStreamSynchronize(g->stream));
    const auto t1 = std::chrono::steady_clock::now();
    StateRef st{W.ucom.p, W.utot.p, W.ctot.p};
    RunInfo info;
    // The vertex weights are final once the run has initialised: into a
    // pinned result array they are copied out on a side stream while the
    // local moving runs (the host link is full duplex).
    cudaPointerAttributes pa{};
    const bool early = out->vertexWeight &&
                       cudaPointerGetAttributes(&pa, out->vertexWeight) == cudaSuccess &&
                       pa.type == cudaMemoryTypeHost;
    cudaGetLastError();
    std::function<void(cudaEvent_t)> hook = [&](cudaEvent_t ready) {
      if (!g->copy_stream) LVG_CUDA(cudaStreamCreateWithFlags(&g->copy_stream, cudaStreamNonBlocking));
      const size_t S = g->base.span;
      W.stage_a.ensure(S);
      LVG_CUDA(cudaStreamWaitEvent(g->copy_stream, ready, 0));
      launch_f32_to_f64(st.vt, W.stage_a.p, S, g->copy_stream);
      LVG_CUDA(cudaMemcpyAsync(out->vertexWeight, W.stage_a.p, S * 8, cudaMemcpyDeviceToHost, g->copy_stream));
    };
    run(g, method, db, prior, st, opt, info, early ? &hook : nullptr);
    fill_result(out, info, g->base.span);
    const auto t2 = std::chrono::steady_clock::now();
    download_result(g, out, st, early);
    if (early) LVG_CUDA(cudaStreamSynchronize(g->copy_stream));
    const auto t3 = std::chrono::steady_clock::now();
    using ms = std::chrono::duration<double, std::milli>;
    g->stats.call_upload_ms = ms(t1 - t0).count();
    g->stats.call_run_ms = ms(t2 - t1).count();
    g->stats.call_download_ms = ms(t3 - t2).count();
    return LVG_OK;
  });
}

// Lay out a compact CSR already in HBM (coff[span+1], ckey/cw[X]) as the
// graph's gapped CSR — room for row_capacity(deg) entries per row, then an
// overflow pool for rows that outgrow their room under batch updates — and
// compute its degree bins, hub plan and total weight. g->ex holds the present
// flags when has_exists.
void init_graph(lvg_graph *g, size_t span, size_t order, size_t X, const uint64_t *coff, const uint32_t *ckey,
                const float *cw, bool has_exists) {
  cudaStream_t s = g->stream;
  g->off.ensure(span + 1);
  g->deg.ensure(span + 1);
  g->cap.ensure(span);
  g->bins.ensure(span + 1);
  g->upd.ensure(UPD_SLOTS);
  g->hupd.ensure(UPD_SLOTS + 8);
  {
    DBuf<uint64_t> cap64, sc;
    cap64.ensure(span);
    sc.ensure(scan_scratch_elems(span));
    launch_row_caps(coff, span, g->deg.p, g->cap.p, cap64.p, s);
    exclusive_scan_u64(cap64.p, g->off.p, span, g->off.p + span, sc.p, s);
    LVG_CUDA(cudaMemcpyAsync(g->hupd.p, g->off.p + span, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    LVG_CUDA(cudaStreamSynchronize(s));
    const size_t rows_end = g->hupd.p[0];
    g->pool_begin = rows_end;
    g->slots = rows_end + rows_end / 8 + 65536;
    g->key.ensure(g->slots);
    g->w.ensure(g->slots);
    LVG_CUDA(cudaMemsetAsync(g->key.p + rows_end, 0, (g->slots - rows_end) * 4, s));
    LVG_CUDA(cudaMemsetAsync(g->w.p + rows_end, 0, (g->slots - rows_end) * 4, s));
    launch_spread_rows(coff, ckey, cw, span, g->off.p, g->cap.p, g->key.p, g->w.p, s);
    g->pool_cursor = rows_end;
    LVG_CUDA(cudaMemsetAsync(g->upd.p, 0, UPD_SLOTS * 8, s));
    LVG_CUDA(cudaStreamSynchronize(s));  // the scratch is freed next
  }
  g->ctr.ensure(1);
  g->hctr.ensure(1);
  LVG_CUDA(cudaMemsetAsync(g->ctr.p, 0, sizeof(Counters), s));
  Level &b = g->base;
  b.span = span; b.order = order; b.edges = X;
  b.off = g->off.p; b.deg = g->deg.p; b.key = g->key.p; b.w = g->w.p; b.ex = has_exists ? g->ex.p : nullptr;
  launch_total_weight(g->w.p, g->slots, g->ctr.p, s);
  DBuf<uint32_t> scratch;
  scratch.ensure(bin_scratch_elems(span + 1, DEFAULT_COLORS_ASYNC));
  compute_bins(g, b, g->deg.p, g->bins.p, scratch.p, DEFAULT_COLORS_ASYNC);  // synchronises
  build_hub_plan(g, b, g->hubplan);
  read_counters(g);
  g->total_weight = g->hctr.p->fp64[0];
}

// ---------------------------------------------------------------- batch apply

// The batch plan, on the device: each list packed as (src << b | dst) keys,
// stably sorted, the first of each run kept (tidyBatchUpdateU's sort +
// unique, inc/batch.hxx:169-192, keeping the first in batch order where the
// reference's unstable sort keeps an unspecified one) into g->u_ds.. /
// g->u_is.., and one UpdRow per touched source vertex into g->u_rows.
struct PlanCounts {
  size_t nd = 0, ni = 0, nrows = 0, max_group = 0;
};

int id_bits(size_t span) {  // bits to hold ids 0..span-1
  int b = 1;
  while (b < 32 && ((span - 1) >> b)) ++b;
  return b;
}

PlanCounts plan_device(lvg_graph *g, const uint32_t *ds, const uint32_t *dd, const float *dw, size_t nd,
                       const uint32_t *is, const uint32_t *id, const float *iw, size_t ni) {
  cudaStream_t s = g->stream;
  const size_t S = g->base.span, n = std::max(nd, ni);
  const int b = id_bits(S);
  g->u_k0.ensure(n); g->u_k1.ensure(n); g->u_v0.ensure(n); g->u_v1.ensure(n);
  g->u_flag.ensure(n + 1); g->u_pos.ensure(n + 1); g->u_pscan.ensure(scan_scratch_elems(n + 1));
  g->u_ds.ensure(nd); g->u_dd.ensure(nd); g->u_dw.ensure(nd);
  g->u_is.ensure(ni); g->u_id.ensure(ni); g->u_iw.ensure(ni);
  g->u_cnt.ensure(4);
  g->hcnt.ensure(4);
  LVG_CUDA(cudaMemsetAsync(g->u_cnt.p, 0, 4 * sizeof(uint32_t), s));
  LVG_CUDA(cudaMemsetAsync(g->upd.p + UPD_MAXG, 0, sizeof(uint64_t), s));
  auto one = [&](const uint32_t *src, const uint32_t *dst, const float *w, size_t m, uint32_t *os, uint32_t *od,
                 float *ow, uint32_t *count) {
    if (!m) return;
    launch_pack_keys(src, dst, m, b, g->u_k0.p, g->u_v0.p, s);
    const bool alt = sort_pairs_u64(g->u_k0.p, g->u_k1.p, g->u_v0.p, g->u_v1.p, m, 2 * b, g->u_tmp, s);
    const uint64_t *k = alt ? g->u_k1.p : g->u_k0.p;
    const uint32_t *v = alt ? g->u_v1.p : g->u_v0.p;
    launch_first_flags(k, m, g->u_flag.p, s);
    exclusive_scan_u32(g->u_flag.p, g->u_pos.p, m, count, g->u_pscan.p, s);
    launch_unpack_keys(k, v, g->u_flag.p, g->u_pos.p, m, b, w, os, od, ow, s);
  };
  one(ds, dd, dw, nd, g->u_ds.p, g->u_dd.p, g->u_dw.p, g->u_cnt.p + 0);
  one(is, id, iw, ni, g->u_is.p, g->u_id.p, g->u_iw.p, g->u_cnt.p + 1);
  g->u_touch.ensure(S + 1); g->u_tpos.ensure(S + 1); g->u_tscan.ensure(scan_scratch_elems(S + 1));
  g->u_rows.ensure(std::min(S, nd + ni));
  launch_plan_rows(g->u_ds.p, g->u_cnt.p + 0, g->u_is.p, g->u_cnt.p + 1, n, g->u_touch.p, g->u_tpos.p,
                   g->u_tscan.p, S, g->u_rows.p, g->upd.p, g->u_cnt.p + 2, s);
  LVG_CUDA(cudaMemcpyAsync(g->hcnt.p, g->u_cnt.p, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  LVG_CUDA(cudaMemcpyAsync(g->hupd.p + UPD_MAXG, g->upd.p + UPD_MAXG, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
  LVG_CUDA(cudaStreamSynchronize(s));
  PlanCounts c;
  c.nd = g->hcnt.p[0];
  c.ni = g->hcnt.p[1];
  c.nrows = g->hcnt.p[2];
  c.max_group = g->hupd.p[UPD_MAXG];
  return c;
}

// Copy every row into a fresh gapped layout whose pool has room for at least
// `need` entries. Row order and contents are kept.
void relayout(lvg_graph *g, size_t need) {
  cudaStream_t s = g->stream;
  const size_t S = g->base.span;
  DBuf<uint64_t> cap64, noff, sc;
  DBuf<uint32_t> ncap, nkey;
  DBuf<float> nw;
  cap64.ensure(S);
  noff.ensure(S + 1);
  sc.ensure(scan_scratch_elems(S));
  ncap.ensure(S);
  launch_fresh_caps(g->deg.p, S, ncap.p, cap64.p, s);
  exclusive_scan_u64(cap64.p, noff.p, S, noff.p + S, sc.p, s);
  LVG_CUDA(cudaMemcpyAsync(g->hupd.p, noff.p + S, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
  LVG_CUDA(cudaStreamSynchronize(s));
  const size_t rows_end = g->hupd.p[0];
  const size_t slots = rows_end + std::max(need, rows_end / 8) + 65536;
  nkey.ensure(slots);
  nw.ensure(slots);
  LVG_CUDA(cudaMemsetAsync(nkey.p + rows_end, 0, (slots - rows_end) * sizeof(uint32_t), s));
  LVG_CUDA(cudaMemsetAsync(nw.p + rows_end, 0, (slots - rows_end) * sizeof(float), s));
  launch_relayout_rows(g->off.p, g->deg.p, g->key.p, g->w.p, S, noff.p, ncap.p, nkey.p, nw.p, s);
  LVG_CUDA(cudaStreamSynchronize(s));
  g->off.swap(noff);
  g->cap.swap(ncap);
  g->key.swap(nkey);
  g->w.swap(nw);
  g->base.off = g->off.p;
  g->base.key = g->key.p;
  g->base.w = g->w.p;
  g->slots = slots;
  g->pool_begin = rows_end;
  g->pool_cursor = rows_end;
}

// Tidy and apply a planned batch (plan_device's lists and rows). The kept
// flags of the tidied batch are left in g->u_keep (deletions, then
// insertions).
void apply_plan(lvg_graph *g, const PlanCounts &pc) {
  const UpdRow *rows = g->u_rows.p;
  const size_t nrows = pc.nrows, nd = pc.nd, ni = pc.ni;
  const uint32_t *dd = g->u_dd.p, *id = g->u_id.p;
  const float *iw = g->u_iw.p;
  if (!nrows) return;
  cudaStream_t s = g->stream;
  Level &b = g->base;
  g->u_pre.ensure(nd + ni);
  g->u_keep.ensure(nd + ni);
  g->u_plan.ensure(nrows);
  g->u_len.ensure(nrows); g->u_src.ensure(nrows); g->u_grow.ensure(nrows);
  g->u_spos.ensure(nrows + 1); g->u_srcpos.ensure(nrows + 1); g->u_gpos.ensure(nrows + 1);
  g->u_scan.ensure(scan_scratch_elems(nrows + 1));
  g->u_wdelta.ensure(1);
  uint8_t *ex = b.ex ? g->ex.p : nullptr;
  uint64_t T = 0, SRC = 0, GROW = 0;
  for (int attempt = 0;; ++attempt) {
    LVG_CUDA(cudaMemsetAsync(g->upd.p, 0, UPD_SLOTS * sizeof(uint64_t), s));
    LVG_CUDA(cudaMemsetAsync(g->u_wdelta.p, 0, sizeof(double), s));
    launch_row_plan(g->off.p, g->deg.p, g->cap.p, g->key.p, g->w.p, rows, nrows, dd, id, iw, nd, g->u_pre.p,
                    g->u_keep.p, g->u_plan.p, g->u_len.p, g->u_src.p, g->u_grow.p, ex, g->upd.p, g->u_wdelta.p, s);
    exclusive_scan_u64(g->u_len.p, g->u_spos.p, nrows, g->u_spos.p + nrows, g->u_scan.p, s);
    exclusive_scan_u64(g->u_src.p, g->u_srcpos.p, nrows, g->u_srcpos.p + nrows, g->u_scan.p, s);
    exclusive_scan_u64(g->u_grow.p, g->u_gpos.p, nrows, g->u_gpos.p + nrows, g->u_scan.p, s);
    unsigned long long *h = g->hupd.p;
    LVG_CUDA(cudaMemcpyAsync(h, g->upd.p, UPD_SLOTS * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    LVG_CUDA(cudaMemcpyAsync(h + 3, g->u_spos.p + nrows, 8, cudaMemcpyDeviceToHost, s));
    LVG_CUDA(cudaMemcpyAsync(h + 4, g->u_srcpos.p + nrows, 8, cudaMemcpyDeviceToHost, s));
    LVG_CUDA(cudaMemcpyAsync(h + 5, g->u_gpos.p + nrows, 8, cudaMemcpyDeviceToHost, s));
    LVG_CUDA(cudaMemcpyAsync(h + 6, g->u_wdelta.p, 8, cudaMemcpyDeviceToHost, s));
    LVG_CUDA(cudaStreamSynchronize(s));
    T = h[3];
    SRC = h[4];
    GROW = h[5];
    if (g->slots - g->pool_cursor >= GROW) break;
    if (attempt) throw Error(LVG_ECUDA, "batch apply: the re-laid-out pool is too small (internal sizing error)");
    relayout(g, GROW);  // fresh capacities: plan again
  }
  const long long edge_delta = (long long)g->hupd.p[UPD_EDGES];
  double wdelta;
  std::memcpy(&wdelta, &g->hupd.p[6], sizeof(double));
  g->u_skey.ensure(T);
  g->u_sw.ensure(T);
  const uint64_t pool = g->pool_cursor;
  launch_merge_items(g->off.p, g->deg.p, g->key.p, g->w.p, rows, nrows, dd, id, iw, nd, g->u_pre.p, g->u_keep.p,
                     g->u_plan.p, g->u_srcpos.p, SRC, g->u_spos.p, g->u_skey.p, g->u_sw.p, s);
  launch_copy_items(g->off.p, rows, nrows, g->u_plan.p, g->u_spos.p, T, g->u_grow.p, g->u_gpos.p, pool, g->u_skey.p,
                    g->u_sw.p, g->key.p, g->w.p, s);
  launch_finish_rows(g->off.p, g->deg.p, g->cap.p, g->key.p, g->w.p, rows, nrows, g->u_plan.p, g->u_grow.p,
                     g->u_gpos.p, pool, s);
  g->pool_cursor += GROW;
  if (ex) {
    launch_count_present(ex, b.span, g->upd.p, s);
    LVG_CUDA(cudaMemcpyAsync(g->hupd.p + UPD_ORDER, g->upd.p + UPD_ORDER, 8, cudaMemcpyDeviceToHost, s));
  }
  LVG_CUDA(cudaStreamSynchronize(s));
  b.edges = size_t((long long)b.edges + edge_delta);
  if (ex) b.order = g->hupd.p[UPD_ORDER];
  g->total_weight += wdelta;
  // degrees changed: new bins and hub plan; the captured iteration is stale
  if (g->iter_exec) {
    cudaGraphExecDestroy(g->iter_exec);
    g->iter_exec = nullptr;
  }
  ensure_ws(g);
  // the aggregation levels' edge buffers grow with 1/16 headroom: sized to the
  // exact count, a stream of insertion batches reallocated them (GBs freed
  // and allocated again) on every apply
  if (b.edges > g->ws->X) g->ws->allocate(b.span, b.edges + b.edges / 16, s);
  compute_bins(g, b, g->deg.p, g->bins.p, g->ws->binscratch.p, b.colors);  // synchronises
  build_hub_plan(g, b, g->hubplan);
}

// Plan, apply and compact the tidied batch into (tds.., tis..), arrays with
// room for nd / ni entries that may be the input arrays themselves (the plan
// has copied them before the compaction writes): what main.cxx:108-109 does
// on the host, here in HBM. Returns the tidied counts and the plan's longest
// insertion run.
PlanCounts tidy_apply(lvg_graph *g, const uint32_t *ds, const uint32_t *dd, const float *dw, size_t nd,
                      const uint32_t *is, const uint32_t *id, const float *iw, size_t ni, uint32_t *tds,
                      uint32_t *tdd, float *tdw, uint32_t *tis, uint32_t *tid, float *tiw) {
  if (!g->rows_sorted) throw Error(LVG_EINVAL, "batch apply needs rows sorted by neighbour id");
  if (nd > 0x7FFFFFFFull || ni > 0x7FFFFFFFull) throw Error(LVG_EINVAL, "batch apply: more than 2^31-1 entries");
  cudaStream_t s = g->stream;
  PlanCounts pc = plan_device(g, ds, dd, dw, nd, is, id, iw, ni);
  apply_plan(g, pc);
  const size_t n = pc.nd + pc.ni;
  PlanCounts out;
  out.max_group = pc.max_group;
  if (n && pc.nrows) {
    g->u_pos.ensure(n + 1);
    g->u_pscan.ensure(scan_scratch_elems(n + 1));
    exclusive_scan_u32(g->u_keep.p, g->u_pos.p, n, g->u_pos.p + n, g->u_pscan.p, s);
    launch_tidy_compact(g->u_ds.p, g->u_dd.p, g->u_dw.p, pc.nd, g->u_keep.p, g->u_pos.p, nullptr, tds, tdd, tdw, s);
    launch_tidy_compact(g->u_is.p, g->u_id.p, g->u_iw.p, pc.ni, g->u_keep.p + pc.nd, g->u_pos.p + pc.nd,
                        g->u_pos.p + pc.nd, tis, tid, tiw, s);
    g->hcnt.ensure(4);
    LVG_CUDA(cudaMemcpyAsync(g->hcnt.p, g->u_pos.p + pc.nd, 4, cudaMemcpyDeviceToHost, s));
    LVG_CUDA(cudaMemcpyAsync(g->hcnt.p + 1, g->u_pos.p + n, 4, cudaMemcpyDeviceToHost, s));
    LVG_CUDA(cudaStreamSynchronize(s));
    out.nd = g->hcnt.p[0];
    out.ni = g->hcnt.p[1] - g->hcnt.p[0];
  }
  return out;
}

}  // namespace

int fail_noalloc(int code, const char *msg) { return fail(code, msg); }

}  // namespace lvg

// ==================================================================== C-ABI

namespace lvg {
namespace {

// Copy a device array of n elements to per-graph host arrays (graph i gets
// elements [vb[i], vb[i+1]) into dst(i)) through two pinned staging chunks:
// each chunk is copied off the device while the previous one is spread into
// the (pageable) host arrays by a few threads.
template <class Dst>
void copy_out_slices(cudaStream_t s, const void *dev, size_t elem, const std::vector<uint64_t> &vb, Dst dst) {
  const size_t n = vb.back(), G = vb.size() - 1;
  if (!n) return;
  const size_t per = std::max<size_t>(1, (size_t(64) << 20) / elem);  // elements per chunk
  HBuf<uint8_t> stage[2];
  stage[0].ensure(per * elem);
  stage[1].ensure(per * elem);
  cudaEvent_t ev[2];
  LVG_CUDA(cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming));
  LVG_CUDA(cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming));
  const size_t chunks = (n + per - 1) / per;
  auto issue = [&](size_t k) {
    const size_t b = k * per, m = std::min(per, n - b);
    LVG_CUDA(cudaMemcpyAsync(stage[k & 1].p, static_cast<const uint8_t *>(dev) + b * elem, m * elem,
                             cudaMemcpyDeviceToHost, s));
    LVG_CUDA(cudaEventRecord(ev[k & 1], s));
  };
  const unsigned T = std::max(1u, std::min(8u, std::thread::hardware_concurrency()));
  size_t g0 = 0;  // first graph that may overlap the current chunk
  issue(0);
  for (size_t k = 0; k < chunks; ++k) {
    if (k + 1 < chunks) issue(k + 1);
    LVG_CUDA(cudaEventSynchronize(ev[k & 1]));
    const size_t b = k * per, e = std::min(n, b + per);
    while (g0 < G && vb[g0 + 1] <= b) ++g0;
    auto spread = [&](size_t lo, size_t hi) {  // element range [lo, hi) of the chunk
      size_t g = std::upper_bound(vb.begin(), vb.end(), lo) - vb.begin() - 1;
      for (; g < G && vb[g] < hi; ++g) {
        const size_t x0 = std::max<size_t>(lo, vb[g]), x1 = std::min<size_t>(hi, vb[g + 1]);
        if (x1 > x0)
          std::memcpy(static_cast<uint8_t *>(dst(g)) + (x0 - vb[g]) * elem, stage[k & 1].p + (x0 - b) * elem,
                      (x1 - x0) * elem);
      }
    };
    std::vector<std::thread> th;
    const size_t step = (e - b + T - 1) / T;
    for (unsigned t = 1; t < T && b + t * step < e; ++t)
      th.emplace_back(spread, b + t * step, std::min(e, b + (t + 1) * step));
    spread(b, std::min(e, b + step));
    for (auto &x : th) x.join();
  }
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
}

}  // namespace
}  // namespace lvg

namespace lvg {
namespace {

void check_tuning(const lvg_tuning &t) {
  if (t.frontier_colors < 1 || t.frontier_colors > MAX_COLORS)
    throw Error(LVG_EINVAL, "tuning: frontier_colors out of 1..32");
  if (t.hub_chunk < 256 || t.hub_chunk > (1u << 20)) throw Error(LVG_EINVAL, "tuning: hub_chunk out of 256..2^20");
  if (t.big_blocks_per_sm < 0 || t.big_blocks_per_sm > 64) throw Error(LVG_EINVAL, "tuning: big_blocks_per_sm");
  if (!(t.frontier_max_fraction >= 0 && t.frontier_max_fraction <= 1))
    throw Error(LVG_EINVAL, "tuning: frontier_max_fraction out of 0..1");
}

// Set a graph's tuning: the hub plan of the uploaded level follows the chunk
// size, and a captured iteration (launch shapes baked in) is dropped.
void apply_tuning(lvg_graph *g, const lvg_tuning &t) {
  check_tuning(t);
  const bool chunks = t.hub_chunk != g->tuning.hub_chunk;
  g->tuning = t;
  if (chunks) build_hub_plan(g, g->base, g->hubplan);
  if (g->iter_exec) {
    cudaGraphExecDestroy(g->iter_exec);
    g->iter_exec = nullptr;
  }
}

// Modularity of a membership already in HBM (the uploaded level's graph).
double modularity_device(lvg_graph *g, const uint32_t *dq, double M, double R) {
  Workspace &W = *g->ws;
  cudaStream_t s = g->stream;
  W.ctot64.ensure(g->base.span);
  launch_modularity(g->base, dq, W.ctot64.p, g->ctr.p, s);
  launch_sq_sum(W.ctot64.p, g->base.span, g->ctr.p, s);
  read_counters(g);
  const double intra = g->hctr.p->fp64[1], sq = g->hctr.p->fp64[2];
  return intra / (2 * M) - R * sq / (4 * M * M);
}

}  // namespace
}  // namespace lvg

extern "C" {

const char *lvg_last_error(void) { return lvg::g_err.c_str(); }

void lvg_options_default(lvg_options *o) {
  if (!o) return;
  o->repeat = 1;
  o->resolution = 1;
  o->tolerance = 1e-2;
  o->aggregationTolerance = 1.0;
  o->toleranceDrop = 10;
  o->maxIterations = 20;
  o->maxPasses = 10;
  o->deterministic = 0;
  o->colors = 0;
}

int lvg_graph_create(size_t span, const uint64_t *offsets, const uint32_t *keys, const float *weights,
                     const uint8_t *exists, lvg_graph **out) {
  if (!out || !offsets || span == 0 || span > 0xFFFFFFFFull) return lvg::fail(LVG_EINVAL, "lvg_graph_create: bad argument");
  *out = nullptr;
  const size_t X = offsets[span];
  if (X && (!keys || !weights)) return lvg::fail(LVG_EINVAL, "lvg_graph_create: null keys/weights");
  if (offsets[0] != 0) return lvg::fail(LVG_EINVAL, "lvg_graph_create: offsets[0] != 0");
  size_t order = 0;
  for (size_t u = 0; u < span; ++u) {
    if (offsets[u + 1] < offsets[u]) return lvg::fail(LVG_EINVAL, "lvg_graph_create: offsets not monotone");
    if (offsets[u + 1] - offsets[u] > 0xE0000000ull) return lvg::fail(LVG_EINVAL, "lvg_graph_create: row too long");
    const bool has = !exists || exists[u];
    order += has;
    if (!has && offsets[u + 1] != offsets[u])
      return lvg::fail(LVG_EINVAL, "lvg_graph_create: absent vertex with edges");
  }
  bool rows_sorted = true;
  for (size_t u = 0; u < span; ++u)
    for (uint64_t i = offsets[u]; i < offsets[u + 1]; ++i) {
      if (keys[i] >= span) return lvg::fail(LVG_EINVAL, "lvg_graph_create: neighbour id >= span");
      if (i > offsets[u] && keys[i] <= keys[i - 1]) rows_sorted = false;
    }
  std::unique_ptr<lvg_graph> g(new lvg_graph());
  lvg::AcctScope acct_(&g->bytes);
  int rc = lvg::guarded([&] {
    LVG_CUDA(cudaGetDevice(&g->device));
    LVG_CUDA(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
    cudaStream_t s = g->stream;
    g->rows_sorted = rows_sorted;
    lvg::DBuf<uint64_t> coff;
    lvg::DBuf<uint32_t> ckey;
    lvg::DBuf<float> cw;
    coff.ensure(span + 1);
    ckey.ensure(X);
    cw.ensure(X);
    LVG_CUDA(cudaMemcpyAsync(coff.p, offsets, (span + 1) * 8, cudaMemcpyHostToDevice, s));
    if (X) {
      LVG_CUDA(cudaMemcpyAsync(ckey.p, keys, X * 4, cudaMemcpyHostToDevice, s));
      LVG_CUDA(cudaMemcpyAsync(cw.p, weights, X * 4, cudaMemcpyHostToDevice, s));
    }
    if (exists) {
      g->ex.ensure(span);
      LVG_CUDA(cudaMemcpyAsync(g->ex.p, exists, span, cudaMemcpyHostToDevice, s));
    }
    lvg::init_graph(g.get(), span, order, X, coff.p, ckey.p, cw.p, exists != nullptr);
    return LVG_OK;
  });
  if (rc != LVG_OK) {
    if (g->stream) cudaStreamDestroy(g->stream);
    return rc;
  }
  *out = g.release();
  return LVG_OK;
}

namespace lvg {
namespace {
int create_generated(const GenSpec &spec, lvg_graph **out) {
  *out = nullptr;
  std::unique_ptr<lvg_graph> g(new lvg_graph());
  AcctScope acct_(&g->bytes);
  int rc = guarded([&] {
    LVG_CUDA(cudaGetDevice(&g->device));
    LVG_CUDA(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
    DBuf<uint64_t> coff;
    DBuf<uint32_t> ckey;
    DBuf<float> cw;
    const size_t X = generate_graph(spec, coff, ckey, cw, g->ex, g->stream);
    g->rows_sorted = true;
    init_graph(g.get(), spec.span, spec.span - 1, X, coff.p, ckey.p, cw.p, true);
    return LVG_OK;
  });
  if (rc != LVG_OK) {
    if (g->stream) cudaStreamDestroy(g->stream);
    return rc;
  }
  *out = g.release();
  return LVG_OK;
}
}  // namespace
}  // namespace lvg

int lvg_graph_create_planted_partition(uint32_t n, uint32_t block, double avg_degree, double p_in, uint64_t seed,
                                       lvg_graph **out) {
  if (!out || n == 0 || n >= 0xFFFFFFFFu || block == 0 || !(avg_degree >= 0) || !(p_in >= 0 && p_in <= 1))
    return lvg::fail(LVG_EINVAL, "lvg_graph_create_planted_partition: bad argument");
  lvg::GenSpec g;
  g.kind = lvg::GenSpec::PP;
  g.span = size_t(n) + 1;
  g.draws = size_t(std::llround(double(n) * avg_degree / 2));
  g.n = n;
  g.block = block;
  g.p_in = p_in;
  g.seed = seed;
  return lvg::create_generated(g, out);
}

int lvg_graph_create_rmat(int scale, double edge_factor, double a, double b, double c, int permute, uint64_t seed,
                          lvg_graph **out) {
  if (!out || scale < 1 || scale > 30 || !(edge_factor >= 0) || a < 0 || b < 0 || c < 0 || a + b + c > 1)
    return lvg::fail(LVG_EINVAL, "lvg_graph_create_rmat: bad argument");
  return lvg::guarded([&] {
    lvg::GenSpec g;
    g.kind = lvg::GenSpec::RMAT;
    g.span = (size_t(1) << scale) + 1;
    g.draws = size_t(std::llround(double(size_t(1) << scale) * edge_factor));
    g.scale = scale;
    g.a = a;
    g.ab = a + b;
    g.abc = a + b + c;
    g.seed = seed;
    if (permute) g.perm = lvg::rmat_permutation(scale, seed);
    return lvg::create_generated(g, out);
  });
}

int lvg_graph_create_from_edges(size_t span, size_t n, const uint32_t *src, const uint32_t *dst, const float *w,
                                lvg_graph **out) {
  if (!out || span == 0 || span > 0xFFFFFFFFull || (n && (!src || !dst)))
    return lvg::fail(LVG_EINVAL, "lvg_graph_create_from_edges: bad argument");
  *out = nullptr;
  for (size_t i = 0; i < n; ++i)
    if (src[i] >= span || dst[i] >= span) return lvg::fail(LVG_EINVAL, "lvg_graph_create_from_edges: id >= span");
  std::unique_ptr<lvg_graph> g(new lvg_graph());
  lvg::AcctScope acct_(&g->bytes);
  int rc = lvg::guarded([&] {
    LVG_CUDA(cudaGetDevice(&g->device));
    LVG_CUDA(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
    cudaStream_t s = g->stream;
    lvg::DBuf<uint32_t> ds, dd, ckey;
    lvg::DBuf<float> dw, cw;
    lvg::DBuf<uint64_t> coff;
    ds.ensure(n); dd.ensure(n); dw.ensure(n);
    if (n) {
      LVG_CUDA(cudaMemcpyAsync(ds.p, src, n * 4, cudaMemcpyHostToDevice, s));
      LVG_CUDA(cudaMemcpyAsync(dd.p, dst, n * 4, cudaMemcpyHostToDevice, s));
      if (w) {
        LVG_CUDA(cudaMemcpyAsync(dw.p, w, n * 4, cudaMemcpyHostToDevice, s));
      } else {
        const float one = 1.0f;
        lvg::launch_fill_f32(dw.p, n, one, s);
      }
    }
    const size_t X = lvg::graph_from_edges(ds.p, dd.p, dw.p, n, span, coff, ckey, cw, g->ex, s);
    ds.release(); dd.release(); dw.release();
    std::vector<uint8_t> ex(span);
    LVG_CUDA(cudaMemcpyAsync(ex.data(), g->ex.p, span, cudaMemcpyDeviceToHost, s));
    LVG_CUDA(cudaStreamSynchronize(s));
    size_t order = 0;
    for (uint8_t e : ex) order += e;
    g->rows_sorted = true;
    lvg::init_graph(g.get(), span, order, X, coff.p, ckey.p, cw.p, true);
    return LVG_OK;
  });
  if (rc != LVG_OK) {
    if (g->stream) cudaStreamDestroy(g->stream);
    return rc;
  }
  *out = g.release();
  return LVG_OK;
}

int lvg_graph_clone(lvg_graph *x, lvg_graph **out) {
  if (!x || !out) return lvg::fail(LVG_EINVAL, "null argument");
  *out = nullptr;
  std::unique_ptr<lvg_graph> g(new lvg_graph());
  lvg::AcctScope acct_(&g->bytes);
  int rc = lvg::guarded([&] {
    LVG_CUDA(cudaSetDevice(x->device));
    g->device = x->device;
    LVG_CUDA(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
    cudaStream_t s = g->stream;
    LVG_CUDA(cudaStreamSynchronize(x->stream));
    const size_t S = x->base.span;
    auto copy = [&](auto &dst, const auto &src, size_t count) {
      dst.ensure(count);
      if (count) LVG_CUDA(cudaMemcpyAsync(dst.p, src.p, count * sizeof(*src.p), cudaMemcpyDeviceToDevice, s));
    };
    copy(g->off, x->off, S + 1);
    copy(g->deg, x->deg, S + 1);
    copy(g->cap, x->cap, S);
    copy(g->key, x->key, x->slots);
    copy(g->w, x->w, x->slots);
    if (x->base.ex) copy(g->ex, x->ex, S);
    g->bins.ensure(S + 1);
    g->upd.ensure(lvg::UPD_SLOTS);
    g->hupd.ensure(lvg::UPD_SLOTS + 8);
    LVG_CUDA(cudaMemsetAsync(g->upd.p, 0, lvg::UPD_SLOTS * 8, s));
    g->slots = x->slots;
    g->pool_begin = x->pool_begin;
    g->pool_cursor = x->pool_cursor;
    g->rows_sorted = x->rows_sorted;
    g->total_weight = x->total_weight;
    g->tuning = x->tuning;
    g->ctr.ensure(1);
    g->hctr.ensure(1);
    LVG_CUDA(cudaMemsetAsync(g->ctr.p, 0, sizeof(Counters), s));
    lvg::Level &b = g->base;
    b.span = S; b.order = x->base.order; b.edges = x->base.edges;
    b.off = g->off.p; b.deg = g->deg.p; b.key = g->key.p; b.w = g->w.p; b.ex = x->base.ex ? g->ex.p : nullptr;
    lvg::DBuf<uint32_t> scratch;
    scratch.ensure(lvg::bin_scratch_elems(S + 1, x->base.colors));
    lvg::compute_bins(g.get(), b, g->deg.p, g->bins.p, scratch.p, x->base.colors);  // synchronises
    lvg::build_hub_plan(g.get(), b, g->hubplan);
    return LVG_OK;
  });
  if (rc != LVG_OK) {
    if (g->stream) cudaStreamDestroy(g->stream);
    return rc;
  }
  *out = g.release();
  return LVG_OK;
}

int lvg_graph_create_union(lvg_graph *const *graphs, size_t n, lvg_graph **out) {
  if (!graphs || !n || !out) return lvg::fail(LVG_EINVAL, "null argument or no graphs");
  *out = nullptr;
  for (size_t i = 0; i < n; ++i) {
    if (!graphs[i]) return lvg::fail(LVG_EINVAL, "null graph");
    if (graphs[i]->uni) return lvg::fail(LVG_EINVAL, "a graph union cannot be part of a union");
    if (graphs[i]->device != graphs[0]->device) return lvg::fail(LVG_EINVAL, "graphs on different devices");
  }
  std::unique_ptr<lvg_graph> g(new lvg_graph());
  lvg::AcctScope acct_(&g->bytes);
  int rc = lvg::guarded([&] {
    using namespace lvg;
    LVG_CUDA(cudaSetDevice(graphs[0]->device));
    g->device = graphs[0]->device;
    LVG_CUDA(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
    cudaStream_t s = g->stream;
    auto U = std::make_unique<UnionInfo>();
    U->n = n;
    U->vb.assign(n + 1, 0);
    U->M.resize(n);
    std::vector<uint64_t> order(n);
    size_t ord = 0;
    for (size_t i = 0; i < n; ++i) {
      const lvg_graph *x = graphs[i];
      LVG_CUDA(cudaStreamSynchronize(x->stream));
      U->vb[i + 1] = U->vb[i] + x->base.span;
      order[i] = x->base.order;
      ord += x->base.order;
      U->M[i] = x->total_weight / 2;
    }
    const size_t S = U->vb[n];
    if (S >= size_t(EMPTY)) throw Error(LVG_EINVAL, "graph union: more than 2^32-2 vertices");
    // compact union CSR: degrees, their scan, rows with ids shifted by the graph's first vertex
    DBuf<uint64_t> coff, sc;
    DBuf<uint32_t> ckey;
    DBuf<float> cw;
    coff.ensure(S + 1);
    sc.ensure(scan_scratch_elems(S + 1));
    g->ex.ensure(S);
    for (size_t i = 0; i < n; ++i) {
      const lvg_graph *x = graphs[i];
      const size_t sp = x->base.span;
      launch_union_degrees(x->base.deg, sp, coff.p + U->vb[i], s);
      if (!sp) continue;
      if (x->base.ex) LVG_CUDA(cudaMemcpyAsync(g->ex.p + U->vb[i], x->base.ex, sp, cudaMemcpyDeviceToDevice, s));
      else LVG_CUDA(cudaMemsetAsync(g->ex.p + U->vb[i], 1, sp, s));
    }
    exclusive_scan_u64(coff.p, coff.p, S, coff.p + S, sc.p, s);
    uint64_t X = 0;  // edges: the degrees' sum
    LVG_CUDA(cudaMemcpyAsync(&X, coff.p + S, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    LVG_CUDA(cudaStreamSynchronize(s));
    ckey.ensure(std::max<size_t>(X, 1));
    cw.ensure(std::max<size_t>(X, 1));
    for (size_t i = 0; i < n; ++i) {
      const lvg_graph *x = graphs[i];
      launch_union_rows(x->base.off, x->base.deg, x->base.key, x->base.w, x->base.span, uint32_t(U->vb[i]), coff.p,
                        ckey.p, cw.p, s);
    }
    std::vector<uint32_t> vb32(n + 1);
    for (size_t i = 0; i <= n; ++i) vb32[i] = uint32_t(U->vb[i]);
    U->vb0.ensure(n + 1);
    U->gid0.ensure(S);
    U->order.ensure(n);
    U->Md.ensure(n);
    LVG_CUDA(cudaMemcpyAsync(U->vb0.p, vb32.data(), (n + 1) * 4, cudaMemcpyHostToDevice, s));
    LVG_CUDA(cudaMemcpyAsync(U->order.p, order.data(), n * 8, cudaMemcpyHostToDevice, s));
    LVG_CUDA(cudaMemcpyAsync(U->Md.p, U->M.data(), n * 8, cudaMemcpyHostToDevice, s));
    launch_fill_gid(U->vb0.p, n, U->gid0.p, s);
    LVG_CUDA(cudaStreamSynchronize(s));
    init_graph(g.get(), S, ord, X, coff.p, ckey.p, cw.p, true);
    // colour classes by each graph's own vertex ids
    g->base.gid = U->gid0.p;
    g->base.gbase = U->vb0.p;
    DBuf<uint32_t> scratch;
    scratch.ensure(bin_scratch_elems(S + 1, DEFAULT_COLORS_ASYNC));
    compute_bins(g.get(), g->base, g->deg.p, g->bins.p, scratch.p, DEFAULT_COLORS_ASYNC);
    build_hub_plan(g.get(), g->base, g->hubplan);
    g->uni = std::move(U);
    return LVG_OK;
  });
  if (rc != LVG_OK) {
    if (g->stream) cudaStreamDestroy(g->stream);
    return rc;
  }
  *out = g.release();
  return LVG_OK;
}

int lvg_union_graphs(const lvg_graph *u, size_t *n) {
  if (!u || !n) return lvg::fail(LVG_EINVAL, "null argument");
  *n = u->uni ? u->uni->n : 0;
  return LVG_OK;
}

int lvg_static_union(lvg_graph *u, const lvg_options *o, lvg_result *results) {
  lvg::AcctScope acct_(u ? &u->bytes : nullptr);
  if (!u || !results) return lvg::fail(LVG_EINVAL, "null graph or results");
  if (!u->uni) return lvg::fail(LVG_EINVAL, "not a graph union (lvg_graph_create_union)");
  return lvg::guarded([&] {
    using namespace lvg;
    LVG_CUDA(cudaSetDevice(u->device));
    lvg_options opt;
    if (o) opt = *o; else lvg_options_default(&opt);
    const auto t0 = std::chrono::steady_clock::now();
    RunInfo info;
    run_union(u, opt, info);
    const auto t1 = std::chrono::steady_clock::now();
    UnionInfo &U = *u->uni;
    Workspace &W = *u->ws;
    cudaStream_t s = u->stream;
    const size_t S = u->base.span;
    W.stage_a.ensure(S);
    W.stage_b.ensure(S);
    launch_f32_to_f64(W.utot.p, W.stage_a.p, S, s);
    launch_f32_to_f64(U.ct.p, W.stage_b.p, S, s);
    for (size_t i = 0; i < U.n; ++i) {
      lvg_result *r = &results[i];
      const size_t sp = U.vb[i + 1] - U.vb[i];
      if (!r->membership) { r->membership = (uint32_t *)std::malloc(sp * 4 + 1); r->owned |= 1; }
      if (!r->vertexWeight) { r->vertexWeight = (double *)std::malloc(sp * 8 + 1); r->owned |= 2; }
      if (!r->communityWeight) { r->communityWeight = (double *)std::malloc(sp * 8 + 1); r->owned |= 4; }
      if (!r->membership || !r->vertexWeight || !r->communityWeight) throw std::bad_alloc();
    }
    copy_out_slices(s, U.q.p, 4, U.vb, [&](size_t i) -> void * { return results[i].membership; });
    copy_out_slices(s, W.stage_a.p, 8, U.vb, [&](size_t i) -> void * { return results[i].vertexWeight; });
    copy_out_slices(s, W.stage_b.p, 8, U.vb, [&](size_t i) -> void * { return results[i].communityWeight; });
    for (size_t i = 0; i < U.n; ++i) {
      lvg_result *r = &results[i];
      const size_t sp = U.vb[i + 1] - U.vb[i];
      const GraphCtl &c = U.hctl.p[i];
      RunInfo ri = info;
      ri.iterations = int(c.l);
      ri.passes = int(c.p);
      ri.affected = c.aff;
      fill_result(r, ri, sp);
    }
    LVG_CUDA(cudaStreamSynchronize(s));
    const auto t2 = std::chrono::steady_clock::now();
    using ms = std::chrono::duration<double, std::milli>;
    u->stats.call_upload_ms = 0;
    u->stats.call_run_ms = ms(t1 - t0).count();
    u->stats.call_download_ms = ms(t2 - t1).count();
    return LVG_OK;
  });
}

int lvg_graph_destroy(lvg_graph *g) {
  if (!g) return LVG_OK;
  cudaSetDevice(g->device);
  if (g->stream) cudaStreamSynchronize(g->stream);
  cudaStream_t s = g->stream;
  delete g;
  if (s) cudaStreamDestroy(s);
  return LVG_OK;
}

size_t lvg_graph_device_bytes(const lvg_graph *g) { return g ? g->bytes : 0; }
size_t lvg_state_device_bytes(const lvg_state *st) { return st ? st->bytes : 0; }
size_t lvg_device_batch_device_bytes(const lvg_device_batch *b) { return b ? b->bytes : 0; }

int lvg_graph_trim(lvg_graph *g, int level) {
  if (!g || level < 1 || level > 2) return lvg::fail(LVG_EINVAL, "lvg_graph_trim: bad argument");
  return lvg::guarded([&] {
    LVG_CUDA(cudaSetDevice(g->device));
    LVG_CUDA(cudaStreamSynchronize(g->stream));
    if (g->iter_exec) {  // the captured iteration refers to the buffers released below
      cudaGraphExecDestroy(g->iter_exec);
      g->iter_exec = nullptr;
    }
    if (g->ws) {
      lvg::Workspace &W = *g->ws;
      W.gkeys.release(); W.gvals.release();
      W.part_key.release(); W.part_val.release(); W.chunk_cnt.release();
    }
    for (auto *d : {&g->u_k0, &g->u_k1, &g->u_len, &g->u_src, &g->u_grow, &g->u_spos, &g->u_srcpos, &g->u_gpos,
                    &g->u_scan})
      d->release();
    for (auto *d : {&g->u_skey, &g->u_pre, &g->u_keep, &g->u_pos, &g->u_pscan, &g->u_v0, &g->u_v1,
                    &g->u_flag, &g->u_touch, &g->u_tpos, &g->u_tscan, &g->u_cnt, &g->u_ds, &g->u_dd, &g->u_is,
                    &g->u_id, &g->b_ds, &g->b_dd, &g->b_is, &g->b_id, &g->b_seg})
      d->release();
    for (auto *d : {&g->u_sw, &g->u_dw, &g->u_iw, &g->b_dw, &g->b_iw}) d->release();
    g->u_tmp.release();
    g->u_rows.release();
    g->u_plan.release();
    g->u_wdelta.release();
    if (level == 2) g->ws.reset();
    return LVG_OK;
  });
}

size_t lvg_graph_span(const lvg_graph *g) { return g ? g->base.span : 0; }
size_t lvg_graph_order(const lvg_graph *g) { return g ? g->base.order : 0; }
size_t lvg_graph_size(const lvg_graph *g) { return g ? g->base.edges : 0; }

int lvg_static(lvg_graph *x, const lvg_options *o, lvg_result *out) {
  return lvg::run_host(x, LVG_METHOD_STATIC, nullptr, nullptr, nullptr, nullptr, o, out);
}

int lvg_naive_dynamic(lvg_graph *y, const lvg_batch *b, const uint32_t *q, const double *qvtot, const double *qctot,
                      const lvg_options *o, lvg_result *out) {
  return lvg::run_host(y, LVG_METHOD_NAIVE, b, q, qvtot, qctot, o, out);
}

int lvg_delta_screening(lvg_graph *y, const lvg_batch *b, const uint32_t *q, const double *qvtot,
                        const double *qctot, const lvg_options *o, lvg_result *out) {
  return lvg::run_host(y, LVG_METHOD_DELTA, b, q, qvtot, qctot, o, out);
}

int lvg_frontier(lvg_graph *y, const lvg_batch *b, const uint32_t *q, const double *qvtot, const double *qctot,
                 const lvg_options *o, lvg_result *out) {
  return lvg::run_host(y, LVG_METHOD_FRONTIER, b, q, qvtot, qctot, o, out);
}

void lvg_result_free(lvg_result *r) {
  if (!r) return;
  if (r->owned & 1) std::free(r->membership);
  if (r->owned & 2) std::free(r->vertexWeight);
  if (r->owned & 4) std::free(r->communityWeight);
  if (r->owned & 1) r->membership = nullptr;
  if (r->owned & 2) r->vertexWeight = nullptr;
  if (r->owned & 4) r->communityWeight = nullptr;
  r->owned = 0;
}

int lvg_edge_weight(lvg_graph *g, double *out) {
  if (!g || !out) return lvg::fail(LVG_EINVAL, "null argument");
  *out = g->total_weight;
  return LVG_OK;
}

int lvg_vertex_weights(lvg_graph *g, double *vtot) {
  lvg::AcctScope acct_(g ? &g->bytes : nullptr);
  if (!g || !vtot) return lvg::fail(LVG_EINVAL, "null argument");
  return lvg::guarded([&] {
    LVG_CUDA(cudaSetDevice(g->device));
    lvg::ensure_ws(g);
    lvg::Workspace &W = *g->ws;
    const size_t S = g->base.span;
    W.stage_a.ensure(S);
    lvg::launch_vertex_weights_f64(g->base, W.stage_a.p, g->stream);
    LVG_CUDA(cudaMemcpyAsync(vtot, W.stage_a.p, S * 8, cudaMemcpyDeviceToHost, g->stream));
    LVG_CUDA(cudaStreamSynchronize(g->stream));
    return LVG_OK;
  });
}

int lvg_community_weights(lvg_graph *g, const uint32_t *membership, const double *vtot, double *ctot) {
  lvg::AcctScope acct_(g ? &g->bytes : nullptr);
  if (!g || !membership || !ctot) return lvg::fail(LVG_EINVAL, "null argument");
  return lvg::guarded([&] {
    LVG_CUDA(cudaSetDevice(g->device));
    const size_t S = g->base.span;
    for (size_t u = 0; u < S; ++u)
      if (membership[u] >= S) throw lvg::Error(LVG_EINVAL, "membership id >= span");
    lvg::ensure_ws(g);
    lvg::Workspace &W = *g->ws;
    cudaStream_t s = g->stream;
    W.stage_a.ensure(S);
    W.stage_b.ensure(S);
    LVG_CUDA(cudaMemcpyAsync(W.com_next.p, membership, S * 4, cudaMemcpyHostToDevice, s));
    if (vtot) LVG_CUDA(cudaMemcpyAsync(W.stage_a.p, vtot, S * 8, cudaMemcpyHostToDevice, s));
    else lvg::launch_vertex_weights_f64(g->base, W.stage_a.p, s);
    lvg::launch_community_weights_f64(W.com_next.p, W.stage_a.p, S, W.stage_b.p, s);
    LVG_CUDA(cudaMemcpyAsync(ctot, W.stage_b.p, S * 8, cudaMemcpyDeviceToHost, s));
    LVG_CUDA(cudaStreamSynchronize(s));
    return LVG_OK;
  });
}

int lvg_modularity(lvg_graph *g, const uint32_t *membership, double M, double R, double *out) {
  lvg::AcctScope acct_(g ? &g->bytes : nullptr);
  if (!g || !membership || !out) return lvg::fail(LVG_EINVAL, "null argument");
  return lvg::guarded([&] {
    LVG_CUDA(cudaSetDevice(g->device));
    const size_t S = g->base.span;
    for (size_t u = 0; u < S; ++u)
      if (membership[u] >= S) throw lvg::Error(LVG_EINVAL, "membership id >= span");
    lvg::ensure_ws(g);
    lvg::Workspace &W = *g->ws;
    cudaStream_t s = g->stream;
    if (M <= 0) M = g->total_weight / 2;
    W.ctot64.ensure(S);
    LVG_CUDA(cudaMemcpyAsync(W.com_next.p, membership, S * 4, cudaMemcpyHostToDevice, s));
    lvg::launch_modularity(g->base, W.com_next.p, W.ctot64.p, g->ctr.p, s);
    lvg::launch_sq_sum(W.ctot64.p, S, g->ctr.p, s);
    lvg::read_counters(g);
    const double intra = g->hctr.p->fp64[1], sq = g->hctr.p->fp64[2];
    *out = intra / (2 * M) - R * sq / (4 * M * M);
    return LVG_OK;
  });
}

int lvg_affected_vertices(lvg_graph *y, int method, const lvg_batch *b, const uint32_t *q, const double *qvtot,
                          const double *qctot, const lvg_options *o, uint8_t *flags, uint8_t *neighbors,
                          uint8_t *communities) {
  lvg::AcctScope acct_(y ? &y->bytes : nullptr);
  if (!y || !flags || method < 0 || method > 3) return lvg::fail(LVG_EINVAL, "bad argument");
  return lvg::guarded([&] {
    LVG_CUDA(cudaSetDevice(y->device));
    lvg_options opt;
    if (o) opt = *o; else lvg_options_default(&opt);
    opt.maxPasses = 0;  // initialise and mark only
    opt.repeat = 1;
    lvg::check_batch(y, b, method == LVG_METHOD_DELTA);
    lvg::ensure_ws(y);
    lvg::Workspace &W = *y->ws;
    lvg::DBatch db;
    lvg::upload_batch(y, method == LVG_METHOD_STATIC ? nullptr : b, y->b_ds, y->b_dd, y->b_dw, y->b_is, y->b_id,
                      y->b_iw, y->b_seg, db);
    lvg::StateRef prior{nullptr, nullptr, nullptr};
    if (method != LVG_METHOD_STATIC) {
      W.prior_q.ensure(W.S); W.prior_vt.ensure(W.S); W.prior_ct.ensure(W.S);
      lvg::upload_prior(y, q, qvtot, qctot, W.prior_q.p, W.prior_vt.p, W.prior_ct.p);
      prior = lvg::StateRef{W.prior_q.p, W.prior_vt.p, W.prior_ct.p};
    }
    lvg::StateRef st{W.ucom.p, W.utot.p, W.ctot.p};
    lvg::RunInfo info;
    lvg::run(y, method, db, prior, st, opt, info);
    const size_t S = y->base.span;
    LVG_CUDA(cudaMemcpyAsync(flags, W.vaff.p, S, cudaMemcpyDeviceToHost, y->stream));
    if (method == LVG_METHOD_DELTA && neighbors) LVG_CUDA(cudaMemcpyAsync(neighbors, W.fn.p, S, cudaMemcpyDeviceToHost, y->stream));
    if (method == LVG_METHOD_DELTA && communities) LVG_CUDA(cudaMemcpyAsync(communities, W.fc.p, S, cudaMemcpyDeviceToHost, y->stream));
    LVG_CUDA(cudaStreamSynchronize(y->stream));
    return LVG_OK;
  });
}

int lvg_aggregate(lvg_graph *g, const uint32_t *membership, uint32_t *renumbered, size_t *num_communities,
                  uint64_t *offsets, uint32_t *keys, double *weights) {
  lvg::AcctScope acct_(g ? &g->bytes : nullptr);
  if (!g || !membership || !renumbered || !num_communities || !offsets) return lvg::fail(LVG_EINVAL, "null argument");
  return lvg::guarded([&] {
    LVG_CUDA(cudaSetDevice(g->device));
    const size_t S = g->base.span, X = g->base.edges;
    for (size_t u = 0; u < S; ++u)
      if (membership[u] >= S) throw lvg::Error(LVG_EINVAL, "membership id >= span");
    if (X && (!keys || !weights)) throw lvg::Error(LVG_EINVAL, "null keys/weights");
    lvg::ensure_ws(g);
    lvg::Workspace &W = *g->ws;
    cudaStream_t s = g->stream;
    LVG_CUDA(cudaMemcpyAsync(W.ucom.p, membership, S * 4, cudaMemcpyHostToDevice, s));
    LVG_CUDA(cudaMemsetAsync(W.cext.p, 0, (S + 1) * sizeof(uint32_t), s));
    lvg::launch_community_flags(g->base, W.ucom.p, W.cext.p, s);
    lvg::exclusive_scan_u32(W.cext.p, W.cext.p, S, &g->ctr.p->cn, W.scan32.p, s);
    lvg::read_counters(g);
    const size_t CN = g->hctr.p->cn;
    lvg::launch_lookup(W.ucom.p, W.cext.p, S, s);
    lvg::Level nl = lvg::aggregate(g, g->base, W.ucom.p, CN, 0, 1);
    std::vector<uint64_t> yoff(CN + 1);
    std::vector<uint32_t> ydeg(CN + 1), yk(X ? X : 1);
    std::vector<float> yw(X ? X : 1);
    LVG_CUDA(cudaMemcpyAsync(renumbered, W.ucom.p, S * 4, cudaMemcpyDeviceToHost, s));
    LVG_CUDA(cudaMemcpyAsync(yoff.data(), nl.off, (CN + 1) * 8, cudaMemcpyDeviceToHost, s));
    if (CN) LVG_CUDA(cudaMemcpyAsync(ydeg.data(), nl.deg, CN * 4, cudaMemcpyDeviceToHost, s));
    if (X) {
      LVG_CUDA(cudaMemcpyAsync(yk.data(), nl.key, X * 4, cudaMemcpyDeviceToHost, s));
      LVG_CUDA(cudaMemcpyAsync(yw.data(), nl.w, X * 4, cudaMemcpyDeviceToHost, s));
    }
    LVG_CUDA(cudaStreamSynchronize(s));
    *num_communities = CN;
    uint64_t k = 0;
    for (size_t c = 0; c < CN; ++c) {
      offsets[c] = k;
      for (uint32_t j = 0; j < ydeg[c]; ++j, ++k) {
        keys[k] = yk[yoff[c] + j];
        weights[k] = yw[yoff[c] + j];
      }
    }
    offsets[CN] = k;
    return LVG_OK;
  });
}

void *lvg_host_alloc(size_t bytes) {
  void *p = nullptr;
  if (cudaMallocHost(&p, bytes ? bytes : 1) != cudaSuccess) return nullptr;
  return p;
}

void lvg_host_free(void *p) {
  if (p) cudaFreeHost(p);
}

int lvg_profiler_start(void) {
  return lvg::guarded([&] {
    LVG_CUDA(cudaProfilerStart());
    return LVG_OK;
  });
}

int lvg_profiler_stop(void) {
  return lvg::guarded([&] {
    LVG_CUDA(cudaProfilerStop());
    return LVG_OK;
  });
}

int lvg_set_device(int device) {
  return lvg::guarded([&] {
    LVG_CUDA(cudaSetDevice(device));
    return LVG_OK;
  });
}

int lvg_set_profiling(lvg_graph *g, int enable) {
  if (!g) return lvg::fail(LVG_EINVAL, "null graph");
  g->profiling = enable != 0;
  return LVG_OK;
}

int lvg_get_stats(const lvg_graph *g, lvg_stats *out) {
  if (!g || !out) return lvg::fail(LVG_EINVAL, "null argument");
  *out = g->stats;
  return LVG_OK;
}

int lvg_state_create(lvg_graph *g, lvg_state **out) {
  if (!g || !out) return lvg::fail(LVG_EINVAL, "null argument");
  *out = nullptr;
  std::unique_ptr<lvg_state> st(new lvg_state());
  lvg::AcctScope acct_(&st->bytes);
  int rc = lvg::guarded([&] {
    LVG_CUDA(cudaSetDevice(g->device));
    const size_t S = g->base.span;
    st->g = g;
    st->device = g->device;
    st->q.ensure(S); st->vt.ensure(S); st->ct.ensure(S);
    LVG_CUDA(cudaMemsetAsync(st->q.p, 0, S * 4, g->stream));
    LVG_CUDA(cudaMemsetAsync(st->vt.p, 0, S * 4, g->stream));
    LVG_CUDA(cudaMemsetAsync(st->ct.p, 0, S * 4, g->stream));
    LVG_CUDA(cudaStreamSynchronize(g->stream));
    return LVG_OK;
  });
  if (rc == LVG_OK) *out = st.release();
  return rc;
}

int lvg_state_set(lvg_state *st, const uint32_t *q, const double *qvtot, const double *qctot) {
  if (!st) return lvg::fail(LVG_EINVAL, "null state");
  return lvg::guarded([&] {
    lvg_graph *g = st->g;
    LVG_CUDA(cudaSetDevice(g->device));
    lvg::ensure_ws(g);
    lvg::upload_prior(g, q, qvtot, qctot, st->q.p, st->vt.p, st->ct.p);
    LVG_CUDA(cudaStreamSynchronize(g->stream));
    return LVG_OK;
  });
}

int lvg_state_get(const lvg_state *st, uint32_t *membership, double *vtot, double *ctot) {
  if (!st) return lvg::fail(LVG_EINVAL, "null state");
  return lvg::guarded([&] {
    lvg_graph *g = st->g;
    LVG_CUDA(cudaSetDevice(g->device));
    lvg::ensure_ws(g);
    lvg::Workspace &W = *g->ws;
    cudaStream_t s = g->stream;
    const size_t S = g->base.span;
    W.stage_a.ensure(S);
    W.stage_b.ensure(S);
    if (membership) LVG_CUDA(cudaMemcpyAsync(membership, st->q.p, S * 4, cudaMemcpyDeviceToHost, s));
    if (vtot) {
      lvg::launch_f32_to_f64(st->vt.p, W.stage_a.p, S, s);
      LVG_CUDA(cudaMemcpyAsync(vtot, W.stage_a.p, S * 8, cudaMemcpyDeviceToHost, s));
    }
    if (ctot) {
      lvg::launch_f32_to_f64(st->ct.p, W.stage_b.p, S, s);
      LVG_CUDA(cudaMemcpyAsync(ctot, W.stage_b.p, S * 8, cudaMemcpyDeviceToHost, s));
    }
    LVG_CUDA(cudaStreamSynchronize(s));
    return LVG_OK;
  });
}

int lvg_state_destroy(lvg_state *st) {
  if (!st) return LVG_OK;
  cudaSetDevice(st->device);
  delete st;  // cudaFree waits for the work that uses the buffers
  return LVG_OK;
}

int lvg_device_batch_create(lvg_graph *g, const lvg_batch *b, lvg_device_batch **out) {
  if (!g || !b || !out) return lvg::fail(LVG_EINVAL, "null argument");
  *out = nullptr;
  std::unique_ptr<lvg_device_batch> db(new lvg_device_batch());
  lvg::AcctScope acct_(&db->bytes);
  int rc = lvg::guarded([&] {
    LVG_CUDA(cudaSetDevice(g->device));
    lvg::check_batch(g, b, false);
    db->g = g;
    db->device = g->device;
    lvg::upload_batch(g, b, db->ds, db->dd, db->dw, db->is, db->id, db->iw, db->seg, db->b);
    LVG_CUDA(cudaStreamSynchronize(g->stream));
    // remember whether the insertions are source-sorted (delta-screening needs it)
    bool sorted = true;
    for (size_t i = 1; i < b->num_insertions; ++i) sorted &= b->ins_src[i] >= b->ins_src[i - 1];
    if (!sorted) db->b.max_group = ~size_t(0);
    return LVG_OK;
  });
  if (rc == LVG_OK) *out = db.release();
  return rc;
}

int lvg_graph_apply_batch(lvg_graph *g, const lvg_batch *b, lvg_batch_buf *tidy) {
  lvg::AcctScope acct_(g ? &g->bytes : nullptr);
  if (!g) return lvg::fail(LVG_EINVAL, "null graph");
  if (g->uni) return lvg::fail(LVG_EINVAL, "batch updates of a graph union are not supported");
  if (tidy && b &&
      ((b->num_deletions && (!tidy->del_src || !tidy->del_dst || !tidy->del_w)) ||
       (b->num_insertions && (!tidy->ins_src || !tidy->ins_dst || !tidy->ins_w))))
    return lvg::fail(LVG_EINVAL, "lvg_graph_apply_batch: null tidy-batch array");
  return lvg::guarded([&] {
    LVG_CUDA(cudaSetDevice(g->device));
    lvg::check_batch(g, b, false);
    if (tidy) tidy->num_deletions = tidy->num_insertions = 0;
    if (!b || !(b->num_deletions + b->num_insertions)) return LVG_OK;
    cudaStream_t s = g->stream;
    lvg::DBatch raw;
    lvg::upload_batch(g, b, g->b_ds, g->b_dd, g->b_dw, g->b_is, g->b_id, g->b_iw, g->b_seg, raw);
    // the tidied batch is compacted over the uploaded one (g->b_*)
    uint32_t *tds = g->b_ds.p, *tdd = g->b_dd.p, *tis = g->b_is.p, *tid = g->b_id.p;
    float *tdw = g->b_dw.p, *tiw = g->b_iw.p;
    const lvg::PlanCounts t = lvg::tidy_apply(g, raw.ds, raw.dd, raw.dw, raw.nd, raw.is, raw.id, raw.iw, raw.ni,
                                              tds, tdd, tdw, tis, tid, tiw);
    if (tidy) {
      if (t.nd) {
        LVG_CUDA(cudaMemcpyAsync(tidy->del_src, tds, t.nd * 4, cudaMemcpyDeviceToHost, s));
        LVG_CUDA(cudaMemcpyAsync(tidy->del_dst, tdd, t.nd * 4, cudaMemcpyDeviceToHost, s));
        LVG_CUDA(cudaMemcpyAsync(tidy->del_w, tdw, t.nd * 4, cudaMemcpyDeviceToHost, s));
      }
      if (t.ni) {
        LVG_CUDA(cudaMemcpyAsync(tidy->ins_src, tis, t.ni * 4, cudaMemcpyDeviceToHost, s));
        LVG_CUDA(cudaMemcpyAsync(tidy->ins_dst, tid, t.ni * 4, cudaMemcpyDeviceToHost, s));
        LVG_CUDA(cudaMemcpyAsync(tidy->ins_w, tiw, t.ni * 4, cudaMemcpyDeviceToHost, s));
      }
      LVG_CUDA(cudaStreamSynchronize(s));
      tidy->num_deletions = t.nd;
      tidy->num_insertions = t.ni;
    }
    return LVG_OK;
  });
}

int lvg_graph_apply_device_batch(lvg_graph *g, lvg_device_batch *b) {
  if (!g || !b) return lvg::fail(LVG_EINVAL, "null argument");
  if (g->uni) return lvg::fail(LVG_EINVAL, "batch updates of a graph union are not supported");
  if (b->g != g) return lvg::fail(LVG_EINVAL, "the batch was created on another graph");
  if (b->applied) return lvg::fail(LVG_EINVAL, "the batch has already been applied");
  return lvg::guarded([&] {
    LVG_CUDA(cudaSetDevice(g->device));
    cudaStream_t s = g->stream;
    // the batch becomes the tidied batch (tidyBatchUpdateU's result), which
    // the dynamic methods then take, as main.cxx:108-125 does
    const lvg::DBatch &r = b->b;
    if (!(r.nd + r.ni)) {
      b->applied = true;
      return LVG_OK;
    }
    // compacted over the batch's own arrays, which the plan has copied
    lvg::AcctScope acct_(&g->bytes);
    const lvg::PlanCounts t = lvg::tidy_apply(g, r.ds, r.dd, r.dw, r.nd, r.is, r.id, r.iw, r.ni, b->ds.p, b->dd.p,
                                              b->dw.p, b->is.p, b->id.p, b->iw.p);
    (void)s;
    b->b.nd = t.nd;
    b->b.ni = t.ni;
    b->b.max_group = t.max_group;  // an upper bound after the filter
    b->applied = true;
    return LVG_OK;
  });
}

int lvg_graph_download(lvg_graph *g, uint64_t *offsets, uint32_t *keys, float *weights, uint8_t *exists) {
  if (!g || !offsets) return lvg::fail(LVG_EINVAL, "null argument");
  return lvg::guarded([&] {
    LVG_CUDA(cudaSetDevice(g->device));
    cudaStream_t s = g->stream;
    const size_t S = g->base.span;
    std::vector<uint64_t> off(S);
    std::vector<uint32_t> deg(S), key(g->slots);
    std::vector<float> w(g->slots);
    LVG_CUDA(cudaMemcpyAsync(off.data(), g->off.p, S * 8, cudaMemcpyDeviceToHost, s));
    LVG_CUDA(cudaMemcpyAsync(deg.data(), g->deg.p, S * 4, cudaMemcpyDeviceToHost, s));
    if (keys) LVG_CUDA(cudaMemcpyAsync(key.data(), g->key.p, g->slots * 4, cudaMemcpyDeviceToHost, s));
    if (weights) LVG_CUDA(cudaMemcpyAsync(w.data(), g->w.p, g->slots * 4, cudaMemcpyDeviceToHost, s));
    if (exists) {
      if (g->base.ex) LVG_CUDA(cudaMemcpyAsync(exists, g->ex.p, S, cudaMemcpyDeviceToHost, s));
      else std::memset(exists, 1, S);
    }
    LVG_CUDA(cudaStreamSynchronize(s));
    offsets[0] = 0;
    for (size_t u = 0; u < S; ++u) {
      const uint64_t o = offsets[u];
      if (keys) std::memcpy(keys + o, key.data() + off[u], deg[u] * 4);
      if (weights) std::memcpy(weights + o, w.data() + off[u], deg[u] * 4);
      offsets[u + 1] = o + deg[u];
    }
    return LVG_OK;
  });
}

int lvg_device_batch_generate(lvg_graph *g, size_t deletions, size_t insertions, uint32_t begin, uint32_t range,
                              float weight, uint64_t seed, lvg_device_batch **out) {
  if (!g || !out) return lvg::fail(LVG_EINVAL, "null argument");
  *out = nullptr;
  if (range == 0 || size_t(begin) + range > g->base.span)
    return lvg::fail(LVG_EINVAL, "lvg_device_batch_generate: [begin, begin+range) outside the span");
  std::unique_ptr<lvg_device_batch> db(new lvg_device_batch());
  lvg::AcctScope acct_(&db->bytes);
  int rc = lvg::guarded([&] {
    LVG_CUDA(cudaSetDevice(g->device));
    db->g = g;
    db->device = g->device;
    size_t nd = 0, ni = 0;
    lvg::generate_batch(g->off.p, g->deg.p, g->key.p, g->w.p, deletions, insertions, begin, range, weight, seed,
                        db->ds, db->dd, db->dw, db->is, db->id, db->iw, nd, ni, g->stream);
    db->seg.ensure(ni + 1);
    lvg::DBatch &d = db->b;
    d = lvg::DBatch{};
    d.ds = db->ds.p; d.dd = db->dd.p; d.dw = db->dw.p;
    d.is = db->is.p; d.id = db->id.p; d.iw = db->iw.p; d.seg = db->seg.p;
    d.nd = nd;
    d.ni = ni;
    d.max_group = ~size_t(0);  // not sorted by source until applied
    return LVG_OK;
  });
  if (rc == LVG_OK) *out = db.release();
  return rc;
}

int lvg_device_batch_download(const lvg_device_batch *b, lvg_batch_buf *out) {
  if (!b || !out) return lvg::fail(LVG_EINVAL, "null argument");
  return lvg::guarded([&] {
    LVG_CUDA(cudaSetDevice(b->device));
    const lvg::DBatch &d = b->b;
    cudaStream_t s = b->g->stream;
    auto get = [&](void *dst, const void *src, size_t bytes) {
      if (bytes && !dst) throw lvg::Error(LVG_EINVAL, "lvg_device_batch_download: null array");
      if (bytes) LVG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s));
    };
    get(out->del_src, d.ds, d.nd * 4); get(out->del_dst, d.dd, d.nd * 4); get(out->del_w, d.dw, d.nd * 4);
    get(out->ins_src, d.is, d.ni * 4); get(out->ins_dst, d.id, d.ni * 4); get(out->ins_w, d.iw, d.ni * 4);
    LVG_CUDA(cudaStreamSynchronize(s));
    out->num_deletions = d.nd;
    out->num_insertions = d.ni;
    return LVG_OK;
  });
}

int lvg_device_batch_size(const lvg_device_batch *b, size_t *deletions, size_t *insertions) {
  if (!b) return lvg::fail(LVG_EINVAL, "null argument");
  if (deletions) *deletions = b->b.nd;
  if (insertions) *insertions = b->b.ni;
  return LVG_OK;
}

int lvg_device_batch_set(lvg_device_batch *db, const lvg_batch *b) {
  if (!db || !b) return lvg::fail(LVG_EINVAL, "null argument");
  lvg_graph *g = db->g;
  lvg::AcctScope acct_(&db->bytes);
  return lvg::guarded([&] {
    LVG_CUDA(cudaSetDevice(g->device));
    lvg::check_batch(g, b, false);
    lvg::upload_batch(g, b, db->ds, db->dd, db->dw, db->is, db->id, db->iw, db->seg, db->b);
    bool sorted = true;
    for (size_t i = 1; i < b->num_insertions; ++i) sorted &= b->ins_src[i] >= b->ins_src[i - 1];
    if (!sorted) db->b.max_group = ~size_t(0);
    db->applied = false;
    LVG_CUDA(cudaStreamSynchronize(g->stream));  // the caller may reuse its arrays
    return LVG_OK;
  });
}

int lvg_device_batch_destroy(lvg_device_batch *b) {
  if (!b) return LVG_OK;
  cudaSetDevice(b->device);
  delete b;  // cudaFree waits for the work that uses the buffers
  return LVG_OK;
}

void lvg_tuning_default(lvg_tuning *t) {
  if (t) *t = lvg::default_tuning();
}

int lvg_graph_get_tuning(const lvg_graph *g, lvg_tuning *t) {
  if (!g || !t) return lvg::fail(LVG_EINVAL, "null argument");
  *t = g->tuning;
  return LVG_OK;
}

int lvg_graph_set_tuning(lvg_graph *g, const lvg_tuning *t) {
  lvg::AcctScope acct_(g ? &g->bytes : nullptr);
  if (!g || !t) return lvg::fail(LVG_EINVAL, "null argument");
  return lvg::guarded([&] {
    LVG_CUDA(cudaSetDevice(g->device));
    LVG_CUDA(cudaStreamSynchronize(g->stream));
    lvg::apply_tuning(g, *t);
    return LVG_OK;
  });
}

int lvg_autotune(lvg_graph *g, int method, const lvg_device_batch *b, const lvg_state *prior, const lvg_options *o,
                 int repeats, lvg_tuning *best, double *best_ms) {
  lvg::AcctScope acct_(g ? &g->bytes : nullptr);
  if (!g || method < 0 || method > 3 || repeats < 1) return lvg::fail(LVG_EINVAL, "bad argument");
  if (g->uni && method != LVG_METHOD_STATIC) return lvg::fail(LVG_EINVAL, "a graph union runs static Louvain only");
  if (!g->uni && method != LVG_METHOD_STATIC && !prior)
    return lvg::fail(LVG_EINVAL, "dynamic methods need a prior state");
  if ((b && b->g != g) || (prior && prior->g != g)) return lvg::fail(LVG_EINVAL, "state/batch belongs to another graph");
  return lvg::guarded([&] {
    using namespace lvg;
    LVG_CUDA(cudaSetDevice(g->device));
    lvg_options opt;
    if (o) opt = *o; else lvg_options_default(&opt);
    opt.repeat = 1;
    ensure_ws(g);
    Workspace &W = *g->ws;
    DBatch db;
    if (b && method != LVG_METHOD_STATIC) db = b->b;
    StateRef pr{nullptr, nullptr, nullptr};
    if (prior) pr = StateRef{prior->q.p, prior->vt.p, prior->ct.p};
    StateRef st{W.ucom.p, W.utot.p, W.ctot.p};
    // per-launch timing off while tuning (restored however the call ends)
    struct Restore {
      lvg_graph *g;
      bool was;
      ~Restore() { g->profiling = was; }
    } restore{g, g->profiling};
    g->profiling = false;
    auto once = [&] {
      RunInfo ri;
      if (g->uni) run_union(g, opt, ri);
      else run(g, method, db, pr, st, opt, ri);
      return double(ri.t);
    };
    // time of a candidate (min over the repeats, after one warm-up run); q:
    // the modularity of its last run, when asked (frontier colour classes)
    auto measure = [&](const lvg_tuning &t, double *q) {
      apply_tuning(g, t);
      once();
      double tm = 1e300;
      for (int r = 0; r < repeats; ++r) tm = std::min(tm, once());
      if (q) *q = modularity_device(g, st.q, g->total_weight / 2, opt.resolution);
      return tm;
    };
    const bool colours = !g->uni && !opt.deterministic && opt.colors <= 0 &&
                         (method == LVG_METHOD_FRONTIER || method == LVG_METHOD_DELTA);
    lvg_tuning cur = g->tuning;
    double qref = 0;
    double tcur = measure(cur, colours ? &qref : nullptr);
    auto try_knob = [&](auto set, std::initializer_list<long> values, bool guard) {
      for (long v : values) {
        lvg_tuning t = cur;
        set(t, v);
        if (!std::memcmp(&t, &cur, sizeof(t))) continue;
        double q = 0;
        const double tm = measure(t, guard ? &q : nullptr);
        if (tm < 0.98 * tcur && (!guard || q >= qref - 1e-3)) {
          cur = t;
          tcur = tm;
        }
      }
    };
    // the class count first (the largest effect), then the launch shapes; twice,
    // since each knob's best value can depend on the others
    const lvg_tuning start = cur;
    for (int round = 0; round < 2; ++round) {
      if (colours) try_knob([](lvg_tuning &t, long v) { t.frontier_colors = int(v); }, {8, 4, 2, 1}, true);
      try_knob([](lvg_tuning &t, long v) { t.hub_chunk = uint32_t(v); }, {2048, 4096, 8192, 16384}, false);
      // concurrent bins and fused small bins together: each one's best value
      // depends on the other (R-MAT s24, DF at 1e-4 |E|, one class: 0.62 ms
      // with concurrent and unfused, 0.78 ms for the best of one at a time)
      try_knob([](lvg_tuning &t, long v) { t.concurrent_bins = int(v >> 1); t.fused_small = int(v & 1); },
               {3, 2, 1, 0}, false);
      try_knob([](lvg_tuning &t, long v) { t.big_blocks_per_sm = int(v); }, {0, 2, 3, 4}, false);
    }
    // confirm the launch shapes against the starting ones (with the chosen
    // class count), measured in turn, since a sub-millisecond run drifts
    // between measurements: shapes that are not 2 % faster on this second
    // look are dropped
    lvg_tuning base = start;
    base.frontier_colors = cur.frontier_colors;
    if (std::memcmp(&cur, &base, sizeof(cur))) {
      double a = 1e300, z = 1e300;
      for (int r = 0; r < 3; ++r) {
        a = std::min(a, measure(cur, nullptr));
        z = std::min(z, measure(base, nullptr));
      }
      if (a < 0.98 * z) {
        tcur = a;
      } else {
        cur = base;
        tcur = z;
      }
    }
    apply_tuning(g, cur);
    if (best) *best = cur;
    if (best_ms) *best_ms = tcur;
    return LVG_OK;
  });
}

int lvg_run_resident(lvg_graph *g, int method, const lvg_device_batch *b, const lvg_state *prior, lvg_state *out,
                     const lvg_options *o, lvg_result *info) {
  lvg::AcctScope acct_(g ? &g->bytes : nullptr);
  if (!g || !out || method < 0 || method > 3) return lvg::fail(LVG_EINVAL, "bad argument");
  if (method != LVG_METHOD_STATIC && !prior) return lvg::fail(LVG_EINVAL, "dynamic methods need a prior state");
  if ((b && b->g != g) || (prior && prior->g != g) || out->g != g)
    return lvg::fail(LVG_EINVAL, "state/batch belongs to another graph");
  if (method == LVG_METHOD_DELTA && b && b->b.max_group == ~size_t(0))
    return lvg::fail(LVG_EINVAL, "delta-screening needs insertions sorted by source vertex");
  return lvg::guarded([&] {
    LVG_CUDA(cudaSetDevice(g->device));
    lvg_options opt;
    if (o) opt = *o; else lvg_options_default(&opt);
    lvg::DBatch db;
    if (b && method != LVG_METHOD_STATIC) db = b->b;
    lvg::StateRef pr{nullptr, nullptr, nullptr};
    if (prior) pr = lvg::StateRef{prior->q.p, prior->vt.p, prior->ct.p};
    lvg::StateRef st{out->q.p, out->vt.p, out->ct.p};
    lvg::RunInfo ri;
    lvg::run(g, method, db, pr, st, opt, ri);
    if (info) lvg::fill_result(info, ri, g->base.span);
    return LVG_OK;
  });
}

}  // extern "C"
