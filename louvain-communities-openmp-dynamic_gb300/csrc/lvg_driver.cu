// lvg_driver.cu — the pass driver, batch apply and graph set-up behind the C-ABI.
//
// The pass driver follows louvainInvokeOmp (inc/louvain.hxx:1120-1221): per
// repetition it initialises membership and weights (fi), marks affected
// vertices (fm), then alternates local moving and aggregation until a pass
// converges in one iteration, maxPasses is reached, or the community count
// stops shrinking below aggregationTolerance. Everything runs on the graph's
// own CUDA stream; the host only reads back the per-iteration gain sum and the
// per-pass community count to take the reference's branch decisions.
#include "lvg_driver.cuh"

namespace lvg {

thread_local std::string g_err;

int fail(int code, const std::string &msg) {
  g_err = msg;
  return code;
}

// Wait for the graph's stream, counted in the call's statistics (host_syncs).
void host_sync(lvg_graph *g) {
  ++g->stats.host_syncs;
  LVG_CUDA(cudaStreamSynchronize(g->stream));
}

void drop_graphs(lvg_graph *g) {
  g->key_seen = false;
  if (g->iter_exec) {
    cudaGraphExecDestroy(g->iter_exec);
    g->iter_exec = nullptr;
  }
  if (g->phase_exec) {
    cudaGraphExecDestroy(g->phase_exec);
    g->phase_exec = nullptr;
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
  host_sync(g);
  if (g->hctr.p->err) {
    unsigned e = g->hctr.p->err;
    LVG_CUDA(cudaMemsetAsync(&g->ctr.p->err, 0, sizeof(unsigned), g->stream));
    if (e & ERR_BAD_ID) throw Error(LVG_EINVAL, "prior membership id >= span (err=" + std::to_string(e) + ")");
    if (e & ERR_WORKLIST) throw Error(LVG_ECUDA, "worklist append outside its degree bin (stale degree bins)");
    throw Error(LVG_ETIMEOUT, "device hash table overflow guard tripped (err=" + std::to_string(e) + ")");
  }
}

void compute_bins(lvg_graph *g, Level &lv, const uint32_t *deg, uint32_t *list, uint32_t *scratch, int colors) {
  g->hbins.ensure(bin_host_elems(MAX_COLORS));
  lv.colors = colors;
  lv.lim = bin_limits_of(g->tuning);
  bin_items_u32(deg, lv.ex, lv.span, colors, list, lv.bin_start, lv.bin_maxdeg, scratch, g->hbins.p, g->stream,
                lv.gid, lv.gbase, lv.lim);
  ++g->stats.host_syncs;  // the bin counts are read back
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
  host_sync(g);
  std::vector<uint4> chunks;
  std::vector<uint64_t> parts, toff(H);
  std::vector<uint8_t> tlog(H);
  std::vector<uint32_t> pages;
  uint64_t part = 0;
  for (int k = 0; k < K; ++k) {
    P.chunk_begin[k] = chunks.size();
    uint64_t slots = 0;  // the class's spill tables, back to back
    P.page_begin[k] = pages.size();
    for (size_t h = P.hub_begin[k]; h < P.hub_begin[k + 1]; ++h) {
      int lg = SPILL_PAGE_LOG;
      while ((uint64_t(1) << lg) < 2ull * degs[h]) ++lg;
      tlog[h] = uint8_t(lg);
      toff[h] = slots;
      slots += uint64_t(1) << lg;
      pages.insert(pages.end(), size_t(1) << (lg - SPILL_PAGE_LOG), uint32_t(h));
      first[h] = uint32_t(chunks.size());
      const uint32_t step = g->tuning.hub_chunk;
      for (uint32_t lo = 0; lo < degs[h]; lo += step) {
        chunks.push_back(make_uint4(uint32_t(h), lo, std::min<uint32_t>(degs[h], lo + step), verts[h]));
        parts.push_back(part + lo);
      }
      part += degs[h];
    }
    P.spill_slots = std::max<size_t>(P.spill_slots, slots);
    P.class_slots[k] = slots;
  }
  P.page_begin[K] = pages.size();
  P.chunk_begin[K] = chunks.size();
  first[H] = uint32_t(chunks.size());
  P.chunks = chunks.size();
  P.part = part;
  hb.hub_first.ensure(H + 1);
  hb.chunk.ensure(chunks.size());
  hb.chunk_part.ensure(chunks.size());
  hb.hub_toff.ensure(H);
  hb.hub_tlog.ensure(H);
  LVG_CUDA(cudaMemcpyAsync(hb.hub_toff.p, toff.data(), H * 8, cudaMemcpyHostToDevice, s));
  LVG_CUDA(cudaMemcpyAsync(hb.hub_tlog.p, tlog.data(), H, cudaMemcpyHostToDevice, s));
  hb.page_hub.ensure(pages.size());
  LVG_CUDA(cudaMemcpyAsync(hb.page_hub.p, pages.data(), pages.size() * 4, cudaMemcpyHostToDevice, s));
  LVG_CUDA(cudaMemcpyAsync(hb.hub_first.p, first.data(), (H + 1) * 4, cudaMemcpyHostToDevice, s));
  LVG_CUDA(cudaMemcpyAsync(hb.chunk.p, chunks.data(), chunks.size() * sizeof(uint4), cudaMemcpyHostToDevice, s));
  LVG_CUDA(cudaMemcpyAsync(hb.chunk_part.p, parts.data(), parts.size() * 8, cudaMemcpyHostToDevice, s));
  host_sync(g);
  P.hub_vertex = hb.hub_vertex.p;
  P.hub_first = hb.hub_first.p;
  P.chunk = hb.chunk.p;
  P.chunk_part = hb.chunk_part.p;
  P.hub_toff = hb.hub_toff.p;
  P.hub_tlog = hb.hub_tlog.p;
  P.page_hub = hb.page_hub.p;
}

// Colour classes of a run: the options' count, else 16 (deterministic), else
// the graph's tuned count for the frontier methods on batches of at most
// frontier_max_fraction entries per edge, else 16 for static Louvain (after
// its first iteration, see first_colors) and 8 for the others.
int colors_for(const lvg_options &o, int method, const lvg_tuning &t, size_t batch_entries = 0,
               size_t edges = 0) {
  int k = o.colors;
  if (k <= 0) {
    const bool small = double(batch_entries) <= t.frontier_max_fraction * double(edges);
    if (o.deterministic) k = DEFAULT_COLORS_SYNC;
    else if ((method == LVG_METHOD_FRONTIER || method == LVG_METHOD_DELTA) && small) k = t.frontier_colors;
    else if (method == LVG_METHOD_STATIC) k = STATIC_COLORS_ASYNC;
    else k = DEFAULT_COLORS_ASYNC;
  }
  return k < 1 ? 1 : (k > MAX_COLORS ? MAX_COLORS : k);
}

// Classes of the first iteration of the first pass (0: as the rest): static
// Louvain in asynchronous mode with the default count starts from singletons,
// where nearly every vertex moves at once and neighbours that decide
// together join each other's old communities; a finer first sweep keeps the
// reference's sequential quality.
int first_colors(const lvg_options &o, int method) {
  return method == LVG_METHOD_STATIC && !o.deterministic && o.colors <= 0 ? FIRST_COLORS_STATIC : 0;
}

// Static Louvain (it starts from singletons; a hub's neighbours stay in
// thousands of communities for several iterations, and the super-vertices of
// the next levels see thousands of neighbour communities too): the hubs whose
// chunks overflow are merged through spill tables (hub_spill_kernel), cleared
// here and left clear by the merge after each class. Scoped: the flag is
// dropped however the phase ends.
struct SpillScope {
  Workspace &W;
  SpillScope(lvg_graph *g, const Level &lv, bool on = true) : W(*g->ws) {
    if (!on || !lv.hub.hubs || !lv.hub.spill_slots) return;
    W.spill_keys.ensure(lv.hub.spill_slots);
    W.spill_vals.ensure(lv.hub.spill_slots);
    LVG_CUDA(cudaMemsetAsync(W.spill_keys.p, 0xFF, lv.hub.spill_slots * sizeof(uint32_t), g->stream));
    LVG_CUDA(cudaMemsetAsync(W.spill_vals.p, 0, lv.hub.spill_slots * sizeof(float), g->stream));
    W.spill_now = true;
  }
  ~SpillScope() { W.spill_now = false; }
};

// Degree bins and hub plan of the uploaded level for k colour classes.
void set_base_colors(lvg_graph *g, int k) {
  if (g->base.colors == k && g->base.lim == bin_limits_of(g->tuning)) return;
  compute_bins(g, g->base, g->deg.p, g->bins.p, g->ws->binscratch.p, k);
  build_hub_plan(g, g->base, g->hubplan);
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
// ------------------------------------------------------- resident hub tables

// The uploaded level's hubs in id order and the vertex -> hub index map, for
// the current graph version. The hubs are the hub plan's (degree bin 11, any
// colour class); their degrees size the build's scratch tables.
void ensure_hub_index(lvg_graph *g) {
  if (g->hub_index_version == g->version) return;
  cudaStream_t s = g->stream;
  const HubPlan &P = g->base.hub;
  const size_t H = P.hubs;
  std::vector<uint32_t> ids(H), degs(H);
  if (H) {
    DBuf<uint32_t> d;
    d.ensure(H);
    launch_gather_u32(P.hub_vertex, H, g->base.deg, d.p, s);
    LVG_CUDA(cudaMemcpyAsync(ids.data(), P.hub_vertex, H * 4, cudaMemcpyDeviceToHost, s));
    LVG_CUDA(cudaMemcpyAsync(degs.data(), d.p, H * 4, cudaMemcpyDeviceToHost, s));
    host_sync(g);
    std::vector<size_t> ord(H);
    for (size_t i = 0; i < H; ++i) ord[i] = i;
    std::sort(ord.begin(), ord.end(), [&](size_t a, size_t b) { return ids[a] < ids[b]; });
    std::vector<uint32_t> si(H), sd(H);
    for (size_t i = 0; i < H; ++i) { si[i] = ids[ord[i]]; sd[i] = degs[ord[i]]; }
    ids.swap(si);
    degs.swap(sd);
  }
  g->hub_deg_h = degs;
  if (ids != g->hub_ids_h || !g->hub_slot.p) {
    const size_t S = g->base.span;
    g->hub_slot.ensure(S);
    LVG_CUDA(cudaMemsetAsync(g->hub_slot.p, 0xFF, S * sizeof(uint32_t), s));
    if (H) {
      g->hub_ids.ensure(H);
      LVG_CUDA(cudaMemcpyAsync(g->hub_ids.p, ids.data(), H * 4, cudaMemcpyHostToDevice, s));
      launch_ht_slots(g->hub_ids.p, H, g->hub_slot.p, s);
    }
    host_sync(g);  // ids is freed next
    g->hub_ids_h.swap(ids);
    ++g->hub_index_gen;
  }
  g->hub_index_version = g->version;
}

// Largest table of a hub: a hub with more than a quarter of this many
// neighbour communities keeps scanning its edges.
constexpr int HT_MAX_LOG = 16;

// Hub tables T of membership q on the current graph version: every hub's
// neighbours counted per community into a scratch table (at least twice its
// degree in slots), the distinct communities counted, then each hub's table
// laid out with four times that many slots (at least 64) and filled.
void build_hub_tables(lvg_graph *g, const uint32_t *q, HubTables &T) {
  ensure_hub_index(g);
  Workspace &W = *g->ws;
  cudaStream_t s = g->stream;
  const size_t H = g->hub_ids_h.size();
  T.hubs = H;
  T.slots = 0;
  if (H) {
    std::vector<uint64_t> soff(H + 1, 0);
    std::vector<uint8_t> slg(H);
    for (size_t h = 0; h < H; ++h) {
      int l = 1;
      while ((uint64_t(1) << l) < 2ull * g->hub_deg_h[h]) ++l;
      slg[h] = uint8_t(l);
      soff[h + 1] = soff[h] + (uint64_t(1) << l);
    }
    const size_t stotal = soff[H];
    W.ht_soff.ensure(H + 1);
    W.ht_slg.ensure(H);
    W.ht_skey.ensure(stotal);
    W.ht_scnt.ensure(stotal);
    W.ht_n.ensure(H);
    LVG_CUDA(cudaMemcpyAsync(W.ht_soff.p, soff.data(), (H + 1) * 8, cudaMemcpyHostToDevice, s));
    LVG_CUDA(cudaMemcpyAsync(W.ht_slg.p, slg.data(), H, cudaMemcpyHostToDevice, s));
    LVG_CUDA(cudaMemsetAsync(W.ht_skey.p, 0xFF, stotal * 4, s));
    LVG_CUDA(cudaMemsetAsync(W.ht_scnt.p, 0, stotal * 4, s));
    launch_ht_scratch(g->base, q, g->hub_slot.p, W.ht_soff.p, W.ht_slg.p, W.ht_skey.p, W.ht_scnt.p, g->ctr.p, s);
    launch_ht_count(H, W.ht_soff.p, W.ht_slg.p, W.ht_skey.p, W.ht_n.p, s);
    std::vector<uint32_t> n(H);
    LVG_CUDA(cudaMemcpyAsync(n.data(), W.ht_n.p, H * 4, cudaMemcpyDeviceToHost, s));
    host_sync(g);
    std::vector<uint64_t> off(H + 1, 0);
    std::vector<uint8_t> lg(H), bad(H, 0);
    for (size_t h = 0; h < H; ++h) {
      int l = 6;
      while ((uint64_t(1) << l) < 4ull * n[h]) ++l;
      if (l > HT_MAX_LOG) {  // too many communities: this hub scans its edges
        l = 1;
        bad[h] = 1;
      }
      lg[h] = uint8_t(l);
      off[h + 1] = off[h] + (uint64_t(1) << l);
    }
    T.slots = off[H];
    AcctScope owner(T.acct ? T.acct : acct_target());  // the tables' own buffers
    T.off.ensure(H + 1);
    T.lg.ensure(H);
    T.bad.ensure(H);
    T.nbad.ensure(1);
    uint32_t nb = 0;
    for (size_t h = 0; h < H; ++h) nb += bad[h];
    LVG_CUDA(cudaMemcpyAsync(T.nbad.p, &nb, 4, cudaMemcpyHostToDevice, s));
    T.key.ensure(T.slots);
    T.cnt.ensure(T.slots);
    LVG_CUDA(cudaMemcpyAsync(T.off.p, off.data(), (H + 1) * 8, cudaMemcpyHostToDevice, s));
    LVG_CUDA(cudaMemcpyAsync(T.lg.p, lg.data(), H, cudaMemcpyHostToDevice, s));
    LVG_CUDA(cudaMemcpyAsync(T.bad.p, bad.data(), H, cudaMemcpyHostToDevice, s));
    LVG_CUDA(cudaMemsetAsync(T.key.p, 0xFF, T.slots * 4, s));
    LVG_CUDA(cudaMemsetAsync(T.cnt.p, 0, T.slots * 4, s));
    launch_ht_fill(H, W.ht_soff.p, W.ht_slg.p, W.ht_skey.p, W.ht_scnt.p, T.view(g->hub_slot.p), s);
    host_sync(g);  // the host arrays above are freed next
  }
  T.version = g->version;
  T.index = g->hub_index_gen;
}

// dst := src (same graph).
void copy_hub_tables(lvg_graph *g, const HubTables &src, HubTables &dst) {
  cudaStream_t s = g->stream;
  const size_t H = src.hubs;
  dst.hubs = H;
  dst.slots = src.slots;
  if (H) {
    AcctScope owner(dst.acct ? dst.acct : acct_target());
    dst.off.ensure(H + 1);
    dst.lg.ensure(H);
    dst.bad.ensure(H);
    dst.nbad.ensure(1);
    LVG_CUDA(cudaMemcpyAsync(dst.nbad.p, src.nbad.p, 4, cudaMemcpyDeviceToDevice, s));
    dst.key.ensure(src.slots);
    dst.cnt.ensure(src.slots);
    LVG_CUDA(cudaMemcpyAsync(dst.off.p, src.off.p, (H + 1) * 8, cudaMemcpyDeviceToDevice, s));
    LVG_CUDA(cudaMemcpyAsync(dst.lg.p, src.lg.p, H, cudaMemcpyDeviceToDevice, s));
    LVG_CUDA(cudaMemcpyAsync(dst.bad.p, src.bad.p, H, cudaMemcpyDeviceToDevice, s));
    LVG_CUDA(cudaMemcpyAsync(dst.key.p, src.key.p, src.slots * 4, cudaMemcpyDeviceToDevice, s));
    LVG_CUDA(cudaMemcpyAsync(dst.cnt.p, src.cnt.p, src.slots * 4, cudaMemcpyDeviceToDevice, s));
  }
  dst.version = src.version;
  dst.index = src.index;
}

// The tables the first pass keeps up to date while it is enqueued (scoped:
// cleared however the pass ends).
struct HubTabScope {
  Workspace &W;
  HubTabScope(lvg_graph *g, const HubTables *t) : W(*g->ws) {
    W.ht_now = t && t->hubs ? t->view(g->hub_slot.p) : HubTabView{};
  }
  ~HubTabScope() { W.ht_now = HubTabView{}; }
};

int bin_stream(int b) { return b <= 4 ? 0 : b <= 8 ? 1 : b == 9 ? 2 : b == 10 ? 3 : -1; }

void enqueue_iteration(lvg_graph *g, const Level &lv, uint32_t *com, tot_t *ctot, const tot_t *tot,
                       const uint8_t *fa, float kr, bool sync, int fused, const int *glog2, const size_t *goff,
                       size_t need, std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> *bin_ev,
                       const UnionCall *uc, bool read_back = true, bool clear_pre = true) {
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
  launch_iter_begin(&g->ctr.p->el_fix, W.wl_count.p, K * NUM_BINS, s);
  for (int k = 0; k < K; ++k) {
    // this class's active vertices of bins 1..NUM_BINS-2 -> worklists
    BinBounds bb;
    for (int b = 0; b <= NUM_BINS; ++b) bb.start[b] = lv.bin_start[k * NUM_BINS + b];
    uint32_t *wlc = W.wl_count.p + size_t(k) * NUM_BINS;
    if (bb.start[NUM_BINS - 1] > bb.start[1]) {
      if (K == 1 && !uc) launch_compact_active_scan(lv, bb, W.vaff.p, fa, W.wl.p, wlc, g->ctr.p, s);
      else launch_compact_active(lv.bins, bb, W.vaff.p, fa, W.wl.p, wlc, s, uc ? lv.gid : nullptr, uc ? uc->gact : nullptr);
    }
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
        a.kr = kr; a.ctr = g->ctr.p; a.unit = lv.unit; a.bin = grp.first;
        a.ht = W.ht_now;
        set_union(a);
        cudaEvent_t b0 = bin_ev ? g->events.record(s) : nullptr;
        launch_move_small(grp.first, grp.second, sync, a, sb, stream_of(grp.first), g->tuning.small_regs);
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
      a.kr = kr; a.ctr = g->ctr.p; a.unit = lv.unit; a.bin = b;
      a.gkeys = need ? W.gkeys.p + goff[b] : nullptr;
      a.gvals = need ? W.gvals.p + goff[b] : nullptr;
      a.glog2 = glog2[b];
      a.big_cap = g->tuning.big_blocks_per_sm;
      a.big_direct = W.first_sweep;
      a.ht = W.ht_now;
      set_union(a);
      cudaEvent_t b0 = bin_ev ? g->events.record(s) : nullptr;
      if (b == NUM_BINS - 1) {
        a.hub = lv.hub;
        a.color = k;
        a.chunk_cnt = W.chunk_cnt.p;
        a.part_key = W.part_key.p;
        a.part_val = W.part_val.p;
        a.hub_kd = W.hub_kd.p;
        a.hub_over = W.hub_over.p;
        a.spill_keys = W.spill_now ? W.spill_keys.p : nullptr;
        a.spill_vals = W.spill_now ? W.spill_vals.p : nullptr;
        a.hub_best = W.hub_best.p;
        // (with resident tables the table kernel runs on its own side
        // stream beside the chunked pair, which only takes bad tables' hubs)
        launch_move_hubs(sync, a, s, conc ? g->aux[4] : nullptr);
      } else {
        launch_move_bin(b, sync, a, stream_of(b));
      }
      if (bin_ev) bin_ev->push_back({b, {b0, g->events.record(s)}});
      ++g->stats.move_launches;
    }
    if (conc) {  // join
      for (int i = 0; i < 5; ++i) {
        LVG_CUDA(cudaEventRecord(g->join_ev[i], g->aux[i]));
        LVG_CUDA(cudaStreamWaitEvent(s, g->join_ev[i], 0));
      }
    }
    if (sync) {
      if (W.ht_now.key)  // the hubs' tables follow the decided moves before they are applied
        launch_ht_sync_moves(lv, lv.bins + lv.color_begin(k), lv.color_end(k) - lv.color_begin(k), W.dec.p, com,
                             W.ht_now, g->ctr.p, s);
      launch_apply_moves(lv.bins + lv.color_begin(k), lv.color_end(k) - lv.color_begin(k), W.dec.p, com, ctot, tot, s);
      launch_merge_marks(W.vaff.p, W.mark.p, lv.span, s);
    }
  }
  // worklists filled while a dynamic-frontier batch was marked serve the
  // first iteration only (in a phase graph iter_end_kernel clears the flag)
  if (K == 1 && !uc && clear_pre) launch_fill_bytes(&g->ctr.p->pre_flag, 0, sizeof(unsigned int), s);
  if (uc) launch_iter_control(uc->n, uc->ctl, uc->gact, uc->fix, uc->M, uc->E, uc->L, g->ctr.p, s);
  if (read_back) LVG_CUDA(cudaMemcpyAsync(g->hctr.p, g->ctr.p, sizeof(Counters), cudaMemcpyDeviceToHost, s));
}

// The whole local-moving phase of the uploaded level as one graph: a
// conditional while node whose body is one iteration (as enqueue_iteration
// issues it) followed by iter_end_kernel, which evaluates the reference's
// stop test (el <= E, or L iterations; inc/louvain.hxx:588-609) on the device
// and sets the node's condition (for a graph union: while any graph is still
// moving, each graph's own test having run in iter_control_kernel). The loop
// is bounded by L whatever the kernels compute. A phase is then one graph
// launch and one synchronisation, instead of one of each per iteration. Any
// failure to build it leaves the per-iteration path in place for this handle.
struct PhaseGraph {
  cudaGraphExec_t exec = nullptr;
  unsigned long long nodes = 0, moves = 0;  // kernel launches (all, local-moving) of one iteration
};
PhaseGraph build_phase(lvg_graph *g, const Level &lv, uint32_t *com, tot_t *ctot, const tot_t *tot, const uint8_t *fa,
                       float kr, bool sync, int fused, const int *glog2, const size_t *goff, size_t need, double M,
                       double E, int L, const UnionCall *uc) {
  cudaStream_t s = g->stream;
  PhaseGraph pg;
  const unsigned long long l0 = launch_counter();
  const unsigned long long m0 = g->stats.move_launches;
  cudaGraph_t graph = nullptr;
  bool fine = cudaGraphCreate(&graph, 0) == cudaSuccess;
  cudaGraphConditionalHandle h{};
  cudaGraphNodeParams cp{};
  cudaGraphNode_t node = nullptr;
  if (fine) fine = cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault) == cudaSuccess;
  if (fine) {
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    fine = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp) == cudaSuccess;
  }
  if (fine) fine = cudaStreamBeginCaptureToGraph(s, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                                 cudaStreamCaptureModeThreadLocal) == cudaSuccess;
  if (fine) {
    try {
      enqueue_iteration(g, lv, com, ctot, tot, fa, kr, sync, fused, glog2, goff, need, nullptr, uc, false, false);
      launch_iter_end(g->ctr.p, M, E, L, uc != nullptr, h, s);
    } catch (const Error &) {
      fine = false;
    }
    cudaGraph_t body = nullptr;
    fine = cudaStreamEndCapture(s, &body) == cudaSuccess && fine;
  }
  pg.nodes = launch_counter() - l0;  // the iteration's kernels and the stop test
  pg.moves = g->stats.move_launches - m0;
  launch_counter() = l0;
  g->stats.move_launches = m0;
  if (!fine || cudaGraphInstantiate(&pg.exec, graph, 0) != cudaSuccess) {
    cudaGetLastError();
    pg.exec = nullptr;
  }
  if (graph) cudaGraphDestroy(graph);
  return pg;
}

// The whole local-moving phase of the uploaded level as one graph: a
// conditional while node whose body is one iteration (as enqueue_iteration
// issues it) followed by iter_end_kernel, which evaluates the reference's
// stop test (el <= E, or L iterations; inc/louvain.hxx:588-609) on the device
// and sets the node's condition (for a graph union: while any graph is still
// moving, each graph's own test having run in iter_control_kernel). The loop
// is bounded by L whatever the kernels compute. A phase is then one graph
// launch and one synchronisation, instead of one of each per iteration. Any
// failure to build it leaves the per-iteration path in place for this handle.
void capture_phase(lvg_graph *g, const Level &lv, uint32_t *com, tot_t *ctot, const tot_t *tot, const uint8_t *fa,
                   float kr, bool sync, int fused, const int *glog2, const size_t *goff, size_t need,
                   const IterKey &key, const UnionCall *uc) {
  if (g->phase_exec) {
    cudaGraphExecDestroy(g->phase_exec);
    g->phase_exec = nullptr;
  }
  const PhaseGraph pg = build_phase(g, lv, com, ctot, tot, fa, kr, sync, fused, glog2, goff, need, key.M, key.E,
                                    key.L, uc);
  g->phase_exec = pg.exec;
  if (!pg.exec) g->no_phase_graphs = true;
  else g->phase_key = key;
}

// The rest of an aggregated level's phase (after its first iteration, which
// ran eagerly and set every kernel's attributes) as one graph built for this
// call, launched once and dropped: the same loop and device-side stop test as
// the uploaded level's phase graph, so the level's remaining iterations cost
// one launch and one synchronisation instead of one of each per iteration
// (an aggregated level's kernels are short, and issuing every class's
// launches from the host each iteration took longer than running them).
// Returns false, having run nothing, when the graph could not be built.
bool run_level_phase(lvg_graph *g, const Level &lv, uint32_t *com, tot_t *ctot, const tot_t *tot, const uint8_t *fa,
                     float kr, bool sync, int fused, const int *glog2, const size_t *goff, size_t need, double M,
                     double E, int L, const UnionCall *uc, int &iters, double &el) {
  cudaStream_t s = g->stream;
  const PhaseGraph pg = build_phase(g, lv, com, ctot, tot, fa, kr, sync, fused, glog2, goff, need, M, E, L, uc);
  if (!pg.exec) {
    g->no_level_graphs = true;
    return false;
  }
  struct Drop {
    cudaGraphExec_t e;
    ~Drop() { cudaGraphExecDestroy(e); }
  } drop{pg.exec};
  launch_fill_bytes(&g->ctr.p->dev_iters, 0, sizeof(unsigned int), s);
  LVG_CUDA(cudaGraphLaunch(pg.exec, s));
  LVG_CUDA(cudaMemcpyAsync(g->hctr.p, g->ctr.p, sizeof(Counters), cudaMemcpyDeviceToHost, s));
  host_sync(g);
  if (g->hctr.p->err) read_counters(g);  // raises the device error
  iters = int(g->hctr.p->dev_iters);
  el = uc ? 0.0 : g->hctr.p->dev_el;
  launch_counter() += pg.nodes * unsigned(iters);
  g->stats.move_launches += pg.moves * unsigned(iters);
  ++g->stats.level_graphs;
  return true;
}

// Capture one iteration of the uploaded level into a CUDA graph (after an
// eager iteration, so every kernel's attributes are already set). A capture
// failure disables graphs for this handle; the eager path stays correct.
void capture_iteration(lvg_graph *g, const Level &lv, uint32_t *com, tot_t *ctot, const tot_t *tot,
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
// The raw outcome of move_phase: iterations run and the last iteration's el.
struct PhaseEnd {
  int l = 0;
  double el = 0;
};

// tail (optional): work to enqueue after the phase and before its one
// synchronisation when the phase runs as one graph; *tail_done tells whether
// it was.
int move_phase(lvg_graph *g, const Level &lv, uint32_t *com, tot_t *ctot, const tot_t *tot, const uint8_t *fa,
               double M, float kr, int L, double E, bool sync, int fused, const UnionCall *uc = nullptr,
               bool iso_clear = false, PhaseEnd *end = nullptr, bool capture = true,
               const std::function<void()> *tail = nullptr, bool *tail_done = nullptr) {
  if (tail_done) *tail_done = false;
  Workspace &W = *g->ws;
  cudaStream_t s = g->stream;
  const int K = lv.colors;
  // Existing degree-0 vertices are processed once and never re-marked: their
  // flags are cleared here (the dynamic-frontier first pass: df_start_kernel
  // left them unmarked, iso_clear).
  if (!iso_clear) {
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
    need += size_t(move_grid_blocks(b, sync, lv.unit, most, g->tuning.big_blocks_per_sm)) << glog2[b];
  }
  if (need) {
    W.gkeys.ensure(need);
    W.gvals.ensure(need);
  }
  if (lv.hub.hubs) {
    W.chunk_cnt.ensure(lv.hub.chunks);
    W.part_key.ensure(lv.hub.part);
    W.part_val.ensure(lv.hub.part);
    if (W.hub_over.n < lv.hub.hubs) {  // the merge resets each mark it reads
      W.hub_over.ensure(lv.hub.hubs);
      LVG_CUDA(cudaMemsetAsync(W.hub_over.p, 0, W.hub_over.n, s));
      W.hub_best.ensure(lv.hub.hubs);
      LVG_CUDA(cudaMemsetAsync(W.hub_best.p, 0, W.hub_best.n * 8, s));
    }
  }
  const bool base = lv.off == g->base.off;
  IterKey key{};
  if (base) {
    const void *ps[34] = {W.spill_now ? W.spill_keys.p : nullptr, lv.off, lv.bins, com, ctot, tot, fa, W.vaff.p,
                          W.mark.p, W.dec.p, W.wl.p, W.wl_count.p,
                          W.gkeys.p, W.gvals.p, W.chunk_cnt.p, W.part_key.p, W.part_val.p, W.hub_kd.p, g->ctr.p,
                          g->hctr.p, lv.hub.chunk, lv.hub.hub_vertex, lv.gid,
                          W.spill_now ? W.spill_vals.p : nullptr, W.hub_over.p, W.hub_best.p, lv.deg,
                          // every buffer of the resident hub tables (a state's tables are
                          // separate allocations: one may move while the others stay)
                          W.ht_now.key, W.ht_now.slot, W.ht_now.cnt, W.ht_now.off, W.ht_now.nbad,
                          W.ht_now.lg, W.ht_now.bad};
    std::memcpy(key.p, ps, sizeof(ps));
    key.n[0] = lv.span; key.n[1] = need; key.n[2] = lv.hub.chunks; key.n[3] = lv.bin_start[K * NUM_BINS];
    key.k[0] = K; key.k[1] = sync | int(lv.unit) << 1; key.k[2] = glog2[9] | glog2[10] << 8 | glog2[11] << 16;
    key.k[3] = fused;
    key.kr = kr;
    key.E = E;
    key.M = M;
    key.L = L;
  }
  const bool graphs = base && capture && !g->profiling && !g->no_graphs;
  const bool phase_graphs = graphs && !g->no_phase_graphs && L > 0;
  // an aggregated level, or the uploaded level on a call that has no phase
  // graph to replay yet: its iterations after the first as one graph built
  // for this call (the uploaded level's phase graph for later calls is
  // captured at the end)
  const bool level_graphs = (!base || phase_graphs) && capture && !g->profiling && !g->no_graphs &&
                            !g->no_level_graphs && g->tuning.level_graphs;
  // Graphs of the uploaded level are captured only for a key that the
  // previous call on the handle had too: a call after a batch apply (whose
  // degrees and bins change the key) would build graphs that no call replays,
  // as a serving loop that applies and runs in turn would on every request.
  const bool key_again = base && g->key_seen && g->seen_key == key;
  if (base) {
    g->seen_key = key;
    g->key_seen = true;
  }
  int l = 0;
  double el = 0;
  if (phase_graphs && g->phase_exec && g->phase_key == key) {
    launch_fill_bytes(&g->ctr.p->dev_iters, 0, sizeof(unsigned int), s);
    LVG_CUDA(cudaGraphLaunch(g->phase_exec, s));
    LVG_CUDA(cudaMemcpyAsync(g->hctr.p, g->ctr.p, sizeof(Counters), cudaMemcpyDeviceToHost, s));
    if (tail) {
      (*tail)();
      if (tail_done) *tail_done = true;
    }
    host_sync(g);
    if (g->hctr.p->err) read_counters(g);  // raises the device error
    l = int(g->hctr.p->dev_iters);
    el = uc ? 0.0 : g->hctr.p->dev_el;  // graph unions: each graph's el is in its GraphCtl
    launch_counter() += (g->iter_nodes + 1) * unsigned(l);
    g->stats.move_launches += g->iter_moves * unsigned(l);
    if (end) { end->l = l; end->el = el; }
    return (l > 1 || el != 0) ? l : 0;
  }
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
    host_sync(g);
    if (g->hctr.p->err) read_counters(g);  // raises the device error
    if (g->profiling) {
      g->stats.move_kernel_ms += elapsed(e0, e1);
      for (auto &be : bin_ev) g->stats.move_bin_ms[be.first] += elapsed(be.second.first, be.second.second);
    }
    if (graphs && !replay && key_again)
      capture_iteration(g, lv, com, ctot, tot, fa, kr, sync, fused, glog2, goff, need, key, uc);
    ++l;
    if (uc) {  // each graph ran its own stop test (iter_control_kernel)
      if (g->hctr.p->gactive == 0) break;
    } else {
      el = double(g->hctr.p->el_fix) / GAIN_FIX / M;
      if (el <= E) break;
    }
    if (level_graphs && l == 1 && l < L) {
      int more = 0;
      if (run_level_phase(g, lv, com, ctot, tot, fa, kr, sync, fused, glog2, goff, need, M, E, L - l, uc, more,
                          el)) {
        l += more;
        break;
      }
    }
  }
  // next time, the whole phase as one graph (every kernel's attributes are set
  // by now)
  if (phase_graphs && key_again && !(g->phase_exec && g->phase_key == key))
    capture_phase(g, lv, com, ctot, tot, fa, kr, sync, fused, glog2, goff, need, key, uc);
  if (end) { end->l = l; end->el = el; }
  return (l > 1 || el != 0) ? l : 0;
}

// ---------------------------------------------------------------- aggregation

// Renumbered membership `com` of level `lv` with CN communities -> next level
// in buffer set `which` (louvainCommunityVerticesOmpW + louvainAggregateOmpW,
// inc/louvain.hxx:1197-1203). Also writes the new level's vertex weights.
Level aggregate(lvg_graph *g, const Level &lv, const uint32_t *com, size_t CN, int which, int colors,
                const uint32_t *ngid, const uint32_t *ngbase) {
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
  // Empty communities never reach a kernel: zero their rows first.
  LVG_CUDA(cudaMemsetAsync(nl.deg, 0, CN * sizeof(uint32_t), s));
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
    a.ctr = g->ctr.p; a.cn = uint32_t(CN);
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
    host_sync(g);
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
    a.ctr = g->ctr.p; a.cn = uint32_t(CN);
    a.gkeys = nullptr; a.gvals = nullptr; a.glog2 = 0;
    AggChunks ch{W.agg_chunk.p, list, W.agg_toff.p, W.agg_tlog.p, W.mpre.p, W.agg_gk.p, W.agg_gv.p, uint32_t(n11)};
    launch_aggregate_chunks(a, ch, chunks.size(), slots, s);
    g->stats.aggregate_launches += 2;
    host_sync(g);  // the host vectors above are freed next
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


// Whether a method's first pass evaluates the hubs from resident tables: the
// delta-screening and dynamic-frontier methods on a unit-weight graph, when
// the tuning keeps them. Naive-dynamic processes every vertex, and millions
// of them move: each move's updates of its hub neighbours' tables then cost
// more than the scans they save (R-MAT s24 at 1e-3 |E|: 10.6 ms with tables,
// 9.6 without).
bool uses_hub_tables(const lvg_graph *g, int method) {
  return (method == LVG_METHOD_DELTA || method == LVG_METHOD_FRONTIER) && g->tuning.hub_tables && g->base.unit;
}

// One call of a method. prior: device prior state (dynamic methods);
// out: where the first level's membership/weights and final totals live.
// on_init (optional) is called once, in the last repetition, with an event
// recorded when the first level's vertex weights (out.vt) are final.
void run(lvg_graph *g, int method, const DBatch &b, StateRef prior, StateRef out, const lvg_options &o,
         RunInfo &info, const std::function<void(cudaEvent_t)> *on_init, HubTables *tprior, HubTables *tout,
         bool vt_ready) {
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
  const int K1 = first_colors(o, method);
  uint32_t *ucom = out.q;
  tot_t *utot = out.vt, *ctot = out.ct;
  g->stats = lvg_stats{};
  const unsigned long long launches0 = launch_counter();
  launch_fill_bytes(g->ctr.p, 0, sizeof(Counters), s);
  // resident hub tables: the dynamic methods on a unit-weight graph, between
  // two states (lvg_run_resident)
  const bool tabs0 = tprior && tout && uses_hub_tables(g, method);
  int l = 0, p = 0;
  for (int r = 0; r < rep; ++r) {
    g->events.reset();
    set_base_colors(g, K1 ? K1 : K);
    // Reset the flags, as the reference does before each repetition (the
    // aggregated levels' membership and weights need no reset:
    // Workspace::allocate).
    launch_fill_bytes(W.vaff.p, 0, S, s);
    // The prior state into place: the reference moves its copies of it
    // (louvainSetupInitialsW, inc/louvain.hxx:1240) in without copying, so
    // the copy stays outside the timed section as its copies do.
    if (method != LVG_METHOD_STATIC) {
      if (prior.q != ucom) LVG_CUDA(cudaMemcpyAsync(ucom, prior.q, S * 4, cudaMemcpyDeviceToDevice, s));
      if (prior.vt != utot)
        LVG_CUDA(cudaMemcpyAsync(utot, prior.vt, S * sizeof(tot_t), cudaMemcpyDeviceToDevice, s));
      if (prior.ct != ctot)
        LVG_CUDA(cudaMemcpyAsync(ctot, prior.ct, S * sizeof(tot_t), cudaMemcpyDeviceToDevice, s));
    }
    // The prior's hub tables into the result state, like its membership and
    // weights: as they are when they describe this graph version; plus this
    // run's batch when they describe the version before it and the batch is
    // the one that made this version; else built (in the timed section) from
    // the prior membership.
    const bool tabs = tabs0 && g->base.hub.hubs > 0;
    int ht_mode = 0;  // 1 copied, 2 copied + the batch's edges, 3 built
    if (tabs) {
      ensure_hub_index(g);
      const bool same_hubs = tprior->index == g->hub_index_gen;
      if (same_hubs && tprior->version == g->version) ht_mode = 1;
      else if (same_hubs && tprior->version != ~0ull && tprior->version + 1 == g->version &&
               b.applied_version == g->version)
        ht_mode = 2;
      else ht_mode = 3;
      if (ht_mode <= 2 && tprior != tout) copy_hub_tables(g, *tprior, *tout);
    }
    cudaEvent_t e0 = g->events.record(s);
    if (ht_mode == 2) {
      const HubTabView v = tout->view(g->hub_slot.p);
      launch_ht_batch(b.ds, b.dd, b.nd, false, ucom, v, g->ctr.p, s);
      launch_ht_batch(b.is, b.id, b.ni, true, ucom, v, g->ctr.p, s);
      tout->version = g->version;
    } else if (ht_mode == 3) {
      build_hub_tables(g, ucom, *tout);
      if (tprior != tout) copy_hub_tables(g, *tout, *tprior);  // the prior's own cache, before any move
      g->stats.hub_tables_built = 1;
    }
    // the vertex weights' side of the batch update, unless the caller made it
    // (vt_ready: one run, its prior's weights updated before it started)
    tot_t *vt_upd = vt_ready && r == 0 ? nullptr : utot;
    // fi: initial membership and weights. Dynamic frontier: fm (the marking)
    // runs in the same pass over the batch (df_start_kernel; its time counts
    // as initialisation), and with one colour class it also lists the marked
    // vertices for the first iteration.
    if (method == LVG_METHOD_STATIC) {
      launch_init_static(g->base, ucom, utot, ctot, s);
    } else if (method == LVG_METHOD_FRONTIER) {
      BinBounds bb{};
      const bool lists = K == 1 && g->base.colors == 1;
      if (lists)
        for (int x = 0; x <= NUM_BINS; ++x) bb.start[x] = g->base.bin_start[x];
      launch_df_start(b.ds, b.dd, b.dw, b.nd, b.is, b.id, b.iw, b.ni, ucom, vt_upd, ctot, g->base, W.vaff.p,
                      lists ? &bb : nullptr, W.wl.p, g->ctr.p, s);
    } else {
      launch_batch_weights(b.ds, b.dw, b.nd, -1.f, ucom, vt_upd, ctot, s);
      launch_batch_weights(b.is, b.iw, b.ni, +1.f, ucom, vt_upd, ctot, s);
    }
    cudaEvent_t e1 = g->events.record(s);
    if (on_init && r == rep - 1) (*on_init)(e1);
    // fm: mark affected vertices.
    const uint8_t *fa = nullptr;
    if (method == LVG_METHOD_STATIC || method == LVG_METHOD_NAIVE) {
      LVG_CUDA(cudaMemsetAsync(W.vaff.p, 1, S, s));
    } else if (method == LVG_METHOD_FRONTIER) {
      // marked by df_start_kernel
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
    const tot_t *tot = utot;
    int which = 0;
    bool ended_by_tail = false;
    for (l = 0, p = 0; M > 0 && P > 0;) {
      if (p == 1) ep1 = g->events.record(s);
      const bool first = p == 0;
      cudaEvent_t a0 = g->events.record(s);
      // the frontier methods' first pass: the small degree bins go in two
      // fused launches per class, with blocks per SM and bin for DF's short
      // worklists (2) or for delta-screening's whole communities (8: with
      // two, its first pass took 2.8x as long on a 4M-vertex graph of
      // average degree 87)
      const int tf = g->tuning.fused_small;
      const int fused = !first || !tf || (method != LVG_METHOD_FRONTIER && method != LVG_METHOD_DELTA) ? 0
                        : tf >= 2                        ? tf
                        : method == LVG_METHOD_FRONTIER  ? 2
                                                         : 8;
      const bool ends = first && method == LVG_METHOD_FRONTIER;  // df_start_kernel left isolated ones unmarked
      // the end of the run, enqueued ahead of the first pass's one
      // synchronisation: if the run ends after this pass (as a frontier run
      // on a small batch does), it needs no other synchronisation
      cudaEvent_t tail_ev = nullptr;
      const std::function<void()> tail = [&] {
        tail_ev = g->events.record(s);
        launch_count_flags(W.vaff.p, S, g->ctr.p, s);
        LVG_CUDA(cudaMemcpyAsync(g->hctr.p, g->ctr.p, sizeof(Counters), cudaMemcpyDeviceToHost, s));
      };
      bool tail_done = false;
      int m;
      if (first && K1 && K1 != K) {
        // the first iteration over K1 classes (not captured: it runs once per
        // call), the rest of the pass over K
        PhaseEnd e1, e2;
        {
          SpillScope spill(g, lv);
          W.first_sweep = true;
          try {
            move_phase(g, lv, com, ctot, tot, fa, M, kr, 1, E, sync, fused, nullptr, ends, &e1, false);
          } catch (...) {
            W.first_sweep = false;
            throw;
          }
          W.first_sweep = false;
        }
        set_base_colors(g, K);
        lv = g->base;
        if (e1.el <= E || L <= 1) {
          m = (e1.l > 1 || e1.el != 0) ? e1.l : 0;
        } else {
          SpillScope spill(g, lv);
          move_phase(g, lv, com, ctot, tot, fa, M, kr, L - 1, E, sync, fused, nullptr, ends, &e2);
          const int lt = 1 + e2.l;
          m = (lt > 1 || e2.el != 0) ? lt : 0;
        }
      } else {
        SpillScope spill(g, lv, method == LVG_METHOD_STATIC);
        HubTabScope hts(g, first && tabs ? tout : nullptr);  // kept up to date by the first pass's moves
        m = move_phase(g, lv, com, ctot, tot, first ? fa : nullptr, M, kr, L, E, sync, fused, nullptr, ends,
                       nullptr, true, first && r == rep - 1 ? &tail : nullptr, &tail_done);
      }
      tl_ev.push_back({a0, tail_done ? tail_ev : g->events.record(s)});
      l += std::max(m, 1);
      ++p;
      if (m <= 1 || p >= P) {
        ended_by_tail = tail_done;
        break;
      }
      const size_t GN = first ? g->base.order : lv.span;
      LVG_CUDA(cudaMemsetAsync(W.cext.p, 0, (lv.span + 1) * sizeof(uint32_t), s));
      launch_community_flags(lv, com, W.cext.p, s);
      exclusive_scan_u32(W.cext.p, W.cext.p, lv.span, &g->ctr.p->cn, W.scan32.p, s);
      read_counters(g);
      const size_t CN = g->hctr.p->cn;
      if (double(CN) / double(GN) >= o.aggregationTolerance) break;
      // the next level's vertex weights: the communities' FP64 totals
      launch_next_vertex_weights(W.cext.p, lv.span, &g->ctr.p->cn, ctot, W.vtot.p, s);
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
    cudaEvent_t eend = ended_by_tail ? tl_ev.back().second : g->events.record(s);
    if (!ended_by_tail) {
      if (r == rep - 1) {
        // the residual affected count (inc/louvain.hxx:1220), read with the
        // same synchronisation that ends the run
        launch_count_flags(W.vaff.p, S, g->ctr.p, s);
        LVG_CUDA(cudaMemcpyAsync(g->hctr.p, g->ctr.p, sizeof(Counters), cudaMemcpyDeviceToHost, s));
      }
      host_sync(g);
    }
    if (r == rep - 1 && g->hctr.p->err) read_counters(g);  // raises the device error
    // the result's hub tables describe its membership if no pass aggregated
    // (which relabels it) and none ran out of room (then they are rebuilt)
    if (tout && !(tabs && p <= 1 && !g->hctr.p->ht_over)) tout->version = ~0ull;
    info.ti += elapsed(e0, e1);
    info.tm += elapsed(e1, e2);
    info.tp += elapsed(e2, ep1 ? ep1 : eend);
    for (auto &pr : tl_ev) info.tl += elapsed(pr.first, pr.second);
    for (auto &pr : ta_ev) info.ta += elapsed(pr.first, pr.second);
    info.t += elapsed(e0, eend);
  }
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
  g->stats.hub_table_slots = g->hctr.p->ht_slots;
  g->stats.hub_table_overflow = g->hctr.p->ht_over;
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
  const int K1 = first_colors(o, LVG_METHOD_STATIC);
  {
    std::vector<float> kr(n);
    for (size_t i = 0; i < n; ++i) kr[i] = U.M[i] > 0 ? float(R / (2.0 * U.M[i])) : 0.f;
    U.kr.ensure(n);
    LVG_CUDA(cudaMemcpyAsync(U.kr.p, kr.data(), n * sizeof(float), cudaMemcpyHostToDevice, s));
    host_sync(g);
  }
  U.fix.ensure(n); U.ctl.ensure(n); U.hctl.ensure(n); U.gact.ensure(n);
  U.gid[0].ensure(S); U.gid[1].ensure(S); U.gbase[0].ensure(n + 1); U.gbase[1].ensure(n + 1);
  U.aggex.ensure(S); U.q.ensure(S); U.ct.ensure(S); U.aff.ensure(S);
  uint32_t *ucom = W.ucom.p;
  tot_t *utot = W.utot.p, *ctot = W.ctot.p;
  g->stats = lvg_stats{};
  const unsigned long long launches0 = launch_counter();
  LVG_CUDA(cudaMemsetAsync(g->ctr.p, 0, sizeof(Counters), s));
  const UnionCall uc0{n, U.kr.p, U.fix.p, U.gact.p, U.ctl.p, U.Md.p, 0.0, L};
  for (int r = 0; r < rep; ++r) {
    g->events.reset();
    set_base_colors(g, K1 ? K1 : K);
    LVG_CUDA(cudaMemsetAsync(W.vaff.p, 0, S, s));
    LVG_CUDA(cudaMemsetAsync(W.vcom.p, 0, S * sizeof(uint32_t), s));
    LVG_CUDA(cudaMemsetAsync(W.vtot.p, 0, S * sizeof(tot_t), s));
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
    const tot_t *tot = utot;
    int which = 0;
    for (int p = 0;; ++p) {
      if (p == 1) ep1 = g->events.record(s);
      const bool first = p == 0;
      launch_pass_begin(n, U.ctl.p, U.gact.p, s);
      UnionCall uc = uc0;
      uc.E = E;
      cudaEvent_t a0 = g->events.record(s);
      if (first && K1 && K1 != K) {
        // as run(): the first iteration over K1 classes, the rest over K (each
        // graph's iteration count and stop test carry on on the device)
        {
          SpillScope spill(g, lv);
          W.first_sweep = true;
          try {
            move_phase(g, lv, com, ctot, tot, nullptr, 0.0, 0.f, 1, E, sync, 0, &uc, false, nullptr, false);
          } catch (...) {
            W.first_sweep = false;
            throw;
          }
          W.first_sweep = false;
        }
        set_base_colors(g, K);
        lv = g->base;
        if (g->hctr.p->gactive && L > 1) {
          SpillScope spill(g, lv);
          move_phase(g, lv, com, ctot, tot, nullptr, 0.0, 0.f, L - 1, E, sync, 0, &uc);
        }
      } else {
        SpillScope spill(g, lv);
        move_phase(g, lv, com, ctot, tot, nullptr, 0.0, 0.f, L, E, sync, 0, &uc);
      }
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
      launch_next_vertex_weights(W.cext.p, lv.span, &g->ctr.p->cn, ctot, W.vtot.p, s);
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
    host_sync(g);
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
  LVG_CUDA(cudaMemcpyAsync(out->membership, st.q, S * 4, cudaMemcpyDeviceToHost, s));
  if (!skip_vw) LVG_CUDA(cudaMemcpyAsync(out->vertexWeight, st.vt, S * sizeof(tot_t), cudaMemcpyDeviceToHost, s));
  LVG_CUDA(cudaMemcpyAsync(out->communityWeight, st.ct, S * sizeof(tot_t), cudaMemcpyDeviceToHost, s));
  LVG_CUDA(cudaStreamSynchronize(s));
}

// cq[k] (optional): cached memberships to compare the uploaded one with
// (g->hctr.p->qdiff[k] after the call).
void upload_prior(lvg_graph *g, const uint32_t *q, const double *qvtot, const double *qctot, uint32_t *dq,
                  tot_t *dvt, tot_t *dct, const uint32_t *const *cq) {
  cudaStream_t s = g->stream;
  const size_t S = g->base.span;
  if (!q || !qvtot || !qctot) throw Error(LVG_EINVAL, "prior state: null array");
  // the device keeps the totals in FP64, as the caller passes them (dvt
  // nullptr: the vertex weights were uploaded already)
  LVG_CUDA(cudaMemcpyAsync(dq, q, S * 4, cudaMemcpyHostToDevice, s));
  if (dvt) LVG_CUDA(cudaMemcpyAsync(dvt, qvtot, S * sizeof(tot_t), cudaMemcpyHostToDevice, s));
  LVG_CUDA(cudaMemcpyAsync(dct, qctot, S * sizeof(tot_t), cudaMemcpyHostToDevice, s));
  // every prior id must be < span (checked on the device; read back before any use)
  if (cq) launch_check_prior(dq, S, uint32_t(S), cq[0], cq[1], g->ctr.p, s);
  else launch_check_ids(dq, S, uint32_t(S), g->ctr.p, s);
  read_counters(g);
}

// The host-call table caches after a batch apply made graph version
// g->version from g->version - 1 with the tidied batch (ds, dd | is, id):
// a cache of the old version gets the batch's edges (each changes one
// neighbour count of a hub), as long as the set of hubs is the same; any
// other cache is dropped.
void advance_host_tables(lvg_graph *g, const uint32_t *ds, const uint32_t *dd, size_t nd, const uint32_t *is,
                         const uint32_t *id, size_t ni) {
  bool any = false;
  for (auto &e : g->htab) {
    if (e.t.version != ~0ull && e.t.version + 1 == g->version) any = true;
    else e.t.version = ~0ull;
  }
  if (!any) return;
  ensure_hub_index(g);
  cudaStream_t s = g->stream;
  for (auto &e : g->htab) {
    if (e.t.version == ~0ull) continue;
    if (e.t.index != g->hub_index_gen || e.t.hubs != g->hub_ids_h.size()) {
      e.t.version = ~0ull;
      continue;
    }
    const HubTabView v = e.t.view(g->hub_slot.p);
    launch_ht_batch(ds, dd, nd, false, e.q.p, v, g->ctr.p, s);
    launch_ht_batch(is, id, ni, true, e.q.p, v, g->ctr.p, s);
    e.t.version = g->version;
  }
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
    StateRef st{W.ucom.p, W.utot.p, W.ctot.p};
    StateRef prior{nullptr, nullptr, nullptr};
    // resident hub tables for a prior that comes from the host: those of a
    // cached membership equal to it (exactly: compared on the device with
    // the upload's id check), else built for it by the run into the least
    // recently used cache
    const bool tabs = opt.repeat <= 1 && uses_hub_tables(g, method) && g->base.hub.hubs > 0;
    HubTables *tprior = nullptr;
    int slot = -1;
    // The vertex weights of a dynamic run are the prior's plus the batch's
    // (louvainUpdateWeightsFromOmpU) and final from there on. Into a pinned
    // result array they are uploaded first, updated, and copied back on a
    // side stream while the rest of the prior uploads (the host link carries
    // both directions at once); their download is over before the run starts
    // (with it in flight, the local-moving phase took 0.70 ms instead of 0.13).
    cudaPointerAttributes pa{};
    const bool early = method != LVG_METHOD_STATIC && opt.repeat <= 1 && qvtot && out->vertexWeight &&
                       cudaPointerGetAttributes(&pa, out->vertexWeight) == cudaSuccess &&
                       pa.type == cudaMemoryTypeHost;
    cudaGetLastError();
    if (early) {
      for (auto &e : g->vt_ev)
        if (!e) LVG_CUDA(cudaEventCreate(&e));
      if (!g->copy_stream) LVG_CUDA(cudaStreamCreateWithFlags(&g->copy_stream, cudaStreamNonBlocking));
      LVG_CUDA(cudaMemcpyAsync(st.vt, qvtot, W.S * sizeof(tot_t), cudaMemcpyHostToDevice, g->stream));
      LVG_CUDA(cudaEventRecord(g->vt_ev[0], g->stream));
      launch_batch_weights(db.ds, db.dw, db.nd, -1.f, nullptr, st.vt, nullptr, g->stream);
      launch_batch_weights(db.is, db.iw, db.ni, +1.f, nullptr, st.vt, nullptr, g->stream);
      LVG_CUDA(cudaEventRecord(g->vt_ev[1], g->stream));
      LVG_CUDA(cudaStreamWaitEvent(g->copy_stream, g->vt_ev[1], 0));
      LVG_CUDA(cudaMemcpyAsync(out->vertexWeight, st.vt, W.S * sizeof(tot_t), cudaMemcpyDeviceToHost,
                               g->copy_stream));
    }
    if (method != LVG_METHOD_STATIC) {
      if (opt.repeat <= 1) {
        // one run: the prior goes straight where the run starts from
        const uint32_t *cq[2] = {nullptr, nullptr};
        if (tabs) {
          ensure_hub_index(g);
          for (int k = 0; k < 2; ++k) {
            const HubTables &t = g->htab[k].t;
            if (t.version == g->version && t.index == g->hub_index_gen && g->htab[k].q.n >= W.S)
              cq[k] = g->htab[k].q.p;
          }
        }
        upload_prior(g, q, qvtot, qctot, st.q, early ? nullptr : st.vt, st.ct, tabs ? cq : nullptr);
        prior = st;
        if (tabs) {
          for (int k = 0; k < 2; ++k)
            if (cq[k] && !g->hctr.p->qdiff[k]) slot = k;
          if (slot < 0) {  // the run builds the tables of this prior into the older cache
            slot = g->htab[0].stamp <= g->htab[1].stamp ? 0 : 1;
            g->htab[slot].q.ensure(W.S);
            LVG_CUDA(cudaMemcpyAsync(g->htab[slot].q.p, st.q, W.S * 4, cudaMemcpyDeviceToDevice, g->stream));
            g->htab[slot].t.version = ~0ull;
          }
          g->htab[slot].stamp = ++g->htab_clock;
          tprior = &g->htab[slot].t;
        }
      } else {  // every repetition starts from the same prior
        W.prior_q.ensure(W.S); W.prior_vt.ensure(W.S); W.prior_ct.ensure(W.S);
        upload_prior(g, q, qvtot, qctot, W.prior_q.p, W.prior_vt.p, W.prior_ct.p);
        prior = StateRef{W.prior_q.p, W.prior_vt.p, W.prior_ct.p};
      }
    }
    LVG_CUDA(cudaStreamSynchronize(g->stream));
    // the early weight download ends before the run's kernels start
    if (early) LVG_CUDA(cudaStreamSynchronize(g->copy_stream));
    const auto t1 = std::chrono::steady_clock::now();
    RunInfo info;
    run(g, method, db, prior, st, opt, info, nullptr, tprior, tabs ? &g->hwork : nullptr, early);
    if (early) {  // the weight update belongs to the run's initialisation
      const float vt_ms = elapsed(g->vt_ev[0], g->vt_ev[1]);
      info.t += vt_ms;
      info.ti += vt_ms;
    }
    if (tabs && g->hwork.version == g->version) {
      // the result's tables, in the other cache (the next call's prior is
      // often this result)
      auto &e = g->htab[1 - slot];
      e.q.ensure(W.S);
      LVG_CUDA(cudaMemcpyAsync(e.q.p, st.q, W.S * 4, cudaMemcpyDeviceToDevice, g->stream));
      copy_hub_tables(g, g->hwork, e.t);
      e.stamp = ++g->htab_clock;
    }
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
  launch_count_nonunit(cw, X, g->ctr.p, s);
  DBuf<uint32_t> scratch;
  scratch.ensure(bin_scratch_elems(span + 1, DEFAULT_COLORS_ASYNC));
  compute_bins(g, b, g->deg.p, g->bins.p, scratch.p, DEFAULT_COLORS_ASYNC);  // synchronises
  build_hub_plan(g, b, g->hubplan);
  read_counters(g);
  g->total_weight = g->hctr.p->fp64[0];
  b.unit = X > 0 && g->hctr.p->nonunit == 0;
}

// ---------------------------------------------------------------- batch apply

// The batch plan, on the device: each list packed as (src << b | dst) keys,
// stably sorted, the first of each run kept (tidyBatchUpdateU's sort +
// unique, inc/batch.hxx:169-192, keeping the first in batch order where the
// reference's unstable sort keeps an unspecified one) into g->u_ds.. /
// g->u_is.., and one UpdRow per touched source vertex into g->u_rows.

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
  ++g->version;  // every cache of the old edges (hub tables) is stale from here on
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
  if (b.unit && ni) {  // an insertion of another weight ends the unit-weight fast path
    LVG_CUDA(cudaMemsetAsync(&g->ctr.p->nonunit, 0, sizeof(unsigned long long), s));
    launch_count_nonunit(iw, ni, g->ctr.p, s);
    LVG_CUDA(cudaMemcpyAsync(&g->hctr.p->nonunit, &g->ctr.p->nonunit, sizeof(unsigned long long),
                             cudaMemcpyDeviceToHost, s));
  }
  if (ex) {
    launch_count_present(ex, b.span, g->upd.p, s);
    LVG_CUDA(cudaMemcpyAsync(g->hupd.p + UPD_ORDER, g->upd.p + UPD_ORDER, 8, cudaMemcpyDeviceToHost, s));
  }
  LVG_CUDA(cudaStreamSynchronize(s));
  if (b.unit && ni && g->hctr.p->nonunit) b.unit = false;
  b.edges = size_t((long long)b.edges + edge_delta);
  if (ex) b.order = g->hupd.p[UPD_ORDER];
  g->total_weight += wdelta;
  // degrees changed: new bins and hub plan; the captured iteration is stale
  drop_graphs(g);
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
  if (pc.nrows) advance_host_tables(g, tds, tdd, out.nd, tis, tid, out.ni);
  return out;
}

int fail_noalloc(int code, const char *msg) { return fail(code, msg); }

}  // namespace lvg
