// lvg_api.cu — the C-ABI entry points (include/louvain_gb300.h) over the
// device graph handles and the pass driver of lvg_driver.cu.
#include "lvg_driver.cuh"

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
    throw Error(LVG_EINVAL, "tuning: frontier_colors out of 1.." + std::to_string(MAX_COLORS));
  if (t.hub_chunk < 256 || t.hub_chunk > (1u << 20)) throw Error(LVG_EINVAL, "tuning: hub_chunk out of 256..2^20");
  if (t.big_blocks_per_sm < 0 || t.big_blocks_per_sm > 64) throw Error(LVG_EINVAL, "tuning: big_blocks_per_sm");
  if (!(t.frontier_max_fraction >= 0 && t.frontier_max_fraction <= 1))
    throw Error(LVG_EINVAL, "tuning: frontier_max_fraction out of 0..1");
  if (t.hub_tables != 0 && t.hub_tables != 1) throw Error(LVG_EINVAL, "tuning: hub_tables is 0 or 1");
  if (t.level_graphs != 0 && t.level_graphs != 1) throw Error(LVG_EINVAL, "tuning: level_graphs is 0 or 1");
  if (t.small_regs != 32 && t.small_regs != 64) throw Error(LVG_EINVAL, "tuning: small_regs is 32 or 64");
  if (t.fused_small < 0 || t.fused_small > 64) throw Error(LVG_EINVAL, "tuning: fused_small out of 0..64");
  if (t.bin_max_degree[0] || t.bin_max_degree[10] || t.bin_max_degree[11])
    throw Error(LVG_EINVAL, "tuning: bin_max_degree[0], [10] and [11] are 0");
  uint32_t prev = 0;
  for (int b = 1; b <= 10; ++b) {
    const uint32_t hi = t.bin_max_degree[b] ? t.bin_max_degree[b] : uint32_t(BIN_MAX_DEGREE[b]);
    if (hi > BIN_MAX_DEGREE[b] || hi < prev)
      throw Error(LVG_EINVAL, "tuning: bin_max_degree[" + std::to_string(b) + "] = " + std::to_string(hi) +
                                  " is beyond the bin's reach (" + std::to_string(BIN_MAX_DEGREE[b]) +
                                  ") or below the previous bin's limit (" + std::to_string(prev) + ")");
    prev = hi;
  }
}

// Set a graph's tuning: the hub plan of the uploaded level follows the chunk
// size, and a captured iteration (launch shapes baked in) is dropped.
void apply_tuning(lvg_graph *g, const lvg_tuning &t) {
  check_tuning(t);
  const bool chunks = t.hub_chunk != g->tuning.hub_chunk;
  const bool bins = !(bin_limits_of(t) == bin_limits_of(g->tuning));
  g->tuning = t;
  if (bins && g->base.bins) {  // the uploaded level regrouped by the new limits
    ensure_ws(g);
    compute_bins(g, g->base, g->deg.p, g->bins.p, g->ws->binscratch.p, g->base.colors);
  }
  if (chunks || bins) build_hub_plan(g, g->base, g->hubplan);
  drop_graphs(g);
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
    b.unit = x->base.unit;
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
    for (size_t i = 0; i < U.n; ++i) {
      lvg_result *r = &results[i];
      const size_t sp = U.vb[i + 1] - U.vb[i];
      if (!r->membership) { r->membership = (uint32_t *)std::malloc(sp * 4 + 1); r->owned |= 1; }
      if (!r->vertexWeight) { r->vertexWeight = (double *)std::malloc(sp * 8 + 1); r->owned |= 2; }
      if (!r->communityWeight) { r->communityWeight = (double *)std::malloc(sp * 8 + 1); r->owned |= 4; }
      if (!r->membership || !r->vertexWeight || !r->communityWeight) throw std::bad_alloc();
    }
    copy_out_slices(s, U.q.p, 4, U.vb, [&](size_t i) -> void * { return results[i].membership; });
    copy_out_slices(s, W.utot.p, sizeof(tot_t), U.vb, [&](size_t i) -> void * { return results[i].vertexWeight; });
    copy_out_slices(s, U.ct.p, sizeof(tot_t), U.vb, [&](size_t i) -> void * { return results[i].communityWeight; });
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
    lvg::drop_graphs(g);  // the captured iteration refers to the buffers released below
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
    // the host calls' hub-table caches (rebuilt by the next call that needs them)
    auto drop = [](lvg::HubTables &t) {
      t.off.release(); t.lg.release(); t.bad.release(); t.key.release(); t.cnt.release(); t.nbad.release();
      t.hubs = t.slots = 0;
      t.version = t.index = ~0ull;
    };
    for (auto &e : g->htab) {
      e.q.release();
      drop(e.t);
    }
    drop(g->hwork);
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
    st->ht.acct = &st->bytes;  // filled by calls on g, released with the state
    st->q.ensure(S); st->vt.ensure(S); st->ct.ensure(S);
    LVG_CUDA(cudaMemsetAsync(st->q.p, 0, S * 4, g->stream));
    LVG_CUDA(cudaMemsetAsync(st->vt.p, 0, S * sizeof(tot_t), g->stream));
    LVG_CUDA(cudaMemsetAsync(st->ct.p, 0, S * sizeof(tot_t), g->stream));
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
    st->ht.version = ~0ull;  // its hub tables described the old membership
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
    cudaStream_t s = g->stream;
    const size_t S = g->base.span;
    if (membership) LVG_CUDA(cudaMemcpyAsync(membership, st->q.p, S * 4, cudaMemcpyDeviceToHost, s));
    if (vtot) LVG_CUDA(cudaMemcpyAsync(vtot, st->vt.p, S * sizeof(tot_t), cudaMemcpyDeviceToHost, s));
    if (ctot) LVG_CUDA(cudaMemcpyAsync(ctot, st->ct.p, S * sizeof(tot_t), cudaMemcpyDeviceToHost, s));
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
    // the batch becomes the tidied batch (tidyBatchUpdateU's result), which
    // the dynamic methods then take, as main.cxx:108-125 does
    const lvg::DBatch &r = b->b;
    if (!(r.nd + r.ni)) {
      b->b.applied_version = g->version;
      b->applied = true;
      return LVG_OK;
    }
    // compacted over the batch's own arrays, which the plan has copied
    lvg::AcctScope acct_(&g->bytes);
    const lvg::PlanCounts t = lvg::tidy_apply(g, r.ds, r.dd, r.dw, r.nd, r.is, r.id, r.iw, r.ni, b->ds.p, b->dd.p,
                                              b->dw.p, b->is.p, b->id.p, b->iw.p);
    b->b.nd = t.nd;
    b->b.ni = t.ni;
    b->b.max_group = t.max_group;  // an upper bound after the filter
    b->b.applied_version = g->version;
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
    db->b.applied_version = ~0ull;
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
      else run(g, method, db, pr, st, opt, ri, nullptr, prior ? const_cast<HubTables *>(&prior->ht) : nullptr,
               &g->ht_tune);
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
    auto try_knob_list = [&](auto set, const std::vector<long> &values, bool guard) {
      for (long v : values) {
        lvg_tuning t = cur;
        set(t, v);
        if (!std::memcmp(&t, &cur, sizeof(t))) continue;
        try {  // e.g. a bin's full reach above a later bin's lowered limit
          check_tuning(t);
        } catch (const Error &) {
          continue;
        }
        double q = 0;
        const double tm = measure(t, guard ? &q : nullptr);
        if (tm < 0.98 * tcur && (!guard || q >= qref - 1e-3)) {
          cur = t;
          tcur = tm;
        }
      }
    };
    auto try_knob = [&](auto set, std::initializer_list<long> values, bool guard) {
      try_knob_list(set, std::vector<long>(values), guard);
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
      // fused: its blocks per SM and bin (the worklists' lengths vary with the
      // batch), and the degree <= 128 launch's register budget (32 registers
      // with spills and 8 blocks per SM, or 64 and 4)
      if (cur.fused_small) {
        try_knob([](lvg_tuning &t, long v) { t.fused_small = int(v); }, {1, 4, 8, 16}, false);
        try_knob([](lvg_tuning &t, long v) { t.small_regs = int(v); }, {32, 64}, false);
      }
      // the degree from which a block per vertex (bin 9's kernel) serves —
      // every warp bin (6-8) reaching above it emptied into bin 9 — jointly
      // with the blocks per SM of those block kernels, since each one's best
      // value depends on the other (R-MAT s24 DF: degrees 129-512 took 46 us
      // as a warp per vertex and the step 0.178 ms, in bin 9's blocks 0.161 ms
      // with as many blocks as fit, but slower with 4 blocks per SM).
      // v = blocks per SM * 1024 + the degree (0: no bin emptied).
      {
        std::vector<long> vs;
        for (long bb : {0, 2, 3, 4})
          for (long from : {0, 256, 128, 64}) vs.push_back(bb * 1024 + from);
        try_knob_list(
            [](lvg_tuning &t, long v) {
              t.big_blocks_per_sm = int(v / 1024);
              const long from = v % 1024;
              for (int b = 6; b <= 8; ++b)
                t.bin_max_degree[b] = from && BIN_MAX_DEGREE[b] > uint64_t(from) ? uint32_t(from) : 0u;
            },
            vs, false);
      }
      // the degree bins: each bin at its full reach, at the previous bin's
      // reach, or emptied (all its degrees handed on to the next bin's wider
      // tile and larger table; after the previous bin was emptied too, a run
      // of bins goes to one kernel); bin 9 also split at 1024. Each candidate
      // is at least the previous bin's limit.
      for (int b = 2; b <= 9; ++b) {
        auto set = [b](lvg_tuning &t, long v) { t.bin_max_degree[b] = uint32_t(v); };
        const long prev = long(bin_limits_of(cur).hi[b - 1]);
        const long half = std::max(prev, long(BIN_MAX_DEGREE[b - 1]));
        if (b == 9) try_knob(set, {0, 1024, half, prev}, false);
        else try_knob(set, {0, half, prev}, false);
      }
      // aggregated levels' iterations as one graph launch per level, or
      // launched from the host iteration by iteration
      try_knob([](lvg_tuning &t, long v) { t.level_graphs = int(v); }, {1, 0}, false);
      // resident hub tables: a large saving where few vertices move (DF), a
      // cost where millions do (each move updates its hub neighbours' tables)
      if (prior && method != LVG_METHOD_STATIC)
        try_knob([](lvg_tuning &t, long v) { t.hub_tables = int(v); }, {1, 0}, false);
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
    // the prior's hub tables are a cache of its membership: filled, never changed in meaning
    lvg::HubTables *tp = prior ? const_cast<lvg::HubTables *>(&prior->ht) : nullptr;
    lvg::run(g, method, db, pr, st, opt, ri, nullptr, tp, &out->ht);
    if (info) lvg::fill_result(info, ri, g->base.span);
    return LVG_OK;
  });
}

}  // extern "C"
