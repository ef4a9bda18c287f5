// lvg_experiment.cpp — the reference's experiment driver (main.cxx) on the GPU
// library, with the reference's command line and log lines.
//
//   louvain_gb300_experiment <file> <rows> <size> <unused> <batchFraction>
//   louvain_gb300_experiment --drift <n> <communities> <edges> <seed> <batchFraction>
//
// As main.cxx:146-166 and runExperiment (main.cxx:60-135): read the first 90 %
// of the temporal edge lines as an undirected graph (readTemporalOmpW +
// symmetrizeOmp), run static Louvain on it, then for each of BATCH_LENGTH
// batches take the next batchFraction * size lines as insertions, tidy and
// apply them to a copy of the base graph (tidyBatchUpdateU +
// applyBatchUpdateOmpU, here in HBM), and run static, naive-dynamic,
// delta-screening and dynamic-frontier Louvain from the previous results,
// printing one line per run in main.cxx's format (main.cxx:77-85), which
// lvg_log.py turns into CSV as the reference's process.js does.
//
// --drift replaces the file by the synthetic temporal stream of
// lvgg_temporal_drift (log-normal communities that drift over time).
// Environment: BATCH_LENGTH (default 1), REPEAT_METHOD (default 5), as the
// reference's compile-time macros.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "louvain_gb300.h"
#include "louvain_gb300_graphgen.h"

namespace {

void log_prefix() {
  const std::time_t s = std::time(nullptr);
  const std::tm *t = std::localtime(&s);
  std::printf("%04d-%02d-%02d %02d:%02d:%02d", t->tm_year + 1900, t->tm_mon + 1, t->tm_mday, t->tm_hour, t->tm_min,
              t->tm_sec);
}

[[noreturn]] void die(const char *what, const char *msg) {
  // the libraries' messages may already open with the failing call's name
  const size_t n = std::strlen(what);
  if (std::strncmp(msg, what, n) == 0 && msg[n] == ':') std::fprintf(stderr, "%s\n", msg);
  else std::fprintf(stderr, "%s: %s\n", what, msg);
  std::exit(1);
}

void check(int rc, const char *what) {
  if (rc != LVG_OK) die(what, lvg_last_error());
}

int env_int(const char *name, int dflt) {
  const char *v = std::getenv(name);
  return v && *v ? std::atoi(v) : dflt;
}

// A host edge stream: a SNAP temporal file, or the synthetic drift stream.
struct Stream {
  lvgg_temporal *file = nullptr;
  lvgg_edges all{};  // the drift stream (undirected, one entry per line)
  size_t pos = 0;
  // The next `lines` lines, both directions (readTemporalDo with symmetric).
  void read(size_t lines, std::vector<uint32_t> &s, std::vector<uint32_t> &d, std::vector<float> &w) {
    s.clear(); d.clear(); w.clear();
    if (file) {
      lvgg_edges e{};
      if (lvgg_temporal_read(file, lines, 1, &e) != 0) die("lvgg_temporal_read", lvgg_last_error());
      s.assign(e.src, e.src + e.n); d.assign(e.dst, e.dst + e.n); w.assign(e.w, e.w + e.n);
      lvgg_edges_free(&e);
      return;
    }
    for (size_t i = 0; i < lines && pos < all.n; ++i, ++pos) {
      s.push_back(all.src[pos]); d.push_back(all.dst[pos]); w.push_back(all.w[pos]);
      s.push_back(all.dst[pos]); d.push_back(all.src[pos]); w.push_back(all.w[pos]);
    }
  }
};

struct Result {
  std::vector<uint32_t> m;
  std::vector<double> vt, ct;
  lvg_result r{};
};

double modularity(lvg_graph *g, const std::vector<uint32_t> &m, double M) {
  double q = 0;
  check(lvg_modularity(g, m.data(), M, 1.0, &q), "lvg_modularity");
  return q;
}

// main.cxx:77-85
void glog(const Result &a, const char *technique, int threads, lvg_graph *y, double M, double df, double inf) {
  std::printf(
      "{-%.3e/+%.3e batchf, %03d threads} -> "
      "{%09.1fms, %09.1fms mark, %09.1fms init, %09.1fms firstpass, %09.1fms locmove, %09.1fms aggr, %.3e aff, "
      "%04d iters, %03d passes, %01.9f modularity} %s\n",
      df, inf, threads, a.r.time, a.r.markingTime, a.r.initializationTime, a.r.firstPassTime, a.r.localMoveTime,
      a.r.aggregationTime, double(a.r.affectedVertices), a.r.iterations, a.r.passes, modularity(y, a.m, M),
      technique);
  std::fflush(stdout);
}

void print_graph(lvg_graph *g, const char *tail) {
  log_prefix();
  std::printf(" order: %zu size: %zu [directed] {}%s\n", lvg_graph_order(g), lvg_graph_size(g), tail);
}

Result run(int method, lvg_graph *y, const lvg_batch *b, const Result *prior, const lvg_options &o) {
  Result a;
  const size_t S = lvg_graph_span(y);
  a.m.resize(S); a.vt.resize(S); a.ct.resize(S);
  a.r.membership = a.m.data(); a.r.vertexWeight = a.vt.data(); a.r.communityWeight = a.ct.data();
  int rc;
  if (method == LVG_METHOD_STATIC) rc = lvg_static(y, &o, &a.r);
  else if (method == LVG_METHOD_NAIVE)
    rc = lvg_naive_dynamic(y, b, prior->m.data(), prior->vt.data(), prior->ct.data(), &o, &a.r);
  else if (method == LVG_METHOD_DELTA)
    rc = lvg_delta_screening(y, b, prior->m.data(), prior->vt.data(), prior->ct.data(), &o, &a.r);
  else rc = lvg_frontier(y, b, prior->m.data(), prior->vt.data(), prior->ct.data(), &o, &a.r);
  check(rc, "louvain");
  return a;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc < 6) {
    std::fprintf(stderr,
                 "usage: %s <file> <rows> <size> <unused> <batchFraction>\n"
                 "       %s --drift <n> <communities> <edges> <seed> <batchFraction>\n",
                 argv[0], argv[0]);
    return 2;
  }
  const bool drift = std::strcmp(argv[1], "--drift") == 0;
  const char *file = argv[1];
  size_t rows = std::strtoull(argv[2], nullptr, 10);
  size_t size = std::strtoull(argv[3], nullptr, 10);
  double batchFraction = std::strtod(argv[5], nullptr);
  Stream in;
  std::string name = file;
  if (drift) {
    const uint32_t n = uint32_t(rows), communities = uint32_t(size);
    const size_t edges = std::strtoull(argv[4], nullptr, 10);
    const uint64_t seed = std::strtoull(argv[5], nullptr, 10);
    if (argc < 7) die("--drift", "missing batchFraction");
    batchFraction = std::strtod(argv[6], nullptr);
    if (lvgg_temporal_drift(n, communities, 1.0, edges, 0.85, std::max<size_t>(1, edges / 20), 0.01, seed,
                            &in.all) != 0)
      die("lvgg_temporal_drift", lvgg_last_error());
    rows = n;
    size = edges;
    name = "/drift/temporal-drift-" + std::to_string(n) + ".txt";
  } else if (lvgg_temporal_open(file, 0, &in.file) != 0) {
    die("lvgg_temporal_open", lvgg_last_error());
  }
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int threads = sms;  // the GPU's SMs stand in for the reference's OpenMP threads
  const int BATCH_LENGTH = env_int("BATCH_LENGTH", 1), REPEAT = env_int("REPEAT_METHOD", 5);
  log_prefix();
  std::printf(" OMP_NUM_THREADS=%d\n", threads);
  log_prefix();
  std::printf(" Loading graph %s ...\n", name.c_str());
  // the first 90 % of the lines, both directions (readTemporalOmpW + symmetrizeOmp)
  std::vector<uint32_t> s, d;
  std::vector<float> w;
  in.read(size_t(0.90 * double(size)), s, d, w);
  lvg_graph *gx = nullptr;
  check(lvg_graph_create_from_edges(rows + 1, s.size(), s.data(), d.data(), w.data(), &gx),
        "lvg_graph_create_from_edges");
  print_graph(gx, " (90%)");
  print_graph(gx, " (symmetrize)");  // the base is read with both directions already
  double M = 0;
  check(lvg_edge_weight(gx, &M), "lvg_edge_weight");
  M /= 2;
  lvg_options o;
  lvg_options_default(&o);
  o.repeat = REPEAT;
  Result b0 = run(LVG_METHOD_STATIC, gx, nullptr, nullptr, o);
  glog(b0, "louvainStaticOmpOriginal", threads, gx, M, 0.0, 0.0);
  Result b2 = b0, b3 = b0, b4 = b0;
  for (int batch = 0; batch < BATCH_LENGTH; ++batch) {
    // y = duplicate(x); tidy + apply the next lines as insertions
    lvg_graph *gy = nullptr;
    check(lvg_graph_clone(gx, &gy), "lvg_graph_clone");
    std::vector<uint32_t> is, id;
    std::vector<float> iw;
    in.read(size_t(batchFraction * double(size)), is, id, iw);
    lvg_batch raw{0, nullptr, nullptr, nullptr, is.size(), is.data(), id.data(), iw.data()};
    std::vector<uint32_t> ts(is.size() + 1), td(is.size() + 1);
    std::vector<float> tw(is.size() + 1);
    lvg_batch_buf tidy{0, nullptr, nullptr, nullptr, 0, ts.data(), td.data(), tw.data()};
    check(lvg_graph_apply_batch(gy, &raw, &tidy), "lvg_graph_apply_batch");
    char tail[64];
    std::snprintf(tail, sizeof tail, " (insertions=%zu)", tidy.num_insertions);
    print_graph(gy, tail);
    double My = 0;
    check(lvg_edge_weight(gy, &My), "lvg_edge_weight");
    My /= 2;
    lvg_batch bt{0, nullptr, nullptr, nullptr, tidy.num_insertions, ts.data(), td.data(), tw.data()};
    Result r1 = run(LVG_METHOD_STATIC, gy, nullptr, nullptr, o);
    glog(r1, "louvainStaticOmp", threads, gy, My, 0.0, batchFraction);
    Result r2 = run(LVG_METHOD_NAIVE, gy, &bt, &b2, o);
    glog(r2, "louvainNaiveDynamicOmp", threads, gy, My, 0.0, batchFraction);
    Result r3 = run(LVG_METHOD_DELTA, gy, &bt, &b3, o);
    glog(r3, "louvainDynamicDeltaScreeningOmp", threads, gy, My, 0.0, batchFraction);
    Result r4 = run(LVG_METHOD_FRONTIER, gy, &bt, &b4, o);
    glog(r4, "louvainDynamicFrontierOmp", threads, gy, My, 0.0, batchFraction);
    b2 = r2; b3 = r3; b4 = r4;
    lvg_graph_destroy(gy);
  }
  std::printf("\n");
  lvg_graph_destroy(gx);
  if (in.file) lvgg_temporal_close(in.file);
  lvgg_edges_free(&in.all);
  return 0;
}
