// ref_harness.cxx — C-ABI harness over the reference's own Louvain headers.
//
// TEST INFRASTRUCTURE ONLY. This file is compiled against the unmodified
// reference headers where they lie (inc/main.hxx), into oracle/_ref/, by
// oracle/Makefile. It is used to pin the C restatement in
// oracle/louvain_oracle.c and to generate the golden fixtures under
// tests/golden/. It never ships in the product path.
//
// Each entry point calls the reference's own functions:
//   ref_louvain      -> louvainStaticOmp / louvainNaiveDynamicOmp /
//                       louvainDynamicDeltaScreeningOmp / louvainDynamicFrontierOmp
//                       (inc/louvain.hxx:1285, 1349, 1542, 1674)
//   ref_vertex_weights  -> louvainVertexWeightsOmpW     (inc/louvain.hxx:210)
//   ref_update_weights  -> louvainUpdateWeightsFromOmpU (inc/louvain.hxx:374)
//   ref_df_mark         -> louvainAffectedVerticesFrontierOmpW      (inc/louvain.hxx:1606)
//   ref_ds_mark         -> louvainAffectedVerticesDeltaScreeningOmpW (inc/louvain.hxx:1441)
//   ref_aggregate       -> the driver's renumber + community-vertices + aggregate
//                          sequence (inc/louvain.hxx:1190-1202)
//   ref_modularity      -> modularityBy (inc/properties.hxx:178)
//   ref_edge_weight     -> edgeWeightOmp (inc/properties.hxx:96)
//   ref_apply_batch     -> tidyBatchUpdateU + applyBatchUpdateOmpU
//                          (inc/batch.hxx:202, 241), in place
//   ref_graph_csr       -> the graph's rows (forEachEdge) as a compact CSR
//   ref_read_temporal   -> readTemporalOmpW + symmetrizeOmp (inc/snap.hxx:212,
//                          inc/symmetrize.hxx:72), as main.cxx:159-161
#include "inc/main.hxx"

#include <cstdint>
#include <cstring>
#include <fstream>
#include <omp.h>

using K = uint32_t;
using V = float;
using W = double;
using G = DiGraph<K, None, V>;

namespace {
vector<tuple<K, K, V>> make_edges(size_t n, const uint32_t *s, const uint32_t *d, const float *w) {
  vector<tuple<K, K, V>> a;
  a.reserve(n);
  for (size_t i = 0; i < n; ++i) a.push_back({s[i], d[i], w[i]});
  return a;
}
}  // namespace

extern "C" {

struct ref_info {
  int iterations, passes;
  float time, markingTime, initializationTime, firstPassTime, localMoveTime, aggregationTime;
  uint64_t affectedVertices;
};

void ref_set_threads(int t) { omp_set_num_threads(t); }

void *ref_graph_new(size_t span, const uint64_t *off, const uint32_t *key, const float *w, const uint8_t *exists) {
  G *g = new G();
  g->respan(span);
  for (size_t u = 0; u < span; ++u)
    if (!exists || exists[u]) g->addVertex(K(u));
  for (size_t u = 0; u < span; ++u)
    for (uint64_t i = off[u]; i < off[u + 1]; ++i) g->addEdge(K(u), key[i], w[i]);
  g->update();
  return g;
}

void ref_graph_free(void *g) { delete static_cast<G *>(g); }

size_t ref_graph_order(void *g) { return static_cast<G *>(g)->order(); }
size_t ref_graph_size(void *g) { return static_cast<G *>(g)->size(); }

double ref_edge_weight(void *g) { return edgeWeightOmp(*static_cast<G *>(g)); }

void ref_vertex_weights(void *gp, double *vtot) {
  const G &x = *static_cast<G *>(gp);
  vector<W> a(x.span());
  louvainVertexWeightsOmpW(a, x);
  std::memcpy(vtot, a.data(), a.size() * sizeof(W));
}

void ref_update_weights(void *gp, size_t nd, const uint32_t *ds, const uint32_t *dd, const float *dw, size_t ni,
                        const uint32_t *is, const uint32_t *id, const float *iw, const uint32_t *vcom, double *vtot,
                        double *ctot) {
  const G &y = *static_cast<G *>(gp);
  size_t S = y.span();
  auto del = make_edges(nd, ds, dd, dw), ins = make_edges(ni, is, id, iw);
  vector<K> c(vcom, vcom + S);
  vector<W> vt(vtot, vtot + S), ct(ctot, ctot + S);
  louvainUpdateWeightsFromOmpU(vt, ct, y, del, ins, c);
  std::memcpy(vtot, vt.data(), S * sizeof(W));
  std::memcpy(ctot, ct.data(), S * sizeof(W));
}

void ref_df_mark(void *gp, size_t nd, const uint32_t *ds, const uint32_t *dd, const float *dw, size_t ni,
                 const uint32_t *is, const uint32_t *id, const float *iw, const uint32_t *vcom, uint8_t *flags) {
  const G &y = *static_cast<G *>(gp);
  size_t S = y.span();
  auto del = make_edges(nd, ds, dd, dw), ins = make_edges(ni, is, id, iw);
  vector<K> c(vcom, vcom + S);
  vector<char> f(S);
  louvainAffectedVerticesFrontierOmpW(f, y, del, ins, c);
  for (size_t u = 0; u < S; ++u) flags[u] = uint8_t(f[u]);
}

void ref_ds_mark(void *gp, size_t nd, const uint32_t *ds, const uint32_t *dd, const float *dw, size_t ni,
                 const uint32_t *is, const uint32_t *id, const float *iw, const uint32_t *vcom, const double *vtot,
                 const double *ctot, double M, double R, uint8_t *vertices, uint8_t *neighbors,
                 uint8_t *communities) {
  const G &y = *static_cast<G *>(gp);
  size_t S = y.span();
  int T = omp_get_max_threads();
  auto del = make_edges(nd, ds, dd, dw), ins = make_edges(ni, is, id, iw);
  vector<K> c(vcom, vcom + S);
  vector<W> vt(vtot, vtot + S), ct(ctot, ctot + S);
  vector<char> fv(S), fn(S), fc(S);
  vector<vector<K> *> vcs(T);
  vector<vector<W> *> vcout(T);
  louvainAllocateHashtablesW(vcs, vcout, S);
  louvainAffectedVerticesDeltaScreeningOmpW(fv, fn, fc, vcs, vcout, y, del, ins, c, vt, ct, M, R);
  louvainFreeHashtablesW(vcs, vcout);
  for (size_t u = 0; u < S; ++u) {
    vertices[u] = uint8_t(fv[u]);
    neighbors[u] = uint8_t(fn[u]);
    communities[u] = uint8_t(fc[u]);
  }
}

// Renumber vcom (span entries, in place) and aggregate. Returns CN; the output
// is the reference's gapped CSR: yoff[CN+1], ydeg[CN], rows at yoff[c].
size_t ref_aggregate(void *gp, uint32_t *vcom, uint64_t *yoff, uint32_t *ydeg, uint32_t *ykey, double *yw) {
  const G &x = *static_cast<G *>(gp);
  size_t S = x.span(), X = x.size();
  int T = omp_get_max_threads();
  vector<K> bufk(T);
  vector<size_t> bufs(T);
  vector<vector<K> *> vcs(T);
  vector<vector<W> *> vcout(T);
  louvainAllocateHashtablesW(vcs, vcout, S);
  vector<K> c(vcom, vcom + S);
  DiGraphCsr<K, None, None, K> cv(S, S);
  DiGraphCsr<K, None, W> z(S, X);
  size_t CN = louvainCommunityExistsOmpW(cv.degrees, x, c);
  louvainRenumberCommunitiesOmpW(c, cv.degrees, bufk, x);
  cv.respan(CN);
  z.respan(CN);
  louvainCommunityVerticesOmpW(cv.offsets, cv.degrees, cv.edgeKeys, bufk, x, c);
  louvainAggregateOmpW(z.offsets, z.degrees, z.edgeKeys, z.edgeValues, bufs, vcs, vcout, x, c, cv.offsets,
                       cv.edgeKeys);
  louvainFreeHashtablesW(vcs, vcout);
  std::memcpy(vcom, c.data(), S * sizeof(K));
  for (size_t i = 0; i <= CN; ++i) yoff[i] = z.offsets[i];
  for (size_t i = 0; i < CN; ++i) ydeg[i] = z.degrees[i];
  std::memcpy(ykey, z.edgeKeys.data(), X * sizeof(K));
  std::memcpy(yw, z.edgeValues.data(), X * sizeof(W));
  return CN;
}

// tidyBatchUpdateU + applyBatchUpdateOmpU, in place, as main.cxx:108-109;
// the tidied batch is written out (room for nd / ni entries).
void ref_apply_batch(void *gp, size_t nd, const uint32_t *ds, const uint32_t *dd, const float *dw, size_t ni,
                     const uint32_t *is, const uint32_t *id, const float *iw, uint32_t *tds, uint32_t *tdd,
                     float *tdw, size_t *tnd, uint32_t *tis, uint32_t *tid, float *tiw, size_t *tni) {
  G &y = *static_cast<G *>(gp);
  auto del = make_edges(nd, ds, dd, dw), ins = make_edges(ni, is, id, iw);
  tidyBatchUpdateU(del, ins, y);
  applyBatchUpdateOmpU(y, del, ins);
  for (size_t i = 0; i < del.size(); ++i) std::tie(tds[i], tdd[i], tdw[i]) = del[i];
  for (size_t i = 0; i < ins.size(); ++i) std::tie(tis[i], tid[i], tiw[i]) = ins[i];
  *tnd = del.size();
  *tni = ins.size();
}

// main.cxx:159-161: readTemporalOmpW(x, file, false, true, rows, lines) then
// x = symmetrizeOmp(x). Returns the graph (free with ref_graph_free).
void *ref_read_temporal(const char *path, size_t rows, size_t lines) {
  G x;
  std::ifstream f(path);
  readTemporalOmpW(x, f, false, true, rows, lines);
  return new G(symmetrizeOmp(x));
}

// Compact CSR of the graph: off[span+1], key/w[size], ex[span]. Returns size.
size_t ref_graph_csr(void *gp, uint64_t *off, uint32_t *key, float *w, uint8_t *ex) {
  const G &x = *static_cast<G *>(gp);
  size_t m = 0;
  off[0] = 0;
  for (size_t u = 0; u < x.span(); ++u) {
    ex[u] = x.hasVertex(K(u)) ? 1 : 0;
    if (ex[u]) x.forEachEdge(K(u), [&](auto v, auto wt) { key[m] = v; w[m] = wt; ++m; });
    off[u + 1] = m;
  }
  return m;
}

double ref_modularity(void *gp, const uint32_t *membership, double M, double R) {
  const G &x = *static_cast<G *>(gp);
  auto fc = [&](auto u) { return membership[u]; };
  return modularityBy(x, fc, M, R);
}

// method: 0 static, 1 naive-dynamic, 2 delta-screening, 3 dynamic frontier.
int ref_louvain(void *gp, int method, size_t nd, const uint32_t *ds, const uint32_t *dd, const float *dw, size_t ni,
                const uint32_t *is, const uint32_t *id, const float *iw, const uint32_t *q, const double *qvtot,
                const double *qctot, int repeat, double resolution, double tolerance, double aggregationTolerance,
                double toleranceDrop, int maxIterations, int maxPasses, uint32_t *membership, double *vtot,
                double *ctot, ref_info *info) {
  const G &y = *static_cast<G *>(gp);
  size_t S = y.span();
  LouvainOptions o(repeat, resolution, tolerance, aggregationTolerance, toleranceDrop, maxIterations, maxPasses);
  auto del = make_edges(nd, ds, dd, dw), ins = make_edges(ni, is, id, iw);
  auto fill = [&](const auto &a) {
    std::memcpy(membership, a.membership.data(), a.membership.size() * sizeof(K));
    std::memcpy(vtot, a.vertexWeight.data(), a.vertexWeight.size() * sizeof(W));
    std::memcpy(ctot, a.communityWeight.data(), a.communityWeight.size() * sizeof(W));
    info->iterations = a.iterations;
    info->passes = a.passes;
    info->time = a.time;
    info->markingTime = a.markingTime;
    info->initializationTime = a.initializationTime;
    info->firstPassTime = a.firstPassTime;
    info->localMoveTime = a.localMoveTime;
    info->aggregationTime = a.aggregationTime;
    info->affectedVertices = a.affectedVertices;
  };
  if (method == 0) {
    fill(louvainStaticOmp(y, o));
    return 0;
  }
  vector<K> qv(q, q + S);
  vector<W> qvt(qvtot, qvtot + S), qct(qctot, qctot + S);
  if (method == 1) fill(louvainNaiveDynamicOmp(y, del, ins, qv, qvt, qct, o));
  else if (method == 2) fill(louvainDynamicDeltaScreeningOmp(y, del, ins, qv, qvt, qct, o));
  else if (method == 3) fill(louvainDynamicFrontierOmp(y, del, ins, qv, qvt, qct, o));
  else return -1;
  return 0;
}

}  // extern "C"
