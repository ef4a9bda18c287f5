// louvain_gb300.hxx — C++ drop-in for the reference's Louvain templates.
//
// Replaces inc/louvain.hxx of puzzlef/louvain-communities-openmp-dynamic for
// callers: the same names and call shapes
//   louvainStaticOmp(x, o)                                   (inc/louvain.hxx:1285)
//   louvainNaiveDynamicOmp(y, del, ins, q, qvtot, qctot, o)  (inc/louvain.hxx:1349)
//   louvainDynamicDeltaScreeningOmp(...)                     (inc/louvain.hxx:1542)
//   louvainDynamicFrontierOmp(...)                           (inc/louvain.hxx:1674)
// with LouvainOptions (inc/louvain.hxx:30-63) and LouvainResult<K, double>
// (inc/louvain.hxx:78-145), running on the GPU through liblouvain_gb300.so.
//
// The graph argument is any type with the reference's graph concept
// (key_type, span(), hasVertex(u), forEachEdge(u, f(v, w)); inc/Graph.hxx):
// it is flattened to CSR and uploaded on each call. A caller that runs several
// methods on one graph can upload it once with DeviceGraph and pass that
// instead. Failures throw std::runtime_error (the reference throws nothing but
// std::bad_alloc). Define LVG_NO_GLOBAL_NAMES to keep the names inside
// namespace louvain_gb300 only.
#pragma once
#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#include "louvain_gb300.h"

namespace louvain_gb300 {

/** Options for the Louvain algorithm (the reference's LouvainOptions, same defaults). */
struct LouvainOptions {
  int repeat;
  double resolution;
  double tolerance;
  double aggregationTolerance;
  double toleranceDrop;
  int maxIterations;
  int maxPasses;
  LouvainOptions(int repeat = 1, double resolution = 1, double tolerance = 1e-2, double aggregationTolerance = 1.0,
                 double toleranceDrop = 10, int maxIterations = 20, int maxPasses = 10)
      : repeat(repeat), resolution(resolution), tolerance(tolerance), aggregationTolerance(aggregationTolerance),
        toleranceDrop(toleranceDrop), maxIterations(maxIterations), maxPasses(maxPasses) {}
};

/** Result of the Louvain algorithm (the reference's LouvainResult). */
template <class K, class W = double>
struct LouvainResult {
  std::vector<K> membership;
  std::vector<W> vertexWeight;
  std::vector<W> communityWeight;
  int iterations = 0;
  int passes = 0;
  float time = 0;
  float markingTime = 0;
  float initializationTime = 0;
  float firstPassTime = 0;
  float localMoveTime = 0;
  float aggregationTime = 0;
  size_t affectedVertices = 0;

  LouvainResult() = default;
  /** From vectors the caller hands over (rvalues); scalar fields as given.
   * Same parameters and defaults as the reference's constructor
   * (inc/louvain.hxx:118-119). */
  LouvainResult(std::vector<K> &&membership, std::vector<W> &&vertexWeight, std::vector<W> &&communityWeight,
                int iterations = 0, int passes = 0, float time = 0, float markingTime = 0,
                float initializationTime = 0, float firstPassTime = 0, float localMoveTime = 0,
                float aggregationTime = 0, size_t affectedVertices = 0)
      : membership(std::move(membership)), vertexWeight(std::move(vertexWeight)),
        communityWeight(std::move(communityWeight)), iterations(iterations), passes(passes), time(time),
        markingTime(markingTime), initializationTime(initializationTime), firstPassTime(firstPassTime),
        localMoveTime(localMoveTime), aggregationTime(aggregationTime), affectedVertices(affectedVertices) {}
  /** From the caller's vectors (lvalues), whose contents are moved in and
   * which are left empty, as the reference's second constructor does
   * (inc/louvain.hxx:139-140). */
  LouvainResult(std::vector<K> &membership, std::vector<W> &vertexWeight, std::vector<W> &communityWeight,
                int iterations = 0, int passes = 0, float time = 0, float markingTime = 0,
                float initializationTime = 0, float firstPassTime = 0, float localMoveTime = 0,
                float aggregationTime = 0, size_t affectedVertices = 0)
      : membership(std::move(membership)), vertexWeight(std::move(vertexWeight)),
        communityWeight(std::move(communityWeight)), iterations(iterations), passes(passes), time(time),
        markingTime(markingTime), initializationTime(initializationTime), firstPassTime(firstPassTime),
        localMoveTime(localMoveTime), aggregationTime(aggregationTime), affectedVertices(affectedVertices) {}
};

namespace detail {

inline void check(int rc, const char *what) {
  if (rc == LVG_OK) return;
  // the library's messages may already open with the failing call's name
  const std::string msg = lvg_last_error(), head = std::string(what) + ":";
  throw std::runtime_error(msg.compare(0, head.size(), head) == 0 ? msg : std::string(what) + ": " + msg);
}

inline lvg_options to_c(const LouvainOptions &o) {
  lvg_options c;
  lvg_options_default(&c);
  c.repeat = o.repeat;
  c.resolution = o.resolution;
  c.tolerance = o.tolerance;
  c.aggregationTolerance = o.aggregationTolerance;
  c.toleranceDrop = o.toleranceDrop;
  c.maxIterations = o.maxIterations;
  c.maxPasses = o.maxPasses;
  return c;
}

template <class K, class W>
LouvainResult<K, W> from_c(lvg_result &r) {
  LouvainResult<K, W> a;
  a.membership.assign(r.membership, r.membership + r.span);
  a.vertexWeight.assign(r.vertexWeight, r.vertexWeight + r.span);
  a.communityWeight.assign(r.communityWeight, r.communityWeight + r.span);
  a.iterations = r.iterations;
  a.passes = r.passes;
  a.time = r.time;
  a.markingTime = r.markingTime;
  a.initializationTime = r.initializationTime;
  a.firstPassTime = r.firstPassTime;
  a.localMoveTime = r.localMoveTime;
  a.aggregationTime = r.aggregationTime;
  a.affectedVertices = r.affectedVertices;
  lvg_result_free(&r);
  return a;
}

// A batch as structure-of-arrays, from the reference's vector<tuple<K,K,V>>.
struct Batch {
  std::vector<uint32_t> ds, dd, is, id;
  std::vector<float> dw, iw;
  lvg_batch c{};
  template <class K, class V>
  Batch(const std::vector<std::tuple<K, K, V>> &del, const std::vector<std::tuple<K, K, V>> &ins) {
    for (const auto &e : del) { ds.push_back(uint32_t(std::get<0>(e))); dd.push_back(uint32_t(std::get<1>(e))); dw.push_back(float(std::get<2>(e))); }
    for (const auto &e : ins) { is.push_back(uint32_t(std::get<0>(e))); id.push_back(uint32_t(std::get<1>(e))); iw.push_back(float(std::get<2>(e))); }
    c.num_deletions = ds.size();
    c.del_src = ds.data(); c.del_dst = dd.data(); c.del_w = dw.data();
    c.num_insertions = is.size();
    c.ins_src = is.data(); c.ins_dst = id.data(); c.ins_w = iw.data();
  }
};

}  // namespace detail

/** A graph uploaded to the GPU once (RAII over lvg_graph). */
class DeviceGraph {
 public:
  template <class G>
  explicit DeviceGraph(const G &x) {
    using K = typename G::key_type;
    static_assert(std::is_integral<K>::value && sizeof(K) <= 4, "vertex ids must fit uint32");
    const size_t S = x.span();
    std::vector<uint64_t> off(S + 1, 0);
    std::vector<uint32_t> keys;
    std::vector<float> w;
    std::vector<uint8_t> ex(S, 0);
    for (size_t u = 0; u < S; ++u) {
      if (x.hasVertex(K(u))) {
        ex[u] = 1;
        x.forEachEdge(K(u), [&](auto v, auto wt) {
          keys.push_back(uint32_t(v));
          w.push_back(float(wt));
        });
      }
      off[u + 1] = keys.size();
    }
    detail::check(lvg_graph_create(S, off.data(), keys.data(), w.data(), ex.data(), &g_), "lvg_graph_create");
  }
  ~DeviceGraph() { if (g_) lvg_graph_destroy(g_); }
  DeviceGraph(const DeviceGraph &) = delete;
  DeviceGraph &operator=(const DeviceGraph &) = delete;
  DeviceGraph(DeviceGraph &&o) noexcept : g_(o.g_) { o.g_ = nullptr; }
  lvg_graph *get() const { return g_; }
  size_t span() const { return lvg_graph_span(g_); }

 private:
  lvg_graph *g_ = nullptr;
};

// ----------------------------------------------------------------- batch update

/** tidyBatchUpdateU(deletions, insertions, y) followed by
 * applyBatchUpdateOmpU(y, deletions, insertions) (inc/batch.hxx:202, 241), as
 * main.cxx:108-109 runs them, on a graph in HBM: the graph is updated in
 * place and the vectors are replaced by the tidied batch (present deletions,
 * absent insertions, sorted by (source, target), unique), ready for the
 * dynamic entry points. */
template <class K, class V>
inline void tidyApplyBatchUpdateOmpU(DeviceGraph &y, std::vector<std::tuple<K, K, V>> &deletions,
                                     std::vector<std::tuple<K, K, V>> &insertions) {
  detail::Batch b(deletions, insertions);
  std::vector<uint32_t> ts(b.ds.size()), td(b.ds.size()), us(b.is.size()), ud(b.is.size());
  std::vector<float> tw(b.ds.size()), uw(b.is.size());
  lvg_batch_buf t{0, ts.data(), td.data(), tw.data(), 0, us.data(), ud.data(), uw.data()};
  detail::check(lvg_graph_apply_batch(y.get(), &b.c, &t), "lvg_graph_apply_batch");
  deletions.clear();
  insertions.clear();
  for (size_t i = 0; i < t.num_deletions; ++i) deletions.emplace_back(K(ts[i]), K(td[i]), V(tw[i]));
  for (size_t i = 0; i < t.num_insertions; ++i) insertions.emplace_back(K(us[i]), K(ud[i]), V(uw[i]));
}

// ----------------------------------------------------------------- entry points

template <class K = uint32_t>
inline LouvainResult<K, double> louvainStaticOmp(const DeviceGraph &x, const LouvainOptions &o = {}) {
  lvg_result r{};
  lvg_options c = detail::to_c(o);
  detail::check(lvg_static(x.get(), &c, &r), "lvg_static");
  return detail::from_c<K, double>(r);
}

template <class G, class = typename G::key_type>
inline auto louvainStaticOmp(const G &x, const LouvainOptions &o = {}) {
  DeviceGraph d(x);
  return louvainStaticOmp<typename G::key_type>(d, o);
}

namespace detail {
template <class K, class V, class W, class F>
LouvainResult<K, double> dynamic_call(F fn, const char *name, const DeviceGraph &y,
                                      const std::vector<std::tuple<K, K, V>> &deletions,
                                      const std::vector<std::tuple<K, K, V>> &insertions, const std::vector<K> &q,
                                      const std::vector<W> &qvtot, const std::vector<W> &qctot,
                                      const LouvainOptions &o) {
  const size_t S = y.span();
  if (q.size() < S || qvtot.size() < S || qctot.size() < S)
    throw std::runtime_error(std::string(name) + ": prior state shorter than the graph's span");
  std::vector<uint32_t> q32(q.begin(), q.begin() + S);
  std::vector<double> vt(qvtot.begin(), qvtot.begin() + S), ct(qctot.begin(), qctot.begin() + S);
  Batch b(deletions, insertions);
  lvg_result r{};
  lvg_options c = to_c(o);
  check(fn(y.get(), &b.c, q32.data(), vt.data(), ct.data(), &c, &r), name);
  return from_c<K, double>(r);
}
}  // namespace detail

template <class K, class V, class W>
inline auto louvainNaiveDynamicOmp(const DeviceGraph &y, const std::vector<std::tuple<K, K, V>> &deletions,
                                   const std::vector<std::tuple<K, K, V>> &insertions, const std::vector<K> &q,
                                   const std::vector<W> &qvtot, const std::vector<W> &qctot,
                                   const LouvainOptions &o = {}) {
  return detail::dynamic_call(lvg_naive_dynamic, "lvg_naive_dynamic", y, deletions, insertions, q, qvtot, qctot, o);
}

template <class K, class V, class W>
inline auto louvainDynamicDeltaScreeningOmp(const DeviceGraph &y, const std::vector<std::tuple<K, K, V>> &deletions,
                                            const std::vector<std::tuple<K, K, V>> &insertions,
                                            const std::vector<K> &q, const std::vector<W> &qvtot,
                                            const std::vector<W> &qctot, const LouvainOptions &o = {}) {
  return detail::dynamic_call(lvg_delta_screening, "lvg_delta_screening", y, deletions, insertions, q, qvtot, qctot,
                              o);
}

template <class K, class V, class W>
inline auto louvainDynamicFrontierOmp(const DeviceGraph &y, const std::vector<std::tuple<K, K, V>> &deletions,
                                      const std::vector<std::tuple<K, K, V>> &insertions, const std::vector<K> &q,
                                      const std::vector<W> &qvtot, const std::vector<W> &qctot,
                                      const LouvainOptions &o = {}) {
  return detail::dynamic_call(lvg_frontier, "lvg_frontier", y, deletions, insertions, q, qvtot, qctot, o);
}

template <class G, class K, class V, class W, class = typename G::key_type>
inline auto louvainNaiveDynamicOmp(const G &y, const std::vector<std::tuple<K, K, V>> &deletions,
                                   const std::vector<std::tuple<K, K, V>> &insertions, const std::vector<K> &q,
                                   const std::vector<W> &qvtot, const std::vector<W> &qctot,
                                   const LouvainOptions &o = {}) {
  DeviceGraph d(y);
  return louvainNaiveDynamicOmp(d, deletions, insertions, q, qvtot, qctot, o);
}

template <class G, class K, class V, class W, class = typename G::key_type>
inline auto louvainDynamicDeltaScreeningOmp(const G &y, const std::vector<std::tuple<K, K, V>> &deletions,
                                            const std::vector<std::tuple<K, K, V>> &insertions,
                                            const std::vector<K> &q, const std::vector<W> &qvtot,
                                            const std::vector<W> &qctot, const LouvainOptions &o = {}) {
  DeviceGraph d(y);
  return louvainDynamicDeltaScreeningOmp(d, deletions, insertions, q, qvtot, qctot, o);
}

template <class G, class K, class V, class W, class = typename G::key_type>
inline auto louvainDynamicFrontierOmp(const G &y, const std::vector<std::tuple<K, K, V>> &deletions,
                                      const std::vector<std::tuple<K, K, V>> &insertions, const std::vector<K> &q,
                                      const std::vector<W> &qvtot, const std::vector<W> &qctot,
                                      const LouvainOptions &o = {}) {
  DeviceGraph d(y);
  return louvainDynamicFrontierOmp(d, deletions, insertions, q, qvtot, qctot, o);
}

}  // namespace louvain_gb300

#ifndef LVG_NO_GLOBAL_NAMES
using louvain_gb300::LouvainOptions;
using louvain_gb300::LouvainResult;
using louvain_gb300::louvainDynamicDeltaScreeningOmp;
using louvain_gb300::louvainDynamicFrontierOmp;
using louvain_gb300::louvainNaiveDynamicOmp;
using louvain_gb300::louvainStaticOmp;
using louvain_gb300::tidyApplyBatchUpdateOmpU;
#endif
