// Uses include/louvain_gb300.hxx the way main.cxx uses inc/louvain.hxx
// (main.cxx:89-126): static on a graph, then the three dynamic methods on the
// updated graph from the static result. The graph type implements the
// reference's graph concept (key_type, span, hasVertex, forEachEdge).
#include <cstdio>
#include <algorithm>
#include <cstdlib>
#include <map>
#include <tuple>
#include <vector>

#include "louvain_gb300.hxx"

struct TinyGraph {
  using key_type = uint32_t;
  using edge_value_type = float;
  std::vector<std::map<uint32_t, float>> rows;
  std::vector<bool> ex;
  size_t span() const { return rows.size(); }
  bool hasVertex(uint32_t u) const { return u < ex.size() && ex[u]; }
  template <class F> void forEachEdge(uint32_t u, F f) const { for (auto &kv : rows[u]) f(kv.first, kv.second); }
  void add(uint32_t u, uint32_t v, float w) { rows[u][v] = w; rows[v][u] = w; }
};

int main() {
  const uint32_t n = 4096, block = 64;
  TinyGraph x;
  x.rows.resize(n + 1);
  x.ex.assign(n + 1, true);
  x.ex[0] = false;  // vertex 0 absent, as in the reference's SNAP graphs
  uint64_t s = 12345;
  auto rnd = [&]() { s = s * 6364136223846793005ull + 1442695040888963407ull; return uint32_t(s >> 33); };
  for (uint32_t i = 0; i < n * 8; ++i) {
    uint32_t u = 1 + rnd() % n, v = (rnd() % 10 < 8) ? 1 + ((u - 1) / block) * block + rnd() % block : 1 + rnd() % n;
    if (u != v) x.add(u, v, 1.0f);
  }
  auto a = louvainStaticOmp(x, {1});
  std::vector<std::tuple<uint32_t, uint32_t, float>> del, ins;
  TinyGraph y = x;
  for (uint32_t i = 0; i < 40; ++i) {
    uint32_t u = 1 + rnd() % n, v = 1 + rnd() % n;
    if (u == v || y.rows[u].count(v)) continue;
    y.add(u, v, 1.0f);
    ins.push_back({std::min(u, v), std::max(u, v), 1.0f});
    ins.push_back({std::max(u, v), std::min(u, v), 1.0f});
  }
  std::sort(ins.begin(), ins.end());
  auto b = louvainNaiveDynamicOmp(y, del, ins, a.membership, a.vertexWeight, a.communityWeight, {1});
  auto c = louvainDynamicDeltaScreeningOmp(y, del, ins, a.membership, a.vertexWeight, a.communityWeight, {1});
  louvain_gb300::DeviceGraph dy(y);
  auto d = louvainDynamicFrontierOmp(dy, del, ins, a.membership, a.vertexWeight, a.communityWeight, {1});
  int bad = 0;
  for (auto *r : {&a, &b, &c, &d}) {
    if (r->membership.size() != n + 1 || r->passes < 1) ++bad;
    for (uint32_t u = 1; u <= n; ++u) if (r->membership[u] > n) ++bad;
  }
  for (uint32_t u = 1; u <= n; ++u) if (a.vertexWeight[u] != double(x.rows[u].size())) ++bad;
  std::printf("static %d passes %d iters %.3f ms | nd %.3f ds %.3f df %.3f ms | bad %d\n", a.passes, a.iterations,
              a.time, b.time, c.time, d.time, bad);
  // main.cxx:108-109 in HBM: tidy + apply an untidy batch to x on the device
  louvain_gb300::DeviceGraph dx(x);
  auto ins2 = ins;
  ins2.push_back(ins[0]);                                     // a duplicate
  ins2.push_back({1u, x.rows[1].begin()->first, 1.0f});       // an edge x already has
  std::reverse(ins2.begin(), ins2.end());                     // unsorted
  auto del2 = del;
  tidyApplyBatchUpdateOmpU(dx, del2, ins2);
  if (ins2 != ins || !del2.empty()) ++bad;                    // the tidied batch
  if (lvg_graph_size(dx.get()) != lvg_graph_size(dy.get())) ++bad;
  double wx = 0, wy = 0;
  lvg_edge_weight(dx.get(), &wx);
  lvg_edge_weight(dy.get(), &wy);
  if (wx != wy) ++bad;
  try {
    std::vector<uint32_t> shortq(3);
    louvainDynamicFrontierOmp(dy, del, ins, shortq, a.vertexWeight, a.communityWeight);
    ++bad;
  } catch (const std::runtime_error &) {
  }
  return bad ? 1 : 0;
}
