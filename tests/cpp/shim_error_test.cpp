// The C++ header's error behaviour, on an input its library refuses before
// any device work (so it runs without a GPU): a graph with a neighbour beyond
// its span makes the entry point throw std::runtime_error with the library's
// message, naming the failing call once. Prints "errors ok".
#include <cstdio>
#include <map>
#include <stdexcept>
#include <string>
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
};

static int expect_throw(const TinyGraph &g, const std::string &want) {
  try {
    louvainStaticOmp(g, {1});
  } catch (const std::runtime_error &e) {
    if (std::string(e.what()) == want) return 0;
    std::printf("message: '%s', expected '%s'\n", e.what(), want.c_str());
    return 1;
  }
  std::printf("no exception, expected '%s'\n", want.c_str());
  return 1;
}

int main() {
  int bad = 0;
  TinyGraph g;
  g.rows.resize(5);
  g.ex.assign(5, true);
  g.rows[1][2] = 1.f;
  g.rows[2][1] = 1.f;
  g.rows[3][7] = 1.f;  // beyond the span of 5
  bad += expect_throw(g, "lvg_graph_create: neighbour id >= span");
  std::printf(bad ? "errors bad %d\n" : "errors ok\n", bad);
  return bad;
}
