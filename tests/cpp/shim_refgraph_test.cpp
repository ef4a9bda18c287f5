// A caller that holds the reference's own graph type: compiled against the
// reference's unmodified headers (its inc/ directory on the include path) and
// include/louvain_gb300.hxx, it builds a DiGraph<uint32_t, None, float>, draws
// a batch with the reference's generateEdgeDeletions / generateEdgeInsertions,
// tidies and applies it with tidyBatchUpdateU + applyBatchUpdateOmpU — the
// sequence of main.cxx:89-126 — and runs each method twice on the same
// inputs: the reference's own template (louvain.hxx:1285-1690) and the shim's
// GPU entry point of the same name. Both results are scored with the
// reference's modularityBy (properties.hxx:178); the GPU's must be within
// 0.005 of the reference's, and every membership must be a valid id.
//
// The shim's names are kept out of the global namespace (LVG_NO_GLOBAL_NAMES)
// because the reference's templates of the same names live there.
#define LVG_NO_GLOBAL_NAMES
#include "inc/main.hxx"

#include <cmath>
#include <cstdio>
#include <random>

#include "louvain_gb300.hxx"

using K = uint32_t;
using V = float;
using Graph = DiGraph<K, None, V>;

template <class R>
static double quality(const Graph &x, const R &a) {
  const double M = edgeWeightOmp(x) / 2;
  return modularityBy(x, [&](auto u) { return a.membership[u]; }, M, 1.0);
}

int main() {
  const K n = 8192, block = 64;
  Graph x;
  x.respan(n + 1);
  for (K u = 1; u <= n; ++u) x.addVertex(u);  // vertex 0 absent, as in the SNAP graphs
  std::mt19937_64 rnd(2024);
  for (K i = 0; i < n * 8; ++i) {
    const K u = 1 + rnd() % n;
    const K v = (rnd() % 10 < 8) ? 1 + ((u - 1) / block) * block + rnd() % block : 1 + rnd() % n;
    if (u == v) continue;
    x.addEdge(u, v, 1.0f);
    x.addEdge(v, u, 1.0f);
  }
  x.update();
  int bad = 0;
  auto check = [&](const char *what, double qr, double qg, const std::vector<K> &m) {
    for (K u = 1; u <= n; ++u)
      if (m[u] > n) ++bad;
    const bool ok = std::fabs(qr - qg) <= 0.005;
    if (!ok) ++bad;
    std::printf("%-8s reference Q %.6f  gpu Q %.6f  %s\n", what, qr, qg, ok ? "ok" : "FAR");
  };
  // static (main.cxx:89)
  auto r0 = ::louvainStaticOmp(x, ::LouvainOptions(1));
  auto g0 = louvain_gb300::louvainStaticOmp(x, louvain_gb300::LouvainOptions(1));
  check("static", quality(x, r0), quality(x, g0), g0.membership);
  // a batch of 1e-3 |E| (main.cxx:101-111), applied to a copy
  auto y = duplicate(x);
  const size_t nb = x.size() / 2000;
  auto deletions = generateEdgeDeletions(rnd, y, nb / 5, 1, n, true);
  auto insertions = generateEdgeInsertions(rnd, y, nb - nb / 5, 1, n, true, V(1));
  tidyBatchUpdateU(deletions, insertions, y);
  applyBatchUpdateOmpU(y, deletions, insertions);
  // the dynamic methods from the reference's static result (main.cxx:119-125)
  auto &q = r0.membership;
  auto &vt = r0.vertexWeight;
  auto &ct = r0.communityWeight;
  auto r1 = ::louvainNaiveDynamicOmp(y, deletions, insertions, q, vt, ct, ::LouvainOptions(1));
  auto g1 = louvain_gb300::louvainNaiveDynamicOmp(y, deletions, insertions, q, vt, ct);
  check("naive", quality(y, r1), quality(y, g1), g1.membership);
  auto r2 = ::louvainDynamicDeltaScreeningOmp(y, deletions, insertions, q, vt, ct, ::LouvainOptions(1));
  auto g2 = louvain_gb300::louvainDynamicDeltaScreeningOmp(y, deletions, insertions, q, vt, ct);
  check("delta", quality(y, r2), quality(y, g2), g2.membership);
  auto r3 = ::louvainDynamicFrontierOmp(y, deletions, insertions, q, vt, ct, ::LouvainOptions(1));
  auto g3 = louvain_gb300::louvainDynamicFrontierOmp(y, deletions, insertions, q, vt, ct);
  check("frontier", quality(y, r3), quality(y, g3), g3.membership);
  // the shim's result type takes the reference result's constructor arguments
  louvain_gb300::LouvainResult<K> copy(std::move(g3.membership), std::move(g3.vertexWeight),
                                       std::move(g3.communityWeight), g3.iterations, g3.passes);
  if (copy.membership.size() != n + 1 || copy.passes != g3.passes) ++bad;
  std::printf("bad %d\n", bad);
  return bad ? 1 : 0;
}
