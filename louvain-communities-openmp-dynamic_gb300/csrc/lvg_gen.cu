// lvg_gen.cu — graphs and batch updates generated in HBM, and the key sort
// behind the device-side batch tidy.
//
// The generators draw from the same counter-based streams as the host
// generators of liblvg_graphgen.so (splitmix64 finaliser on (seed, stream,
// index)), so a graph made here equals lvgg_planted_partition / lvgg_rmat
// row for row. Each draw is independent of the others, so every thread makes
// its own draws; the undirected pairs are then symmetrised as packed
// (u << b | v) keys, sorted and deduplicated into a sorted-row CSR.
//
// Sorting is cub::DeviceRadixSort (the toolkit's sort), used only here: for
// graph generation and the batch tidy, never inside Louvain's passes.
#include <cub/device/device_radix_sort.cuh>

#include "lvg_internal.cuh"

namespace lvg {
namespace {

__host__ __device__ inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// One independent stream per (seed, stream, index); the host generator's.
struct DRng {
  uint64_t s;
  __device__ DRng(uint64_t seed, uint64_t stream, uint64_t idx) {
    s = mix64(mix64(seed ^ mix64(stream + 0x632BE59BD9B4E019ull)) ^ idx);
  }
  __device__ uint64_t next() {
    s += 0x9E3779B97F4A7C15ull;
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  __device__ double uniform() { return double(next() >> 11) * 0x1.0p-53; }
  __device__ uint64_t below(uint64_t n) { return __umul64hi(next(), n); }
};

#define GEN_STRIDE(i, n) \
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < (n); i += size_t(gridDim.x) * blockDim.x)

// Both directions of draw i as packed keys; a self-pair becomes two sentinels.
__device__ __forceinline__ void emit_pair(uint64_t *keys, size_t i, uint32_t u, uint32_t v, int b,
                                          uint64_t sentinel) {
  const bool keep = u != v;
  keys[2 * i] = keep ? (uint64_t(u) << b | v) : sentinel;
  keys[2 * i + 1] = keep ? (uint64_t(v) << b | u) : sentinel;
}

// lvgg_planted_partition's draws: u uniform in 1..n; with probability p_in v
// is uniform in u's block, else uniform in 1..n.
__global__ void pp_draws_kernel(uint32_t n, uint32_t block, double p_in, uint64_t seed, size_t draws, int b,
                                uint64_t sentinel, uint64_t *keys) {
  GEN_STRIDE(i, draws) {
    DRng r(seed, 1, i);
    const uint32_t u = 1 + uint32_t(r.below(n));
    uint32_t v;
    if (r.uniform() < p_in) {
      const uint32_t b0 = ((u - 1) / block) * block;
      const uint32_t bn = min(block, n - b0);
      v = 1 + b0 + uint32_t(r.below(bn));
    } else {
      v = 1 + uint32_t(r.below(n));
    }
    emit_pair(keys, i, u, v, b, sentinel);
  }
}

// lvgg_rmat's draws: one quadrant choice per level, then the permutation.
__global__ void rmat_draws_kernel(int scale, double a, double ab, double abc, const uint32_t *perm, uint64_t seed,
                                  size_t draws, int b, uint64_t sentinel, uint64_t *keys) {
  GEN_STRIDE(i, draws) {
    DRng r(seed, 2, i);
    uint64_t u = 0, v = 0;
    for (int l = 0; l < scale; ++l) {
      const double x = r.uniform();
      const uint64_t bu = x >= ab, bv = (x >= a && x < ab) || x >= abc;
      u = (u << 1) | bu;
      v = (v << 1) | bv;
    }
    if (perm) {
      u = perm[u];
      v = perm[v];
    }
    emit_pair(keys, i, uint32_t(u + 1), uint32_t(v + 1), b, sentinel);
  }
}

// First occurrence of each key below the sentinel.
__global__ void unique_flags_kernel(const uint64_t *keys, size_t n, uint64_t sentinel, uint32_t *flag) {
  GEN_STRIDE(i, n) flag[i] = keys[i] < sentinel && (i == 0 || keys[i] != keys[i - 1]);
}

__global__ void compact_keys_kernel(const uint64_t *keys, const uint32_t *flag, const uint32_t *pos, size_t n,
                                    uint64_t *out) {
  GEN_STRIDE(i, n) if (flag[i]) out[pos[i]] = keys[i];
}

// Row u starts at the first unique key whose source is >= u.
__global__ void csr_offsets_kernel(const uint64_t *ukeys, size_t m, size_t span, int b, uint64_t *off) {
  GEN_STRIDE(u, span + 1) {
    const uint64_t x = uint64_t(u) << b;
    size_t lo = 0, hi = m;
    while (lo < hi) {
      const size_t mid = (lo + hi) >> 1;
      if (ukeys[mid] < x) lo = mid + 1; else hi = mid;
    }
    off[u] = lo;
  }
}

__global__ void csr_rows_kernel(const uint64_t *ukeys, size_t m, int b, uint32_t *key, float *w) {
  const uint64_t mask = (uint64_t(1) << b) - 1;
  GEN_STRIDE(i, m) {
    key[i] = uint32_t(ukeys[i] & mask);
    w[i] = 1.0f;
  }
}

__global__ void present_kernel(size_t span, uint8_t *ex) {
  GEN_STRIDE(u, span) ex[u] = u > 0;
}

// generateEdgeDeletions (inc/batch.hxx:105-117) with removeRandomEdge
// (:30-58): a source uniform in [begin, begin+range), retried up to 5 times
// while it has no edge, then a uniform neighbour; both directions. Draw l
// uses stream 5, index l. ok[l] = 1 when the draw produced an edge.
__global__ void gen_deletions_kernel(const uint64_t *off, const uint32_t *deg, const uint32_t *key, const float *w,
                                     size_t nd, uint32_t begin, uint32_t range, uint64_t seed, uint32_t *src,
                                     uint32_t *dst, float *wt, uint32_t *ok) {
  GEN_STRIDE(l, nd) {
    DRng r(seed, 5, l);
    bool got = false;
    uint32_t u = 0, v = 0;
    float x = 0.f;
    for (int t = 0; t < 5 && !got; ++t) {
      u = begin + uint32_t(double(range) * r.uniform());
      const uint32_t d = deg[u];
      if (d == 0) continue;
      const uint32_t vi = uint32_t(r.uniform() * double(d));
      v = key[off[u] + vi];
      x = w[off[u] + vi];
      got = true;
    }
    ok[l] = got;
    src[2 * l] = u; dst[2 * l] = v; wt[2 * l] = x;
    src[2 * l + 1] = v; dst[2 * l + 1] = u; wt[2 * l + 1] = x;
  }
}

// generateEdgeInsertions (inc/batch.hxx:131-143) with addRandomEdge
// (:68-83): both endpoints uniform in [begin, begin+range), both directions,
// weight `weight`. Draw l uses stream 6, index l.
__global__ void gen_insertions_kernel(size_t ni, uint32_t begin, uint32_t range, float weight, uint64_t seed,
                                      uint32_t *src, uint32_t *dst, float *wt) {
  GEN_STRIDE(l, ni) {
    DRng r(seed, 6, l);
    const uint32_t u = begin + uint32_t(double(range) * r.uniform());
    const uint32_t v = begin + uint32_t(double(range) * r.uniform());
    src[2 * l] = u; dst[2 * l] = v; wt[2 * l] = weight;
    src[2 * l + 1] = v; dst[2 * l + 1] = u; wt[2 * l + 1] = weight;
  }
}

// Drop the failed deletion draws (both directions of draw l at 2l, 2l+1).
__global__ void compact_draws_kernel(const uint32_t *src, const uint32_t *dst, const float *wt, size_t nd,
                                     const uint32_t *ok, const uint32_t *pos, uint32_t *osrc, uint32_t *odst,
                                     float *ow) {
  GEN_STRIDE(l, nd) {
    if (!ok[l]) continue;
    const size_t o = 2 * size_t(pos[l]);
    osrc[o] = src[2 * l]; odst[o] = dst[2 * l]; ow[o] = wt[2 * l];
    osrc[o + 1] = src[2 * l + 1]; odst[o + 1] = dst[2 * l + 1]; ow[o + 1] = wt[2 * l + 1];
  }
}

// Edge i of a list as a packed key, with its index.
__global__ void edge_keys_kernel(const uint32_t *src, const uint32_t *dst, size_t n, int b, uint64_t *key,
                                 uint32_t *val) {
  GEN_STRIDE(i, n) {
    key[i] = uint64_t(src[i]) << b | dst[i];
    val[i] = uint32_t(i);
  }
}

// The last of each run of equal keys (the stable sort keeps stream order, so
// that is the last occurrence: LazyBitset's set_union_last).
__global__ void last_flags_kernel(const uint64_t *key, size_t n, uint32_t *flag) {
  GEN_STRIDE(i, n) flag[i] = i + 1 == n || key[i] != key[i + 1];
}

__global__ void compact_edges_kernel(const uint64_t *key, const uint32_t *val, const uint32_t *flag,
                                     const uint32_t *pos, size_t n, const float *w, uint64_t *ukey, float *uw) {
  GEN_STRIDE(i, n) {
    if (!flag[i]) continue;
    ukey[pos[i]] = key[i];
    uw[pos[i]] = w[val[i]];
  }
}

__global__ void csr_keys_kernel(const uint64_t *ukeys, size_t m, int b, uint32_t *key) {
  const uint64_t mask = (uint64_t(1) << b) - 1;
  GEN_STRIDE(i, m) key[i] = uint32_t(ukeys[i] & mask);
}

// Vertices 1..span-1 and every endpoint are present (addVerticesIfU over
// 1..rows, then addEdge's addVertex, inc/snap.hxx:167, inc/Graph.hxx:318).
__global__ void endpoints_present_kernel(const uint32_t *src, const uint32_t *dst, size_t n, uint8_t *ex) {
  GEN_STRIDE(i, n) {
    ex[src[i]] = 1;
    ex[dst[i]] = 1;
  }
}

int bits_for(uint64_t x) {  // bits to hold values 0..x
  int b = 1;
  while (b < 64 && (x >> b)) ++b;
  return b;
}

}  // namespace

// Seeded Fisher-Yates on one stream, as lvgg_rmat permutes (sequential).
std::vector<uint32_t> rmat_permutation(int scale, uint64_t seed) {
  const uint64_t n = uint64_t(1) << scale;
  std::vector<uint32_t> perm(n);
  for (uint64_t i = 0; i < n; ++i) perm[i] = uint32_t(i);
  uint64_t st = mix64(mix64(seed ^ mix64(7 + 0x632BE59BD9B4E019ull)) ^ 0);
  for (uint64_t i = n - 1; i > 0; --i) {
    st += 0x9E3779B97F4A7C15ull;
    uint64_t z = st;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    const uint64_t j = uint64_t((unsigned __int128)z * (i + 1) >> 64);
    std::swap(perm[i], perm[j]);
  }
  return perm;
}

// ------------------------------------------------------------------- sorts

bool sort_keys_u64(uint64_t *k0, uint64_t *k1, size_t n, int end_bit, DBuf<uint8_t> &tmp, cudaStream_t s) {
  if (n > size_t(0x7FFFFFFF)) throw Error(LVG_EINVAL, "sort: more than 2^31-1 keys");
  cub::DoubleBuffer<uint64_t> d(k0, k1);
  size_t bytes = 0;
  LVG_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, bytes, d, int(n), 0, end_bit, s));
  tmp.ensure(bytes);
  LVG_CUDA(cub::DeviceRadixSort::SortKeys(tmp.p, bytes, d, int(n), 0, end_bit, s));
  return d.selector != 0;
}

bool sort_pairs_u64(uint64_t *k0, uint64_t *k1, uint32_t *v0, uint32_t *v1, size_t n, int end_bit,
                    DBuf<uint8_t> &tmp, cudaStream_t s) {
  if (n > size_t(0x7FFFFFFF)) throw Error(LVG_EINVAL, "sort: more than 2^31-1 keys");
  cub::DoubleBuffer<uint64_t> d(k0, k1);
  cub::DoubleBuffer<uint32_t> e(v0, v1);
  size_t bytes = 0;
  LVG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, bytes, d, e, int(n), 0, end_bit, s));
  tmp.ensure(bytes);
  LVG_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, bytes, d, e, int(n), 0, end_bit, s));
  return d.selector != 0;
}

// --------------------------------------------------------------- graphs

// Draw, symmetrise, sort and deduplicate; the result is a compact CSR in
// HBM (coff[span+1], ckey/cw[X], ex[span]). Returns X.
size_t generate_graph(const GenSpec &g, DBuf<uint64_t> &coff, DBuf<uint32_t> &ckey, DBuf<float> &cw,
                      DBuf<uint8_t> &ex, cudaStream_t s) {
  const size_t span = g.span, draws = g.draws;
  if (2 * draws > size_t(0x7FFFFFFF)) throw Error(LVG_EINVAL, "generator: more than 2^30 draws");
  const int b = bits_for(span);
  const uint64_t sentinel = uint64_t(span) << b;  // above every (u < span) key
  const int end_bit = std::min(64, 2 * b + 1);
  const size_t n = 2 * draws;
  DBuf<uint64_t> k0, k1;
  DBuf<uint32_t> flag, pos, perm, scan;
  DBuf<uint8_t> tmp;
  k0.ensure(n);
  k1.ensure(n);
  if (g.kind == GenSpec::PP) {
    pp_draws_kernel<<<grid_for(draws, 256), 256, 0, s>>>(g.n, g.block, g.p_in, g.seed, draws, b, sentinel, k0.p);
  } else {
    if (!g.perm.empty()) {
      perm.ensure(g.perm.size());
      LVG_CUDA(cudaMemcpyAsync(perm.p, g.perm.data(), g.perm.size() * 4, cudaMemcpyHostToDevice, s));
    }
    rmat_draws_kernel<<<grid_for(draws, 256), 256, 0, s>>>(g.scale, g.a, g.ab, g.abc, g.perm.empty() ? nullptr : perm.p,
                                                           g.seed, draws, b, sentinel, k0.p);
  }
  LVG_CHECK_LAUNCH();
  const bool alt = n ? sort_keys_u64(k0.p, k1.p, n, end_bit, tmp, s) : false;
  const uint64_t *sorted = alt ? k1.p : k0.p;
  uint64_t *uniq = alt ? k0.p : k1.p;
  flag.ensure(n + 1);
  pos.ensure(n + 1);
  scan.ensure(scan_scratch_elems(n + 1));
  size_t m = 0;
  if (n) {
    unique_flags_kernel<<<grid_for(n, 256), 256, 0, s>>>(sorted, n, sentinel, flag.p);
    LVG_CHECK_LAUNCH();
    exclusive_scan_u32(flag.p, pos.p, n, pos.p + n, scan.p, s);
    compact_keys_kernel<<<grid_for(n, 256), 256, 0, s>>>(sorted, flag.p, pos.p, n, uniq);
    LVG_CHECK_LAUNCH();
    uint32_t cnt = 0;
    LVG_CUDA(cudaMemcpyAsync(&cnt, pos.p + n, 4, cudaMemcpyDeviceToHost, s));
    LVG_CUDA(cudaStreamSynchronize(s));
    m = cnt;
  }
  coff.ensure(span + 1);
  ckey.ensure(m);
  cw.ensure(m);
  ex.ensure(span);
  csr_offsets_kernel<<<grid_for(span + 1, 256), 256, 0, s>>>(uniq, m, span, b, coff.p);
  LVG_CHECK_LAUNCH();
  if (m) {
    csr_rows_kernel<<<grid_for(m, 256), 256, 0, s>>>(uniq, m, b, ckey.p, cw.p);
    LVG_CHECK_LAUNCH();
  }
  present_kernel<<<grid_for(span, 256), 256, 0, s>>>(span, ex.p);
  LVG_CHECK_LAUNCH();
  LVG_CUDA(cudaStreamSynchronize(s));  // the scratch is freed next
  return m;
}

// The graph of an edge list (device arrays src/dst/w of n entries, ids <
// span): rows sorted by neighbour id, duplicates merged keeping the last
// weight in list order. Returns X.
size_t graph_from_edges(const uint32_t *src, const uint32_t *dst, const float *w, size_t n, size_t span,
                        DBuf<uint64_t> &coff, DBuf<uint32_t> &ckey, DBuf<float> &cw, DBuf<uint8_t> &ex,
                        cudaStream_t s) {
  if (n > size_t(0x7FFFFFFF)) throw Error(LVG_EINVAL, "edge list: more than 2^31-1 entries");
  const int b = bits_for(span);
  DBuf<uint64_t> k0, k1;
  DBuf<uint32_t> v0, v1, flag, pos, scan;
  DBuf<uint8_t> tmp;
  k0.ensure(n); k1.ensure(n); v0.ensure(n); v1.ensure(n);
  size_t m = 0;
  const uint64_t *uniq = k1.p;
  if (n) {
    edge_keys_kernel<<<grid_for(n, 256), 256, 0, s>>>(src, dst, n, b, k0.p, v0.p);
    LVG_CHECK_LAUNCH();
    const bool alt = sort_pairs_u64(k0.p, k1.p, v0.p, v1.p, n, 2 * b, tmp, s);
    const uint64_t *sk = alt ? k1.p : k0.p;
    const uint32_t *sv = alt ? v1.p : v0.p;
    uint64_t *uk = alt ? k0.p : k1.p;
    flag.ensure(n + 1); pos.ensure(n + 1); scan.ensure(scan_scratch_elems(n + 1));
    cw.ensure(n);
    last_flags_kernel<<<grid_for(n, 256), 256, 0, s>>>(sk, n, flag.p);
    LVG_CHECK_LAUNCH();
    exclusive_scan_u32(flag.p, pos.p, n, pos.p + n, scan.p, s);
    compact_edges_kernel<<<grid_for(n, 256), 256, 0, s>>>(sk, sv, flag.p, pos.p, n, w, uk, cw.p);
    LVG_CHECK_LAUNCH();
    uint32_t cnt = 0;
    LVG_CUDA(cudaMemcpyAsync(&cnt, pos.p + n, 4, cudaMemcpyDeviceToHost, s));
    LVG_CUDA(cudaStreamSynchronize(s));
    m = cnt;
    uniq = uk;
  }
  coff.ensure(span + 1);
  ckey.ensure(m);
  cw.ensure(m);
  ex.ensure(span);
  csr_offsets_kernel<<<grid_for(span + 1, 256), 256, 0, s>>>(uniq, m, span, b, coff.p);
  LVG_CHECK_LAUNCH();
  if (m) {
    csr_keys_kernel<<<grid_for(m, 256), 256, 0, s>>>(uniq, m, b, ckey.p);
    LVG_CHECK_LAUNCH();
  }
  present_kernel<<<grid_for(span, 256), 256, 0, s>>>(span, ex.p);
  LVG_CHECK_LAUNCH();
  if (n) {
    endpoints_present_kernel<<<grid_for(n, 256), 256, 0, s>>>(src, dst, n, ex.p);
    LVG_CHECK_LAUNCH();
  }
  LVG_CUDA(cudaStreamSynchronize(s));  // the scratch is freed next
  return m;
}

// --------------------------------------------------------------- batches

void generate_batch(const uint64_t *off, const uint32_t *deg, const uint32_t *key, const float *w, size_t nd,
                    size_t ni, uint32_t begin, uint32_t range, float weight, uint64_t seed, DBuf<uint32_t> &ds,
                    DBuf<uint32_t> &dd, DBuf<float> &dw, DBuf<uint32_t> &is, DBuf<uint32_t> &id,
                    DBuf<float> &iw, size_t &out_nd, size_t &out_ni, cudaStream_t s) {
  if (nd > size_t(0x3FFFFFFF) || ni > size_t(0x3FFFFFFF)) throw Error(LVG_EINVAL, "generator: batch too large");
  DBuf<uint32_t> ts, td, ok, pos, scan;
  DBuf<float> tw;
  is.ensure(2 * ni);
  id.ensure(2 * ni);
  iw.ensure(2 * ni);
  if (ni) {
    gen_insertions_kernel<<<grid_for(ni, 256), 256, 0, s>>>(ni, begin, range, weight, seed, is.p, id.p, iw.p);
    LVG_CHECK_LAUNCH();
  }
  ds.ensure(2 * nd);
  dd.ensure(2 * nd);
  dw.ensure(2 * nd);
  uint32_t kept = 0;
  if (nd) {
    ts.ensure(2 * nd); td.ensure(2 * nd); tw.ensure(2 * nd);
    ok.ensure(nd + 1); pos.ensure(nd + 1); scan.ensure(scan_scratch_elems(nd + 1));
    gen_deletions_kernel<<<grid_for(nd, 256), 256, 0, s>>>(off, deg, key, w, nd, begin, range, seed, ts.p, td.p, tw.p,
                                                           ok.p);
    LVG_CHECK_LAUNCH();
    exclusive_scan_u32(ok.p, pos.p, nd, pos.p + nd, scan.p, s);
    compact_draws_kernel<<<grid_for(nd, 256), 256, 0, s>>>(ts.p, td.p, tw.p, nd, ok.p, pos.p, ds.p, dd.p, dw.p);
    LVG_CHECK_LAUNCH();
    LVG_CUDA(cudaMemcpyAsync(&kept, pos.p + nd, 4, cudaMemcpyDeviceToHost, s));
  }
  LVG_CUDA(cudaStreamSynchronize(s));
  out_nd = 2 * size_t(kept);
  out_ni = 2 * ni;
}

}  // namespace lvg
