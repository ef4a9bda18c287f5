// lvg_graphgen.cpp — seeded synthetic graphs and batch updates (host, OpenMP).
//
// Conventions follow the reference's graph inputs: ids 1..n with vertex 0
// absent (inc/snap.hxx:133), sorted rows (inc/_bitset.hxx:227-262), tidy
// batches (inc/batch.hxx:202-209) applied as remove-then-add
// (inc/batch.hxx:241-248). The RNG is counter based, so results do not depend
// on the number of OpenMP threads.
#include "louvain_gb300_graphgen.h"

#include <omp.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

namespace {

thread_local std::string g_err;

int fail(int code, const char *msg) {
  g_err = msg;
  return code;
}

inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// One independent stream per (seed, stream, index).
struct Rng {
  uint64_t s;
  Rng(uint64_t seed, uint64_t stream, uint64_t idx) {
    s = mix64(mix64(seed ^ mix64(stream + 0x632BE59BD9B4E019ull)) ^ idx);
  }
  uint64_t next() {
    s += 0x9E3779B97F4A7C15ull;
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return double(next() >> 11) * 0x1.0p-53; }
  uint64_t below(uint64_t n) { return uint64_t((unsigned __int128)next() * n >> 64); }
};

template <class T>
T *xalloc(size_t n) {
  void *p = std::malloc(std::max<size_t>(n, 1) * sizeof(T));
  if (!p) throw std::bad_alloc();
  return static_cast<T *>(p);
}

// Build a symmetric, deduplicated, row-sorted CSR from undirected pairs
// (self-loops already removed). All ids 1..span-1 exist.
void build_symmetric_csr(size_t span, const std::vector<uint32_t> &eu, const std::vector<uint32_t> &ev,
                         lvgg_csr *out) {
  const size_t P = eu.size();
  std::vector<uint64_t> cnt(span + 1, 0);
  #pragma omp parallel for schedule(static)
  for (size_t i = 0; i < P; ++i) {
    __atomic_fetch_add(&cnt[eu[i]], 1, __ATOMIC_RELAXED);
    __atomic_fetch_add(&cnt[ev[i]], 1, __ATOMIC_RELAXED);
  }
  std::vector<uint64_t> off(span + 1, 0);
  for (size_t u = 0; u < span; ++u) off[u + 1] = off[u] + cnt[u];
  std::vector<uint32_t> rows(off[span]);
  std::vector<uint64_t> cur(off.begin(), off.end() - 1);
  #pragma omp parallel for schedule(static)
  for (size_t i = 0; i < P; ++i) {
    uint64_t a = __atomic_fetch_add(&cur[eu[i]], 1, __ATOMIC_RELAXED);
    rows[a] = ev[i];
    uint64_t b = __atomic_fetch_add(&cur[ev[i]], 1, __ATOMIC_RELAXED);
    rows[b] = eu[i];
  }
  // Sort and deduplicate each row; record the unique degree.
  std::vector<uint64_t> udeg(span + 1, 0);
  #pragma omp parallel for schedule(dynamic, 1024)
  for (size_t u = 0; u < span; ++u) {
    uint32_t *b = rows.data() + off[u], *e = rows.data() + off[u + 1];
    std::sort(b, e);
    udeg[u] = uint64_t(std::unique(b, e) - b);
  }
  out->span = span;
  out->offsets = xalloc<uint64_t>(span + 1);
  out->offsets[0] = 0;
  for (size_t u = 0; u < span; ++u) out->offsets[u + 1] = out->offsets[u] + udeg[u];
  out->num_edges = out->offsets[span];
  out->keys = xalloc<uint32_t>(out->num_edges);
  out->weights = xalloc<float>(out->num_edges);
  out->exists = xalloc<uint8_t>(span);
  #pragma omp parallel for schedule(dynamic, 1024)
  for (size_t u = 0; u < span; ++u) {
    std::memcpy(out->keys + out->offsets[u], rows.data() + off[u], udeg[u] * sizeof(uint32_t));
    std::fill(out->weights + out->offsets[u], out->weights + out->offsets[u + 1], 1.0f);
    out->exists[u] = u > 0;
  }
}

bool has_edge(const lvgg_csr *x, uint32_t u, uint32_t v) {
  const uint32_t *b = x->keys + x->offsets[u], *e = x->keys + x->offsets[u + 1];
  return std::binary_search(b, e, v);
}

}  // namespace

extern "C" {

const char *lvgg_last_error(void) { return g_err.c_str(); }

void lvgg_csr_free(lvgg_csr *g) {
  if (!g) return;
  std::free(g->offsets);
  std::free(g->keys);
  std::free(g->weights);
  std::free(g->exists);
  std::memset(g, 0, sizeof(*g));
}

void lvgg_batch_free(lvgg_batch *b) {
  if (!b) return;
  std::free(b->del_src);
  std::free(b->del_dst);
  std::free(b->del_w);
  std::free(b->ins_src);
  std::free(b->ins_dst);
  std::free(b->ins_w);
  std::memset(b, 0, sizeof(*b));
}

int lvgg_planted_partition(uint32_t n, uint32_t block, double avg_degree, double p_in, uint64_t seed,
                           lvgg_csr *out) {
  if (!out || n == 0 || block == 0 || avg_degree < 0 || p_in < 0 || p_in > 1)
    return fail(-EINVAL, "lvgg_planted_partition: bad argument");
  std::memset(out, 0, sizeof(*out));
  try {
    const size_t draws = size_t(std::llround(double(n) * avg_degree / 2));
    std::vector<uint32_t> eu(draws), ev(draws);
    std::vector<uint8_t> keep(draws);
    #pragma omp parallel for schedule(static)
    for (size_t i = 0; i < draws; ++i) {
      Rng r(seed, 1, i);
      uint32_t u = 1 + uint32_t(r.below(n));
      uint32_t v;
      if (r.uniform() < p_in) {
        uint32_t b0 = ((u - 1) / block) * block;
        uint32_t bn = std::min<uint32_t>(block, n - b0);
        v = 1 + b0 + uint32_t(r.below(bn));
      } else {
        v = 1 + uint32_t(r.below(n));
      }
      eu[i] = u; ev[i] = v; keep[i] = u != v;
    }
    size_t k = 0;
    for (size_t i = 0; i < draws; ++i)
      if (keep[i]) { eu[k] = eu[i]; ev[k] = ev[i]; ++k; }
    eu.resize(k); ev.resize(k);
    build_symmetric_csr(size_t(n) + 1, eu, ev, out);
  } catch (const std::bad_alloc &) {
    lvgg_csr_free(out);
    return fail(-ENOMEM, "lvgg_planted_partition: out of memory");
  }
  return 0;
}

int lvgg_rmat(int scale, double edge_factor, double a, double b, double c, int permute, uint64_t seed,
              lvgg_csr *out) {
  if (!out || scale < 1 || scale > 31 || edge_factor < 0 || a < 0 || b < 0 || c < 0 || a + b + c > 1)
    return fail(-EINVAL, "lvgg_rmat: bad argument");
  std::memset(out, 0, sizeof(*out));
  try {
    const uint64_t n = uint64_t(1) << scale;
    const size_t draws = size_t(std::llround(double(n) * edge_factor));
    std::vector<uint32_t> perm;
    if (permute) {
      // Seeded Fisher-Yates on one stream (sequential, deterministic).
      perm.resize(n);
      for (uint64_t i = 0; i < n; ++i) perm[i] = uint32_t(i);
      Rng r(seed, 7, 0);
      for (uint64_t i = n - 1; i > 0; --i) std::swap(perm[i], perm[r.below(i + 1)]);
    }
    std::vector<uint32_t> eu(draws), ev(draws);
    std::vector<uint8_t> keep(draws);
    const double ab = a + b, abc = a + b + c;
    #pragma omp parallel for schedule(static)
    for (size_t i = 0; i < draws; ++i) {
      Rng r(seed, 2, i);
      uint64_t u = 0, v = 0;
      for (int l = 0; l < scale; ++l) {
        double x = r.uniform();
        uint64_t bu = x >= ab, bv = (x >= a && x < ab) || x >= abc;
        u = (u << 1) | bu;
        v = (v << 1) | bv;
      }
      if (permute) { u = perm[u]; v = perm[v]; }
      eu[i] = uint32_t(u + 1); ev[i] = uint32_t(v + 1); keep[i] = u != v;
    }
    size_t k = 0;
    for (size_t i = 0; i < draws; ++i)
      if (keep[i]) { eu[k] = eu[i]; ev[k] = ev[i]; ++k; }
    eu.resize(k); ev.resize(k);
    build_symmetric_csr(size_t(n) + 1, eu, ev, out);
  } catch (const std::bad_alloc &) {
    lvgg_csr_free(out);
    return fail(-ENOMEM, "lvgg_rmat: out of memory");
  }
  return 0;
}

int lvgg_random_batch(const lvgg_csr *x, size_t num_updates, double insertion_fraction, uint64_t seed,
                      lvgg_batch *out) {
  if (!x || !out || insertion_fraction < 0 || insertion_fraction > 1)
    return fail(-EINVAL, "lvgg_random_batch: bad argument");
  std::memset(out, 0, sizeof(*out));
  const size_t ni = size_t(std::llround(double(num_updates) * insertion_fraction));
  const size_t nd = num_updates - ni;
  const size_t S = x->span;
  try {
    // Existing vertex ids, for uniform pair sampling.
    std::vector<uint32_t> ids;
    ids.reserve(S);
    for (size_t u = 0; u < S; ++u)
      if (!x->exists || x->exists[u]) ids.push_back(uint32_t(u));
    std::vector<uint64_t> dels, inss;  // canonical (min<<32 | max) pairs
    Rng rd(seed, 3, 0), ri(seed, 4, 0);
    const size_t E = x->num_edges;
    // Deletions: uniform over directed edge slots = uniform over undirected edges.
    for (size_t tries = 0; E > 0 && dels.size() < nd && tries < 64; ++tries) {
      while (dels.size() < nd) {
        uint64_t j = rd.below(E);
        uint32_t u = uint32_t(std::upper_bound(x->offsets, x->offsets + S + 1, j) - x->offsets - 1);
        uint32_t v = x->keys[j];
        uint64_t p = u < v ? (uint64_t(u) << 32 | v) : (uint64_t(v) << 32 | u);
        dels.push_back(p);
      }
      std::sort(dels.begin(), dels.end());
      dels.erase(std::unique(dels.begin(), dels.end()), dels.end());
    }
    // Insertions: uniform vertex pairs, u != v, edge absent.
    for (size_t tries = 0; ids.size() > 1 && inss.size() < ni && tries < 64; ++tries) {
      size_t guard = 0;
      while (inss.size() < ni && guard < 64 * (ni + 1)) {
        ++guard;
        uint32_t u = ids[ri.below(ids.size())], v = ids[ri.below(ids.size())];
        if (u == v || has_edge(x, u, v)) continue;
        inss.push_back(u < v ? (uint64_t(u) << 32 | v) : (uint64_t(v) << 32 | u));
      }
      std::sort(inss.begin(), inss.end());
      inss.erase(std::unique(inss.begin(), inss.end()), inss.end());
    }
    auto emit = [&](const std::vector<uint64_t> &pairs, size_t &cnt, uint32_t *&src, uint32_t *&dst, float *&w,
                    bool existing) {
      std::vector<uint64_t> dir;
      dir.reserve(2 * pairs.size());
      for (uint64_t p : pairs) {
        uint32_t u = uint32_t(p >> 32), v = uint32_t(p);
        dir.push_back(uint64_t(u) << 32 | v);
        dir.push_back(uint64_t(v) << 32 | u);
      }
      std::sort(dir.begin(), dir.end());
      cnt = dir.size();
      src = xalloc<uint32_t>(cnt); dst = xalloc<uint32_t>(cnt); w = xalloc<float>(cnt);
      for (size_t i = 0; i < cnt; ++i) {
        src[i] = uint32_t(dir[i] >> 32);
        dst[i] = uint32_t(dir[i]);
        w[i] = 1.0f;
        if (existing) {
          const uint32_t *b = x->keys + x->offsets[src[i]], *e = x->keys + x->offsets[src[i] + 1];
          w[i] = x->weights[std::lower_bound(b, e, dst[i]) - x->keys];
        }
      }
    };
    emit(dels, out->num_deletions, out->del_src, out->del_dst, out->del_w, true);
    emit(inss, out->num_insertions, out->ins_src, out->ins_dst, out->ins_w, false);
  } catch (const std::bad_alloc &) {
    lvgg_batch_free(out);
    return fail(-ENOMEM, "lvgg_random_batch: out of memory");
  }
  return 0;
}

int lvgg_reference_batch(const lvgg_csr *x, size_t deletions, size_t insertions, uint32_t begin, uint32_t range,
                         float weight, uint64_t seed, lvgg_batch *out) {
  if (!x || !out || range == 0 || size_t(begin) + range > x->span)
    return fail(-EINVAL, "lvgg_reference_batch: bad argument");
  std::memset(out, 0, sizeof(*out));
  try {
    std::vector<uint32_t> ds, dd;
    std::vector<float> dw;
    for (size_t l = 0; l < deletions; ++l) {
      Rng r(seed, 5, l);
      for (int t = 0; t < 5; ++t) {
        const uint32_t u = begin + uint32_t(double(range) * r.uniform());
        const uint64_t d = x->offsets[u + 1] - x->offsets[u];
        if (d == 0) continue;
        const uint64_t j = x->offsets[u] + uint64_t(uint32_t(r.uniform() * double(d)));
        const uint32_t v = x->keys[j];
        ds.push_back(u); dd.push_back(v); dw.push_back(x->weights[j]);
        ds.push_back(v); dd.push_back(u); dw.push_back(x->weights[j]);
        break;
      }
    }
    out->num_deletions = ds.size();
    out->del_src = xalloc<uint32_t>(ds.size());
    out->del_dst = xalloc<uint32_t>(ds.size());
    out->del_w = xalloc<float>(ds.size());
    std::copy(ds.begin(), ds.end(), out->del_src);
    std::copy(dd.begin(), dd.end(), out->del_dst);
    std::copy(dw.begin(), dw.end(), out->del_w);
    out->num_insertions = 2 * insertions;
    out->ins_src = xalloc<uint32_t>(2 * insertions);
    out->ins_dst = xalloc<uint32_t>(2 * insertions);
    out->ins_w = xalloc<float>(2 * insertions);
    for (size_t l = 0; l < insertions; ++l) {
      Rng r(seed, 6, l);
      const uint32_t u = begin + uint32_t(double(range) * r.uniform());
      const uint32_t v = begin + uint32_t(double(range) * r.uniform());
      out->ins_src[2 * l] = u; out->ins_dst[2 * l] = v; out->ins_w[2 * l] = weight;
      out->ins_src[2 * l + 1] = v; out->ins_dst[2 * l + 1] = u; out->ins_w[2 * l + 1] = weight;
    }
  } catch (const std::bad_alloc &) {
    lvgg_batch_free(out);
    return fail(-ENOMEM, "lvgg_reference_batch: out of memory");
  }
  return 0;
}

// ------------------------------------------------------------ temporal

}  // extern "C"

struct lvgg_temporal {
  std::FILE *f = nullptr;
  int weighted = 0;
  std::vector<char> buf;
};

namespace {

// "u v [w] ..." -> true when at least u and v parse (strtoull/strtod as
// readTemporalDoOmp parses, inc/snap.hxx:85-90).
bool parse_line(const char *line, int weighted, uint64_t &u, uint64_t &v, double &w) {
  char *e = nullptr;
  u = std::strtoull(line, &e, 10);
  if (e == line) return false;
  const char *p = e;
  v = std::strtoull(p, &e, 10);
  if (e == p) return false;
  w = 1;
  if (weighted) {
    p = e;
    double x = std::strtod(p, &e);
    if (e != p && x != 0) w = x;
  }
  return true;
}

void edges_alloc(lvgg_edges *e, size_t n) {
  e->n = n;
  e->src = xalloc<uint32_t>(n);
  e->dst = xalloc<uint32_t>(n);
  e->w = xalloc<float>(n);
}

}  // namespace

extern "C" {

void lvgg_edges_free(lvgg_edges *e) {
  if (!e) return;
  std::free(e->src);
  std::free(e->dst);
  std::free(e->w);
  std::memset(e, 0, sizeof(*e));
}

int lvgg_temporal_open(const char *path, int weighted, lvgg_temporal **out) {
  if (!path || !out) return fail(-EINVAL, "lvgg_temporal_open: bad argument");
  *out = nullptr;
  std::FILE *f = std::fopen(path, "r");
  if (!f) return fail(-ENOENT, "lvgg_temporal_open: cannot open the file");
  lvgg_temporal *t = new (std::nothrow) lvgg_temporal();
  if (!t) {
    std::fclose(f);
    return fail(-ENOMEM, "lvgg_temporal_open: out of memory");
  }
  t->f = f;
  t->weighted = weighted;
  t->buf.resize(1 << 16);
  *out = t;
  return 0;
}

int lvgg_temporal_read(lvgg_temporal *t, size_t lines, int symmetric, lvgg_edges *out) {
  if (!t || !out) return fail(-EINVAL, "lvgg_temporal_read: bad argument");
  std::memset(out, 0, sizeof(*out));
  try {
    std::vector<uint32_t> s, d;
    std::vector<float> w;
    for (size_t i = 0; i < lines; ++i) {
      if (!std::fgets(t->buf.data(), int(t->buf.size()), t->f)) break;
      uint64_t u, v;
      double x;
      if (!parse_line(t->buf.data(), t->weighted, u, v, x)) break;
      if (u > 0xFFFFFFFEull || v > 0xFFFFFFFEull) return fail(-EINVAL, "lvgg_temporal_read: id does not fit 32 bits");
      s.push_back(uint32_t(u)); d.push_back(uint32_t(v)); w.push_back(float(x));
      if (symmetric) { s.push_back(uint32_t(v)); d.push_back(uint32_t(u)); w.push_back(float(x)); }
    }
    edges_alloc(out, s.size());
    std::copy(s.begin(), s.end(), out->src);
    std::copy(d.begin(), d.end(), out->dst);
    std::copy(w.begin(), w.end(), out->w);
  } catch (const std::bad_alloc &) {
    lvgg_edges_free(out);
    return fail(-ENOMEM, "lvgg_temporal_read: out of memory");
  }
  return 0;
}

void lvgg_temporal_close(lvgg_temporal *t) {
  if (!t) return;
  if (t->f) std::fclose(t->f);
  delete t;
}

int lvgg_temporal_write(const char *path, const lvgg_edges *e) {
  if (!path || !e) return fail(-EINVAL, "lvgg_temporal_write: bad argument");
  std::FILE *f = std::fopen(path, "w");
  if (!f) return fail(-ENOENT, "lvgg_temporal_write: cannot create the file");
  for (size_t i = 0; i < e->n; ++i) std::fprintf(f, "%u %u %zu\n", e->src[i], e->dst[i], i);
  return std::fclose(f) == 0 ? 0 : fail(-EIO, "lvgg_temporal_write: write failed");
}

int lvgg_csr_from_edges(size_t rows, const lvgg_edges *e, lvgg_csr *out) {
  if (!e || !out || rows >= 0xFFFFFFFFull) return fail(-EINVAL, "lvgg_csr_from_edges: bad argument");
  std::memset(out, 0, sizeof(*out));
  const size_t S = rows + 1;
  for (size_t i = 0; i < e->n; ++i)
    if (e->src[i] >= S || e->dst[i] >= S) return fail(-EINVAL, "lvgg_csr_from_edges: id > rows");
  try {
    // per source, in stream order; then sort by target keeping the last of equal targets
    std::vector<uint64_t> cnt(S + 1, 0);
    for (size_t i = 0; i < e->n; ++i) ++cnt[e->src[i] + 1];
    for (size_t u = 0; u < S; ++u) cnt[u + 1] += cnt[u];
    std::vector<uint64_t> cur(cnt.begin(), cnt.end() - 1);
    std::vector<uint64_t> idx(e->n);
    for (size_t i = 0; i < e->n; ++i) idx[cur[e->src[i]]++] = i;
    std::vector<uint64_t> deg(S, 0);
    #pragma omp parallel for schedule(dynamic, 1024)
    for (size_t u = 0; u < S; ++u) {
      uint64_t *b = idx.data() + cnt[u], *f = idx.data() + cnt[u + 1];
      std::stable_sort(b, f, [&](uint64_t a, uint64_t c) { return e->dst[a] < e->dst[c]; });
      size_t m = 0;
      for (uint64_t *p = b; p < f; ++p) {
        if (m && e->dst[b[m - 1]] == e->dst[*p]) b[m - 1] = *p;  // the last duplicate wins
        else b[m++] = *p;
      }
      deg[u] = m;
    }
    out->span = S;
    out->offsets = xalloc<uint64_t>(S + 1);
    out->offsets[0] = 0;
    for (size_t u = 0; u < S; ++u) out->offsets[u + 1] = out->offsets[u] + deg[u];
    out->num_edges = out->offsets[S];
    out->keys = xalloc<uint32_t>(out->num_edges);
    out->weights = xalloc<float>(out->num_edges);
    out->exists = xalloc<uint8_t>(S);
    #pragma omp parallel for schedule(dynamic, 1024)
    for (size_t u = 0; u < S; ++u) {
      for (uint64_t j = 0; j < deg[u]; ++j) {
        const uint64_t i = idx[cnt[u] + j];
        out->keys[out->offsets[u] + j] = e->dst[i];
        out->weights[out->offsets[u] + j] = e->w[i];
      }
      out->exists[u] = u > 0;  // vertices 1..rows (addVerticesIfU, inc/snap.hxx:167)
    }
    for (size_t i = 0; i < e->n; ++i) out->exists[e->src[i]] = out->exists[e->dst[i]] = 1;
  } catch (const std::bad_alloc &) {
    lvgg_csr_free(out);
    return fail(-ENOMEM, "lvgg_csr_from_edges: out of memory");
  }
  return 0;
}

int lvgg_temporal_drift(uint32_t n, uint32_t communities, double sigma, size_t edges, double p_in,
                        size_t drift_every, double drift, uint64_t seed, lvgg_edges *out) {
  if (!out || n == 0 || communities == 0 || communities > n || sigma < 0 || p_in < 0 || p_in > 1 || drift < 0 ||
      drift > 1)
    return fail(-EINVAL, "lvgg_temporal_drift: bad argument");
  std::memset(out, 0, sizeof(*out));
  try {
    // community sizes ~ log-normal(0, sigma), scaled to n; vertices assigned in id order
    std::vector<double> wsz(communities);
    double tot = 0;
    for (uint32_t c = 0; c < communities; ++c) {
      Rng r(seed, 8, c);
      const double u1 = std::max(r.uniform(), 1e-300), u2 = r.uniform();
      const double z = std::sqrt(-2 * std::log(u1)) * std::cos(6.283185307179586 * u2);
      wsz[c] = std::exp(sigma * z);
      tot += wsz[c];
    }
    std::vector<uint32_t> com(size_t(n) + 1, 0);
    std::vector<std::vector<uint32_t>> members(communities);
    uint32_t v = 1;
    double acc = 0;
    for (uint32_t c = 0; c < communities && v <= n; ++c) {
      acc += wsz[c];
      const uint32_t end = (c + 1 == communities) ? n : uint32_t(std::min<double>(n, std::llround(acc / tot * n)));
      for (; v <= end; ++v) { com[v] = c; members[c].push_back(v); }
      if (members[c].empty() && v <= n) { com[v] = c; members[c].push_back(v); ++v; }
    }
    edges_alloc(out, edges);
    size_t e = 0;
    for (size_t epoch = 0; e < edges; ++epoch) {
      const size_t end = std::min(edges, e + (drift_every ? drift_every : edges));
      #pragma omp parallel for schedule(static)
      for (size_t i = e; i < end; ++i) {
        Rng r(seed, 9, i);
        const uint32_t a = 1 + uint32_t(r.below(n));
        uint32_t b;
        const std::vector<uint32_t> &m = members[com[a]];
        if (r.uniform() < p_in && m.size() > 1) b = m[r.below(m.size())];
        else b = 1 + uint32_t(r.below(n));
        out->src[i] = a;
        out->dst[i] = b;
        out->w[i] = 1.0f;
      }
      e = end;
      if (drift > 0 && e < edges) {  // a fraction of the vertices changes community
        Rng r(seed, 10, epoch);
        const size_t moves = size_t(std::llround(drift * n));
        for (size_t k = 0; k < moves; ++k) {
          const uint32_t x = 1 + uint32_t(r.below(n));
          const uint32_t c = uint32_t(r.below(communities));
          if (c == com[x]) continue;
          auto &old = members[com[x]];
          old.erase(std::find(old.begin(), old.end(), x));
          members[c].push_back(x);
          com[x] = c;
        }
      }
    }
  } catch (const std::bad_alloc &) {
    lvgg_edges_free(out);
    return fail(-ENOMEM, "lvgg_temporal_drift: out of memory");
  }
  return 0;
}

int lvgg_apply_batch(const lvgg_csr *x, const lvgg_batch *b, lvgg_csr *y) {
  if (!x || !b || !y) return fail(-EINVAL, "lvgg_apply_batch: bad argument");
  std::memset(y, 0, sizeof(*y));
  const size_t S = x->span;
  for (size_t i = 0; i < b->num_deletions; ++i)
    if (b->del_src[i] >= S || b->del_dst[i] >= S) return fail(-EINVAL, "lvgg_apply_batch: deletion id >= span");
  for (size_t i = 0; i < b->num_insertions; ++i)
    if (b->ins_src[i] >= S || b->ins_dst[i] >= S) return fail(-EINVAL, "lvgg_apply_batch: insertion id >= span");
  try {
    // Per-row ranges of the (src, dst)-sorted batch.
    auto ranges = [&](const uint32_t *src, size_t n, std::vector<uint64_t> &beg) {
      beg.assign(S + 1, 0);
      for (size_t i = 0; i < n; ++i) ++beg[src[i] + 1];
      for (size_t u = 0; u < S; ++u) beg[u + 1] += beg[u];
    };
    std::vector<uint64_t> db, ib;
    ranges(b->del_src, b->num_deletions, db);
    ranges(b->ins_src, b->num_insertions, ib);
    // Merge row u: (old \ deletions) U insertions, sorted; an insertion of an
    // existing key overwrites its weight (the reference's LazyBitset keeps the last).
    auto merge_row = [&](size_t u, uint32_t *ok, float *ow) -> size_t {
      const uint32_t *k = x->keys + x->offsets[u];
      const float *w = x->weights + x->offsets[u];
      size_t n = x->offsets[u + 1] - x->offsets[u];
      size_t i = 0, d = db[u], de = db[u + 1], s = ib[u], se = ib[u + 1], m = 0;
      while (i < n || s < se) {
        if (s < se && (i >= n || b->ins_dst[s] <= k[i])) {
          if (i < n && b->ins_dst[s] == k[i]) ++i;
          if (ok) { ok[m] = b->ins_dst[s]; ow[m] = b->ins_w[s]; }
          ++m; ++s;
          continue;
        }
        while (d < de && b->del_dst[d] < k[i]) ++d;
        if (d < de && b->del_dst[d] == k[i]) { ++i; continue; }
        if (ok) { ok[m] = k[i]; ow[m] = w[i]; }
        ++m; ++i;
      }
      return m;
    };
    std::vector<uint64_t> deg(S);
    #pragma omp parallel for schedule(dynamic, 1024)
    for (size_t u = 0; u < S; ++u) deg[u] = merge_row(u, nullptr, nullptr);
    y->span = S;
    y->offsets = xalloc<uint64_t>(S + 1);
    y->offsets[0] = 0;
    for (size_t u = 0; u < S; ++u) y->offsets[u + 1] = y->offsets[u] + deg[u];
    y->num_edges = y->offsets[S];
    y->keys = xalloc<uint32_t>(y->num_edges);
    y->weights = xalloc<float>(y->num_edges);
    y->exists = xalloc<uint8_t>(S);
    #pragma omp parallel for schedule(dynamic, 1024)
    for (size_t u = 0; u < S; ++u) {
      merge_row(u, y->keys + y->offsets[u], y->weights + y->offsets[u]);
      y->exists[u] = x->exists ? x->exists[u] : 1;
    }
  } catch (const std::bad_alloc &) {
    lvgg_csr_free(y);
    return fail(-ENOMEM, "lvgg_apply_batch: out of memory");
  }
  return 0;
}

}  // extern "C"
