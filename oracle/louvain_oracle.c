/*
 * louvain_oracle.c — CPU restatement of the reference's Louvain hot path.
 *
 * TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and the CPU
 * legs of bench.py may load this library, and only as the checker or as the
 * timed CPU baseline. The product (liblouvain_gb300.so) never calls it.
 *
 * Parity is pinned: tests/test_oracle_golden.py checks every function here
 * against fixtures produced by the reference's own code (oracle/ref_harness.cxx
 * compiled against the unmodified headers), and a 1-thread run of
 * orc_louvain() reproduces the reference's 1-thread membership bit for bit.
 *
 * Restated functions (reference file:line):
 *   orc_edge_weight      edgeWeight / edgeWeightOmp        inc/properties.hxx:81-106
 *   orc_vertex_weights   louvainVertexWeightsOmpW          inc/louvain.hxx:210-218
 *   orc_update_weights   louvainUpdateWeightsFromOmpU      inc/louvain.hxx:374-388
 *   orc_df_mark          louvainAffectedVerticesFrontierOmpW      inc/louvain.hxx:1606-1624
 *   orc_ds_mark          louvainAffectedVerticesDeltaScreeningOmpW inc/louvain.hxx:1441-1486
 *   orc_renumber         louvainCommunityExistsOmpW + louvainRenumberCommunitiesOmpW
 *                        inc/louvain.hxx:668-682, 941-945
 *   orc_aggregate        louvainCommunityVerticesOmpW + louvainAggregateOmpW
 *                        inc/louvain.hxx:800-812, 897-912, 987-992
 *   orc_modularity       modularityBy                      inc/properties.hxx:178-191
 *   orc_louvain          louvainInvokeOmp with the four entries' fi/fm/fa
 *                        inc/louvain.hxx:1120-1221, 1285, 1349, 1542, 1674
 *                        (async moves louvainMoveOmpW :588-609, ΔQ
 *                        deltaModularity inc/properties.hxx:253-256)
 *   orc_apply_batch      tidyBatchUpdateU + applyBatchUpdateOmpU
 *                        inc/batch.hxx:154-209, 241-248 (DiGraph::removeEdge /
 *                        addEdge inc/Graph.hxx:318-357), as main.cxx:108-109
 *   orc_louvain_sync     the project's deterministic colour-class rule
 *                        (no reference counterpart; replays the GPU's
 *                        deterministic mode with the same types — FP64
 *                        vertex weights and community totals, FP32 edge
 *                        weights and link sums — and the same operation
 *                        order, so the two must agree bit for bit).
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ types */

typedef struct orc_options {
  int repeat;
  double resolution, tolerance, aggregationTolerance, toleranceDrop;
  int maxIterations, maxPasses;
} orc_options;

typedef struct orc_info {
  int iterations, passes;
  float time, markingTime, initializationTime, firstPassTime, localMoveTime, aggregationTime;
  uint64_t affectedVertices;
} orc_info;

/* A CSR graph: row u is key[off[u] .. off[u]+degree(u)); degree(u) is deg[u]
 * when deg is given (the reference's gapped DiGraphCsr), else off[u+1]-off[u].
 * Weights are float (input graphs) or double (aggregated graphs, as the
 * reference's DiGraphCsr<K,None,double>). */
typedef struct G {
  size_t span, order, size;
  const uint64_t *off;
  const uint32_t *deg;
  const uint32_t *key;
  const float *wf;
  const double *wd;
  const uint8_t *ex;
} G;

static inline int g_has(const G *g, size_t u) { return !g->ex || g->ex[u]; }
static inline uint64_t g_beg(const G *g, size_t u) { return g->off[u]; }
static inline uint64_t g_end(const G *g, size_t u) { return g->deg ? g->off[u] + g->deg[u] : g->off[u + 1]; }
static inline double g_w(const G *g, uint64_t i) { return g->wf ? (double)g->wf[i] : g->wd[i]; }

static G make_graph(size_t span, const uint64_t *off, const uint32_t *key, const float *w, const uint8_t *ex) {
  G g;
  memset(&g, 0, sizeof(g));
  g.span = span; g.off = off; g.key = key; g.wf = w; g.ex = ex;
  for (size_t u = 0; u < span; ++u)
    if (g_has(&g, u)) { ++g.order; g.size += off[u + 1] - off[u]; }
  return g;
}

/* ΔQ of moving a vertex from community D to C (inc/properties.hxx:253-256). */
static inline double delta_modularity(double vcout, double vdout, double vtot, double ctot, double dtot, double M,
                                      double R) {
  return (vcout - vdout) / M - R * vtot * (vtot + ctot - dtot) / (2 * M * M);
}

/* Per-thread scan table: dense values + first-touch key list (inc/louvain.hxx:152-182, 406-438). */
typedef struct Table {
  uint32_t *keys;
  size_t n;
  double *val;
} Table;

static Table *tables_new(int T, size_t S) {
  Table *t = (Table *)calloc((size_t)T, sizeof(Table));
  for (int i = 0; i < T; ++i) {
    t[i].keys = (uint32_t *)malloc((S + 1) * sizeof(uint32_t));
    t[i].val = (double *)calloc(S + 1, sizeof(double));
    t[i].n = 0;
  }
  return t;
}

static void tables_free(Table *t, int T) {
  for (int i = 0; i < T; ++i) { free(t[i].keys); free(t[i].val); }
  free(t);
}

static inline void table_clear(Table *t) {
  for (size_t i = 0; i < t->n; ++i) t->val[t->keys[i]] = 0;
  t->n = 0;
}

/* louvainScanCommunityW: the key is appended when its value is still zero. */
static inline void table_add(Table *t, uint32_t c, double w) {
  if (!t->val[c]) t->keys[t->n++] = c;
  t->val[c] += w;
}

static inline void scan_communities(Table *t, const G *g, size_t u, const uint32_t *vcom, int self) {
  for (uint64_t i = g_beg(g, u), e = g_end(g, u); i < e; ++i) {
    uint32_t v = g->key[i];
    if (!self && v == u) continue;
    table_add(t, vcom[v], g_w(g, i));
  }
}

/* louvainChooseCommunity (inc/louvain.hxx:455-464): strict '>' in scan order
 * starting from (0, 0), so community 0 doubles as "no move". */
static inline uint32_t choose_community(const Table *t, size_t u, const uint32_t *vcom, const double *vtot,
                                        const double *ctot, double M, double R, double *emax_out) {
  uint32_t cmax = 0, d = vcom[u];
  double emax = 0;
  for (size_t i = 0; i < t->n; ++i) {
    uint32_t c = t->keys[i];
    if (c == d) continue;
    double e = delta_modularity(t->val[c], t->val[d], vtot[u], ctot[c], ctot[d], M, R);
    if (e > emax) { emax = e; cmax = c; }
  }
  *emax_out = emax;
  return cmax;
}

/* ------------------------------------------------------ exported helpers */

double orc_edge_weight(size_t span, const uint64_t *off, const uint32_t *key, const float *w, const uint8_t *ex) {
  G g = make_graph(span, off, key, w, ex);
  double a = 0;
  for (size_t u = 0; u < span; ++u) {
    if (!g_has(&g, u)) continue;
    double b = 0;
    for (uint64_t i = g_beg(&g, u); i < g_end(&g, u); ++i) b += g_w(&g, i);
    a += b;
  }
  return a;
}

static void vertex_weights(const G *g, double *vtot) {
  #pragma omp parallel for schedule(dynamic, 2048)
  for (size_t u = 0; u < g->span; ++u) {
    if (!g_has(g, u)) continue;
    for (uint64_t i = g_beg(g, u); i < g_end(g, u); ++i) vtot[u] += g_w(g, i);
  }
}

/* vtot must be zero-initialised by the caller, as in the reference. */
void orc_vertex_weights(size_t span, const uint64_t *off, const uint32_t *key, const float *w, const uint8_t *ex,
                        double *vtot) {
  G g = make_graph(span, off, key, w, ex);
  vertex_weights(&g, vtot);
}

/* Sequential in batch order: deletions subtract, then insertions add. */
void orc_update_weights(size_t nd, const uint32_t *ds, const uint32_t *dd, const float *dw, size_t ni,
                        const uint32_t *is, const uint32_t *id, const float *iw, const uint32_t *vcom, double *vtot,
                        double *ctot) {
  (void)dd; (void)id;
  for (size_t i = 0; i < nd; ++i) { uint32_t u = ds[i]; vtot[u] -= dw[i]; ctot[vcom[u]] -= dw[i]; }
  for (size_t i = 0; i < ni; ++i) { uint32_t u = is[i]; vtot[u] += iw[i]; ctot[vcom[u]] += iw[i]; }
}

void orc_df_mark(size_t span, size_t nd, const uint32_t *ds, const uint32_t *dd, size_t ni, const uint32_t *is,
                 const uint32_t *id, const uint32_t *vcom, uint8_t *flags) {
  memset(flags, 0, span);
  for (size_t i = 0; i < nd; ++i) if (vcom[ds[i]] == vcom[dd[i]]) flags[ds[i]] = 1;
  for (size_t i = 0; i < ni; ++i) if (vcom[is[i]] != vcom[id[i]]) flags[is[i]] = 1;
}

static void ds_mark(const G *g, size_t nd, const uint32_t *ds, const uint32_t *dd, size_t ni, const uint32_t *is,
                    const uint32_t *id, const float *iw, const uint32_t *vcom, const double *vtot,
                    const double *ctot, double M, double R, uint8_t *vertices, uint8_t *neighbors,
                    uint8_t *communities, Table *t) {
  size_t S = g->span;
  memset(vertices, 0, S); memset(neighbors, 0, S); memset(communities, 0, S);
  for (size_t i = 0; i < nd; ++i) {
    uint32_t u = ds[i], v = dd[i];
    if (vcom[u] != vcom[v]) continue;
    vertices[u] = 1; neighbors[u] = 1; communities[vcom[v]] = 1;
  }
  /* Insertions grouped by source (the batch is sorted by source). */
  for (size_t i = 0; i < ni;) {
    uint32_t u = is[i];
    table_clear(t);
    for (; i < ni && is[i] == u; ++i) {
      uint32_t v = id[i];
      if (vcom[u] == vcom[v]) continue;
      table_add(t, vcom[v], iw[i]);
    }
    double e;
    uint32_t c = choose_community(t, u, vcom, vtot, ctot, M, R, &e);
    if (e <= 0) continue;
    vertices[u] = 1; neighbors[u] = 1; communities[c] = 1;
  }
  table_clear(t);
  for (size_t u = 0; u < S; ++u) {
    if (!g_has(g, u)) continue;
    if (neighbors[u])
      for (uint64_t i = g_beg(g, u); i < g_end(g, u); ++i) vertices[g->key[i]] = 1;
    if (communities[vcom[u]]) vertices[u] = 1;
  }
}

void orc_ds_mark(size_t span, const uint64_t *off, const uint32_t *key, const float *w, const uint8_t *ex,
                 size_t nd, const uint32_t *ds, const uint32_t *dd, size_t ni, const uint32_t *is,
                 const uint32_t *id, const float *iw, const uint32_t *vcom, const double *vtot, const double *ctot,
                 double M, double R, uint8_t *vertices, uint8_t *neighbors, uint8_t *communities) {
  G g = make_graph(span, off, key, w, ex);
  Table *t = tables_new(1, span);
  ds_mark(&g, nd, ds, dd, ni, is, id, iw, vcom, vtot, ctot, M, R, vertices, neighbors, communities, t);
  tables_free(t, 1);
}

/* Existence flags + order-preserving renumber over the first `len` entries of
 * vcom (the whole array, as louvainLookupCommunitiesOmpU does). Returns CN. */
static size_t renumber(const G *g, uint32_t *vcom, size_t len, uint32_t *cext) {
  size_t S = g->span, C = 0;
  memset(cext, 0, S * sizeof(uint32_t));
  for (size_t u = 0; u < S; ++u) {
    if (!g_has(g, u)) continue;
    if (!cext[vcom[u]]) ++C;
    cext[vcom[u]] = 1;
  }
  uint32_t acc = 0;
  for (size_t c = 0; c < S; ++c) { uint32_t t = cext[c]; cext[c] = acc; acc += t; }
  for (size_t u = 0; u < len; ++u) vcom[u] = cext[vcom[u]];
  return C;
}

size_t orc_renumber(size_t span, const uint8_t *ex, uint32_t *vcom) {
  G g;
  memset(&g, 0, sizeof(g));
  g.span = span; g.ex = ex;
  uint32_t *cext = (uint32_t *)malloc(span * sizeof(uint32_t));
  size_t C = renumber(&g, vcom, span, cext);
  free(cext);
  return C;
}

/* Aggregated graph, gapped like the reference (yoff = exclusive scan of the
 * communities' total degree; ydeg = emitted entries). */
typedef struct Agg {
  size_t C, cap;
  uint64_t *off;
  uint32_t *deg, *key;
  double *w;
} Agg;

static void aggregate(const G *g, const uint32_t *vcom, size_t C, Agg *y, Table *tabs) {
  size_t S = g->span;
  /* Community -> member CSR: count, exclusive scan, atomic-cursor scatter. */
  uint32_t *coff = (uint32_t *)calloc(C + 1, sizeof(uint32_t));
  uint32_t *cdeg = (uint32_t *)calloc(C + 1, sizeof(uint32_t));
  uint32_t *cedg = (uint32_t *)malloc((S + 1) * sizeof(uint32_t));
  #pragma omp parallel for schedule(static, 2048)
  for (size_t u = 0; u < S; ++u) {
    if (!g_has(g, u)) continue;
    #pragma omp atomic
    ++coff[vcom[u]];
  }
  uint32_t acc = 0;
  for (size_t c = 0; c < C; ++c) { uint32_t t = coff[c]; coff[c] = acc; acc += t; }
  coff[C] = acc;
  #pragma omp parallel for schedule(static, 2048)
  for (size_t u = 0; u < S; ++u) {
    if (!g_has(g, u)) continue;
    uint32_t c = vcom[u], n;
    #pragma omp atomic capture
    { n = cdeg[c]; ++cdeg[c]; }
    cedg[coff[c] + n] = (uint32_t)u;
  }
  /* Row capacity = total degree of the community. */
  memset(y->off, 0, (C + 1) * sizeof(uint64_t));
  #pragma omp parallel for schedule(static, 2048)
  for (size_t u = 0; u < S; ++u) {
    if (!g_has(g, u)) continue;
    uint64_t d = g_end(g, u) - g_beg(g, u);
    #pragma omp atomic
    y->off[vcom[u]] += d;
  }
  uint64_t a2 = 0;
  for (size_t c = 0; c < C; ++c) { uint64_t t = y->off[c]; y->off[c] = a2; a2 += t; }
  y->off[C] = a2;
  y->C = C;
  #pragma omp parallel for schedule(dynamic, 2048)
  for (size_t c = 0; c < C; ++c) {
    Table *t = &tabs[omp_get_thread_num()];
    uint32_t n = coff[c + 1] - coff[c];
    y->deg[c] = 0;
    if (n == 0) continue;
    table_clear(t);
    for (uint32_t j = coff[c]; j < coff[c + 1]; ++j) scan_communities(t, g, cedg[j], vcom, 1);
    for (size_t i = 0; i < t->n; ++i) {
      uint32_t d = t->keys[i];
      uint64_t p = y->off[c] + y->deg[c]++;
      y->key[p] = d;
      y->w[p] = t->val[d];
    }
  }
  free(coff); free(cdeg); free(cedg);
}

/* Aggregate for a given (unrenumbered) membership; writes the renumbered
 * membership back. yoff[CN+1], ydeg[CN], ykey/yw with capacity = edges. */
size_t orc_aggregate(size_t span, const uint64_t *off, const uint32_t *key, const float *w, const uint8_t *ex,
                     uint32_t *vcom, uint64_t *yoff, uint32_t *ydeg, uint32_t *ykey, double *yw) {
  G g = make_graph(span, off, key, w, ex);
  uint32_t *cext = (uint32_t *)malloc(span * sizeof(uint32_t));
  size_t C = renumber(&g, vcom, span, cext);
  free(cext);
  int T = omp_get_max_threads();
  Table *t = tables_new(T, span);
  Agg y = {C, g.size, yoff, ydeg, ykey, yw};
  aggregate(&g, vcom, C, &y, t);
  tables_free(t, T);
  return C;
}

double orc_modularity(size_t span, const uint64_t *off, const uint32_t *key, const float *w, const uint8_t *ex,
                      const uint32_t *membership, double M, double R) {
  G g = make_graph(span, off, key, w, ex);
  double *cin = (double *)calloc(span, sizeof(double)), *ctot = (double *)calloc(span, sizeof(double));
  for (size_t u = 0; u < span; ++u) {
    if (!g_has(&g, u)) continue;
    uint32_t c = membership[u];
    for (uint64_t i = g_beg(&g, u); i < g_end(&g, u); ++i) {
      uint32_t d = membership[g.key[i]];
      double x = g_w(&g, i);
      if (c == d) cin[c] += x;
      ctot[c] += x;
    }
  }
  double a = 0;
  for (size_t c = 0; c < span; ++c) a += cin[c] / (2 * M) - R * pow(ctot[c] / (2 * M), 2);
  free(cin); free(ctot);
  return a;
}

/* ------------------------------------------------ async local-moving phase */

/* louvainMoveOmpW (inc/louvain.hxx:588-609). fa == NULL means every vertex
 * may move. Returns the iteration count, 0 if already converged. */
static int move_async(const G *g, uint32_t *vcom, double *ctot, uint8_t *vaff, const double *vtot, double M,
                      double R, int L, double E, const uint8_t *fa, Table *tabs) {
  size_t S = g->span;
  int l = 0;
  double el = 0;
  while (l < L) {
    el = 0;
    #pragma omp parallel for schedule(dynamic, 2048) reduction(+ : el)
    for (size_t u = 0; u < S; ++u) {
      Table *t = &tabs[omp_get_thread_num()];
      if (!g_has(g, u)) continue;
      if ((fa && !fa[u]) || !vaff[u]) continue;
      table_clear(t);
      scan_communities(t, g, u, vcom, 0);
      double e;
      uint32_t c = choose_community(t, u, vcom, vtot, ctot, M, R, &e);
      if (c) {
        uint32_t d = vcom[u];
        #pragma omp atomic
        ctot[d] -= vtot[u];
        #pragma omp atomic
        ctot[c] += vtot[u];
        vcom[u] = c;
        for (uint64_t i = g_beg(g, u); i < g_end(g, u); ++i) vaff[g->key[i]] = 1;
      }
      vaff[u] = 0;
      el += e;
    }
    ++l;
    if (el <= E) break;
  }
  return (l > 1 || el) ? l : 0;
}

/* ------------------------------------------------------------ pass driver */

enum { ORC_STATIC = 0, ORC_NAIVE = 1, ORC_DELTA = 2, ORC_FRONTIER = 3 };

typedef struct Batch {
  size_t nd, ni;
  const uint32_t *ds, *dd, *is, *id;
  const float *dw, *iw;
} Batch;

static double now_ms(void) { return omp_get_wtime() * 1000.0; }

/* louvainInvokeOmp (inc/louvain.hxx:1120-1221) with the entries' fi/fm/fa. */
int orc_louvain(size_t span, const uint64_t *off, const uint32_t *key, const float *w, const uint8_t *ex,
                int method, size_t nd, const uint32_t *ds, const uint32_t *dd, const float *dw, size_t ni,
                const uint32_t *is, const uint32_t *id, const float *iw, const uint32_t *q, const double *qvtot,
                const double *qctot, const orc_options *o, int threads, uint32_t *membership, double *vtot_out,
                double *ctot_out, orc_info *info) {
  if (method < 0 || method > 3) return -1;
  int saved = omp_get_max_threads();
  if (threads > 0) omp_set_num_threads(threads);
  G x = make_graph(span, off, key, w, ex);
  Batch b = {nd, ni, ds, dd, is, id, dw, iw};
  size_t S = span, X = x.size;
  double R = o->resolution;
  int L = o->maxIterations, P = o->maxPasses, l = 0, p = 0;
  double M = 0;
  {
    double a = 0;
    #pragma omp parallel for schedule(auto) reduction(+ : a)
    for (size_t u = 0; u < S; ++u) {
      if (!g_has(&x, u)) continue;
      double s = 0;
      for (uint64_t i = g_beg(&x, u); i < g_end(&x, u); ++i) s += g_w(&x, i);
      a += s;
    }
    M = a / 2;
  }
  int T = omp_get_max_threads();
  uint8_t *vaff = (uint8_t *)calloc(S, 1);
  uint32_t *ucom = (uint32_t *)calloc(S, sizeof(uint32_t)), *vcom = (uint32_t *)calloc(S, sizeof(uint32_t));
  double *utot = (double *)calloc(S, sizeof(double)), *vtot = (double *)calloc(S, sizeof(double));
  double *ctot = (double *)calloc(S, sizeof(double));
  uint32_t *cext = (uint32_t *)calloc(S, sizeof(uint32_t));
  uint8_t *fv = NULL, *fn = NULL, *fcm = NULL;
  if (method == ORC_DELTA) { fv = (uint8_t *)calloc(S, 1); fn = (uint8_t *)calloc(S, 1); fcm = (uint8_t *)calloc(S, 1); }
  Table *tabs = tables_new(T, S);
  /* Two gapped CSR buffers with capacity X (aggregationTolerance <= 1). */
  size_t cap = X > 0 ? X : 1;
  Agg ya = {0, cap, (uint64_t *)calloc(S + 1, 8), (uint32_t *)calloc(S + 1, 4), (uint32_t *)malloc(cap * 4), (double *)malloc(cap * 8)};
  Agg za = {0, cap, (uint64_t *)calloc(S + 1, 8), (uint32_t *)calloc(S + 1, 4), (uint32_t *)malloc(cap * 4), (double *)malloc(cap * 8)};
  float tm = 0, ti = 0, tp = 0, tl = 0, ta = 0, tt = 0;
  for (int r = 0; r < o->repeat; ++r) {
    double E = o->tolerance;
    memset(vaff, 0, S); memset(ucom, 0, S * 4); memset(vcom, 0, S * 4);
    memset(utot, 0, S * 8); memset(vtot, 0, S * 8); memset(ctot, 0, S * 8);
    double t0m = now_ms();
    /* fi: initialise membership and weights. */
    double a = now_ms();
    if (method == ORC_STATIC) {
      vertex_weights(&x, utot);
      for (size_t u = 0; u < S; ++u) if (g_has(&x, u)) { ucom[u] = (uint32_t)u; ctot[u] = utot[u]; }
    } else {
      memcpy(ucom, q, S * 4); memcpy(utot, qvtot, S * 8); memcpy(ctot, qctot, S * 8);
      orc_update_weights(b.nd, b.ds, b.dd, b.dw, b.ni, b.is, b.id, b.iw, ucom, utot, ctot);
    }
    ti += (float)(now_ms() - a);
    /* fm: mark affected vertices. */
    a = now_ms();
    if (method == ORC_STATIC || method == ORC_NAIVE) memset(vaff, 1, S);
    else if (method == ORC_FRONTIER) orc_df_mark(S, b.nd, b.ds, b.dd, b.ni, b.is, b.id, ucom, vaff);
    else {
      ds_mark(&x, b.nd, b.ds, b.dd, b.ni, b.is, b.id, b.iw, ucom, utot, ctot, M, R, fv, fn, fcm, &tabs[0]);
      memcpy(vaff, fv, S);
    }
    tm += (float)(now_ms() - a);
    double t0 = now_ms(), t1 = t0;
    G y;
    memset(&y, 0, sizeof(y));
    for (l = 0, p = 0; M > 0 && P > 0;) {
      if (p == 1) t1 = now_ms();
      int first = p == 0, m;
      a = now_ms();
      if (first) m = move_async(&x, ucom, ctot, vaff, utot, M, R, L, E, method == ORC_DELTA ? fv : NULL, tabs);
      else m = move_async(&y, vcom, ctot, vaff, vtot, M, R, L, E, NULL, tabs);
      tl += (float)(now_ms() - a);
      l += m > 1 ? m : 1;
      ++p;
      if (m <= 1 || p >= P) break;
      const G *gx = first ? &x : &y;
      size_t GN = gx->order;
      uint32_t *cur = first ? ucom : vcom;
      /* Count communities first; break before renumbering (inc/louvain.hxx:1190-1192). */
      size_t CN = 0;
      {
        memset(cext, 0, gx->span * 4);
        for (size_t u = 0; u < gx->span; ++u) {
          if (!g_has(gx, u)) continue;
          if (!cext[cur[u]]) ++CN;
          cext[cur[u]] = 1;
        }
      }
      if ((double)CN / (double)GN >= o->aggregationTolerance) break;
      renumber(gx, cur, S, cext);
      if (!first) for (size_t u = 0; u < S; ++u) ucom[u] = vcom[ucom[u]];
      a = now_ms();
      aggregate(gx, cur, CN, &za, tabs);
      ta += (float)(now_ms() - a);
      Agg tmp = ya; ya = za; za = tmp;
      memset(&y, 0, sizeof(y));
      y.span = CN; y.order = CN; y.off = ya.off; y.deg = ya.deg; y.key = ya.key; y.wd = ya.w;
      for (size_t c = 0; c < CN; ++c) y.size += ya.deg[c];
      memset(vtot, 0, CN * 8);
      memset(vaff, 1, CN);
      vertex_weights(&y, vtot);
      for (size_t u = 0; u < CN; ++u) { vcom[u] = (uint32_t)u; ctot[u] = vtot[u]; }
      E /= o->toleranceDrop;
    }
    if (p > 1) for (size_t u = 0; u < S; ++u) ucom[u] = vcom[ucom[u]];
    if (p <= 1) t1 = now_ms();
    tp += (float)(t1 - t0);
    tt += (float)(now_ms() - t0m);
  }
  uint64_t aff = 0;
  for (size_t u = 0; u < S; ++u) aff += vaff[u] == 1;
  memcpy(membership, ucom, S * 4);
  memcpy(vtot_out, utot, S * 8);
  memcpy(ctot_out, ctot, S * 8);
  int rep = o->repeat > 0 ? o->repeat : 1;
  info->iterations = l; info->passes = p;
  info->time = tt / rep; info->markingTime = tm / rep; info->initializationTime = ti / rep;
  info->firstPassTime = tp / rep; info->localMoveTime = tl / rep; info->aggregationTime = ta / rep;
  info->affectedVertices = aff;
  tables_free(tabs, T);
  free(vaff); free(ucom); free(vcom); free(utot); free(vtot); free(ctot); free(cext);
  free(fv); free(fn); free(fcm);
  free(ya.off); free(ya.deg); free(ya.key); free(ya.w);
  free(za.off); free(za.deg); free(za.key); free(za.w);
  omp_set_num_threads(saved);
  return 0;
}

/* ======================================================================
 * Deterministic colour-class replay (the project's own rule).
 *
 * Vertices are split into K classes by a hash of their id (color_of). An
 * iteration visits the classes in order. Within a class every active vertex
 * decides from the same state (membership, community totals and flags as
 * left by the previous classes), then all decisions of the class are applied
 * and the neighbour marks of its movers are merged into the flags.
 * Per vertex u the gain of joining community c is, in exactly this
 * operation order,
 *     g(c) = (k_c - k_d) - (float)w_u * (float)((w_u + t_c) - t_d) * kr,   kr = (float)(R/(2M)),
 * with the vertex weight w_u and the community totals t_c, t_d in FP64 (as the
 * reference's W) and everything else in FP32;
 * which is M times the reference's ΔQ. The best c != d is the largest g > 0,
 * ties going to the lowest community id. A best c of 0 does not move (the
 * reference's "if (c)"). The convergence sum adds, per vertex, the best gain
 * as a 2^-16 fixed-point integer: el = (Σ llrint(g*65536)) / 65536 / M.
 * A processed vertex clears its flag; a mover marks its neighbours v != u.
 * Edge weights and the per-vertex link sums k_c are FP32, vertex weights and
 * community totals FP64. A super-vertex's weight is its community's total.
 * Sums of integer weights are exact in any order (below 2^24 in FP32, 2^53
 * in FP64), which is the domain in which the GPU's deterministic mode and
 * this replay agree bit for bit.
 * ==================================================================== */

static inline uint32_t color_of(uint32_t u, uint32_t k) {
  uint32_t h = u * 0x9E3779B1u;
  h ^= h >> 16;
  return h % k;
}

typedef struct GF {
  size_t span, order;
  const uint64_t *off;
  const uint32_t *key;
  const float *w;
  const uint8_t *ex;
} GF;

static inline int gf_has(const GF *g, size_t u) { return !g->ex || g->ex[u]; }

typedef struct TableF {
  uint32_t *keys;
  size_t n;
  float *val;
  uint8_t *seen;
} TableF;

static inline float gain_of(float kc, float kd, double wu, double tc, double td, float kr) {
  float a = kc - kd;
  float c = (float)((wu + tc) - td);
  float d = (float)wu * c;
  float e = d * kr;
  return a - e;
}

static int move_sync(const GF *g, uint32_t *vcom, double *ctot, uint8_t *vaff, uint8_t *mark, uint32_t *dec,
                     const double *vtot, double M, float kr, int L, double E, const uint8_t *fa, TableF *tabs,
                     int K) {
  size_t S = g->span;
  int l = 0;
  double el = 0;
  while (l < L) {
    int64_t elfix = 0;
    for (int col = 0; col < K; ++col) {
      #pragma omp parallel for schedule(dynamic, 2048) reduction(+ : elfix)
      for (size_t u = 0; u < S; ++u) {
        TableF *t = &tabs[omp_get_thread_num()];
        dec[u] = 0xFFFFFFFFu;
        if (color_of((uint32_t)u, (uint32_t)K) != (uint32_t)col) continue;
        if (!gf_has(g, u) || (fa && !fa[u]) || !vaff[u]) continue;
        t->n = 0;
        for (uint64_t i = g->off[u]; i < g->off[u + 1]; ++i) {
          uint32_t v = g->key[i];
          if (v == u) continue;
          uint32_t c = vcom[v];
          if (!t->seen[c]) { t->seen[c] = 1; t->val[c] = 0; t->keys[t->n++] = c; }
          t->val[c] += g->w[i];
        }
        uint32_t d = vcom[u];
        float kd = t->seen[d] ? t->val[d] : 0.0f;
        uint32_t best = 0;
        float bg = 0;
        int found = 0;
        for (size_t i = 0; i < t->n; ++i) {
          uint32_t c = t->keys[i];
          if (c == d) continue;
          float gc = gain_of(t->val[c], kd, vtot[u], ctot[c], ctot[d], kr);
          if (gc > 0 && (!found || gc > bg || (gc == bg && c < best))) { found = 1; bg = gc; best = c; }
        }
        for (size_t i = 0; i < t->n; ++i) t->seen[t->keys[i]] = 0;
        if (found) elfix += (int64_t)llrint((double)bg * 65536.0);
        if (found && best != 0) {
          dec[u] = best;
          for (uint64_t i = g->off[u]; i < g->off[u + 1]; ++i)
            if (g->key[i] != u) mark[g->key[i]] = 1;
        }
        vaff[u] = 0;
      }
      /* apply the class's decisions, then merge its marks */
      for (size_t u = 0; u < S; ++u) {
        uint32_t c = dec[u];
        if (c == 0xFFFFFFFFu) continue;
        uint32_t d = vcom[u];
        ctot[d] -= vtot[u];
        ctot[c] += vtot[u];
        vcom[u] = c;
      }
      for (size_t u = 0; u < S; ++u)
        if (mark[u]) { vaff[u] = 1; mark[u] = 0; }
    }
    el = (double)elfix / 65536.0 / M;
    ++l;
    if (el <= E) break;
  }
  return (l > 1 || el) ? l : 0;
}

/* Deterministic aggregation: rows sorted by neighbour community, FP32 sums in
 * member order (exact for integer weights). Output CSR (compact). */
static size_t aggregate_f(const GF *g, const uint32_t *vcom, size_t C, uint64_t *yoff, uint32_t *ykey, float *yw,
                          TableF *tabs) {
  size_t S = g->span;
  uint32_t *coff = (uint32_t *)calloc(C + 1, 4), *cedg = (uint32_t *)malloc((S + 1) * 4), *cur;
  for (size_t u = 0; u < S; ++u) if (gf_has(g, u)) ++coff[vcom[u] + 1];
  for (size_t c = 0; c < C; ++c) coff[c + 1] += coff[c];
  cur = (uint32_t *)malloc((C + 1) * 4);
  memcpy(cur, coff, (C + 1) * 4);
  for (size_t u = 0; u < S; ++u) if (gf_has(g, u)) cedg[cur[vcom[u]]++] = (uint32_t)u;
  uint64_t *deg = (uint64_t *)calloc(C + 1, 8);
  /* pass 1: distinct neighbour communities; pass 2: write sorted rows */
  for (int pass = 0; pass < 2; ++pass) {
    #pragma omp parallel for schedule(dynamic, 256)
    for (size_t c = 0; c < C; ++c) {
      TableF *t = &tabs[omp_get_thread_num()];
      t->n = 0;
      for (uint32_t j = coff[c]; j < coff[c + 1]; ++j) {
        uint32_t u = cedg[j];
        for (uint64_t i = g->off[u]; i < g->off[u + 1]; ++i) {
          uint32_t d = vcom[g->key[i]];
          if (!t->seen[d]) { t->seen[d] = 1; t->val[d] = 0; t->keys[t->n++] = d; }
          t->val[d] += g->w[i];
        }
      }
      if (pass == 0) deg[c] = t->n;
      else {
        /* insertion sort is fine for small rows; use qsort-like simple sort */
        uint32_t *k = t->keys;
        size_t n = t->n;
        for (size_t i = 1; i < n; ++i) {
          uint32_t x = k[i];
          size_t j = i;
          while (j > 0 && k[j - 1] > x) { k[j] = k[j - 1]; --j; }
          k[j] = x;
        }
        for (size_t i = 0; i < n; ++i) { ykey[yoff[c] + i] = k[i]; yw[yoff[c] + i] = t->val[k[i]]; }
      }
      for (size_t i = 0; i < t->n; ++i) t->seen[t->keys[i]] = 0;
    }
    if (pass == 0) {
      yoff[0] = 0;
      for (size_t c = 0; c < C; ++c) yoff[c + 1] = yoff[c] + deg[c];
    }
  }
  size_t E = yoff[C];
  free(coff); free(cedg); free(cur); free(deg);
  return E;
}

int orc_louvain_sync(size_t span, const uint64_t *off, const uint32_t *key, const float *w, const uint8_t *ex,
                     int method, size_t nd, const uint32_t *ds, const uint32_t *dd, const float *dw, size_t ni,
                     const uint32_t *is, const uint32_t *id, const float *iw, const uint32_t *q,
                     const double *qvtot, const double *qctot, const orc_options *o, int threads, int colors,
                     uint32_t *membership, double *vtot_out, double *ctot_out, orc_info *info) {
  if (colors < 1) colors = 1;
  if (method < 0 || method > 3) return -1;
  int saved = omp_get_max_threads();
  if (threads > 0) omp_set_num_threads(threads);
  size_t S = span;
  GF x = {span, 0, off, key, w, ex};
  size_t X = 0;
  for (size_t u = 0; u < S; ++u) if (gf_has(&x, u)) { ++x.order; X += off[u + 1] - off[u]; }
  /* M in FP64 (as the device reduces it). */
  double M = 0;
  for (size_t u = 0; u < S; ++u) {
    if (!gf_has(&x, u)) continue;
    double s = 0;
    for (uint64_t i = off[u]; i < off[u + 1]; ++i) s += w[i];
    M += s;
  }
  M /= 2;
  double R = o->resolution;
  float kr = (float)(R / (2.0 * M));
  int L = o->maxIterations, P = o->maxPasses, l = 0, p = 0;
  int T = omp_get_max_threads();
  TableF *tabs = (TableF *)calloc((size_t)T, sizeof(TableF));
  for (int i = 0; i < T; ++i) {
    tabs[i].keys = (uint32_t *)malloc((S + 1) * 4);
    tabs[i].val = (float *)calloc(S + 1, 4);
    tabs[i].seen = (uint8_t *)calloc(S + 1, 1);
  }
  uint8_t *vaff = (uint8_t *)calloc(S, 1), *mark = (uint8_t *)calloc(S, 1);
  uint32_t *ucom = (uint32_t *)calloc(S, 4), *vcom = (uint32_t *)calloc(S, 4), *dec = (uint32_t *)calloc(S, 4);
  double *utot = (double *)calloc(S, 8), *vtot = (double *)calloc(S, 8), *ctot = (double *)calloc(S, 8);
  uint32_t *cext = (uint32_t *)calloc(S, 4);
  uint8_t *fv = NULL;
  size_t cap = X > 0 ? X : 1;
  uint64_t *yoff = (uint64_t *)calloc(S + 1, 8), *zoff = (uint64_t *)calloc(S + 1, 8);
  uint32_t *ykey = (uint32_t *)malloc(cap * 4), *zkey = (uint32_t *)malloc(cap * 4);
  float *yw = (float *)malloc(cap * 4), *zw = (float *)malloc(cap * 4);
  if (method == ORC_STATIC) {
    for (size_t u = 0; u < S; ++u) {
      if (!gf_has(&x, u)) continue;
      double s = 0;
      for (uint64_t i = off[u]; i < off[u + 1]; ++i) s += w[i];
      utot[u] = s; ucom[u] = (uint32_t)u; ctot[u] = s;
    }
    memset(vaff, 1, S);
  } else {
    memcpy(ucom, q, S * 4);
    for (size_t u = 0; u < S; ++u) { utot[u] = qvtot[u]; ctot[u] = qctot[u]; }
    for (size_t i = 0; i < nd; ++i) { utot[ds[i]] -= dw[i]; ctot[ucom[ds[i]]] -= dw[i]; }
    for (size_t i = 0; i < ni; ++i) { utot[is[i]] += iw[i]; ctot[ucom[is[i]]] += iw[i]; }
    if (method == ORC_NAIVE) memset(vaff, 1, S);
    else if (method == ORC_FRONTIER) orc_df_mark(S, nd, ds, dd, ni, is, id, ucom, vaff);
    else {
      /* The delta-screening marking reads the FP64 totals, as the reference does. */
      uint8_t *fn = (uint8_t *)calloc(S, 1), *fcm = (uint8_t *)calloc(S, 1);
      fv = (uint8_t *)calloc(S, 1);
      orc_ds_mark(span, off, key, w, ex, nd, ds, dd, ni, is, id, iw, ucom, utot, ctot, M, R, fv, fn, fcm);
      memcpy(vaff, fv, S);
      free(fn); free(fcm);
    }
  }
  double E = o->tolerance;
  GF y = {0, 0, yoff, ykey, yw, NULL};
  for (l = 0, p = 0; M > 0 && P > 0;) {
    int first = p == 0, m;
    if (first) m = move_sync(&x, ucom, ctot, vaff, mark, dec, utot, M, kr, L, E, fv, tabs, colors);
    else m = move_sync(&y, vcom, ctot, vaff, mark, dec, vtot, M, kr, L, E, NULL, tabs, colors);
    l += m > 1 ? m : 1;
    ++p;
    if (m <= 1 || p >= P) break;
    const GF *gx = first ? &x : &y;
    uint32_t *cur = first ? ucom : vcom;
    size_t GN = gx->order, CN = 0;
    memset(cext, 0, gx->span * 4);
    for (size_t u = 0; u < gx->span; ++u) {
      if (!gf_has(gx, u)) continue;
      if (!cext[cur[u]]) ++CN;
      cext[cur[u]] = 1;
    }
    if ((double)CN / (double)GN >= o->aggregationTolerance) break;
    /* renumber; a super-vertex's weight is its community's total */
    uint32_t acc = 0;
    for (size_t c = 0; c < gx->span; ++c) {
      uint32_t t = cext[c];
      cext[c] = acc;
      if (t) vtot[acc] = ctot[c];
      acc += t;
    }
    for (size_t u = 0; u < S; ++u) cur[u] = cext[cur[u]];
    if (!first) for (size_t u = 0; u < S; ++u) ucom[u] = vcom[ucom[u]];
    aggregate_f(gx, cur, CN, zoff, zkey, zw, tabs);
    uint64_t *t1 = yoff; yoff = zoff; zoff = t1;
    uint32_t *t2 = ykey; ykey = zkey; zkey = t2;
    float *t3 = yw; yw = zw; zw = t3;
    y.span = CN; y.order = CN; y.off = yoff; y.key = ykey; y.w = yw; y.ex = NULL;
    memset(vaff, 1, CN);
    for (size_t u = 0; u < CN; ++u) { vcom[u] = (uint32_t)u; ctot[u] = vtot[u]; }
    E /= o->toleranceDrop;
  }
  if (p > 1) for (size_t u = 0; u < S; ++u) ucom[u] = vcom[ucom[u]];
  uint64_t aff = 0;
  for (size_t u = 0; u < S; ++u) aff += vaff[u] == 1;
  memcpy(membership, ucom, S * 4);
  for (size_t u = 0; u < S; ++u) { vtot_out[u] = utot[u]; ctot_out[u] = ctot[u]; }
  memset(info, 0, sizeof(*info));
  info->iterations = l; info->passes = p; info->affectedVertices = aff;
  for (int i = 0; i < T; ++i) { free(tabs[i].keys); free(tabs[i].val); free(tabs[i].seen); }
  free(tabs);
  free(vaff); free(mark); free(ucom); free(vcom); free(dec); free(utot); free(vtot); free(ctot);
  free(cext); free(fv); free(yoff); free(zoff); free(ykey); free(zkey); free(yw); free(zw);
  omp_set_num_threads(saved);
  return 0;
}

/* ------------------------------------------------------------ batch apply */

typedef struct orc_edge { uint32_t u, v; size_t i; } orc_edge;

static int cmp_edge(const void *a, const void *b) {
  const orc_edge *x = (const orc_edge *)a, *y = (const orc_edge *)b;
  if (x->u != y->u) return x->u < y->u ? -1 : 1;
  if (x->v != y->v) return x->v < y->v ? -1 : 1;
  return x->i < y->i ? -1 : x->i > y->i;
}

static int row_has(const uint64_t *off, const uint32_t *key, const uint8_t *ex, uint32_t u, uint32_t v) {
  if (ex && !ex[u]) return 0;
  for (uint64_t j = off[u]; j < off[u + 1]; ++j)
    if (key[j] == v) return 1;
  return 0;
}

/* tidyBatchUpdateU for one list: keep the edges whose presence in x equals
 * `present` (filterEdgesByExistenceU, inc/batch.hxx:154-161), sort by
 * (source, target) and drop duplicates, keeping the first in batch order
 * (sortEdgesByIdU + uniqueEdgesU, :169-192; the reference's unstable sort
 * keeps an unspecified one). Returns the kept count; indices into the input
 * in *out. */
static size_t tidy_list(const uint64_t *off, const uint32_t *key, const uint8_t *ex, size_t n, const uint32_t *s,
                        const uint32_t *d, int present, size_t *out) {
  orc_edge *e = malloc((n ? n : 1) * sizeof(orc_edge));
  size_t m = 0, k = 0;
  for (size_t i = 0; i < n; ++i)
    if (row_has(off, key, ex, s[i], d[i]) == present) { e[m].u = s[i]; e[m].v = d[i]; e[m].i = i; ++m; }
  qsort(e, m, sizeof(orc_edge), cmp_edge);
  for (size_t i = 0; i < m; ++i) {
    if (i && e[i].u == e[i - 1].u && e[i].v == e[i - 1].v) continue;
    out[k++] = e[i].i;
  }
  free(e);
  return k;
}

/* Order (key | weight bits << 32) pairs by key. */
static int cmp_kw(const void *a, const void *b) {
  const uint32_t x = (uint32_t)*(const uint64_t *)a, y = (uint32_t)*(const uint64_t *)b;
  return x < y ? -1 : x > y;
}

/* tidyBatchUpdateU + applyBatchUpdateOmpU, as main.cxx:108-109 runs them:
 * the batch is tidied against x, then its deletions are removed and its
 * insertions added (DiGraph::removeEdge / addEdge, inc/Graph.hxx:318-357),
 * an added edge making both endpoints present; rows stay sorted by
 * neighbour id. Ids must be < span. Outputs: the graph (yoff[span+1],
 * ykey/yw with room for off[span]+ni entries, yex[span]) and the tidied
 * batch (tds/tdd/tdw with room for nd, tis/tid/tiw for ni; counts in
 * *tnd, *tni). Returns the edge count of the result. */
size_t orc_apply_batch(size_t span, const uint64_t *off, const uint32_t *key, const float *w, const uint8_t *ex,
                       size_t nd, const uint32_t *ds, const uint32_t *dd, const float *dw, size_t ni,
                       const uint32_t *is, const uint32_t *id, const float *iw, uint64_t *yoff, uint32_t *ykey,
                       float *yw, uint8_t *yex, uint32_t *tds, uint32_t *tdd, float *tdw, size_t *tnd,
                       uint32_t *tis, uint32_t *tid, float *tiw, size_t *tni) {
  size_t *kd = malloc((nd ? nd : 1) * sizeof(size_t)), *ki = malloc((ni ? ni : 1) * sizeof(size_t));
  const size_t md = tidy_list(off, key, ex, nd, ds, dd, 1, kd);
  const size_t mi = tidy_list(off, key, ex, ni, is, id, 0, ki);
  for (size_t t = 0; t < md; ++t) { tds[t] = ds[kd[t]]; tdd[t] = dd[kd[t]]; tdw[t] = dw[kd[t]]; }
  for (size_t t = 0; t < mi; ++t) { tis[t] = is[ki[t]]; tid[t] = id[ki[t]]; tiw[t] = iw[ki[t]]; }
  *tnd = md;
  *tni = mi;
  for (size_t u = 0; u < span; ++u) yex[u] = ex ? ex[u] : 1;
  for (size_t t = 0; t < mi; ++t) { yex[tis[t]] = 1; yex[tid[t]] = 1; }
  /* the tidied lists are sorted by source: walk them row by row */
  size_t m = 0, a = 0, c = 0;
  yoff[0] = 0;
  for (size_t u = 0; u < span; ++u) {
    const uint64_t o = m;
    const size_t a0 = a;
    while (a < md && tds[a] == u) ++a;
    for (uint64_t j = off[u]; j < off[u + 1]; ++j) {
      int gone = 0;
      for (size_t t = a0; t < a && !gone; ++t) gone = tdd[t] == key[j];
      if (gone) continue;
      ykey[m] = key[j];
      yw[m] = w[j];
      ++m;
    }
    for (; c < mi && tis[c] == u; ++c) { ykey[m] = tid[c]; yw[m] = tiw[c]; ++m; }
    const size_t n = m - o;
    if (n > 1) {
      uint64_t *kw = malloc(n * sizeof(uint64_t));
      for (size_t j = 0; j < n; ++j) {
        uint32_t wb;
        memcpy(&wb, &yw[o + j], 4);
        kw[j] = ((uint64_t)ykey[o + j]) | ((uint64_t)wb << 32);
      }
      qsort(kw, n, sizeof(uint64_t), cmp_kw);
      for (size_t j = 0; j < n; ++j) {
        const uint32_t wb = (uint32_t)(kw[j] >> 32);
        ykey[o + j] = (uint32_t)kw[j];
        memcpy(&yw[o + j], &wb, 4);
      }
      free(kw);
    }
    yoff[u + 1] = m;
  }
  free(kd);
  free(ki);
  return m;
}
