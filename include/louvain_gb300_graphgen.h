/*
 * louvain_gb300_graphgen.h — seeded synthetic graphs and batch updates (host only).
 *
 * These stand in for the reference's inputs. The reference reads SNAP temporal
 * edge lists (inc/snap.hxx:41-212), generates random batches
 * (inc/batch.hxx:100-140), tidies them (inc/batch.hxx:202-209) and applies them
 * to a copy of the graph (inc/batch.hxx:241-248). The datasets are not shipped,
 * so these generators produce seeded graphs with the reference's conventions:
 *   - vertex ids are 1..n and vertex 0 never exists (inc/snap.hxx:133), so the
 *     span is n+1;
 *   - rows are sorted ascending by neighbour id, as the reference's LazyBitset
 *     adjacency is (inc/_bitset.hxx:227-262);
 *   - graphs are undirected: every edge is stored in both directions, without
 *     self-loops or duplicates, with unit float weights.
 *
 * Every generator draws from counter-based random streams keyed by
 * (seed, stream, index), so the output does not depend on the thread count.
 * Memory is allocated by the library; release it with lvgg_csr_free /
 * lvgg_batch_free. Functions return 0 on success and a negative errno-style
 * code on failure (see lvgg_last_error()).
 *
 * This library has no CUDA dependency: the reference's CPU arm of the
 * benchmark links it without loading any GPU code.
 */
#ifndef LOUVAIN_GB300_GRAPHGEN_H
#define LOUVAIN_GB300_GRAPHGEN_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/** A CSR graph on the host: row u is keys[offsets[u] .. offsets[u+1]). */
typedef struct lvgg_csr {
  size_t    span;       /* number of vertex slots (max id + 1) */
  size_t    num_edges;  /* directed edges = offsets[span] */
  uint64_t *offsets;    /* [span+1] */
  uint32_t *keys;       /* [num_edges] neighbour ids, sorted within each row */
  float    *weights;    /* [num_edges] */
  uint8_t  *exists;     /* [span] 1 if the vertex exists (vertex 0 never does) */
} lvgg_csr;

/** A tidy batch update: both directions of each undirected edge, sorted by (src, dst), unique. */
typedef struct lvgg_batch {
  size_t    num_deletions;
  size_t    num_insertions;
  uint32_t *del_src, *del_dst;  /* [num_deletions] */
  float    *del_w;              /* [num_deletions] weight of the removed edge */
  uint32_t *ins_src, *ins_dst;  /* [num_insertions] */
  float    *ins_w;              /* [num_insertions] */
} lvgg_batch;

/**
 * Planted-partition graph: n vertices (ids 1..n) in consecutive blocks of
 * `block` vertices; round(n*avg_degree/2) undirected draws. Each draw picks u
 * uniformly, then v uniformly inside u's block with probability p_in, else
 * uniformly over all vertices. Self-loops are dropped, then the edges are
 * symmetrized and deduplicated.
 */
int lvgg_planted_partition(uint32_t n, uint32_t block, double avg_degree, double p_in,
                           uint64_t seed, lvgg_csr *out);

/**
 * R-MAT graph: 2^scale vertices (ids 1..2^scale), round(edge_factor*2^scale)
 * undirected draws with quadrant probabilities (a, b, c, 1-a-b-c). If permute
 * is non-zero, vertex ids are relabelled by a seeded random permutation (as
 * Graph500 does), so that id order carries no degree information. Self-loops
 * dropped, symmetrized, deduplicated.
 */
int lvgg_rmat(int scale, double edge_factor, double a, double b, double c, int permute,
              uint64_t seed, lvgg_csr *out);

/**
 * Random batch on graph x: num_updates undirected updates, of which
 * round(num_updates*insertion_fraction) are insertions of uniformly random
 * vertex pairs (u != v, edge absent) and the rest deletions of uniformly
 * sampled existing undirected edges (edge-uniform). The batch is returned tidy:
 * both directions, sorted by (src, dst), unique.
 */
int lvgg_random_batch(const lvgg_csr *x, size_t num_updates, double insertion_fraction,
                      uint64_t seed, lvgg_batch *out);

/** y = x with the batch's deletions removed and insertions added (rows stay sorted). */
int lvgg_apply_batch(const lvgg_csr *x, const lvgg_batch *b, lvgg_csr *y);

/* A random untidy batch as the reference draws one:
 * generateEdgeDeletions(rnd, x, deletions, begin, range, true) and
 * generateEdgeInsertions(rnd, x, insertions, begin, range, true, weight)
 * (inc/batch.hxx:105-143): a deletion picks a source uniform in
 * [begin, begin+range), retried up to 5 times while it has no edge, then a
 * uniform neighbour; an insertion picks both endpoints uniform in the range;
 * both directions are emitted. Each draw has its own counter-based stream,
 * so the result equals lvg_device_batch_generate's on the same graph. */
int lvgg_reference_batch(const lvgg_csr *x, size_t deletions, size_t insertions, uint32_t begin, uint32_t range,
                         float weight, uint64_t seed, lvgg_batch *out);

/* ---- Temporal edge streams (the reference's SNAP temporal input). */

/** An edge list in stream order. */
typedef struct lvgg_edges {
  size_t    n;
  uint32_t *src, *dst;
  float    *w;
} lvgg_edges;

typedef struct lvgg_temporal lvgg_temporal;
/** Open a SNAP temporal file ("u v [w] [t]" per line, as inc/snap.hxx:41-140 reads it). */
int lvgg_temporal_open(const char *path, int weighted, lvgg_temporal **out);
/**
 * The next `lines` lines as edges (both directions when symmetric, as
 * readTemporalDo emits them, inc/snap.hxx:41-60; weight 1 unless weighted).
 * Stops early at the end of the file or a line that does not parse.
 */
int lvgg_temporal_read(lvgg_temporal *t, size_t lines, int symmetric, lvgg_edges *out);
void lvgg_temporal_close(lvgg_temporal *t);
/** Write edges as a SNAP temporal file: "u v t" lines, t = stream index (one line per edge). */
int lvgg_temporal_write(const char *path, const lvgg_edges *e);

/**
 * The graph readTemporalOmpW builds from an edge list (inc/snap.hxx:160-212):
 * vertices 1..rows exist (and any endpoint of an edge), rows sorted by
 * neighbour id, duplicate edges merged keeping the last weight. Ids must be
 * <= rows.
 */
int lvgg_csr_from_edges(size_t rows, const lvgg_edges *e, lvgg_csr *out);

/**
 * A synthetic temporal stream with drifting communities (stands in for the
 * SNAP temporal datasets): n vertices (ids 1..n) in `communities` groups of
 * log-normal sizes (sigma), `edges` undirected edges in time order, each
 * intra-community with probability p_in (else uniform); every
 * `drift_every` edges, a fraction `drift` of the vertices move to a random
 * community. One line per undirected edge (as the SNAP files are).
 */
int lvgg_temporal_drift(uint32_t n, uint32_t communities, double sigma, size_t edges, double p_in,
                        size_t drift_every, double drift, uint64_t seed, lvgg_edges *out);
void lvgg_edges_free(lvgg_edges *e);

void lvgg_csr_free(lvgg_csr *g);
void lvgg_batch_free(lvgg_batch *b);

/** Message of the last failure on this thread ("" if none). */
const char *lvgg_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
