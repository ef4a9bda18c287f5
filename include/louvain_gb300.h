/*
 * louvain_gb300.h — C-ABI of the GB300-native Louvain library.
 *
 * This is the drop-in boundary for the Louvain hot path of
 * puzzlef/louvain-communities-openmp-dynamic (inc/louvain.hxx). The four run
 * entry points replace the reference's four public templates; the options and
 * result records mirror LouvainOptions and LouvainResult<K, double> field for
 * field. Behind the ABI every step runs as hand-written sm_103a CUDA kernels
 * on one GPU; there is no CPU fallback (a call on a machine without a usable
 * GPU fails with LVG_ECUDA).
 *
 * Conventions (as in the reference):
 *   - vertex ids are uint32 (K = uint32_t), edge weights float (TYPE float,
 *     main.cxx:19), result weights double (LOUVAIN_WEIGHT_TYPE, inc/louvain.hxx:67);
 *   - a graph has `span` vertex slots; a slot may be absent (`exists[u] == 0`),
 *     as vertex 0 of the reference's SNAP graphs is (inc/snap.hxx:133);
 *   - a batch lists both directions of each undirected update; the
 *     delta-screening entry requires insertions sorted by source
 *     (inc/louvain.hxx:1432-1433), and checks it.
 *
 * Threading: calls on distinct graph handles may run concurrently from
 * different host threads; calls on one handle must be serialised by the
 * caller. Every call runs on the handle's own CUDA stream.
 *
 * Errors: every function that returns int returns LVG_OK (0) or a negative
 * status; the message of the last failure on the calling thread is
 * lvg_last_error(). Arguments are checked before any device work; NULL is
 * refused with LVG_EINVAL, except by the *_destroy functions, which accept it
 * as free() does.
 */
#ifndef LOUVAIN_GB300_H
#define LOUVAIN_GB300_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. The reference has none: it returns by value, throws only
 * std::bad_alloc and compiles its ASSERTs out (inc/_debug.hxx:215-227). */
#define LVG_OK        0
#define LVG_EINVAL   (-22)   /* bad argument: id >= span, unsorted DS batch, size mismatch */
#define LVG_ENOMEM   (-12)   /* device or host allocation failed */
#define LVG_ETIMEOUT (-62)   /* a bounded device loop hit its cap (hash table overflow guard) */
#define LVG_ECUDA    (-1000) /* CUDA runtime error (no device, launch failure, ...), or a
                                 device-side invariant check (a worklist append outside
                                 its degree bin) */

/* Options. Mirrors LouvainOptions (inc/louvain.hxx:30-63) with the same
 * defaults, including aggregationTolerance = 1.0 (inc/louvain.hxx:60). */
typedef struct lvg_options {
  int    repeat;                /* runs to average the timings over [1] */
  double resolution;            /* modularity resolution R [1] */
  double tolerance;             /* local-moving convergence tolerance [1e-2] */
  double aggregationTolerance;  /* stop when communities/vertices >= this [1.0] */
  double toleranceDrop;         /* tolerance divisor after each pass [10] */
  int    maxIterations;         /* local-moving iterations per pass [20] */
  int    maxPasses;             /* passes [10] */
  /* Extension (no reference counterpart): 0 = asynchronous moves with the
   * reference's semantics; 1 = deterministic synchronous moves (every
   * decision reads the previous iteration's state, ties go to the lowest
   * community id), reproducible bit for bit. */
  int    deterministic;
  /* Extension: colour classes per local-moving sweep (1..64; 0 = default:
   * 16 deterministic; asynchronous static Louvain 64 in its first iteration,
   * where every vertex is a singleton, then 16; the other asynchronous
   * methods 8, or the graph's tuned frontier_colors for DF and DS). Vertices
   * are split into classes by a hash of their id and each iteration visits
   * the classes in turn, so most neighbours see each other's moves within
   * the iteration, as in the reference's sequential sweep. */
  int    colors;
} lvg_options;

/* Fill *o with the reference's defaults. Replaces LouvainOptions::LouvainOptions
 * (inc/louvain.hxx:60). */
void lvg_options_default(lvg_options *o);

/* Result. Mirrors LouvainResult<uint32_t, double> (inc/louvain.hxx:78-145).
 * Array fields: if the caller leaves a pointer NULL, the library allocates it
 * (malloc, span entries) and lvg_result_free() releases it; a non-NULL pointer
 * is taken as a caller-owned buffer of `span` entries and is filled in place
 * (use lvg_host_alloc() for pinned buffers). */
typedef struct lvg_result {
  size_t    span;
  uint32_t *membership;       /* community of each vertex (last level, renumbered) */
  double   *vertexWeight;     /* total edge weight of each vertex (first pass) */
  double   *communityWeight;  /* last pass's community totals; entries past the live ids are stale */
  int       iterations;       /* local-moving iterations over all passes */
  int       passes;           /* passes performed */
  float     time;             /* ms, mean over repeats: init + mark + passes */
  float     markingTime;      /* ms, marking affected vertices */
  float     initializationTime; /* ms, initial membership and weights */
  float     firstPassTime;    /* ms, first pass */
  float     localMoveTime;    /* ms, all local-moving phases */
  float     aggregationTime;  /* ms, all aggregation phases */
  size_t    affectedVertices; /* flags still set after the run (inc/louvain.hxx:1220) */
  int       owned;            /* bit 0/1/2: membership/vertexWeight/communityWeight allocated by the library */
} lvg_result;

/* A batch update (host arrays). Replaces the reference's
 * vector<tuple<K,K,V>> deletions / insertions. */
typedef struct lvg_batch {
  size_t          num_deletions;
  const uint32_t *del_src, *del_dst;
  const float    *del_w;
  size_t          num_insertions;
  const uint32_t *ins_src, *ins_dst;
  const float    *ins_w;
} lvg_batch;

/* A graph resident on the GPU (CSR: offsets, neighbour ids, weights). */
typedef struct lvg_graph lvg_graph;

/* Upload a CSR graph. offsets[span+1], keys/weights[offsets[span]];
 * exists[span] may be NULL (every slot exists). Replaces the reference's
 * graph argument `const G& x` (inc/louvain.hxx:1285): the G concept
 * (span/order/size/hasVertex/forEachEdge, inc/Graph.hxx:59-150) flattened. */
int lvg_graph_create(size_t span, const uint64_t *offsets, const uint32_t *keys, const float *weights,
                     const uint8_t *exists, lvg_graph **out);
int lvg_graph_destroy(lvg_graph *g);
/* Device bytes held by a graph: its gapped CSR, workspace and scratch. */
size_t lvg_graph_device_bytes(const lvg_graph *g);
/* Release scratch a graph keeps between calls: level 1 the global hash
 * tables and the batch-apply scratch, level 2 also the workspace. Later calls
 * allocate again what they need. */
int lvg_graph_trim(lvg_graph *g, int level);
/* G::span(), G::order(), G::size() (inc/Graph.hxx:59-80). */
size_t lvg_graph_span(const lvg_graph *g);
size_t lvg_graph_order(const lvg_graph *g);
size_t lvg_graph_size(const lvg_graph *g);

/* Static Louvain. Replaces louvainStaticOmp(x, o) (inc/louvain.hxx:1285). */
int lvg_static(lvg_graph *x, const lvg_options *o, lvg_result *out);

/* Naive-dynamic Louvain on the updated graph y, from the prior membership q
 * and weights qvtot/qctot (span entries each). Replaces
 * louvainNaiveDynamicOmp(y, deletions, insertions, q, qvtot, qctot, o)
 * (inc/louvain.hxx:1349). */
int lvg_naive_dynamic(lvg_graph *y, const lvg_batch *b, const uint32_t *q, const double *qvtot,
                      const double *qctot, const lvg_options *o, lvg_result *out);

/* Delta-screening dynamic Louvain. Replaces louvainDynamicDeltaScreeningOmp
 * (inc/louvain.hxx:1542). Insertions must be sorted by source (LVG_EINVAL otherwise). */
int lvg_delta_screening(lvg_graph *y, const lvg_batch *b, const uint32_t *q, const double *qvtot,
                        const double *qctot, const lvg_options *o, lvg_result *out);

/* Dynamic-frontier Louvain. Replaces louvainDynamicFrontierOmp
 * (inc/louvain.hxx:1674). */
int lvg_frontier(lvg_graph *y, const lvg_batch *b, const uint32_t *q, const double *qvtot,
                 const double *qctot, const lvg_options *o, lvg_result *out);

/* Affected-vertex marking alone: applies the batch to the prior weights and
 * marks the vertices a method would start from, without running the passes.
 * method LVG_METHOD_FRONTIER replaces louvainAffectedVerticesFrontierOmpW
 * (inc/louvain.hxx:1606); LVG_METHOD_DELTA replaces
 * louvainAffectedVerticesDeltaScreeningOmpW (inc/louvain.hxx:1441) and also
 * returns its neighbour and community flags (either pointer may be NULL);
 * LVG_METHOD_NAIVE / LVG_METHOD_STATIC mark every slot. flags[span]. */
int lvg_affected_vertices(lvg_graph *y, int method, const lvg_batch *b, const uint32_t *q, const double *qvtot,
                          const double *qctot, const lvg_options *o, uint8_t *flags, uint8_t *neighbors,
                          uint8_t *communities);

/* One aggregation step for a given membership: renumbers the communities in
 * id order (louvainCommunityExistsOmpW + louvainRenumberCommunitiesOmpW,
 * inc/louvain.hxx:668, 941) and builds the super-vertex graph
 * (louvainCommunityVerticesOmpW + louvainAggregateOmpW, :800, :987).
 * renumbered[span] receives the renumbered membership, *num_communities the
 * community count, offsets[CN+1] / keys / weights the super-vertex CSR
 * (compact; keys/weights need room for lvg_graph_size(g) entries). Row order
 * within a super-vertex is unspecified, as in the reference. */
int lvg_aggregate(lvg_graph *g, const uint32_t *membership, uint32_t *renumbered, size_t *num_communities,
                  uint64_t *offsets, uint32_t *keys, double *weights);

/* Release the library-owned arrays of a result (LouvainResult's destructor). */
void lvg_result_free(lvg_result *r);

/* Modularity of a membership on graph g, reduced in FP64 on the GPU.
 * Replaces modularityBy (inc/properties.hxx:178) as used by main.cxx:48-51.
 * M <= 0 means "half the total edge weight of g". */
int lvg_modularity(lvg_graph *g, const uint32_t *membership, double M, double R, double *out);

/* Total edge weight of g (FP64 on the GPU). Replaces edgeWeightOmp
 * (inc/properties.hxx:96). */
int lvg_edge_weight(lvg_graph *g, double *out);
/* louvainVertexWeightsOmpW (inc/louvain.hxx:210-218): vtot[u] = sum of u's
 * edge weights (self-loops included), accumulated in FP64; vtot[span]. */
int lvg_vertex_weights(lvg_graph *g, double *vtot);
/* louvainCommunityWeightsOmpW (inc/louvain.hxx:247-256) and the totals of
 * louvainInitializeFromOmpW (:325-335): ctot[c] = sum of vtot[u] over the
 * vertices u with membership[u] == c, in FP64; vtot NULL = the graph's
 * vertex weights. membership, vtot, ctot: [span]; ids must be < span. */
int lvg_community_weights(lvg_graph *g, const uint32_t *membership, const double *vtot, double *ctot);

/* Pinned host memory for result buffers and batches (no reference counterpart). */
void *lvg_host_alloc(size_t bytes);
void  lvg_host_free(void *p);

/* ---- Device-resident inputs (no reference counterpart). The reference keeps
 * its graph, batch and prior state in host memory; these keep them in HBM so a
 * caller that applies many batches (a serving loop) pays no host<->device copy
 * per call. */

/* Methods of lvg_run_resident. */
#define LVG_METHOD_STATIC    0
#define LVG_METHOD_NAIVE     1
#define LVG_METHOD_DELTA     2
#define LVG_METHOD_FRONTIER  3

/* Membership, vertex weights and community weights of a graph (span entries
 * each) in HBM. Weights are held in FP32 on the device. */
typedef struct lvg_state lvg_state;
int lvg_state_create(lvg_graph *g, lvg_state **out);
/* Upload (q, qvtot, qctot) from host arrays of span entries. */
int lvg_state_set(lvg_state *st, const uint32_t *q, const double *qvtot, const double *qctot);
/* Download into host arrays of span entries; any pointer may be NULL. */
int lvg_state_get(const lvg_state *st, uint32_t *membership, double *vtot, double *ctot);
/* A state or device batch may be destroyed before or after its graph; every
 * other call on it needs the graph alive. */
int lvg_state_destroy(lvg_state *st);
size_t lvg_state_device_bytes(const lvg_state *st);

/* A validated batch in HBM. */
typedef struct lvg_device_batch lvg_device_batch;
int lvg_device_batch_create(lvg_graph *g, const lvg_batch *b, lvg_device_batch **out);
/* Replace a device batch's contents with a new host batch (its buffers grow
 * as needed and are reused: no allocation once they are large enough). */
int lvg_device_batch_set(lvg_device_batch *db, const lvg_batch *b);
int lvg_device_batch_destroy(lvg_device_batch *b);
size_t lvg_device_batch_device_bytes(const lvg_device_batch *b);

/* Caller-owned arrays that receive a batch; the counts are written back. */
typedef struct lvg_batch_buf {
  size_t    num_deletions;
  uint32_t *del_src, *del_dst;
  float    *del_w;
  size_t    num_insertions;
  uint32_t *ins_src, *ins_dst;
  float    *ins_w;
} lvg_batch_buf;

/* Tidy a batch against the graph and apply it in place, on the GPU.
 * Replaces the host-side pair main.cxx:108-109 runs before each dynamic call:
 * tidyBatchUpdateU(deletions, insertions, y) (inc/batch.hxx:202-209) keeps the
 * deletions whose edge is present and the insertions whose edge is absent,
 * sorted by (source, target) without duplicates, and
 * applyBatchUpdateOmpU(y, deletions, insertions) (inc/batch.hxx:241-248)
 * removes and adds them; an added edge makes both endpoints present. The
 * batch may be unsorted and hold duplicates (the first in batch order is
 * kept; the reference keeps an unspecified one). Ids must be < span (the
 * graph does not grow its span). Only the touched rows are rewritten: the
 * graph keeps per-row slack and an overflow pool. Needs the rows given to
 * lvg_graph_create sorted by neighbour id (LVG_EINVAL otherwise).
 * `tidy` (may be NULL; arrays with room for b's counts) receives the tidied
 * batch, which is what the dynamic methods take. */
int lvg_graph_apply_batch(lvg_graph *g, const lvg_batch *b, lvg_batch_buf *tidy);
/* The same for a batch in HBM (created on this graph); the batch is replaced
 * by the tidied batch, ready for lvg_run_resident. A batch applies once
 * (LVG_EINVAL the second time). */
int lvg_graph_apply_device_batch(lvg_graph *g, lvg_device_batch *b);

/* ---- Generators in HBM (no reference counterpart; the same draws as the
 * host generators of louvain_gb300_graphgen.h, so the graphs equal
 * lvgg_planted_partition / lvgg_rmat row for row). */
int lvg_graph_create_planted_partition(uint32_t n, uint32_t block, double avg_degree, double p_in, uint64_t seed,
                                       lvg_graph **out);
int lvg_graph_create_rmat(int scale, double edge_factor, double a, double b, double c, int permute, uint64_t seed,
                          lvg_graph **out);
/* The graph readTemporalOmpW + symmetrizeOmp build from an edge list
 * (inc/snap.hxx:160-216, main.cxx:159-161), built in HBM: n directed edges
 * (src, dst, w; w NULL = weight 1), ids < span; vertices 1..span-1 and every
 * endpoint present; rows sorted; duplicates merged keeping the last weight. */
int lvg_graph_create_from_edges(size_t span, size_t n, const uint32_t *src, const uint32_t *dst, const float *w,
                                lvg_graph **out);
/* A copy of a graph in HBM (main.cxx's `auto y = duplicate(x)`). */
int lvg_graph_clone(lvg_graph *x, lvg_graph **out);
/* A random batch drawn on the device as the reference draws one:
 * generateEdgeDeletions(rnd, y, deletions, begin, range, true) and
 * generateEdgeInsertions(rnd, y, insertions, begin, range, true, weight)
 * (inc/batch.hxx:105-143), each draw from its own counter-based stream
 * instead of one mt19937 (lvgg_reference_batch draws the same on the host).
 * The batch is untidy; lvg_graph_apply_device_batch tidies and applies it. */
int lvg_device_batch_generate(lvg_graph *g, size_t deletions, size_t insertions, uint32_t begin, uint32_t range,
                              float weight, uint64_t seed, lvg_device_batch **out);
/* Entry counts of a device batch, and a copy of it into host arrays. */
int lvg_device_batch_size(const lvg_device_batch *b, size_t *deletions, size_t *insertions);
int lvg_device_batch_download(const lvg_device_batch *b, lvg_batch_buf *out);

/* Download the graph as a compact CSR: offsets[span+1], keys/weights[size],
 * exists[span] (any of keys/weights/exists may be NULL). Rows come out in
 * the order they are held (sorted when the uploaded rows were). */
int lvg_graph_download(lvg_graph *g, uint64_t *offsets, uint32_t *keys, float *weights, uint8_t *exists);

/* Run a method on device-resident inputs: prior state `prior` (ignored by
 * LVG_METHOD_STATIC) and batch `b` (NULL for static); the result state is
 * written to `out` (out may equal prior: updated in place). `info` receives
 * the scalar fields of the result; its arrays are not touched. */
int lvg_run_resident(lvg_graph *g, int method, const lvg_device_batch *b, const lvg_state *prior, lvg_state *out,
                     const lvg_options *o, lvg_result *info);

/* ---- Serving loop (no reference counterpart; the reference runs one graph
 * and one batch at a time, main.cxx:101-135). A server keeps many graphs and
 * their community state in HBM and answers batch updates: each request is a
 * host batch for one graph, which a worker uploads, tidies and applies to the
 * graph in HBM (lvg_graph_apply_device_batch) before running `method` from
 * the graph's current state (lvg_run_resident), whose result replaces it.
 * Requests for one graph run in arrival order; different graphs run
 * concurrently, one worker thread each, on their own streams. */
typedef struct lvg_server lvg_server;
typedef struct lvg_server_options {
  int         workers;     /* host worker threads = requests in flight (default 8) */
  size_t      hbm_budget;  /* admission budget in bytes for resident graphs (default 120 GiB) */
  int         method;      /* LVG_METHOD_NAIVE / _DELTA / _FRONTIER (default FRONTIER) */
  lvg_options louvain;     /* options of every run */
  size_t      coalesce;    /* 0 (default): one request per run; else serve a graph's queued requests as
                              one batch of up to this many entries (their union, tidied and applied at
                              once). Every request of such a group gets the group's result; a group
                              ends before a request that inserts or deletes an edge an earlier
                              request of the group inserts, or inserts one it deletes, so the graph
                              after a group equals the graph after its requests one by one */
} lvg_server_options;
typedef struct lvg_request_info {
  uint64_t ticket;
  int      graph, status;
  double   queue_ms, apply_ms, run_ms, latency_ms;  /* latency = submit to completion */
  int      iterations, passes;
  uint64_t affected;
  size_t   tidy_deletions, tidy_insertions;         /* the batch after the tidy */
  uint64_t group;      /* ticket of the first request of the run that answered this one */
  int      coalesced;  /* requests answered by that run (1: served alone) */
} lvg_request_info;
typedef struct lvg_server_stats_t {
  uint64_t completed, failed, updates;  /* updates = batch entries of completed requests */
  size_t   graphs, hbm_reserved;
  double   p50_ms, p99_ms, max_ms, mean_ms;  /* request latency */
  double   wall_s, updates_per_s, requests_per_s;
  double   mean_queue_ms, mean_apply_ms, mean_run_ms;  /* where a request's time goes */
} lvg_server_stats_t;
void lvg_server_options_default(lvg_server_options *o);
/* Estimated device bytes of a resident graph (the admission rule). */
size_t lvg_graph_footprint(size_t span, size_t edges);
int lvg_server_create(const lvg_server_options *o, lvg_server **out);
/* Add a graph (LVG_ENOMEM when its footprint does not fit the budget). Its
 * state starts from (q, qvtot, qctot), or from static Louvain when q is NULL.
 * With take_ownership the server destroys the graph at the end. */
int lvg_server_add_graph(lvg_server *sv, lvg_graph *g, int take_ownership, const uint32_t *q, const double *qvtot,
                         const double *qctot, int *graph_id);
/* Change the coalescing cap (lvg_server_options.coalesce) of a running
 * server; groups formed afterwards use it. */
int lvg_server_set_coalesce(lvg_server *sv, size_t coalesce);
/* Queue a batch for a graph (copied; the caller's arrays may be reused). */
int lvg_server_submit(lvg_server *sv, int graph_id, const lvg_batch *b, uint64_t *ticket);
/* Wait for a request; returns its status. Each ticket can be waited once. */
int lvg_server_wait(lvg_server *sv, uint64_t ticket, lvg_request_info *info);
/* Wait until every queued request has completed. */
int lvg_server_drain(lvg_server *sv);
int lvg_server_stats(lvg_server *sv, int reset, lvg_server_stats_t *out);
/* A graph's current state (after its queued requests), into host arrays. */
int lvg_server_membership(lvg_server *sv, int graph_id, uint32_t *membership, double *vtot, double *ctot);
lvg_graph *lvg_server_graph(lvg_server *sv, int graph_id);
/* Static Louvain on many graphs at once (no reference counterpart; the
 * reference runs one graph per process): `workers` host threads each take the
 * next graph and run lvg_static on its own stream, so the GPU overlaps the
 * graphs' kernels; with trim > 0 each graph is trimmed (lvg_graph_trim) after
 * its run, so only `workers` workspaces are held at a time. results[i] as
 * lvg_static fills it. Returns the first failure's status (the other graphs
 * still run). */
int lvg_static_many(lvg_graph *const *graphs, size_t n, const lvg_options *o, int workers, int trim,
                    lvg_result *results);
/* Graph unions (no reference counterpart; the batched form of
 * louvainStaticOmp, inc/louvain.hxx:1180-1215, over many graphs): the graphs'
 * CSRs copied back to back into one graph in HBM, graph i owning vertices
 * [vb[i], vb[i+1]) with its ids shifted by vb[i] (the sources are unchanged
 * and may be destroyed afterwards). */
int lvg_graph_create_union(lvg_graph *const *graphs, size_t n, lvg_graph **out);
/* Graphs in a union (0 for a plain graph). */
int lvg_union_graphs(const lvg_graph *u, size_t *n);
/* Static Louvain on every graph of a union in one run: each level's local
 * moving is one set of launches over all graphs still moving, and each graph
 * keeps its own M, colour classes (by its own ids), iteration and pass tests,
 * so results[i] equals lvg_static on graph i alone — bit for bit in
 * deterministic mode with integer weights (membership, weights, iterations,
 * passes, affectedVertices); the time fields are the whole run's. The other
 * methods and batch updates reject a union (LVG_EINVAL). */
int lvg_static_union(lvg_graph *u, const lvg_options *o, lvg_result *results);
/* Drains, stops the workers, frees the states and owned graphs. */
int lvg_server_destroy(lvg_server *sv);

/* Per-call device statistics of the last run on g (no reference
 * counterpart; used for the roofline figures): kernel time of the
 * local-moving launches and the work they did. */
typedef struct lvg_stats {
  double   move_kernel_ms;     /* sum of local-moving launch durations (CUDA events) */
  uint64_t move_launches;      /* local-moving kernel launches */
  uint64_t move_vertices;      /* vertices processed (active) */
  uint64_t move_edges;         /* edges scanned by processed vertices */
  uint64_t moves;              /* vertices that changed community */
  double   aggregate_kernel_ms;
  uint64_t aggregate_edges;    /* edges read by aggregation */
  uint64_t aggregate_launches;
  uint64_t kernel_launches;    /* all kernels launched by the last call */
  /* Per degree bin of the local-moving kernels (bin b holds degrees in
   * (4,8,16,32,64,128,256,512,2048,8192 boundaries), bin 0 = degree 0,
   * bin 11 = above 8192): launch time, vertices processed, edges scanned. */
  double   move_bin_ms[12];
  uint64_t move_bin_vertices[12];
  uint64_t move_bin_edges[12];
  /* Host-array entry points (lvg_static/.../lvg_frontier): wall-clock time of
   * the call's three parts — batch + prior upload, the run, result download. */
  double   call_upload_ms, call_run_ms, call_download_ms;
  /* Vertices of each degree bin whose distinct neighbour communities did not
   * fit the bin's shared-memory table (redone with a table in HBM; bin 11:
   * hub merges), and hub chunks that handed their raw pairs on. */
  uint64_t move_bin_overflow[12];
  uint64_t hub_chunk_overflow;
  /* Resident hub tables (lvg_tuning.hub_tables): slots read by the table
   * evaluations, tables that ran out of room (their hubs scanned their edges
   * instead), and whether the call built the tables (1) or took them from
   * its prior state (0). */
  uint64_t hub_table_slots;
  uint64_t hub_table_overflow;
  uint64_t hub_tables_built;
  /* Times the last call waited for the GPU (stream synchronisations of the
   * run: with the local-moving phase replayed as one graph, a dynamic-frontier
   * run that ends after one pass waits once). */
  uint64_t host_syncs;
  /* Aggregated levels whose local-moving iterations after the first ran as
   * one graph launch (lvg_tuning.level_graphs). */
  uint64_t level_graphs;
} lvg_stats;
/* Enable (1) or disable (0) per-launch event timing for calls on g. */
int lvg_set_profiling(lvg_graph *g, int enable);

/* ---- Tuning (no reference counterpart). Launch-shape choices of a graph's
 * local-moving launches that leave Louvain's arithmetic unchanged, except
 * frontier_colors (the colour classes of the frontier methods in
 * asynchronous mode, whose choice lvg_autotune guards by modularity). */
typedef struct lvg_tuning {
  int      frontier_colors;    /* colour classes of DF and DS when lvg_options.colors == 0
                                  and deterministic == 0 (default 8) */
  int      concurrent_bins;    /* 1: a class's degree bins run concurrently on side streams (default 1) */
  int      fused_small;        /* the frontier methods' first pass runs bins 1-8 as two launches per
                                  class: 0 no (separate launches), 1 yes with the method's blocks per
                                  SM and bin (2 for DF's short worklists, 8 for delta-screening's whole
                                  communities), k >= 2 yes with k (default 0) */
  uint32_t hub_chunk;          /* edges per chunk of a vertex above degree 8192 (256..1<<20; default 4096) */
  int      big_blocks_per_sm;  /* resident blocks per SM of the degree 513-8192 kernels (0 = as many
                                  as fit; default 0) */
  double   frontier_max_fraction;  /* frontier_colors applies to batches of at most this many
                                      entries per edge of the graph; larger batches (whose
                                      frontiers cover much of the graph) keep 8 classes
                                      (default 1e-3) */
  int      hub_tables;         /* 1: the neighbour counts per community of every vertex above
                                  degree 8192 of a unit-weight graph are kept with each state
                                  (lvg_run_resident) and cached by the graph for the host-array
                                  calls, so that the delta-screening and dynamic-frontier first
                                  passes evaluate such a vertex from its table instead of its
                                  edges; naive-dynamic, whose every vertex moves, always scans
                                  (same results; default 1) */
  uint32_t bin_max_degree[12]; /* the local-moving degree bins: bin b (1..9) takes vertex degrees
                                  up to bin_max_degree[b] (0 = its full reach: 4, 8, 16, 32, 64,
                                  128, 256, 512, 2048 for b = 1..9), above the previous bin's;
                                  each bin's tile width and hash-table capacity are those of its
                                  full reach, so a lower limit hands the bin's upper degrees to
                                  the next bin's wider tile and larger table, and a limit equal
                                  to the previous bin's empties the bin. Entries 0, 10 and 11
                                  are 0 (bin 10 ends at degree 8192, the hubs' threshold).
                                  Same results in deterministic mode (default all 0) */
  int      level_graphs;       /* 1: on every aggregated level, the local-moving iterations after
                                  the first run as one CUDA graph launch (a conditional while
                                  node with the stop test on the device) built for that level;
                                  0: one launch sequence and one synchronisation per iteration
                                  (same results; default 1) */
  int      small_regs;         /* registers a thread of the fused launch of degree bins 1-6
                                  (fused_small): 32 (8 resident blocks per SM, some values kept
                                  in local memory) or 64 (4 blocks per SM, none); default 64 */
} lvg_tuning;
void lvg_tuning_default(lvg_tuning *t);
int lvg_graph_get_tuning(const lvg_graph *g, lvg_tuning *t);
int lvg_graph_set_tuning(lvg_graph *g, const lvg_tuning *t);
/* The autotuner: coordinate descent over the knobs of lvg_tuning on this
 * graph and workload (method, batch and prior as lvg_run_resident takes
 * them; a graph union takes LVG_METHOD_STATIC and runs lvg_static_union).
 * Each candidate is run once to warm up and then `repeats` times; the
 * fastest (minimum of LouvainResult::time) is kept when it beats the current
 * choice by 2 %, and a frontier_colors candidate only when its modularity is
 * within 1e-3 of the starting choice's. Two rounds over the knobs, the colour
 * classes first. The result is set on the graph and returned in *best (time
 * in *best_ms). */
int lvg_autotune(lvg_graph *g, int method, const lvg_device_batch *b, const lvg_state *prior, const lvg_options *o,
                 int repeats, lvg_tuning *best, double *best_ms);
int lvg_get_stats(const lvg_graph *g, lvg_stats *out);

/* ---- Modularity without device allocation. No counterpart in the reference.
 * For callers that cannot allocate device memory when they call in (a host
 * framework that has reserved the GPU's memory for its own pool, a
 * latency-critical loop that must not pay cudaMalloc's cost and implicit
 * synchronisation, or a deployment that forbids allocation after start-up).
 * Same result as lvg_modularity, but every pointer is a caller-owned DEVICE
 * pointer: offsets[span+1], keys/weights[offsets[span]] (never NULL, even for
 * a graph without edges), exists[span] (may be NULL: every slot exists),
 * membership[span], and out (one double, written on
 * the device). M <= 0 means half the total edge weight. `stream` is a
 * cudaStream_t (NULL: the default stream); the call is asynchronous on it.
 * The function allocates nothing: its scratch is a fixed device array of
 * LVG_NOALLOC_MAX_SPAN doubles (8 MiB) that every GPU loading the library
 * holds until the process exits; spans above that return LVG_EINVAL. The
 * first call on a device looks up that array's device address (make that
 * first call before any stream capture). All calls share the array: calls
 * that overlap on the GPU (other streams, other host threads) race and must
 * be serialised by the caller. An id >= span in membership or keys makes
 * *out NaN. */
#define LVG_NOALLOC_MAX_SPAN (1u << 20)
int lvg_modularity_noalloc(size_t span, const uint64_t *offsets, const uint32_t *keys, const float *weights,
                           const uint8_t *exists, const uint32_t *membership, double M, double R, double *out,
                           void *stream);

/* Start / stop the CUDA profiler's collection (cudaProfilerStart/Stop), so a
 * profiler started with collection off captures only the bracketed calls. */
int lvg_profiler_start(void);
int lvg_profiler_stop(void);

/* Make `device` the calling thread's current GPU; handles created afterwards
 * live on it (no reference counterpart: the reference is CPU only). */
int lvg_set_device(int device);

/* Message of the last failure on the calling thread ("" if none). */
const char *lvg_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
