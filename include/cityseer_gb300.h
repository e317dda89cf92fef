/*
 * cityseer_gb300.h -- C-ABI of libcsgpu.so, the GB300 (sm_103a) implementation of cityseer's
 * localised network centrality (cityseer-api v4.24.0, rust/src/centrality.rs).
 *
 * Conventions
 *  - Plain C types only.  Pointers named *_dev are CUDA device pointers owned by the caller; the
 *    library never frees them.  `stream` is a cudaStream_t passed as void* (NULL = legacy stream).
 *  - Every entry point returns a cs_status; cs_last_error() gives the message of the last failure
 *    on the calling thread.  No C++ exception crosses this boundary.
 *  - Node indices are the reference's StableGraph indices in [0, n_bound); removed nodes simply
 *    have no edges and are never sources.
 *  - Output accumulators are caller-zeroed f64 arrays laid out [metric][threshold][n_bound], the
 *    reference's MetricResult rows (rust/src/common.rs:18-35) stacked per metric.
 */
#ifndef CITYSEER_GB300_H
#define CITYSEER_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t cs_status;
#define CS_OK 0
#define CS_ERR_ARG 1        /* invalid argument (mirrors the reference's PyValueError paths) */
#define CS_ERR_CAPACITY 2   /* workspace too small for a source's reach; retried internally */
#define CS_ERR_CUDA 3       /* CUDA runtime error (no device, launch failure, ...) */
#define CS_ERR_TIMEOUT 4    /* a bounded device-side wait gave up */
#define CS_ERR_INTERNAL 5   /* a device-side consistency check failed */

#define CS_MAX_THRESHOLDS 16  /* thresholds per launch; the host layer splits longer lists */
#define CS_MAX_DEGREE 32      /* max out-degree of a node supported by the replay kernels */

/* Device-resident primal CSR.  Built by cityseer_gb300.device from a NetworkStructure.
 * in_*  : per node u, the edges v->u in petgraph Incoming order (newest first); searches relax
 *         these (rust/src/centrality.rs:1389-1405).
 * out_* : per node v, the edges v->u sorted by (u, newest first); used to replay the order in
 *         which the reference offers candidates to v (rust/src/centrality.rs:1413-1437).
 * *_seglen / *_segimp: length / imp_factor of the edge looked up by get_edge_length_unchecked
 *         (rust/src/graph.rs:1278-1314) for that edge's reverse direction. */
typedef struct {
    int32_t n_bound;
    int32_t n_edges;            /* directed edges in each CSR */
    int32_t max_out_degree;
    const int32_t *in_ptr_dev;  /* [n_bound + 1] */
    const int32_t *in_nb_dev;   /* [n_edges] edge source v of v->u */
    const float *in_w_dev;      /* [n_edges] travel seconds of v->u (impedance applied) */
    const float *in_seglen_dev; /* [n_edges] */
    const float *in_segimp_dev; /* [n_edges] */
    const int32_t *out_ptr_dev; /* [n_bound + 1] */
    const int32_t *out_to_dev;  /* [n_edges] edge target u of v->u */
    const float *out_w_dev;     /* [n_edges] travel seconds of v->u (impedance applied) */
    const uint8_t *out_cnt_dev; /* [n_edges] 1 = counts once for the circuit rank's edge set */
    const float *out_seglen_dev;/* [n_edges] */
    const float *node_w_dev;    /* [n_bound] node weight */
} cs_primal_graph;

/* Device-resident dual CSR for simplest (angular) routing (rust/src/centrality.rs:533-775):
 * per dual node, its outgoing dual edges in petgraph Outgoing order (newest first). */
typedef struct {
    int32_t n_bound;
    int32_t n_edges;
    int32_t max_out_degree;
    const int32_t *ptr_dev;     /* [n_bound + 1] */
    const int32_t *to_dev;      /* [n_edges] */
    const float *w_dev;         /* [n_edges] travel seconds, no impedance */
    const float *ang_dev;       /* [n_edges] angle_sum */
    const float *len_dev;       /* [n_edges] length */
    const uint8_t *exit_slot_dev;  /* [n_edges] slot of the shared primal node at the edge source */
    const uint8_t *entry_slot_dev; /* [n_edges] slot of the shared primal node at the edge target */
    const int32_t *rptr_dev;    /* [n_bound + 1] incoming edges (reverse CSR of the same edges) */
    const int32_t *rfrom_dev;   /* [n_edges] source node of each incoming edge */
    const int32_t *rid_dev;     /* [n_edges] index of that edge in the forward arrays */
    /* Packed 16-byte edge records (cs_dual_pack), required by the centrality calls (the tree calls
     * read the plain arrays): fwd_pack [n_edges] in forward order = target state (2 to + entry_slot)
     * | exit_slot << 31, then the f32 bits of w, angle_sum and length; rev_pack [n_edges] in reverse
     * order = offering state (2 from + 1 - exit_slot) | entry_slot << 31, w, angle_sum, length.
     * 16-byte aligned; n_bound < 2^30. */
    const void *fwd_pack_dev;
    const void *rev_pack_dev;
} cs_dual_graph;

/* One centrality call.  Thresholds are the reference's resolved (distances, betas, seconds)
 * triple from pair_distances_betas_time (rust/src/common.rs:239-270). */
typedef struct {
    int32_t k;                               /* number of thresholds, 1..CS_MAX_THRESHOLDS */
    uint32_t distances[CS_MAX_THRESHOLDS];   /* metres */
    float betas[CS_MAX_THRESHOLDS];
    uint32_t seconds[CS_MAX_THRESHOLDS];
    float speed_m_s;
    float tolerance;              /* validated decimal tolerance, >= 1e-4 */
    float angular_scaling_unit;   /* simplest only */
    float farness_scaling_offset; /* simplest only */
    int32_t compute_closeness;
    int32_t compute_betweenness;
    int32_t track_reach;          /* count reachability_totals (sampling / source subset) */
    int64_t n_sources;
    const int32_t *sources_dev;   /* [n_sources] node indices to process, in order */
    const float *src_wt_dev;      /* [n_bound] per-source weight (node weight / sampling p) */
    const uint8_t *eligible_dev;  /* [n_bound] source_eligible (pair weights 0.5 vs 1.0) */
} cs_query;

/* A data layer assigned to street nodes (DataMap.node_data_map, rust/src/data.rs:380-510), as
 * device arrays.  Assignments are indexed a: node_ptr delimits each node's assignments (in the
 * map's order); assign_entry / assign_dist / assign_node / assign_rank give each one's data entry,
 * distance to the node (f32 of the f64), node and rank within the node's list.  entry_group is the
 * entry's dedupe key as a group id, entry_class its land-use class (-1: not an accessibility key);
 * group_ptr / group_assign list each group's assignments. */
typedef struct {
    int32_t n_entries;
    int32_t n_assign;
    int32_t n_groups;
    const int32_t *node_ptr_dev;     /* [n_bound + 1] */
    const int32_t *assign_entry_dev; /* [n_assign] */
    const float *assign_dist_dev;    /* [n_assign] */
    const int32_t *assign_node_dev;  /* [n_assign] */
    const int32_t *assign_rank_dev;  /* [n_assign] */
    const int32_t *entry_group_dev;  /* [n_entries] */
    const int32_t *entry_class_dev;  /* [n_entries] */
    const int32_t *group_ptr_dev;    /* [n_groups + 1] */
    const int32_t *group_assign_dev; /* [n_assign] */
} cs_data_map;

/* Launch plan: how many concurrent per-source searches and how much workspace they need. */
typedef struct {
    int32_t n_slots;      /* concurrent searches (one warp each) */
    int32_t cap;          /* reached-set capacity per search */
    int32_t threads_per_block;
    int32_t blocks;
    float delta_seconds;  /* band width of the label-correcting search; <= 0 picks a default */
    int32_t lanes;        /* accumulator lanes per reached node */
    int32_t variant;      /* register budget: 2, 3 or 4 resident 256-thread blocks per SM for every
                           * launch; 0 (default): slots sized for 4, and each launch takes 3 for
                           * shortest-path and OD centrality, 4 for segments, trees and accessibility */
    int32_t max_degree;   /* batches: largest out-degree over the jobs */
    int32_t n_bound;      /* node bound the slot geometry was sized for (set by the planners) */
    int32_t cta_blocks;   /* shortest-path plans: blocks of the block-per-source kernel whose scratch
                             the workspace holds (0: the per-warp kernel serves every source) */
    size_t workspace_bytes;
} cs_plan;

/* One job of a batched launch: a graph, a mode (0 shortest, 1 segment, 3 both from one search per
 * source), its thresholds, sources and outputs.  Many jobs of
 * uneven size run in one persistent launch (cs_batch_run), each source an item of a device queue. */
typedef struct {
    cs_primal_graph g;
    int32_t mode;             /* 0 = centrality_shortest, 1 = segment_centrality */
    int32_t k;
    uint32_t distances[CS_MAX_THRESHOLDS];
    float betas[CS_MAX_THRESHOLDS];
    uint32_t seconds[CS_MAX_THRESHOLDS];
    float speed_m_s;
    float tolerance;
    float delta_seconds;      /* per-job band width (autotuned); <= 0: default */
    int32_t compute_closeness;
    int32_t compute_betweenness;
    int32_t n_sources;
    const int32_t *sources_dev;
    const float *src_wt_dev;
    const uint8_t *eligible_dev;
    double *out_dev;          /* [7 (shortest) or 4 (segment)][k][n_bound], zeroed by the caller */
    double *bucket_dev;       /* [3][k][n_bound] scratch for shortest closeness: zero before the first run;
                                 every successful run leaves it zero again */
    double *out2_dev;         /* mode 3 (shortest + segment from one search per source): the segment rows
                                 [4][k][n_bound]; out_dev holds the shortest rows */
    int64_t item_begin;       /* first queue item of this job (set by cs_batch_prepare) */
} cs_batch_job;

/* One simplest-path (dual graph) job of a batched launch: outputs [4][k][n_bound] as
 * cs_centrality_simplest writes them (density, farness, harmonic, betweenness). */
typedef struct {
    cs_dual_graph g;
    int32_t k;
    uint32_t seconds[CS_MAX_THRESHOLDS];
    float tolerance;
    float angular_scaling_unit;
    float farness_scaling_offset;
    int32_t compute_closeness;
    int32_t compute_betweenness;
    int32_t n_sources;
    const int32_t *sources_dev;
    const float *src_wt_dev;
    const uint8_t *eligible_dev;
    double *out_dev;
    double *bucket_dev;       /* [3][k][n_bound] when compute_closeness: zero before the first run; every
                                 successful run leaves it zero */
    int64_t item_begin;       /* first queue item of this job (set by cs_dual_batch_prepare) */
} cs_dual_batch_job;

/* Outputs: f64 rows [metric][k][n_bound]; reach_dev: u32[k] (may be NULL when !track_reach). */
typedef struct {
    double *out_dev;
    uint32_t *reach_dev;
} cs_outputs;

/* Thread-local message of the last failing call. */
size_t cs_last_error(char *buf, size_t len);

/* Host-side threshold conversions, f32-exact restatements of rust/src/common.rs:99-270.
 * mode: 0 = distances given, 1 = betas given, 2 = minutes given.  On success fills all three
 * output arrays (length k).  min_threshold_wt < 0 selects the default MIN_THRESH_WT. */
cs_status cs_pair_distances_betas_time(float speed_m_s, int32_t mode, int32_t k, const uint32_t *distances,
                                       const float *betas, const float *minutes, float min_threshold_wt,
                                       uint32_t *out_distances, float *out_betas, uint32_t *out_seconds);

/* Host-side per-edge travel seconds, rust/src/centrality.rs:961-1007 (edge_travel_seconds with the
 * Tobler slope penalty).  has_z/z per node may be NULL.  seconds: NaN for street edges. */
cs_status cs_edge_travel_seconds(int64_t n_edges, const int32_t *src, const int32_t *dst, const float *length,
                                 const float *imp_factor, const float *seconds, const uint8_t *has_z,
                                 const double *z, float speed_m_s, int32_t use_impedance, float *out);

/* Plans a call: n_slots/cap/threads/blocks and the workspace size.  cap <= 0 picks a default;
 * max_slots <= 0 uses every resident warp; mem_budget_bytes <= 0 means no budget.
 * mode: 0 = centrality_shortest, 1 = segment_centrality, 2 = trees (isochrones). */
cs_status cs_plan_primal(const cs_primal_graph *g, int32_t mode, int32_t k, int32_t cap, int32_t max_slots,
                         int64_t mem_budget_bytes, cs_plan *plan);
/* Fills a dual CSR's packed edge records (cs_dual_graph.fwd_pack_dev / rev_pack_dev, each
 * [n_edges] x 16 bytes, 16-byte aligned) from its plain arrays, w_dev included: one record per edge
 * so that a search reads an edge with one 128-bit load.  Stream-ordered. */
cs_status cs_dual_pack(const cs_dual_graph *g, void *fwd_pack_dev, void *rev_pack_dev, void *stream);

cs_status cs_plan_dual(const cs_dual_graph *g, int32_t mode, int32_t k, int32_t cap, int32_t max_slots,
                       int64_t mem_budget_bytes, cs_plan *plan);

/* Clean-state initialisation of a workspace planned by cs_plan_dual. */
cs_status cs_dual_workspace_init(const cs_plan *plan, int32_t n_bound, void *workspace_dev, size_t workspace_bytes,
                                 void *stream);

/* Puts a freshly allocated workspace into the clean state every call expects (and leaves).
 * Call once after allocating it, and again after any call that returned an error. */
cs_status cs_workspace_init(const cs_plan *plan, int32_t n_bound, void *workspace_dev, size_t workspace_bytes,
                            void *stream);

/* Replaces NetworkStructure.centrality_shortest (rust/src/centrality.rs:1624-1874).
 * out rows: 0 density, 1 farness, 2 cycles, 3 harmonic, 4 beta, 5 betweenness, 6 betweenness_beta.
 * Sources whose reach exceeds plan->cap are re-run with a larger capacity inside the call. */
cs_status cs_centrality_shortest(const cs_primal_graph *g, const cs_query *q, const cs_plan *plan,
                                 void *workspace_dev, size_t workspace_bytes, cs_outputs out, void *stream);

/* Allocation-free variant of cs_centrality_shortest, for callers that cannot allocate device memory
 * when they call (a host application that owns all device memory through its own pool, a plugin
 * with a fixed memory budget, code that must not block or fail on an allocation).  It has no
 * counterpart in the reference: the Rust code allocates per call.  Its scratch is one static 64 MiB
 * device array, held by every GPU that loads the library's device code until the process exits;
 * no workspace is passed and nothing is allocated.  Same inputs, outputs and results as
 * cs_centrality_shortest.  Graphs whose single search needs more than 64 MiB of scratch are
 * rejected with CS_ERR_ARG.  All calls share the array and each call clears what must start at
 * zero; calls that overlap on the GPU race, so issue them one after another.  Every call looks up
 * the array's address (cudaGetSymbolAddress) in the caller's current device and context.  Under
 * lazy module loading (the CUDA default) the device code, and with it the array, is loaded on the
 * first call into this library on a device: make one call while setting up, before the device's
 * memory goes to the caller's pool and before any stream capture. */
cs_status cs_centrality_shortest_noalloc(const cs_primal_graph *g, const cs_query *q, cs_outputs out, void *stream);

/* Replaces NetworkStructure.centrality_simplest (rust/src/centrality.rs:1880-2132) on a dual graph.
 * out rows: 0 density, 1 farness, 2 harmonic, 3 betweenness.  Workspaces from cs_plan_dual are put
 * in their clean state by cs_dual_workspace_init.  Setting CS_DUAL_FORCE_EXACT=1 in the environment
 * runs every source through the exact sequential search (a check of the parallel path). */
cs_status cs_centrality_simplest(const cs_dual_graph *g, const cs_query *q, const cs_plan *plan,
                                 void *workspace_dev, size_t workspace_bytes, cs_outputs out, void *stream);

/* Replaces NetworkStructure.betweenness_od_shortest (rust/src/centrality.rs:2419-2540): shortest-path
 * betweenness weighted by a sparse origin-destination matrix (OdMatrix, :56-91).  od_ptr_dev
 * [n_bound + 1] delimits each origin node's row of od_dst_dev (destination nodes, ascending, no
 * repeats) and od_w_dev (trip weights).  q->sources_dev lists the live origins that have a row; the
 * query's closeness, sampling and reach fields are ignored (source weight 1, no post-scale).  Plans
 * from cs_plan_primal (mode 0, same k) serve this call.  out rows: 0 node_betweenness,
 * 1 node_betweenness_beta ([2][k][n_bound], zeroed by the caller). */
cs_status cs_betweenness_od_shortest(const cs_primal_graph *g, const cs_query *q, const int32_t *od_ptr_dev,
                                     const int32_t *od_dst_dev, const float *od_w_dev, const cs_plan *plan,
                                     void *workspace_dev, size_t workspace_bytes, cs_outputs out, void *stream);

/* Replaces NetworkStructure.segment_centrality (rust/src/centrality.rs:2134-2407).
 * out rows: 0 segment_density, 1 segment_harmonic, 2 segment_beta, 3 segment_betweenness.
 * q->sources_dev lists the live sources (segment centrality has no sampling). */
cs_status cs_segment_centrality(const cs_primal_graph *g, const cs_query *q, const cs_plan *plan,
                                void *workspace_dev, size_t workspace_bytes, cs_outputs out, void *stream);

/* Replaces DataMap.accessibility (rust/src/data.rs:605-740) with angular = False: per listed source
 * (q->sources_dev, the live nodes), a shortest-path search to the largest threshold, then its
 * reachable entries (aggregate_to_src_idx, :513-602: network + assignment distance within the
 * threshold, the nearest entry of each dedupe key) summed per class and threshold: unweighted
 * (count) and weighted (clipped_beta_wt with max_curve_wts[k], common.rs:339-348) rows
 * [n_classes][k][n_bound], zeroed by the caller, and the nearest distance within the largest
 * threshold [n_classes][n_bound] as f32 bits, set to +inf by the caller.  q's betas and seconds are
 * pair_distances_betas_time's; its sampling, closeness and betweenness fields are ignored.  Plans
 * from cs_plan_primal (mode 2) serve this call. */
cs_status cs_accessibility(const cs_primal_graph *g, const cs_data_map *dm, const cs_query *q,
                           const float *max_curve_wts, int32_t n_classes, const cs_plan *plan, void *workspace_dev,
                           size_t workspace_bytes, double *unweighted_dev, double *weighted_dev,
                           uint32_t *nearest_dev, void *stream);

/* Replaces NetworkStructure.dijkstra_tree_shortest (rust/src/centrality.rs:1141-1200, 1500-1508)
 * for a batch of sources: per query q, visited nodes in settle order with their agg_seconds and
 * predecessor.  count_dev[q] = number visited, or minus that number when it exceeds row_cap (the
 * rows are then not written); rows are row_cap wide. */
cs_status cs_tree_shortest(const cs_primal_graph *g, int32_t n_queries, const int32_t *src_dev, uint32_t max_seconds,
                           float speed_m_s, const cs_plan *plan, void *workspace_dev, size_t workspace_bytes,
                           int32_t row_cap, int32_t *count_dev, int32_t *node_dev, float *agg_seconds_dev,
                           int32_t *pred_dev, void *stream);

/* Same for dijkstra_tree_simplest (rust/src/centrality.rs:1202-1332, 1510-1521) on a dual graph:
 * per query, reached dual nodes in first-reach order with their final simpl_dist, agg_seconds and
 * node-level predecessor (-1 for the source).  count_dev[q] = number reached, or minus that number
 * when it exceeds row_cap.  The plan and workspace come from cs_plan_dual_tree /
 * cs_dual_tree_workspace_init; queries whose search outgrows the plan's capacity are redone in the
 * call at full size. */
cs_status cs_plan_dual_tree(const cs_dual_graph *g, int32_t cap, int32_t max_slots, int64_t mem_budget_bytes,
                            cs_plan *plan);
cs_status cs_dual_tree_workspace_init(const cs_plan *plan, void *workspace_dev, size_t workspace_bytes, void *stream);
cs_status cs_tree_simplest(const cs_dual_graph *g, int32_t n_queries, const int32_t *src_dev, uint32_t max_seconds,
                           float speed_m_s, const cs_plan *plan, void *workspace_dev, size_t workspace_bytes,
                           int32_t row_cap, int32_t *count_dev, int32_t *node_dev, float *simpl_dev,
                           float *agg_seconds_dev, int32_t *pred_dev, void *stream);

/* Batched persistent form (no reference counterpart: the reference runs one graph per call).
 * cs_batch_prepare fills item_begin for jobs[0..n_jobs) (host array) and returns the item count.
 * cs_batch_plan sizes one workspace for all jobs (largest graph, degree, lanes; cap = reach capacity).
 * cs_batch_run enqueues the whole batch on `stream`: a header reset, one persistent launch over
 * every item, and one launch for the closeness threshold prefixes of all jobs (which re-zeroes the
 * buckets).  jobs_dev is a device copy of the prepared host array.  With flags & CS_BATCH_ASYNC the
 * call neither synchronises nor retries (it can be captured in a CUDA graph); cs_batch_status /
 * cs_batch_failed then report the overflowed items, which contributed nothing (run them again, e.g.
 * as a batch without CS_BATCH_ASYNC).  Without the flag, overflowed items are redone inside the
 * call at growing capacities. */
#define CS_BATCH_ASYNC 1
cs_status cs_batch_prepare(cs_batch_job *jobs_host, int32_t n_jobs, int64_t *n_items);
cs_status cs_batch_plan(const cs_batch_job *jobs_host, int32_t n_jobs, int32_t cap, int32_t max_slots,
                        int64_t mem_budget_bytes, cs_plan *plan);
cs_status cs_batch_run(const cs_batch_job *jobs_host, const cs_batch_job *jobs_dev, int32_t n_jobs, const cs_plan *plan,
                       void *workspace_dev, size_t workspace_bytes, int32_t flags, void *stream);
cs_status cs_batch_status(void *workspace_dev, int64_t *n_overflowed, int64_t *sources_done, void *stream);
/* After a CS_BATCH_ASYNC launch: the global item indices of the overflowed items (first max_items
 * of *n_failed) so that the caller can run them again, e.g. as a synchronous batch (which retries
 * at full capacity).  Overflowed items contributed nothing to the outputs. */
cs_status cs_batch_failed(void *workspace_dev, const cs_plan *plan, int32_t *items_host, int32_t max_items,
                          int64_t *n_failed, void *stream);

/* Device counters of the last call on this thread: sources done, edges relaxed, nodes settled
 * (used for throughput and roofline accounting) and the number of kernels it launched. */
cs_status cs_last_counters(int64_t *sources, int64_t *edges_relaxed, int64_t *nodes_settled, int64_t *launches);

/* Per-phase SM cycles of the last call on this thread, summed over warps: 0 search, 1 sort,
 * 2 predecessor replay, 3 closeness, 4 sigma, 5 backward sweep, 6 scratch reset.  After a
 * simplest-path call: 0 search, 1 sort, 2 replay, 3 node best + closeness, 4 backward sweep,
 * 5 scratch reset, 6 exact heap search; 7 holds the number of replay rounds instead.  Entries 8-15
 * (n <= 16) are diagnostics: 8 the live progress count; after a simplest-path call 9-11 the
 * replayed states whose route came out below / above their search key / unreached, 12-14 the
 * replay rounds that ended with the routes out of order / an unreached state offered to / a state
 * reached outside the search's set, 15 the states that later replay rounds kept from the round
 * before. */
cs_status cs_last_phase_cycles(int64_t *cycles, int32_t n);

/* Source-indexed plan built on the device without synchronising (prepare_source_sampling with
 * source_indices, rust/src/centrality.rs:1032-1104): src_wt[s] = node_w[s] and eligible[s] = 1 for
 * each listed source, zero elsewhere (node_w: f32[n_bound]). */
cs_status cs_source_weights(const int32_t *sources_dev, int64_t n_sources, const float *node_w_dev, int32_t n_bound,
                            float *src_wt_dev, uint8_t *eligible_dev, void *stream);

/* Batched simplest-path form: many queries on many dual graphs in one persistent launch, as
 * cs_batch_* does for the primal.  cs_dual_batch_run with CS_BATCH_ASYNC neither synchronises nor
 * redoes anything; cs_dual_batch_failed then lists the items that overflowed or whose replay
 * disagreed (they contributed nothing; run them again as a synchronous batch, which redoes them at
 * growing capacities, then with the widened and the exact heap search). */
cs_status cs_dual_batch_prepare(cs_dual_batch_job *jobs_host, int32_t n_jobs, int64_t *n_items);
cs_status cs_dual_batch_plan(const cs_dual_batch_job *jobs_host, int32_t n_jobs, int32_t cap, int32_t max_slots,
                             int64_t mem_budget_bytes, cs_plan *plan);
cs_status cs_dual_batch_run(const cs_dual_batch_job *jobs_host, const cs_dual_batch_job *jobs_dev, int32_t n_jobs,
                            const cs_plan *plan, void *workspace_dev, size_t workspace_bytes, int32_t flags,
                            void *stream);
cs_status cs_dual_batch_failed(void *workspace_dev, const cs_plan *plan, int32_t *items_host, int32_t max_items,
                               int64_t *n_items, void *stream);

/* Sources of the last call on this thread that overflowed their slot's capacity (and were run again
 * at a larger one) and, for simplest-path calls, whose replay disagreed with the label-correcting
 * search (and were run again with the exact heap search). */
cs_status cs_last_retries(int64_t *overflowed, int64_t *inexact);

/* sizeof of cs_primal_graph, cs_dual_graph, cs_query, cs_plan, cs_outputs, cs_batch_job,
 * cs_dual_batch_job (first n). */
cs_status cs_abi_sizes(int32_t *out, int32_t n);

/* Live progress of the call running on a workspace (NetworkStructure.progress, rust/src/graph.rs:
 * 387-415): the sources its kernels have completed so far (a call resets the count when it starts;
 * sources redone after an overflow count twice).  Reads the workspace header on a stream of its own,
 * so it can be called from another host thread while the call's kernels run. */
cs_status cs_workspace_progress(const void *workspace_dev, int64_t *sources_done);

/* Number of SMs of the current device (0 on failure). */
int32_t cs_device_sm_count(void);

/* Diagnostic (no counterpart in the reference): out[i] = w[i] * exp(-(beta[i] * cost[i])) as the
 * betweenness kernels evaluate the beta-weighted seeds (f64 result of an exact f32 x f32 product,
 * the exp taken in double-float arithmetic on the f32 pipe); the reference takes the f64 exp
 * (rust/src/centrality.rs:1806-1808).  All pointers are device arrays of n elements. */
cs_status cs_debug_seed_exp(const float *w_dev, const float *beta_dev, const float *cost_dev, double *out_dev,
                            int64_t n, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* CITYSEER_GB300_H */
