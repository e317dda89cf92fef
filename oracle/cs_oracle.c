/*
 * cs_oracle.c -- CPU restatement of cityseer v4.24.0 `rustalgos` localised network centrality.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the correctness oracle and the timed CPU baseline
 * ("port") for the GPU implementation in cityseer_gb300/.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU legs may load it.  The product path never links or calls it.
 *
 * Every function follows the reference source line by line (paths relative to the cityseer-api
 * project root) and keeps the reference's data structures (node_bound sized per-source state
 * vectors, Rust std BinaryHeap ordering, petgraph reverse-insertion adjacency order, f32
 * arithmetic in the same operation order, f64 accumulation) so that it reproduces the reference's
 * results including its tie behaviour, and its cost profile when timed.
 *
 * Build: see oracle/Makefile (-O2 -ffp-contract=off: Rust never contracts a*b+c into an FMA).
 * Third-party crates restated here (pinned in rust/Cargo.lock of the reference):
 *   petgraph 0.8.3 StableGraph   -> per-node linked lists, newest edge first (og_graph below)
 *   Rust std BinaryHeap          -> hp_push / hp_pop (sift_up, sift_down_to_bottom)
 *   atomic_float 1.1.0 AtomicF64 -> add_f64_atomic (CAS loop)
 */
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define TIE_EPSILON 1e-4f                 /* rust/src/centrality.rs:28 */
#define ANGULAR_ROUTE_TIE_BREAK_FACTOR 1e-6f /* rust/src/centrality.rs:24 */
#define F32_EPSILON 1.1920929e-07f

/* ------------------------------------------------------------------------------------------ */
/* Graph (rust/src/graph.rs:24-122, 381-391).                                                  */
/* ------------------------------------------------------------------------------------------ */
typedef struct {
    int32_t n_bound;          /* node slots (StableGraph node_bound) */
    int32_t n_edges;          /* edge slots in insertion order (edge_bound) */
    const uint8_t *node_exists;
    const uint8_t *live;
    const float *weight;
    const uint8_t *has_z;
    const double *z;
    const int32_t *e_src;
    const int32_t *e_dst;
    const uint8_t *e_exists;
    const int64_t *e_idx;     /* EdgePayload.edge_idx */
    const float *e_len;       /* EdgePayload.length */
    const float *e_ang;       /* EdgePayload.angle_sum */
    const float *e_imp;       /* EdgePayload.imp_factor */
    const float *e_sec;       /* EdgePayload.seconds (NaN for street edges) */
    const int32_t *e_shared;  /* shared_primal_node_key as an interned id, -1 = None */
    int32_t is_dual;
} og_graph_desc;

typedef struct {
    og_graph_desc d;
    int32_t *out_head, *out_next; /* petgraph outgoing list: newest edge first */
    int32_t *in_head, *in_next;   /* petgraph incoming list: newest edge first */
    int32_t *node_list;           /* node_indices(): ascending existing indices */
    int32_t n_nodes;
    int32_t *slots;               /* dual endpoint slots [n_bound][2] (-1 empty) */
    int32_t slots_ok;             /* 1 when every dual node has <= 2 distinct keys */
} og_graph;

og_graph *og_graph_new(const og_graph_desc *d) {
    og_graph *g = (og_graph *)calloc(1, sizeof(og_graph));
    g->d = *d;
    int32_t n = d->n_bound, m = d->n_edges;
    g->out_head = (int32_t *)malloc(sizeof(int32_t) * (n > 0 ? n : 1));
    g->in_head = (int32_t *)malloc(sizeof(int32_t) * (n > 0 ? n : 1));
    g->out_next = (int32_t *)malloc(sizeof(int32_t) * (m > 0 ? m : 1));
    g->in_next = (int32_t *)malloc(sizeof(int32_t) * (m > 0 ? m : 1));
    for (int32_t i = 0; i < n; i++) g->out_head[i] = g->in_head[i] = -1;
    /* petgraph add_edge prepends the new edge to both endpoint lists. */
    for (int32_t e = 0; e < m; e++) {
        g->out_next[e] = g->in_next[e] = -1;
        if (!d->e_exists[e]) continue;
        int32_t s = d->e_src[e], t = d->e_dst[e];
        g->out_next[e] = g->out_head[s];
        g->out_head[s] = e;
        g->in_next[e] = g->in_head[t];
        g->in_head[t] = e;
    }
    g->node_list = (int32_t *)malloc(sizeof(int32_t) * (n > 0 ? n : 1));
    g->n_nodes = 0;
    for (int32_t i = 0; i < n; i++)
        if (d->node_exists[i]) g->node_list[g->n_nodes++] = i;
    /* dual_node_endpoint_slots (rust/src/centrality.rs:533-566): edge_references() order. */
    g->slots = (int32_t *)malloc(sizeof(int32_t) * 2 * (n > 0 ? n : 1));
    for (int32_t i = 0; i < 2 * n; i++) g->slots[i] = -1;
    g->slots_ok = 1;
    for (int32_t e = 0; e < m; e++) {
        if (!d->e_exists[e]) continue;
        int32_t key = d->e_shared ? d->e_shared[e] : -1;
        if (key < 0) { g->slots_ok = 0; continue; }
        int32_t ends[2] = {d->e_src[e], d->e_dst[e]};
        for (int k = 0; k < 2; k++) {
            int32_t *sl = &g->slots[2 * ends[k]];
            if (sl[0] == key || sl[1] == key) continue;
            if (sl[0] < 0) sl[0] = key;
            else if (sl[1] < 0) sl[1] = key;
            else g->slots_ok = 0;
        }
    }
    return g;
}

void og_graph_free(og_graph *g) {
    if (!g) return;
    free(g->out_head); free(g->in_head); free(g->out_next); free(g->in_next);
    free(g->node_list); free(g->slots); free(g);
}

int32_t og_slots_ok(const og_graph *g) { return g->slots_ok; }

/* ------------------------------------------------------------------------------------------ */
/* Rust std BinaryHeap<NodeDistance> with reversed total_cmp (rust/src/centrality.rs:357-386). */
/* ------------------------------------------------------------------------------------------ */
typedef struct { int64_t idx; float metric; } hent;
typedef struct { hent *a; int64_t len, cap; } heap_t;

static inline int32_t tkey(float f) {
    int32_t i;
    memcpy(&i, &f, 4);
    return i ^ (int32_t)(((uint32_t)(i >> 31)) >> 1);
}
/* Ord for NodeDistance: other.metric.total_cmp(&self.metric). Returns -1/0/1. */
static inline int hcmp(hent x, hent y) {
    int32_t kx = tkey(x.metric), ky = tkey(y.metric);
    return (ky > kx) - (ky < kx);
}
static void hp_sift_up(heap_t *h, int64_t start, int64_t pos) {
    hent elem = h->a[pos];
    while (pos > start) {
        int64_t parent = (pos - 1) / 2;
        if (hcmp(elem, h->a[parent]) <= 0) break;
        h->a[pos] = h->a[parent];
        pos = parent;
    }
    h->a[pos] = elem;
}
static void hp_push(heap_t *h, int64_t idx, float metric) {
    if (h->len == h->cap) {
        h->cap = h->cap ? h->cap * 2 : 64;
        h->a = (hent *)realloc(h->a, sizeof(hent) * h->cap);
    }
    h->a[h->len].idx = idx;
    h->a[h->len].metric = metric;
    h->len++;
    hp_sift_up(h, 0, h->len - 1);
}
static void hp_sift_down_to_bottom(heap_t *h, int64_t pos) {
    int64_t end = h->len, start = pos;
    hent elem = h->a[pos];
    int64_t child = 2 * pos + 1;
    int64_t lim = end >= 2 ? end - 2 : 0;
    while (child <= lim && end >= 2) {
        child += (hcmp(h->a[child], h->a[child + 1]) <= 0);
        h->a[pos] = h->a[child];
        pos = child;
        child = 2 * pos + 1;
    }
    if (child == end - 1) {
        h->a[pos] = h->a[child];
        pos = child;
    }
    h->a[pos] = elem;
    hp_sift_up(h, start, pos);
}
static int hp_pop(heap_t *h, hent *out) {
    if (h->len == 0) return 0;
    hent item = h->a[--h->len];
    if (h->len > 0) {
        hent t = h->a[0];
        h->a[0] = item;
        item = t;
        hp_sift_down_to_bottom(h, 0);
    }
    *out = item;
    return 1;
}

/* ------------------------------------------------------------------------------------------ */
/* Edge travel time (rust/src/centrality.rs:961-1007).                                         */
/* ------------------------------------------------------------------------------------------ */
static inline float slope_penalty(const og_graph *g, int32_t from, int32_t to, float length_2d) {
    if (length_2d <= 0.0f) return 1.0f;
    if (g->d.has_z && g->d.has_z[from] && g->d.has_z[to]) {
        float slope = (float)(g->d.z[to] - g->d.z[from]) / length_2d;
        const float FLAT_FACTOR = 0.839457f;
        float slope_factor = expf(-3.5f * fabsf(slope + 0.05f));
        return FLAT_FACTOR / slope_factor;
    }
    return 1.0f;
}
static inline float edge_travel_seconds(const og_graph *g, int32_t from, int32_t to, int32_t e,
                                        float speed, int use_imp) {
    if (!isnan(g->d.e_sec[e])) return g->d.e_sec[e];
    float len = g->d.e_len[e];
    float slope_pen = slope_penalty(g, from, to, len);
    float imp = use_imp ? g->d.e_imp[e] : 1.0f;
    return (len * imp * slope_pen) / speed;
}

float og_edge_travel_seconds(const og_graph *g, int32_t e, float speed, int32_t use_imp) {
    return edge_travel_seconds(g, g->d.e_src[e], g->d.e_dst[e], e, speed, use_imp);
}

/* ------------------------------------------------------------------------------------------ */
/* Thresholds (rust/src/common.rs:10-12, 99-270).                                              */
/* ------------------------------------------------------------------------------------------ */
#define MIN_THRESH_WT 0.01831563888873418f
#define OG_ERR_ARG (-1)

/* betas_from_distances (common.rs:134-165). Returns 0 or OG_ERR_ARG. */
int og_betas_from_distances(const uint32_t *dist, int32_t k, float mtw, int32_t has_mtw, float *betas) {
    if (k <= 0) return OG_ERR_ARG;
    float m = has_mtw ? mtw : MIN_THRESH_WT;
    for (int i = 1; i < k; i++) if (dist[i] <= dist[i - 1]) return OG_ERR_ARG;
    for (int i = 0; i < k; i++) {
        if (dist[i] == 0) return OG_ERR_ARG;
        float beta = -logf(m) / (float)dist[i];
        betas[i] = roundf(beta * 100000.0f) / 100000.0f;
    }
    return 0;
}
/* distances_from_betas (common.rs:99-131) */
int og_distances_from_betas(const float *betas, int32_t k, float mtw, int32_t has_mtw, uint32_t *dist) {
    if (k <= 0) return OG_ERR_ARG;
    float m = has_mtw ? mtw : MIN_THRESH_WT;
    for (int i = 1; i < k; i++) if (betas[i] >= betas[i - 1]) return OG_ERR_ARG;
    for (int i = 0; i < k; i++) {
        if (betas[i] <= 0.0f) return OG_ERR_ARG;
        float d = roundf(logf(m) / -betas[i]);
        if (d <= 0.0f) return OG_ERR_ARG;
        dist[i] = (uint32_t)d;
    }
    return 0;
}
/* seconds_from_distances (common.rs:203-237) */
int og_seconds_from_distances(const uint32_t *dist, int32_t k, float speed, uint32_t *secs) {
    if (k <= 0 || speed <= 0.0f) return OG_ERR_ARG;
    for (int i = 1; i < k; i++) if (dist[i] <= dist[i - 1]) return OG_ERR_ARG;
    for (int i = 0; i < k; i++) {
        if (dist[i] == 0) return OG_ERR_ARG;
        float t = roundf((float)dist[i] / speed);
        if (t <= 0.0f) return OG_ERR_ARG;
        secs[i] = (uint32_t)t;
    }
    return 0;
}
/* distances_from_seconds (common.rs:167-201) */
int og_distances_from_seconds(const uint32_t *secs, int32_t k, float speed, uint32_t *dist) {
    if (k <= 0 || speed <= 0.0f) return OG_ERR_ARG;
    for (int i = 1; i < k; i++) if (secs[i] <= secs[i - 1]) return OG_ERR_ARG;
    for (int i = 0; i < k; i++) {
        if (secs[i] == 0) return OG_ERR_ARG;
        float d = roundf((float)secs[i] * speed);
        if (d <= 0.0f) return OG_ERR_ARG;
        dist[i] = (uint32_t)d;
    }
    return 0;
}
/* minutes -> seconds step of pair_distances_betas_time (common.rs:260-265) */
void og_seconds_from_minutes(const float *minutes, int32_t k, uint32_t *secs) {
    for (int i = 0; i < k; i++) {
        float s = roundf(minutes[i] * 60.0f);
        secs[i] = s <= 0.0f ? 0u : (s >= 4294967295.0f ? 4294967295u : (uint32_t)s);
    }
}

/* ------------------------------------------------------------------------------------------ */
/* Atomic f64 (atomic_float::AtomicF64::fetch_add: CAS loop).                                  */
/* ------------------------------------------------------------------------------------------ */
static inline void add_f64_atomic(double *p, double v) {
    uint64_t *up = (uint64_t *)p;
    uint64_t old = __atomic_load_n(up, __ATOMIC_RELAXED), nw;
    do {
        double o, n;
        memcpy(&o, &old, 8);
        n = o + v;
        memcpy(&nw, &n, 8);
    } while (!__atomic_compare_exchange_n(up, &old, nw, 1, __ATOMIC_RELAXED, __ATOMIC_RELAXED));
}

/* ------------------------------------------------------------------------------------------ */
/* Brandes traversal (rust/src/centrality.rs:388-424, 1344-1494, 577-775).                     */
/* ------------------------------------------------------------------------------------------ */
typedef struct {
    uint8_t visited;
    int32_t npred, cap;
    int64_t *preds;    /* SmallVec<[usize; 2]> */
    int64_t inl[2];
    double sigma;
    int64_t node_idx;
    float route_cost;
    float agg_seconds;
} bstate;

typedef struct {
    int64_t *visited;  int64_t n_visited;   /* visited_state_indices */
    int64_t *reached;  int64_t n_reached;   /* reached_node_indices */
    bstate *state;     int64_t n_state;
    float *best_route_cost;
    float *best_agg_seconds;
} btrav;

static inline void st_init(bstate *s, int64_t node_idx) {
    s->visited = 0; s->npred = 0; s->cap = 2; s->preds = s->inl;
    s->sigma = 0.0; s->node_idx = node_idx;
    s->route_cost = INFINITY; s->agg_seconds = INFINITY;
}
static inline void st_push(bstate *s, int64_t p) {
    if (s->npred == s->cap) {
        int32_t nc = s->cap * 2;
        int64_t *np = (int64_t *)malloc(sizeof(int64_t) * nc);
        memcpy(np, s->preds, sizeof(int64_t) * s->npred);
        if (s->preds != s->inl) free(s->preds);
        s->preds = np; s->cap = nc;
    }
    s->preds[s->npred++] = p;
}
static inline int st_contains(const bstate *s, int64_t p) {
    for (int32_t i = 0; i < s->npred; i++) if (s->preds[i] == p) return 1;
    return 0;
}
static inline void st_clear(bstate *s) { s->npred = 0; }

static void btrav_free(btrav *t) {
    for (int64_t i = 0; i < t->n_state; i++)
        if (t->state[i].preds != t->state[i].inl) free(t->state[i].preds);
    free(t->state); free(t->visited); free(t->reached);
    free(t->best_route_cost); free(t->best_agg_seconds);
}

/* reached_node_indices (centrality.rs:459-466) */
static void fill_reached(btrav *t, int64_t n) {
    t->reached = (int64_t *)malloc(sizeof(int64_t) * (n > 0 ? n : 1));
    t->n_reached = 0;
    for (int64_t i = 0; i < n; i++)
        if (isfinite(t->best_route_cost[i])) t->reached[t->n_reached++] = i;
}

static void push_visited(btrav *t, int64_t *cap, int64_t idx) {
    if (t->n_visited == *cap) {
        *cap = *cap ? *cap * 2 : 256;
        t->visited = (int64_t *)realloc(t->visited, sizeof(int64_t) * *cap);
    }
    t->visited[t->n_visited++] = idx;
}

/* dijkstra_brandes_shortest (centrality.rs:1344-1494) */
static void dijkstra_brandes_shortest(const og_graph *g, int64_t src, uint32_t max_seconds, float speed,
                                      float tolerance, btrav *t) {
    int64_t n = g->d.n_bound;
    memset(t, 0, sizeof(*t));
    t->n_state = n;
    t->state = (bstate *)malloc(sizeof(bstate) * (n > 0 ? n : 1));
    for (int64_t i = 0; i < n; i++) st_init(&t->state[i], i);
    t->best_route_cost = (float *)malloc(sizeof(float) * (n > 0 ? n : 1));
    t->best_agg_seconds = (float *)malloc(sizeof(float) * (n > 0 ? n : 1));
    for (int64_t i = 0; i < n; i++) t->best_route_cost[i] = t->best_agg_seconds[i] = INFINITY;
    int64_t vcap = 0;
    bstate *S = t->state;
    S[src].sigma = 1.0; S[src].route_cost = 0.0f; S[src].agg_seconds = 0.0f;
    t->best_route_cost[src] = 0.0f; t->best_agg_seconds[src] = 0.0f;
    heap_t h = {0};
    hp_push(&h, src, 0.0f);
    hent it;
    const float maxs = (float)max_seconds;
    while (hp_pop(&h, &it)) {
        int64_t si = it.idx;
        if (S[si].visited) continue;
        S[si].visited = 1;
        push_visited(t, &vcap, si);
        int64_t cur = S[si].node_idx;
        for (int32_t e = g->in_head[cur]; e >= 0; e = g->in_next[e]) {
            int64_t nb = g->d.e_src[e];
            if (nb == cur) continue;
            float es = edge_travel_seconds(g, (int32_t)nb, (int32_t)cur, e, speed, 1);
            float cand = S[si].agg_seconds + es;
            if (cand > maxs) continue;
            if (S[nb].visited) continue;
            float cand_route = cand * speed;
            int improved = cand < S[nb].agg_seconds;
            int tied = cand <= S[nb].agg_seconds * (1.0f + TIE_EPSILON);
            if (improved) {
                if (cand < S[nb].agg_seconds * (1.0f - TIE_EPSILON)) {
                    st_clear(&S[nb]);
                    S[nb].sigma = S[si].sigma;
                } else {
                    S[nb].sigma += S[si].sigma;
                }
                S[nb].route_cost = cand_route;
                S[nb].agg_seconds = cand;
                st_push(&S[nb], si);
                hp_push(&h, nb, cand_route);
            } else if (tied && !st_contains(&S[nb], si)) {
                if (cand < S[nb].agg_seconds) S[nb].agg_seconds = cand;
                st_push(&S[nb], si);
                S[nb].sigma += S[si].sigma;
            }
            t->best_route_cost[nb] = S[nb].route_cost;
            t->best_agg_seconds[nb] = S[nb].agg_seconds;
        }
    }
    free(h.a);
    /* Phase 2 (centrality.rs:1444-1483) */
    if (tolerance > TIE_EPSILON) {
        int64_t *visit_pos = (int64_t *)malloc(sizeof(int64_t) * (n > 0 ? n : 1));
        for (int64_t i = 0; i < n; i++) visit_pos[i] = INT64_MAX;
        for (int64_t p = 0; p < t->n_visited; p++) visit_pos[t->visited[p]] = p;
        for (int64_t p = 0; p < t->n_visited; p++) {
            st_clear(&S[t->visited[p]]);
            S[t->visited[p]].sigma = 0.0;
        }
        S[src].sigma = 1.0;
        for (int64_t pos = 0; pos < t->n_visited; pos++) {
            int64_t u = t->visited[pos];
            int64_t un = S[u].node_idx;
            for (int32_t e = g->in_head[un]; e >= 0; e = g->in_next[e]) {
                int64_t v = g->d.e_src[e];
                if (v == u) continue;
                if (visit_pos[v] <= pos) continue;
                float es = edge_travel_seconds(g, (int32_t)v, (int32_t)un, e, speed, 1);
                float ps = S[u].agg_seconds + es;
                if (ps <= S[v].agg_seconds * (1.0f + tolerance) && !st_contains(&S[v], u)) {
                    st_push(&S[v], u);
                    S[v].sigma += S[u].sigma;
                }
            }
        }
        free(visit_pos);
    }
    fill_reached(t, n);
}

static inline int64_t ang_state_idx(int64_t node, int64_t slot) { return node * 2 + slot; }
static inline int slot_pos(const og_graph *g, int64_t node, int32_t key) {
    const int32_t *sl = &g->slots[2 * node];
    if (sl[0] == key) return 0;
    if (sl[1] == key) return 1;
    return -1;
}

/* dijkstra_brandes_angular (centrality.rs:577-775) */
static void dijkstra_brandes_angular(const og_graph *g, int64_t src, uint32_t max_seconds, float speed,
                                     float tolerance, btrav *t) {
    int64_t n = g->d.n_bound, ns = n * 2;
    memset(t, 0, sizeof(*t));
    t->n_state = ns;
    t->state = (bstate *)malloc(sizeof(bstate) * (ns > 0 ? ns : 1));
    for (int64_t i = 0; i < ns; i++) st_init(&t->state[i], i / 2);
    t->best_route_cost = (float *)malloc(sizeof(float) * (n > 0 ? n : 1));
    t->best_agg_seconds = (float *)malloc(sizeof(float) * (n > 0 ? n : 1));
    for (int64_t i = 0; i < n; i++) t->best_route_cost[i] = t->best_agg_seconds[i] = INFINITY;
    int64_t vcap = 0;
    bstate *S = t->state;
    heap_t h = {0};
    t->best_route_cost[src] = 0.0f; t->best_agg_seconds[src] = 0.0f;
    for (int slot = 0; slot < 2; slot++) {
        int64_t s = ang_state_idx(src, slot);
        S[s].sigma = 1.0; S[s].route_cost = 0.0f; S[s].agg_seconds = 0.0f;
        hp_push(&h, s, 0.0f);
    }
    const float maxs = (float)max_seconds;
    hent it;
    while (hp_pop(&h, &it)) {
        int64_t si = it.idx;
        if (S[si].visited) continue;
        S[si].visited = 1;
        push_visited(t, &vcap, si);
        int64_t cur = S[si].node_idx;
        int64_t entry = si % 2;
        for (int32_t e = g->out_head[cur]; e >= 0; e = g->out_next[e]) {
            int64_t nx = g->d.e_dst[e];
            int32_t key = g->d.e_shared[e];
            int cs = slot_pos(g, cur, key);
            if (cs != 1 - entry) continue;
            int ns2 = slot_pos(g, nx, key);
            int64_t nsi = ang_state_idx(nx, ns2);
            float es = edge_travel_seconds(g, (int32_t)cur, (int32_t)nx, e, speed, 0);
            float cand_s = S[si].agg_seconds + es;
            if (cand_s > maxs) continue;
            if (S[nsi].visited) continue;
            float cand_r = S[si].route_cost + g->d.e_ang[e] + (ANGULAR_ROUTE_TIE_BREAK_FACTOR * g->d.e_len[e]);
            float cur_cost = S[nsi].route_cost;
            int improved = cand_r < cur_cost;
            int tied = cand_r <= cur_cost * (1.0f + TIE_EPSILON);
            if (improved) {
                if (cand_r < cur_cost * (1.0f - TIE_EPSILON)) {
                    st_clear(&S[nsi]);
                    S[nsi].sigma = S[si].sigma;
                } else {
                    S[nsi].sigma += S[si].sigma;
                }
                S[nsi].route_cost = cand_r;
                S[nsi].agg_seconds = cand_s;
                st_push(&S[nsi], si);
                hp_push(&h, nsi, cand_r);
            } else if (tied && !st_contains(&S[nsi], si)) {
                if (cand_s < S[nsi].agg_seconds) S[nsi].agg_seconds = cand_s;
                st_push(&S[nsi], si);
                S[nsi].sigma += S[si].sigma;
            }
            int64_t nn = S[nsi].node_idx;
            float best = t->best_route_cost[nn];
            if (cand_r < best * (1.0f - TIE_EPSILON)) {
                t->best_route_cost[nn] = cand_r;
                t->best_agg_seconds[nn] = cand_s;
            } else if (cand_r <= best * (1.0f + TIE_EPSILON)) {
                t->best_agg_seconds[nn] = fminf(t->best_agg_seconds[nn], cand_s);
            }
        }
    }
    free(h.a);
    if (tolerance > TIE_EPSILON) {
        int64_t *visit_pos = (int64_t *)malloc(sizeof(int64_t) * (ns > 0 ? ns : 1));
        for (int64_t i = 0; i < ns; i++) visit_pos[i] = INT64_MAX;
        for (int64_t p = 0; p < t->n_visited; p++) visit_pos[t->visited[p]] = p;
        for (int64_t p = 0; p < t->n_visited; p++) {
            st_clear(&S[t->visited[p]]);
            S[t->visited[p]].sigma = 0.0;
        }
        for (int slot = 0; slot < 2; slot++) S[ang_state_idx(src, slot)].sigma = 1.0;
        for (int64_t pos = 0; pos < t->n_visited; pos++) {
            int64_t u = t->visited[pos];
            int64_t un = S[u].node_idx;
            int64_t entry = u % 2;
            for (int32_t e = g->out_head[un]; e >= 0; e = g->out_next[e]) {
                int64_t nx = g->d.e_dst[e];
                int32_t key = g->d.e_shared[e];
                if (slot_pos(g, un, key) != 1 - entry) continue;
                int64_t v = ang_state_idx(nx, slot_pos(g, nx, key));
                if (visit_pos[v] <= pos) continue;
                float cand_r = S[u].route_cost + g->d.e_ang[e] + (ANGULAR_ROUTE_TIE_BREAK_FACTOR * g->d.e_len[e]);
                if (cand_r <= S[v].route_cost * (1.0f + tolerance) && !st_contains(&S[v], u)) {
                    st_push(&S[v], u);
                    S[v].sigma += S[u].sigma;
                }
            }
        }
        free(visit_pos);
    }
    fill_reached(t, n);
}

/* sorted_brandes_state_indices (centrality.rs:777-791): stable sort, descending route_cost. */
static void merge_sort_desc(int64_t *a, int64_t *tmp, int64_t n, const bstate *S) {
    for (int64_t w = 1; w < n; w *= 2) {
        for (int64_t lo = 0; lo < n; lo += 2 * w) {
            int64_t mid = lo + w < n ? lo + w : n, hi = lo + 2 * w < n ? lo + 2 * w : n;
            int64_t i = lo, j = mid, k = lo;
            while (i < mid && j < hi) {
                /* take right only if strictly "less" under the comparator (b.rc cmp a.rc) */
                float ra = S[a[i]].route_cost, rb = S[a[j]].route_cost;
                if (ra < rb) tmp[k++] = a[j++]; /* rb greater -> comes first */
                else tmp[k++] = a[i++];
            }
            while (i < mid) tmp[k++] = a[i++];
            while (j < hi) tmp[k++] = a[j++];
        }
        memcpy(a, tmp, sizeof(int64_t) * n);
    }
}
static int64_t sorted_state_indices(const btrav *t, int64_t **out) {
    int64_t *a = (int64_t *)malloc(sizeof(int64_t) * (t->n_visited > 0 ? t->n_visited : 1));
    int64_t n = 0;
    for (int64_t i = 0; i < t->n_visited; i++)
        if (t->state[t->visited[i]].sigma > 0.0) a[n++] = t->visited[i];
    int64_t *tmp = (int64_t *)malloc(sizeof(int64_t) * (n > 0 ? n : 1));
    merge_sort_desc(a, tmp, n, t->state);
    free(tmp);
    *out = a;
    return n;
}

/* best_angular_target_states (centrality.rs:793-821) */
static int best_angular_target_states(const btrav *t, int64_t node, float sec_thr, float tol, int64_t *out) {
    int cnt = 0;
    float brc = t->best_route_cost[node], bas = t->best_agg_seconds[node];
    if (!isfinite(brc) || !isfinite(bas) || bas > sec_thr) return 0;
    for (int slot = 0; slot < 2; slot++) {
        int64_t si = ang_state_idx(node, slot);
        const bstate *s = &t->state[si];
        if (s->sigma == 0.0 || s->agg_seconds > sec_thr) continue;
        if (s->route_cost <= brc * (1.0f + tol)) out[cnt++] = si;
    }
    return cnt;
}

/* brandes_backprop_with_beta (centrality.rs:823-873); include mode 0 = route_cost <= thr,
   1 = agg_seconds <= thr.  Credits go straight to the output rows. */
static void brandes_backprop(const btrav *t, const int64_t *sorted, int64_t ns, int64_t src,
                             const double *seed, const double *seed_b, int include_mode, float thr,
                             double *out_b, double *out_bb, double wt, int atomic) {
    double *delta = (double *)calloc(t->n_state > 0 ? t->n_state : 1, sizeof(double));
    double *delta_b = (double *)calloc(t->n_state > 0 ? t->n_state : 1, sizeof(double));
    for (int64_t q = 0; q < ns; q++) {
        int64_t si = sorted[q];
        const bstate *s = &t->state[si];
        int inc = include_mode == 0 ? (s->route_cost <= thr) : (s->agg_seconds <= thr);
        if (!inc) continue;
        double sw = s->sigma;
        if (sw == 0.0) continue;
        double dep = seed[si] + delta[si];
        double dep_b = seed_b[si] + delta_b[si];
        if (dep == 0.0 && dep_b == 0.0) continue;
        for (int32_t p = 0; p < s->npred; p++) {
            int64_t pi = s->preds[p];
            double sv = t->state[pi].sigma;
            if (sv == 0.0) continue;
            double f = sv / sw;
            delta[pi] += f * dep;
            delta_b[pi] += f * dep_b;
        }
        if (s->node_idx == src) continue;
        double credit = dep - seed[si];
        double credit_b = dep_b - seed_b[si];
        if (credit > 0.0 || credit_b > 0.0) {
            double c = credit > 0.0 ? credit : 0.0, cb = credit_b > 0.0 ? credit_b : 0.0;
            int64_t v = s->node_idx;
            if (c > 0.0) {
                if (atomic) add_f64_atomic(&out_b[v], c * wt); else out_b[v] += c * wt;
            }
            if (cb > 0.0 && out_bb) {
                if (atomic) add_f64_atomic(&out_bb[v], cb * wt); else out_bb[v] += cb * wt;
            }
        }
    }
    free(delta); free(delta_b);
}

/* circuit_ranks_from_traversal (centrality.rs:470-526): HashSet of (min,max,edge_idx). */
typedef struct { int64_t a, b, c; uint8_t used; } hkey;
static uint64_t hmix(int64_t a, int64_t b, int64_t c) {
    uint64_t h = (uint64_t)a * 0x9E3779B97F4A7C15ull ^ ((uint64_t)b + 0x632BE59BD9B4E019ull) * 0xBF58476D1CE4E5B9ull;
    h ^= ((uint64_t)c + 0x94D049BB133111EBull) * 0x2545F4914F6CDD1Dull;
    h ^= h >> 31;
    return h;
}
static void circuit_ranks(const og_graph *g, const btrav *t, const uint32_t *dist, int k, float *rank) {
    int64_t node_counts[64] = {0}, edge_counts[64] = {0};
    for (int64_t r = 0; r < t->n_reached; r++) {
        float c = t->best_route_cost[t->reached[r]];
        for (int i = 0; i < k; i++) if (c <= (float)dist[i]) node_counts[i]++;
    }
    int64_t cap = 64;
    while (cap < 4 * (t->n_reached * 4 + 16)) cap *= 2;
    hkey *tab = (hkey *)calloc(cap, sizeof(hkey));
    for (int64_t r = 0; r < t->n_reached; r++) {
        int64_t u = t->reached[r];
        for (int32_t e = g->out_head[u]; e >= 0; e = g->out_next[e]) {
            int64_t v = g->d.e_dst[e];
            if (v == u) continue;
            if (!isfinite(t->best_route_cost[v])) continue;
            int64_t a = u < v ? u : v, b = u < v ? v : u, c = g->d.e_idx[e];
            uint64_t hh = hmix(a, b, c) & (uint64_t)(cap - 1);
            int fresh = 1;
            while (tab[hh].used) {
                if (tab[hh].a == a && tab[hh].b == b && tab[hh].c == c) { fresh = 0; break; }
                hh = (hh + 1) & (uint64_t)(cap - 1);
            }
            if (!fresh) continue;
            tab[hh].used = 1; tab[hh].a = a; tab[hh].b = b; tab[hh].c = c;
            float ec = fmaxf(t->best_route_cost[u], t->best_route_cost[v]);
            for (int i = 0; i < k; i++) if (ec <= (float)dist[i]) edge_counts[i]++;
        }
    }
    free(tab);
    for (int i = 0; i < k; i++) {
        if (node_counts[i] == 0) rank[i] = 0.0f;
        else {
            int64_t r = edge_counts[i] - node_counts[i] + 1;
            rank[i] = (float)(r > 0 ? r : 0);
        }
    }
}

/* ------------------------------------------------------------------------------------------ */
/* Source plan (centrality.rs:1032-1139): resolved on the host, passed in as arrays.           */
/* ------------------------------------------------------------------------------------------ */
typedef struct {
    int32_t k;
    const uint32_t *distances;
    const float *betas;
    const uint32_t *seconds;
    int32_t compute_closeness, compute_betweenness;
    float speed;
    float tolerance;           /* validated decimal tolerance (>= TIE_EPSILON) */
    float angular_scaling_unit, farness_scaling_offset;
    int64_t n_sources;
    const int64_t *sources;    /* processing list (source_indices or node_indices) */
    const uint8_t *eligible;   /* source_eligible[node_bound] */
    const float *src_wt;       /* per-node source weight after sampling (sample_source_weight) */
    const uint8_t *src_take;   /* per-node: 1 if sample_source_weight returned Some */
    int32_t track_reach;       /* sampling or source-indexed */
    int32_t nthreads;
    /* betweenness_od_shortest: per origin node o, destinations od_dst[od_ptr[o] .. od_ptr[o+1]) with
       trip weights od_w (OdMatrix, centrality.rs:56-91, one entry per pair) */
    const int64_t *od_ptr;
    const int64_t *od_dst;
    const float *od_w;
} og_args;

typedef struct {
    const og_graph *g;
    const og_args *a;
    double *out;               /* [M][K][n_bound] */
    uint32_t *reach;           /* [K] */
    int64_t next;              /* work counter */
    int mode;                  /* 0 shortest, 1 simplest, 2 segment */
    int atomic;
} job_t;

static void run_shortest_source(job_t *J, int64_t src) {
    const og_graph *g = J->g;
    const og_args *a = J->a;
    int64_t n = g->d.n_bound;
    int k = a->k;
    if (!a->eligible[src]) return;
    if (!a->src_take[src]) return;
    float wt = a->src_wt[src];
    uint32_t maxs = 0;
    for (int i = 0; i < k; i++) if (a->seconds[i] > maxs) maxs = a->seconds[i];
    btrav t;
    dijkstra_brandes_shortest(g, src, maxs, a->speed, a->tolerance, &t);
    float cycles_wt = wt / g->d.weight[src];
    double *O = J->out;
#define ROW(m, i) (O + ((int64_t)(m) * k + (i)) * n)
    if (a->compute_closeness) {
        float rank[64];
        circuit_ranks(g, &t, a->distances, k, rank);
        for (int64_t r = 0; r < t.n_reached; r++) {
            int64_t to = t.reached[r];
            if (to == src) continue;
            if (!isfinite(t.best_agg_seconds[to])) continue;
            float c = t.best_route_cost[to];
            if (a->track_reach)
                for (int i = 0; i < k; i++)
                    if (c <= (float)a->distances[i]) __atomic_fetch_add(&J->reach[i], 1u, __ATOMIC_RELAXED);
            for (int i = 0; i < k; i++) {
                float beta = a->betas[i];
                if (c <= (float)a->distances[i]) {
                    double v0 = (double)wt, v1 = (double)(c * wt), v2 = (double)(rank[i] * cycles_wt);
                    double v3 = (double)((1.0f / c) * wt), v4 = (double)(expf(-beta * c) * wt);
                    if (J->atomic) {
                        add_f64_atomic(&ROW(0, i)[to], v0); add_f64_atomic(&ROW(1, i)[to], v1);
                        add_f64_atomic(&ROW(2, i)[to], v2); add_f64_atomic(&ROW(3, i)[to], v3);
                        add_f64_atomic(&ROW(4, i)[to], v4);
                    } else {
                        ROW(0, i)[to] += v0; ROW(1, i)[to] += v1; ROW(2, i)[to] += v2;
                        ROW(3, i)[to] += v3; ROW(4, i)[to] += v4;
                    }
                }
            }
        }
    }
    if (a->compute_betweenness) {
        int64_t *sorted;
        int64_t ns = sorted_state_indices(&t, &sorted);
        double *seed = (double *)calloc(t.n_state > 0 ? t.n_state : 1, sizeof(double));
        double *seed_b = (double *)calloc(t.n_state > 0 ? t.n_state : 1, sizeof(double));
        for (int i = 0; i < k; i++) {
            float thr = (float)a->distances[i];
            double beta = (double)a->betas[i];
            memset(seed, 0, sizeof(double) * t.n_state);
            memset(seed_b, 0, sizeof(double) * t.n_state);
            for (int64_t r = 0; r < t.n_reached; r++) {
                int64_t to = t.reached[r];
                if (to == src) continue;
                if (t.best_route_cost[to] > thr) continue;
                double pc = a->eligible[to] ? 0.5 : 1.0;
                double pb = pc * exp(-beta * (double)t.best_route_cost[to]);
                seed[to] += pc;
                seed_b[to] += pb;
            }
            brandes_backprop(&t, sorted, ns, src, seed, seed_b, 0, thr, ROW(5, i), ROW(6, i), (double)wt, J->atomic);
        }
        free(seed); free(seed_b); free(sorted);
    }
#undef ROW
    btrav_free(&t);
}

/* betweenness_od_shortest, one source (centrality.rs:2471-2533): live origins with a row only;
   out: [2][K][n_bound] (betweenness, betweenness_beta), source weight 1. */
static void run_od_source(job_t *J, int64_t src) {
    const og_graph *g = J->g;
    const og_args *a = J->a;
    int64_t n = g->d.n_bound;
    int k = a->k;
    if (!g->d.live[src]) return;
    int64_t r0 = a->od_ptr[src], r1 = a->od_ptr[src + 1];
    if (r1 <= r0) return;
    uint32_t maxs = 0;
    for (int i = 0; i < k; i++) if (a->seconds[i] > maxs) maxs = a->seconds[i];
    btrav t;
    dijkstra_brandes_shortest(g, src, maxs, a->speed, a->tolerance, &t);
    int64_t *sorted;
    int64_t ns = sorted_state_indices(&t, &sorted);
    double *seed = (double *)calloc(t.n_state > 0 ? t.n_state : 1, sizeof(double));
    double *seed_b = (double *)calloc(t.n_state > 0 ? t.n_state : 1, sizeof(double));
    for (int i = 0; i < k; i++) {
        float thr = (float)a->distances[i];
        double beta = (double)a->betas[i];
        memset(seed, 0, sizeof(double) * t.n_state);
        memset(seed_b, 0, sizeof(double) * t.n_state);
        for (int64_t r = r0; r < r1; r++) {
            int64_t dest = a->od_dst[r];
            if (t.best_route_cost[dest] > thr) continue;
            double w = (double)a->od_w[r];
            seed[dest] += w;
            seed_b[dest] += w * exp(-beta * (double)t.best_route_cost[dest]);
        }
        brandes_backprop(&t, sorted, ns, src, seed, seed_b, 0, thr, J->out + (int64_t)i * n,
                         J->out + ((int64_t)k + i) * n, 1.0, J->atomic);
    }
    free(seed); free(seed_b); free(sorted);
    btrav_free(&t);
}

static void run_simplest_source(job_t *J, int64_t src) {
    const og_graph *g = J->g;
    const og_args *a = J->a;
    int64_t n = g->d.n_bound;
    int k = a->k;
    if (!a->eligible[src]) return;
    if (!a->src_take[src]) return;
    float wt = a->src_wt[src];
    uint32_t maxs = 0;
    for (int i = 0; i < k; i++) if (a->seconds[i] > maxs) maxs = a->seconds[i];
    btrav t;
    dijkstra_brandes_angular(g, src, maxs, a->speed, a->tolerance, &t);
    double *O = J->out;
#define ROW(m, i) (O + ((int64_t)(m) * k + (i)) * n)
    if (a->compute_closeness) {
        for (int64_t r = 0; r < t.n_reached; r++) {
            int64_t to = t.reached[r];
            if (to == src) continue;
            float bsd = t.best_route_cost[to], bas = t.best_agg_seconds[to];
            if (!isfinite(bsd) || !isfinite(bas)) continue;
            if (a->track_reach)
                for (int i = 0; i < k; i++)
                    if (bas <= (float)a->seconds[i]) __atomic_fetch_add(&J->reach[i], 1u, __ATOMIC_RELAXED);
            for (int i = 0; i < k; i++) {
                if (bas <= (float)a->seconds[i]) {
                    float far_ang = a->farness_scaling_offset + (bsd / a->angular_scaling_unit);
                    float harm_ang = 1.0f + (bsd / a->angular_scaling_unit);
                    double v0 = (double)wt, v1 = (double)(far_ang * wt), v2 = (double)((1.0f / harm_ang) * wt);
                    if (J->atomic) {
                        add_f64_atomic(&ROW(0, i)[to], v0); add_f64_atomic(&ROW(1, i)[to], v1);
                        add_f64_atomic(&ROW(2, i)[to], v2);
                    } else {
                        ROW(0, i)[to] += v0; ROW(1, i)[to] += v1; ROW(2, i)[to] += v2;
                    }
                }
            }
        }
    }
    if (a->compute_betweenness) {
        int64_t *sorted;
        int64_t ns = sorted_state_indices(&t, &sorted);
        double *seed = (double *)calloc(t.n_state > 0 ? t.n_state : 1, sizeof(double));
        double *seed_b = (double *)calloc(t.n_state > 0 ? t.n_state : 1, sizeof(double));
        for (int i = 0; i < k; i++) {
            float thr = (float)a->seconds[i];
            memset(seed, 0, sizeof(double) * t.n_state);
            for (int64_t r = 0; r < t.n_reached; r++) {
                int64_t to = t.reached[r];
                if (to == src) continue;
                int64_t bs[2];
                int nb = best_angular_target_states(&t, to, thr, a->tolerance, bs);
                if (nb == 0) continue;
                double pc = a->eligible[to] ? 0.5 : 1.0;
                double st = 0.0;
                for (int q = 0; q < nb; q++) st += t.state[bs[q]].sigma;
                if (st == 0.0) continue;
                for (int q = 0; q < nb; q++) seed[bs[q]] += pc * (t.state[bs[q]].sigma / st);
            }
            brandes_backprop(&t, sorted, ns, src, seed, seed_b, 1, thr, ROW(3, i), NULL, (double)wt, J->atomic);
        }
        free(seed); free(seed_b); free(sorted);
    }
#undef ROW
    btrav_free(&t);
}

/* ------------------------------------------------------------------------------------------ */
/* Single-predecessor trees (centrality.rs:1141-1332, 1524-1611; graph.rs:251-315).           */
/* ------------------------------------------------------------------------------------------ */
typedef struct {
    uint8_t visited, discovered;
    int64_t pred;          /* -1 = None */
    float short_dist, simpl_dist;
    int64_t origin_seg, last_seg; /* -1 = None */
    float agg_seconds;
} nvisit;
typedef struct { uint8_t visited; int64_t start, end, edge_idx; } evisit;

static void nvisit_init(nvisit *v) {
    v->visited = 0; v->discovered = 0; v->pred = -1;
    v->short_dist = INFINITY; v->simpl_dist = INFINITY;
    v->origin_seg = -1; v->last_seg = -1; v->agg_seconds = INFINITY;
}

/* dijkstra_tree_shortest_inner (centrality.rs:1141-1200) */
int64_t og_tree_shortest(const og_graph *g, int64_t src, uint32_t max_seconds, float speed,
                         int64_t *visited_out, nvisit *tree) {
    int64_t n = g->d.n_bound, nv = 0;
    for (int64_t i = 0; i < n; i++) nvisit_init(&tree[i]);
    tree[src].agg_seconds = 0.0f; tree[src].discovered = 1; tree[src].short_dist = 0.0f;
    heap_t h = {0};
    hp_push(&h, src, 0.0f);
    hent it;
    const float maxs = (float)max_seconds;
    while (hp_pop(&h, &it)) {
        int64_t u = it.idx;
        if (tree[u].visited) continue;
        tree[u].visited = 1;
        visited_out[nv++] = u;
        for (int32_t e = g->in_head[u]; e >= 0; e = g->in_next[e]) {
            int64_t nb = g->d.e_src[e];
            if (nb == u || tree[nb].visited) continue;
            if (tree[u].pred >= 0 && nb == tree[u].pred) continue;
            float es = edge_travel_seconds(g, (int32_t)nb, (int32_t)u, e, speed, 1);
            float ts = tree[u].agg_seconds + es;
            if (ts > maxs) continue;
            if (ts < tree[nb].agg_seconds) {
                tree[nb].short_dist = ts * speed;
                tree[nb].agg_seconds = ts;
                tree[nb].pred = u;
                tree[nb].discovered = 1;
                hp_push(&h, nb, ts);
            }
        }
    }
    free(h.a);
    return nv;
}

/* dijkstra_tree_angular (centrality.rs:1202-1332) */
int64_t og_tree_simplest(const og_graph *g, int64_t src, uint32_t max_seconds, float speed,
                         int64_t *visited_out, nvisit *tree) {
    int64_t n = g->d.n_bound, ns = 2 * n, nv = 0;
    typedef struct { uint8_t visited; int64_t pred; float rm, sd, as; } ats;
    ats *S = (ats *)malloc(sizeof(ats) * (ns > 0 ? ns : 1));
    for (int64_t i = 0; i < ns; i++) { S[i].visited = 0; S[i].pred = -1; S[i].rm = S[i].sd = S[i].as = INFINITY; }
    uint8_t *reached = (uint8_t *)calloc(n > 0 ? n : 1, 1);
    for (int64_t i = 0; i < n; i++) nvisit_init(&tree[i]);
    visited_out[nv++] = src;
    reached[src] = 1;
    tree[src].discovered = 1; tree[src].visited = 1; tree[src].simpl_dist = 0.0f; tree[src].agg_seconds = 0.0f;
    heap_t h = {0};
    for (int slot = 0; slot < 2; slot++) {
        int64_t s = ang_state_idx(src, slot);
        S[s].rm = 0.0f; S[s].sd = 0.0f; S[s].as = 0.0f;
        hp_push(&h, s, 0.0f);
    }
    const float maxs = (float)max_seconds;
    hent it;
    while (hp_pop(&h, &it)) {
        int64_t si = it.idx;
        if (S[si].visited) continue;
        S[si].visited = 1;
        int64_t cur = si / 2, entry = si % 2;
        for (int32_t e = g->out_head[cur]; e >= 0; e = g->out_next[e]) {
            int64_t nx = g->d.e_dst[e];
            int32_t key = g->d.e_shared[e];
            if (slot_pos(g, cur, key) != 1 - entry) continue;
            int64_t nsi = ang_state_idx(nx, slot_pos(g, nx, key));
            float es = edge_travel_seconds(g, (int32_t)cur, (int32_t)nx, e, speed, 0);
            float cs = S[si].as + es;
            if (cs > maxs) continue;
            float csimpl = S[si].sd + g->d.e_ang[e];
            float cm = csimpl + (ANGULAR_ROUTE_TIE_BREAK_FACTOR * g->d.e_len[e]);
            int improved = cm + TIE_EPSILON < S[nsi].rm;
            int tied = fabsf(cm - S[nsi].rm) <= TIE_EPSILON;
            if (improved || (tied && cs < S[nsi].as && si != nsi)) {
                S[nsi].rm = cm; S[nsi].sd = csimpl; S[nsi].as = cs; S[nsi].pred = si;
                hp_push(&h, nsi, cm);
                nvisit *nv2 = &tree[nx];
                if (!reached[nx]) { reached[nx] = 1; visited_out[nv++] = nx; }
                int node_improved = csimpl + TIE_EPSILON < nv2->simpl_dist;
                int node_tied = fabsf(csimpl - nv2->simpl_dist) <= TIE_EPSILON;
                if (!nv2->discovered || node_improved || (node_tied && cs < nv2->agg_seconds)) {
                    nv2->discovered = 1; nv2->visited = 1;
                    nv2->simpl_dist = csimpl; nv2->agg_seconds = cs; nv2->pred = cur;
                }
            }
        }
    }
    free(h.a); free(S); free(reached);
    return nv;
}

/* dijkstra_tree_segment (centrality.rs:1524-1611). edge ids are edge slot indices. */
int64_t og_tree_segment(const og_graph *g, int64_t src, uint32_t max_seconds, float speed,
                        int64_t *visited_out, nvisit *tree, int64_t *vedges_out, int64_t *n_vedges,
                        evisit *emap) {
    int64_t n = g->d.n_bound, m = g->d.n_edges, nv = 0, ne = 0;
    for (int64_t i = 0; i < n; i++) nvisit_init(&tree[i]);
    for (int64_t i = 0; i < m; i++) { emap[i].visited = 0; emap[i].start = emap[i].end = emap[i].edge_idx = -1; }
    tree[src].short_dist = 0.0f; tree[src].agg_seconds = 0.0f; tree[src].discovered = 1;
    heap_t h = {0};
    hp_push(&h, src, 0.0f);
    hent it;
    const float maxs = (float)max_seconds;
    while (hp_pop(&h, &it)) {
        int64_t u = it.idx;
        if (tree[u].visited) continue;
        tree[u].visited = 1;
        visited_out[nv++] = u;
        for (int32_t e = g->in_head[u]; e >= 0; e = g->in_next[e]) {
            int64_t nb = g->d.e_src[e];
            if (nb == u) {
                vedges_out[ne++] = e;
                emap[e].visited = 1; emap[e].start = u; emap[e].end = nb; emap[e].edge_idx = g->d.e_idx[e];
                continue;
            }
            if (tree[nb].visited) continue;
            vedges_out[ne++] = e;
            emap[e].visited = 1; emap[e].start = u; emap[e].end = nb; emap[e].edge_idx = g->d.e_idx[e];
            float es = edge_travel_seconds(g, (int32_t)nb, (int32_t)u, e, speed, 1);
            float ts = tree[u].agg_seconds + es;
            if (ts > maxs) continue;
            if (ts < tree[nb].agg_seconds) {
                int64_t origin = (u == src) ? e : tree[u].origin_seg;
                tree[nb].short_dist = ts * speed;
                tree[nb].agg_seconds = ts;
                tree[nb].pred = u;
                tree[nb].origin_seg = origin;
                tree[nb].last_seg = e;
                tree[nb].discovered = 1;
                hp_push(&h, nb, ts);
            }
        }
    }
    free(h.a);
    *n_vedges = ne;
    return nv;
}

/* get_edge_length_unchecked / impedance (graph.rs:1278-1314): first edge start->end whose
   payload edge_idx matches, in petgraph edges_connecting order (outgoing list of start). */
static int32_t find_edge(const og_graph *g, int64_t start, int64_t end, int64_t edge_idx) {
    for (int32_t e = g->out_head[start]; e >= 0; e = g->out_next[e])
        if (g->d.e_dst[e] == end && g->d.e_idx[e] == edge_idx) return e;
    return -1;
}

static void run_segment_source(job_t *J, int64_t src, int64_t *visited, nvisit *tree, int64_t *vedges, evisit *emap) {
    const og_graph *g = J->g;
    const og_args *a = J->a;
    int64_t n = g->d.n_bound;
    int k = a->k;
    if (!g->d.live[src]) return;
    uint32_t maxs = 0;
    for (int i = 0; i < k; i++) if (a->seconds[i] > maxs) maxs = a->seconds[i];
    int64_t ne;
    int64_t nv = og_tree_segment(g, src, maxs, a->speed, visited, tree, vedges, &ne, emap);
    double *O = J->out;
#define ROW(m, i) (O + ((int64_t)(m) * k + (i)) * n)
#define ADD(p, v) do { if (J->atomic) add_f64_atomic((p), (v)); else *(p) += (v); } while (0)
    for (int64_t q = 0; q < ne; q++) {
        const evisit *ev = &emap[vedges[q]];
        int64_t sn = ev->start, en = ev->end, eidx = ev->edge_idx;
        const nvisit *vn = &tree[sn], *vm = &tree[en];
        if (!isfinite(vn->short_dist) && !isfinite(vm->short_dist)) continue;
        if (a->compute_closeness) {
            int n_nearer = vn->short_dist <= vm->short_dist;
            float A = n_nearer ? vn->short_dist : vm->short_dist, A_imp = A;
            float B = n_nearer ? vm->short_dist : vn->short_dist, B_imp = B;
            int32_t fe = find_edge(g, sn, en, eidx);
            float elen = g->d.e_len[fe], imp = g->d.e_imp[fe];
            float C = (elen + A + B) / 2.0f, D = C;
            float C_imp = A_imp + (C - A) * imp, D_imp = C_imp;
            for (int i = k - 1; i >= 0; i--) {
                float df = (float)a->distances[i];
                float beta = a->betas[i], neg_beta = -beta;
                float inv_neg_beta = beta != 0.0f ? 1.0f / neg_beta : 0.0f;
                if (A < df) {
                    float cc = C, cci = C_imp;
                    if (cc > df) { cc = df; cci = A_imp + (df - A) * imp; }
                    ADD(&ROW(0, i)[src], (double)(cc - A));
                    float sh = A_imp < 1.0f ? logf(cci) : logf(fmaxf(cci / A_imp, F32_EPSILON));
                    ADD(&ROW(1, i)[src], (double)sh);
                    float bet = beta == 0.0f ? cci - A_imp : (expf(neg_beta * cci) - expf(neg_beta * A_imp)) * inv_neg_beta;
                    ADD(&ROW(2, i)[src], (double)bet);
                }
                if (B == D) continue;
                if (B <= df) {
                    float cd = D, cdi = D_imp;
                    if (cd > df) { cd = df; cdi = B_imp + (df - B) * imp; }
                    ADD(&ROW(0, i)[src], (double)(cd - B));
                    float sh = B_imp < 1.0f ? logf(cdi) : logf(fmaxf(cdi / B_imp, F32_EPSILON));
                    ADD(&ROW(1, i)[src], (double)sh);
                    float bet = beta == 0.0f ? cdi - B_imp : (expf(neg_beta * cdi) - expf(neg_beta * B_imp)) * inv_neg_beta;
                    ADD(&ROW(2, i)[src], (double)bet);
                }
            }
        }
    }
    if (a->compute_betweenness) {
        for (int64_t q = 0; q < nv; q++) {
            int64_t to = visited[q];
            if (to <= src) continue;
            const nvisit *tv = &tree[to];
            if (!isfinite(tv->short_dist)) continue;
            const evisit *oe = &emap[tv->origin_seg], *le = &emap[tv->last_seg];
            float o_len = g->d.e_len[find_edge(g, oe->start, oe->end, oe->edge_idx)];
            float l_len = g->d.e_len[find_edge(g, le->start, le->end, le->edge_idx)];
            float min_span = tv->short_dist - o_len - l_len;
            float o_1 = min_span, o_2 = min_span + o_len, l_1 = min_span, l_2 = min_span + l_len;
            int64_t cp = tv->pred;
            while (cp >= 0) {
                if (cp == src) break;
                for (int i = k - 1; i >= 0; i--) {
                    float df = (float)a->distances[i];
                    float beta = a->betas[i];
                    if (min_span <= df) {
                        float o2s = fminf(o_2, df), l2s = fminf(l_2, df);
                        float auc;
                        if (beta == 0.0f) auc = (o2s - o_1) + (l2s - l_1);
                        else {
                            float nb = -beta, inb = 1.0f / nb;
                            auc = (expf(nb * o2s) - expf(nb * o_1)) * inb + (expf(nb * l2s) - expf(nb * l_1)) * inb;
                        }
                        if (isfinite(auc) && auc >= 0.0f) ADD(&ROW(3, i)[cp], (double)auc);
                    }
                }
                cp = tree[cp].pred;
            }
        }
    }
#undef ADD
#undef ROW
}

/* ------------------------------------------------------------------------------------------ */
/* Drivers: sequential (deterministic order, nthreads <= 1) or a pthread pool over sources     */
/* with atomic f64 accumulation, mirroring the rayon par_iter (centrality.rs:1702-1836).       */
/* ------------------------------------------------------------------------------------------ */
static void *worker(void *arg) {
    job_t *J = (job_t *)arg;
    const og_graph *g = J->g;
    int64_t n = g->d.n_bound, m = g->d.n_edges;
    int64_t *visited = NULL, *vedges = NULL;
    nvisit *tree = NULL;
    evisit *emap = NULL;
    if (J->mode == 2) {
        visited = (int64_t *)malloc(sizeof(int64_t) * (n > 0 ? n : 1));
        vedges = (int64_t *)malloc(sizeof(int64_t) * (m + 1));
        tree = (nvisit *)malloc(sizeof(nvisit) * (n > 0 ? n : 1));
        emap = (evisit *)malloc(sizeof(evisit) * (m + 1));
    }
    for (;;) {
        int64_t i = __atomic_fetch_add(&J->next, 1, __ATOMIC_RELAXED);
        if (i >= J->a->n_sources) break;
        int64_t src = J->a->sources[i];
        if (J->mode == 0) run_shortest_source(J, src);
        else if (J->mode == 1) run_simplest_source(J, src);
        else if (J->mode == 3) run_od_source(J, src);
        else run_segment_source(J, src, visited, tree, vedges, emap);
    }
    free(visited); free(vedges); free(tree); free(emap);
    return NULL;
}

static int run_job(job_t *J) {
    int nt = J->a->nthreads;
    if (nt <= 1) {
        J->atomic = 0;
        worker(J);
        return 0;
    }
    J->atomic = 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nt);
    for (int i = 0; i < nt; i++) pthread_create(&th[i], NULL, worker, J);
    for (int i = 0; i < nt; i++) pthread_join(th[i], NULL);
    free(th);
    return 0;
}

/* out: [7][K][n_bound] (density, farness, cycles, harmonic, beta, betweenness, betweenness_beta) */
int og_centrality_shortest(const og_graph *g, const og_args *a, double *out, uint32_t *reach) {
    if (a->k <= 0 || a->k > 64) return OG_ERR_ARG;
    job_t J = {g, a, out, reach, 0, 0, 0};
    return run_job(&J);
}
/* out: [4][K][n_bound] (density, farness, harmonic, betweenness) */
int og_centrality_simplest(const og_graph *g, const og_args *a, double *out, uint32_t *reach) {
    if (a->k <= 0 || a->k > 64 || !g->slots_ok) return OG_ERR_ARG;
    job_t J = {g, a, out, reach, 0, 1, 0};
    return run_job(&J);
}
/* out: [4][K][n_bound] (segment density, harmonic, beta, betweenness) */
int og_segment_centrality(const og_graph *g, const og_args *a, double *out) {
    if (a->k <= 0 || a->k > 64) return OG_ERR_ARG;
    job_t J = {g, a, out, NULL, 0, 2, 0};
    return run_job(&J);
}

/* out: [2][K][n_bound] (betweenness, betweenness_beta); a->sources = node_indices; every destination
   index is below n_bound (the caller checks). */
int og_betweenness_od(const og_graph *g, const og_args *a, double *out) {
    if (a->k <= 0 || a->k > 64 || !a->od_ptr || !a->od_dst || !a->od_w) return OG_ERR_ARG;
    job_t J = {g, a, out, NULL, 0, 3, 0};
    return run_job(&J);
}

/* Per-source diagnostic: the Brandes traversal's per-node results (shortest, or simplest per
   state) for exact-parity tests of distances, predecessor lists and sigma.
   agg/route: [n_state]; npred: [n_state]; preds: [n_state * pmax] (-1 padded); sigma: [n_state];
   order: [n_state] visited order.  Returns the number of visited states, or -1 if a state has
   more than pmax predecessors. */
int64_t og_brandes_debug(const og_graph *g, int32_t angular, int64_t src, uint32_t max_seconds, float speed,
                         float tolerance, float *agg, float *route, int32_t *npred, int64_t *preds, int32_t pmax,
                         double *sigma, int64_t *order, float *best_route, float *best_agg) {
    btrav t;
    if (angular) dijkstra_brandes_angular(g, src, max_seconds, speed, tolerance, &t);
    else dijkstra_brandes_shortest(g, src, max_seconds, speed, tolerance, &t);
    int64_t res = t.n_visited;
    for (int64_t i = 0; i < t.n_state; i++) {
        agg[i] = t.state[i].agg_seconds;
        route[i] = t.state[i].route_cost;
        npred[i] = t.state[i].npred;
        sigma[i] = t.state[i].sigma;
        if (t.state[i].npred > pmax) res = -1;
        for (int32_t p = 0; p < pmax; p++) preds[i * pmax + p] = p < t.state[i].npred ? t.state[i].preds[p] : -1;
    }
    for (int64_t i = 0; i < t.n_visited; i++) order[i] = t.visited[i];
    for (int64_t i = 0; i < g->d.n_bound; i++) { best_route[i] = t.best_route_cost[i]; best_agg[i] = t.best_agg_seconds[i]; }
    btrav_free(&t);
    return res;
}

int32_t og_sizeof_nvisit(void) { return (int32_t)sizeof(nvisit); }
int32_t og_sizeof_evisit(void) { return (int32_t)sizeof(evisit); }
int32_t og_sizeof_args(void) { return (int32_t)sizeof(og_args); }
int32_t og_sizeof_desc(void) { return (int32_t)sizeof(og_graph_desc); }

/* dual endpoint slots per node (2 entries, -1 empty) as computed above (test accessor) */
void og_get_slots(const og_graph *g, int32_t *out) {
    memcpy(out, g->slots, sizeof(int32_t) * 2 * (size_t)g->d.n_bound);
}

/* ------------------------------------------------------------------------------------------ */
/* Data aggregation (rust/src/data.rs:513-602 aggregate_to_src_idx, :605-740 accessibility).   */
/* ------------------------------------------------------------------------------------------ */
/* node_data_map as CSR: per node, its (entry, node_dist) assignments in the map's Vec order
   (data.rs:484-499); entry_group: the entry's dedupe key as a group id. */
typedef struct {
    int64_t n_entries, n_groups;
    const int64_t *nd_ptr;     /* [n_bound + 1] */
    const int64_t *nd_entry;   /* [n_assign] */
    const double *nd_dist;     /* [n_assign] */
    const int64_t *entry_group;/* [n_entries] */
} og_data;

/* aggregate_to_src_idx: entry_dist[e] = the reachable entry's total distance (f32), NaN when the
   entry is not in the result map.  Scratch: group_best [n_groups] f32, group_entry [n_groups]. */
int64_t og_aggregate(const og_graph *g, const og_data *d, int64_t src, uint32_t max_seconds, float speed,
                     int32_t angular, float *entry_dist, float *group_best, int64_t *group_entry) {
    const int64_t n = g->d.n_bound;
    int64_t *visited = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    nvisit *tree = (nvisit *)malloc(sizeof(nvisit) * (size_t)(n > 0 ? n : 1));
    const int64_t nv = angular ? og_tree_simplest(g, src, max_seconds, speed, visited, tree)
                               : og_tree_shortest(g, src, max_seconds, speed, visited, tree);
    for (int64_t q = 0; q < d->n_groups; q++) { group_best[q] = INFINITY; group_entry[q] = -1; }
    for (int64_t e = 0; e < d->n_entries; e++) entry_dist[e] = NAN;
    const float max_walk_dist = (float)max_seconds * speed;
    for (int64_t i = 0; i < nv; i++) {
        const int64_t node = visited[i];
        const nvisit *nvz = &tree[node];
        if (nvz->agg_seconds >= (float)max_seconds) continue;
        for (int64_t a = d->nd_ptr[node]; a < d->nd_ptr[node + 1]; a++) {
            const int64_t e = d->nd_entry[a];
            const float network_dist = nvz->agg_seconds * speed;
            const float total = network_dist + (float)d->nd_dist[a];
            if (!(total <= max_walk_dist)) continue;
            const int64_t q = d->entry_group[e];
            if (group_entry[q] < 0 || total < group_best[q]) {  /* vacant, or strictly better */
                group_best[q] = total;
                group_entry[q] = e;
            }
        }
    }
    int64_t cnt = 0;
    for (int64_t q = 0; q < d->n_groups; q++)
        if (group_entry[q] >= 0) { entry_dist[group_entry[q]] = group_best[q]; cnt++; }
    free(visited);
    free(tree);
    return cnt;
}

/* accessibility (data.rs:605-740) for live sources: entry_class [n_entries] (-1: not an
   accessibility key), k thresholds (distances, betas, max curve weights), out rows
   unweighted/weighted [n_classes][k][n_bound] (zeroed) and nearest [n_classes][n_bound] (NaN). */
int og_accessibility(const og_graph *g, const og_data *d, const int32_t *entry_class, int32_t n_classes, int32_t k,
                     const uint32_t *distances, const float *betas, const float *mcw, uint32_t max_seconds,
                     float speed, int32_t angular, double *unweighted, double *weighted, double *nearest) {
    const int64_t n = g->d.n_bound;
    uint32_t max_dist = 0;
    for (int32_t i = 0; i < k; i++) if (distances[i] > max_dist) max_dist = distances[i];
    float *edist = (float *)malloc(sizeof(float) * (size_t)(d->n_entries > 0 ? d->n_entries : 1));
    float *gb = (float *)malloc(sizeof(float) * (size_t)(d->n_groups > 0 ? d->n_groups : 1));
    int64_t *ge = (int64_t *)malloc(sizeof(int64_t) * (size_t)(d->n_groups > 0 ? d->n_groups : 1));
    for (int64_t src = 0; src < n; src++) {
        if (!g->d.node_exists[src] || !g->d.live[src]) continue;
        og_aggregate(g, d, src, max_seconds, speed, angular, edist, gb, ge);
        for (int64_t e = 0; e < d->n_entries; e++) {
            const float data_dist = edist[e];
            if (isnan(data_dist)) continue;
            const int32_t c = entry_class[e];
            if (c < 0) continue;
            for (int32_t i = 0; i < k; i++) {
                if (!(data_dist <= (float)distances[i])) continue;
                unweighted[((size_t)c * k + i) * n + src] += 1.0;
                /* clipped_beta_wt (common.rs:339-348) */
                const float raw = expf(-betas[i] * data_dist);
                const float wt = fminf(raw, mcw[i]) / mcw[i];
                weighted[((size_t)c * k + i) * n + src] += (double)wt;
                if (distances[i] == max_dist) {
                    double *cur = &nearest[(size_t)c * n + src];
                    if (isnan(*cur) || (double)data_dist < *cur) *cur = (double)data_dist;
                }
            }
        }
    }
    free(edist);
    free(gb);
    free(ge);
    return 0;
}
