// cs_primal.cu -- GB300 kernels for shortest-path node centrality, OD-weighted betweenness, segment
// centrality and shortest-path trees (isochrones) on the primal graph.
//
// Reference behaviour (cityseer-api v4.24.0):
//   centrality_shortest        rust/src/centrality.rs:1624-1874
//   dijkstra_brandes_shortest  rust/src/centrality.rs:1344-1494
//   circuit_ranks_from_traversal rust/src/centrality.rs:470-526
//   brandes_backprop_with_beta rust/src/centrality.rs:823-873
//   betweenness_od_shortest    rust/src/centrality.rs:2419-2540
//   segment_centrality         rust/src/centrality.rs:2134-2407
//   dijkstra_tree_segment      rust/src/centrality.rs:1524-1611
//   dijkstra_tree_shortest_inner rust/src/centrality.rs:1141-1200
//
// Design (one warp per source; persistent warps pull sources from a work counter, and in the
// block-synchronous form the warps of a block run each phase together):
//  1. Bounded label-correcting search ("near-far" banded Bellman-Ford) from the source over
//     reversed edges.  Every relaxation is fl(d[u] + w) with w >= 0, so the least fixpoint is
//     unique and bit-identical to the reference's heap Dijkstra whatever the relaxation order.
//  2. Warp sort of the reached set by distance (cs_sort.cuh: distance buckets, or LSD radix): the
//     reference's settle order.
//  3. Replay, per reached node and in parallel, of the exact sequence of candidate offers the
//     heap Dijkstra would make to it (offering neighbours in settle order), through the
//     reference's Phase-1 tie rules (and Phase 2 when tolerance > 1e-4).  This reproduces its
//     multi-predecessor lists; sigma follows chunk by chunk in settle order in the same pass.
//  4. Closeness into target rows and circuit ranks; one backward Brandes sweep carrying all K
//     thresholds (a state beyond threshold k contributes nothing to lane k, so one sweep equals
//     the reference's K sweeps).
// Per-slot scratch: dense dist/aux arrays over node_bound (reset touched entries only) plus
// compact per-reached-node arrays of capacity `cap`; sources that overflow `cap` are redone inside
// the same API call at 4x the capacity, then 4x again, up to cap = node_bound.
#include <cstdio>
#include <cstring>
#include <string>
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "cs_common.cuh"
#include "cs_cta.cuh"
#include "cs_seed.cuh"
#include "cs_sort.cuh"

namespace cs {

struct SlotPtrs {
    float *dist;
    uint32_t *aux;
    int32_t *rl;
    uint2 *qa, *qb, *qf;  // (node, dist bits) entries, capacity 2 * cap
    uint32_t *kb;
    int32_t *vb;
    int32_t *ord;
    float *sd;
    double *sig;
    uint8_t *np;
    int32_t *pr;
    double *dl;
    float *fa, *fb;
    int32_t *eb;
};

__host__ __device__ inline size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

__host__ __device__ inline size_t compact_bytes(size_t cap, int P, int L) {
    size_t b = 0;
    b += 4 * al256(cap * 4);      // rl kb vb ord
    b += 3 * al256(cap * 16);     // qa qb qf: 2 * cap entries of 8 bytes
    b += al256(cap * 4);          // sd
    b += al256(cap * 8);          // sig
    b += al256(cap);              // np
    b += al256(cap * 4 * (size_t)P);  // pr
    b += al256(cap * 8 * (size_t)L);  // dl
    b += 3 * al256(cap * 4);      // fa fb eb
    return b;
}

__host__ __device__ inline SlotPtrs slot_ptrs(char *dense, size_t dense_stride, char *compact, size_t cap, int P,
                                              int L, int slot, int n_bound) {
    SlotPtrs s;
    char *d = dense + dense_stride * (size_t)slot;
    s.dist = (float *)d;
    s.aux = (uint32_t *)(d + al256((size_t)n_bound * 4));
    char *c = compact + compact_bytes(cap, P, L) * (size_t)slot;
    size_t o = 0;
    s.rl = (int32_t *)(c + o); o += al256(cap * 4);
    s.qa = (uint2 *)(c + o); o += al256(cap * 16);
    s.qb = (uint2 *)(c + o); o += al256(cap * 16);
    s.qf = (uint2 *)(c + o); o += al256(cap * 16);
    s.kb = (uint32_t *)(c + o); o += al256(cap * 4);
    s.vb = (int32_t *)(c + o); o += al256(cap * 4);
    s.ord = (int32_t *)(c + o); o += al256(cap * 4);
    s.sd = (float *)(c + o); o += al256(cap * 4);
    s.sig = (double *)(c + o); o += al256(cap * 8);
    s.np = (uint8_t *)(c + o); o += al256(cap);
    s.pr = (int32_t *)(c + o); o += al256(cap * 4 * (size_t)P);
    s.dl = (double *)(c + o); o += al256(cap * 8 * (size_t)L);
    s.fa = (float *)(c + o); o += al256(cap * 4);
    s.fb = (float *)(c + o); o += al256(cap * 4);
    s.eb = (int32_t *)(c + o); o += al256(cap * 4);
    return s;
}

// BOTH: batched jobs only.  OD: betweenness seeded by an origin-destination matrix.
// ACCESS: accessibility sums over data assigned to the reached nodes.
enum Mode { MODE_SHORTEST = 0, MODE_SEGMENT = 1, MODE_TREE = 2, MODE_BOTH = 3, MODE_OD = 4, MODE_ACCESS = 5 };

struct PrimalParams {
    cs_primal_graph g;
    int32_t k;
    float dk[MAXK];
    float beta[MAXK];
    float maxsec;
    float speed;
    float tol;
    float delta;
    int32_t closeness, betweenness, track_reach;
    const int32_t *src_list;
    int64_t n_src;
    const float *src_wt;
    const uint8_t *eligible;
    double *out;
    double *bucket;  // [3][K][N] threshold-bucketed closeness terms (density, farness, harmonic)
    double *out2;    // MODE_BOTH: segment rows [4][K][N] (out holds the shortest rows)
    uint32_t *reach;
    WsHeader *hdr;
    int32_t *failed;  // [fail_cap] indices (into src_list) of sources that overflowed
    int32_t fail_cap;
    char *dense;
    size_t dense_stride;
    char *compact;
    int32_t cap, P, L;
    int32_t n_slots;
    int32_t rerun;
    const int32_t *remap;  // rerun: indices into src_list of the sources to redo
    int32_t mode;
    int32_t row_cap;
    int32_t *t_count, *t_node, *t_pred;
    float *t_agg;
    // MODE_OD: per origin node, its row [od_ptr[o], od_ptr[o+1]) of destinations (ascending) and weights
    const int32_t *od_ptr, *od_dst;
    const float *od_w;
    int32_t radix_sort;  // settle-order sort: 0 distance buckets, 1 LSD radix
    // MODE_ACCESS: the data map (cs_data_map) and the per-class rows
    cs_data_map dm;
    float mcw[MAXK];   // max curve weights (clip_wts_curve)
    float max_dist;    // the largest distance threshold (metres)
    double *acc_unw, *acc_wt;  // [n_classes][K][n_bound]
    uint32_t *acc_near;        // [n_classes][n_bound] f32 bits of the nearest distance
};

// ------------------------------------------------------------------------------------------
// 1. Banded label-correcting search.  Returns R (reached count incl. source) or -1 on overflow.
//    Queues hold (node, distance-at-push) entries with lazy deletion: an entry is live only while
//    its distance still equals the node's, so no flag atomics are needed to de-duplicate.
// ------------------------------------------------------------------------------------------
constexpr int DEG_FAST = 8;  // edges per node loaded together; higher degrees loop
// Backward sweep: predecessors per lane kept in shared memory (row and f64 factor); a node's
// further predecessors (high-degree graphs) are read from the per-source scratch.
constexpr int BW_COLS = 8;
__host__ __device__ constexpr int bw_cols(int pm) { return pm < BW_COLS ? pm : BW_COLS; }

__device__ __forceinline__ void push_entries(bool first, int route, int v, float c, int &R, int &nnext, int &nfar,
                                             int cap, int qcap, const SlotPtrs &s, uint2 *nxt, unsigned lt) {
    const unsigned mf = __ballot_sync(FULL, first);
    const unsigned mn = __ballot_sync(FULL, route == 1);
    const unsigned mr = __ballot_sync(FULL, route == 2);
    if (first) {
        const int q = R + __popc(mf & lt);
        if (q < cap) s.rl[q] = v;
    }
    if (route == 1) {
        const int q = nnext + __popc(mn & lt);
        if (q < qcap) nxt[q] = make_uint2((unsigned)v, __float_as_uint(c));
    }
    if (route == 2) {
        const int q = nfar + __popc(mr & lt);
        if (q < qcap) s.qf[q] = make_uint2((unsigned)v, __float_as_uint(c));
    }
    R += __popc(mf);
    nnext += __popc(mn);
    nfar += __popc(mr);
}

#ifndef CS_PHASE_INLINE
#define CS_PHASE_INLINE
#endif

// dmax: an upper bound of every reached distance (the last band's end, at most the cutoff).
CS_PHASE_INLINE __device__ int warp_search(const PrimalParams &p, const SlotPtrs &s, int src, long long &relaxed,
                                           float &dmax) {
    const int lane = lane_id();
    const unsigned lt = lanemask_lt();
    const int cap = p.cap;
    const int qcap = 2 * cap;
    const int32_t *__restrict__ in_ptr = p.g.in_ptr_dev;
    const int32_t *__restrict__ in_nb = p.g.in_nb_dev;
    const float *__restrict__ in_w = p.g.in_w_dev;
    const float maxsec = p.maxsec, delta = p.delta;  // in registers (p may live in shared memory)
    float *dist = s.dist;
    if (lane == 0) {
        dist[src] = 0.0f;
        s.rl[0] = src;
        s.qa[0] = make_uint2((unsigned)src, 0u);
    }
    __syncwarp();
    int R = 1, nnear = 1, nfar = 0;
    uint2 *cur = s.qa, *nxt = s.qb;
    float T = delta;
    float fmn = __int_as_float(INF_BITS);  // this lane's smallest distance queued far since the last split
    bool overflow = false;
    while (true) {
        while (nnear > 0) {
            int nnext = 0;
            for (int base = 0; base < nnear; base += 32) {
                const int i = base + lane;
                uint2 ent = make_uint2(0u, 0u);
                if (i < nnear) ent = cur[i];
                const int u = (int)ent.x;
                const float du = (i < nnear) ? __ldcg(&dist[u]) : 0.0f;
                const bool live = (i < nnear) && (__float_as_uint(du) == ent.y);
                const int beg = live ? __ldg(&in_ptr[u]) : 0;
                const int deg = live ? __ldg(&in_ptr[u + 1]) - beg : 0;
                relaxed += deg;
                // load this node's first DEG_FAST edges together, then issue their atomics together
                int vv[DEG_FAST];
                float cc[DEG_FAST];
                int old[DEG_FAST];
#pragma unroll
                for (int j = 0; j < DEG_FAST; j++) {
                    vv[j] = u;
                    cc[j] = 0.0f;
                    if (j < deg) {
                        vv[j] = __ldg(&in_nb[beg + j]);
                        cc[j] = fadd(du, __ldg(&in_w[beg + j]));
                    }
                }
#pragma unroll
                for (int j = 0; j < DEG_FAST; j++) {
                    old[j] = 0;
                    if (j < deg && vv[j] != u && cc[j] <= maxsec)
                        old[j] = atomicMin((int *)&dist[vv[j]], __float_as_int(cc[j]));
                }
                const int maxdeg = warp_max_i(deg);
#pragma unroll
                for (int j = 0; j < DEG_FAST; j++) {
                    if (j >= maxdeg) break;
                    const bool imp = (j < deg) && vv[j] != u && cc[j] <= maxsec && __float_as_int(cc[j]) < old[j];
                    const int route = imp ? (cc[j] < T ? 1 : 2) : 0;
                    if (route == 2) fmn = fminf(fmn, cc[j]);
                    push_entries(imp && old[j] == INF_BITS, route, vv[j], cc[j], R, nnext, nfar, cap, qcap, s, nxt,
                                 lt);
                }
                // rare high-degree nodes: remaining edges one at a time
                for (int j = DEG_FAST; j < maxdeg; j++) {
                    int v = u;
                    float c = 0.0f;
                    bool imp = false, first = false;
                    if (j < deg) {
                        v = __ldg(&in_nb[beg + j]);
                        c = fadd(du, __ldg(&in_w[beg + j]));
                        if (v != u && c <= maxsec) {
                            const int o = atomicMin((int *)&dist[v], __float_as_int(c));
                            imp = __float_as_int(c) < o;
                            first = imp && o == INF_BITS;
                        }
                    }
                    const int route = imp ? (c < T ? 1 : 2) : 0;
                    if (route == 2) fmn = fminf(fmn, c);
                    push_entries(first, route, v, c, R, nnext, nfar, cap, qcap, s, nxt, lt);
                }
            }
            __syncwarp();
            if (R > cap || nnext > qcap || nfar > qcap) { overflow = true; break; }
            uint2 *t = cur; cur = nxt; nxt = t;
            nnear = nnext;
        }
        if (overflow) break;
        if (nfar == 0) break;
        // Next band: [mn, mn + delta) from the smallest queued far distance (the lanes' minima over
        // the pushes and over the entries the last split kept), strictly above mn even when delta is
        // below mn's ulp.  One streaming pass over the far queue, by the queued distances: entries
        // that died since they were queued are dropped when their band runs.
        const float mn = warp_min_f(fmn);
        T = fmaxf(fadd(mn, delta), __int_as_float(__float_as_int(mn) + 1));
        fmn = __int_as_float(INF_BITS);
        int nn = 0, nf2 = 0;
        for (int base = 0; base < nfar; base += 32) {
            const int i = base + lane;
            const bool act = i < nfar;
            const uint2 ent = act ? s.qf[i] : make_uint2(0u, 0u);
            const float d = __uint_as_float(ent.y);
            const bool tonear = act && d < T;
            const bool keep = act && !tonear;
            if (keep) fmn = fminf(fmn, d);
            const unsigned mt = __ballot_sync(FULL, tonear);
            const unsigned mk = __ballot_sync(FULL, keep);
            __syncwarp();
            if (tonear) cur[nn + __popc(mt & lt)] = ent;
            if (keep) s.qf[nf2 + __popc(mk & lt)] = ent;
            nn += __popc(mt);
            nf2 += __popc(mk);
            __syncwarp();
        }
        nnear = nn;
        nfar = nf2;
    }
    __syncwarp();
    dmax = fminf(T, maxsec);
    if (overflow) return -1;  // the slot's dense state is dirty: the caller resets it
    return R;
}

// ------------------------------------------------------------------------------------------
// 2. Warp LSD radix sort of the reached set by distance (cs_sort.cuh): the settle order.
// ------------------------------------------------------------------------------------------
// The distance-bucket sort (3 passes) unless p.radix_sort selects the 4-pass LSD radix sort; both
// give the same order (ascending distance, ties in reached-list order).
__device__ __forceinline__ void warp_sort(const PrimalParams &p, const SlotPtrs &s, int R, float dmax, uint32_t *hist) {
    const float *dist = s.dist;
    auto key_of = [dist](int v) { return (uint32_t)__float_as_int(__ldcg(&dist[v])); };
    if (p.radix_sort) warp_radix_sort(R, s.rl, key_of, s.kb, s.vb, (uint32_t *)s.sd, s.ord, hist);
    else warp_bucket_sort(R, dmax, s.rl, key_of, s.kb, s.vb, (uint32_t *)s.sd, s.ord, hist);
}

// ------------------------------------------------------------------------------------------
// 3. Offer replay for the node at sorted position i.  Everything per node stays in registers:
//    the kernel is instantiated for a maximum out-degree PM (8 for street graphs, 32 otherwise)
//    and all per-edge arrays are fixed-size and fully unrolled.
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ float route_cost(float secs, float speed) { return fmul(secs, speed); }

// Reached out-neighbours of v: slot j holds out-CSR edge beg + j (pos -1: unreached or self loop).
template <int PM>
struct Nb {
    int pos[PM];
    float d[PM];
    int beg, deg;
};

template <int PM>
__device__ __forceinline__ void load_nb(const PrimalParams &p, const SlotPtrs &s, int v, int R, Nb<PM> &nb,
                                        bool &bad) {
    nb.beg = __ldg(&p.g.out_ptr_dev[v]);
    nb.deg = min(__ldg(&p.g.out_ptr_dev[v + 1]) - nb.beg, PM);
    int uu[PM];
    uint32_t aa[PM];
#pragma unroll
    for (int j = 0; j < PM; j++) uu[j] = (j < nb.deg) ? __ldg(&p.g.out_to_dev[nb.beg + j]) : v;
#pragma unroll
    for (int j = 0; j < PM; j++) aa[j] = (uu[j] != v) ? s.aux[uu[j]] : 0u;
#pragma unroll
    for (int j = 0; j < PM; j++) {
        const bool ok = aa[j] != 0u && aa[j] <= (uint32_t)R;
        if (aa[j] > (uint32_t)R) bad = true;  // scratch not clean: refuse to index
        nb.pos[j] = ok ? (int)aa[j] - 1 : -1;
        nb.d[j] = ok ? s.sd[aa[j] - 1] : 0.0f;
    }
}

// Offers to the node at position i are the reached neighbours settled before it, taken in order of
// the offering node's position (parallel edges keep list order).  Candidate seconds per slot:
template <int PM>
__device__ __forceinline__ unsigned offer_cands(const PrimalParams &p, const Nb<PM> &nb, int i, float *c) {
    unsigned todo = 0;
#pragma unroll
    for (int j = 0; j < PM; j++) {
        const bool off = nb.pos[j] >= 0 && nb.pos[j] < i;
        c[j] = off ? fadd(nb.d[j], __ldg(&p.g.out_w_dev[nb.beg + j])) : 0.0f;
        if (off) todo |= 1u << j;
    }
    return todo;
}

// next offer in settle order: lowest position, then lowest slot
template <int PM>
__device__ __forceinline__ int next_offer(const Nb<PM> &nb, unsigned todo, const float *c, int &bp, float &bc) {
    int best = -1;
    bp = 0x7fffffff;
    bc = 0.0f;
#pragma unroll
    for (int j = 0; j < PM; j++) {
        if (((todo >> j) & 1u) && nb.pos[j] < bp) {
            bp = nb.pos[j];
            best = j;
            bc = c[j];
        }
    }
    return best;
}

template <int PM>
__device__ __forceinline__ bool pos_in(const Nb<PM> &nb, unsigned mask, int pos) {
    bool has = false;
#pragma unroll
    for (int j = 0; j < PM; j++) has |= ((mask >> j) & 1u) && nb.pos[j] == pos;
    return has;
}

// Phase-1 (+ Phase-2) predecessor replay, rust/src/centrality.rs:1413-1437 and 1444-1483.
// Returns the predecessor slots as a bit mask; ok = false if the replayed distance does not
// reproduce the searched one (internal inconsistency).
template <int PM>
__device__ __forceinline__ unsigned replay_brandes(const PrimalParams &p, const Nb<PM> &nb, int i, float dv,
                                                   bool &ok) {
    const float one_plus = 1.0f + TIE_EPSILON;
    const float one_minus = 1.0f - TIE_EPSILON;
    float c[PM];
    const unsigned todo = offer_cands<PM>(p, nb, i, c);
    unsigned t = todo, pm = 0u;
    float cur = __int_as_float(INF_BITS);
    while (t) {
        int bp;
        float bc;
        const int best = next_offer<PM>(nb, t, c, bp, bc);
        t &= ~(1u << best);
        if (bc > p.maxsec) continue;
        const bool improved = bc < cur;
        const bool tied = bc <= fmul(cur, one_plus);
        if (improved) {
            if (bc < fmul(cur, one_minus)) pm = 0u;
            pm |= 1u << best;
            cur = bc;
        } else if (tied && !pos_in<PM>(nb, pm, bp)) {
            pm |= 1u << best;
        }
    }
    ok = __float_as_int(cur) == __float_as_int(dv);
    if (p.tol > TIE_EPSILON) {
        const float lim = fmul(dv, 1.0f + p.tol);
        pm = 0u;
        t = todo;
        while (t) {
            int bp;
            float bc;
            const int best = next_offer<PM>(nb, t, c, bp, bc);
            t &= ~(1u << best);
            if (bc <= lim && !pos_in<PM>(nb, pm, bp)) pm |= 1u << best;
        }
    }
    return pm;
}

// Strict-< single predecessor (dijkstra_tree_* / dijkstra_tree_segment): the first offer in settle
// order that reaches the final distance.  Returns its slot or -1; ok as above.
template <int PM>
__device__ __forceinline__ int replay_first_min(const PrimalParams &p, const Nb<PM> &nb, int i, float dv, bool &ok) {
    float c[PM];
    unsigned t = offer_cands<PM>(p, nb, i, c);
    float cur = __int_as_float(INF_BITS);
    int pick = -1;
    while (t) {
        int bp;
        float bc;
        const int best = next_offer<PM>(nb, t, c, bp, bc);
        t &= ~(1u << best);
        if (bc > p.maxsec) continue;
        if (bc < cur) {
            cur = bc;
            pick = best;
        }
    }
    ok = __float_as_int(cur) == __float_as_int(dv);
    return pick;
}

// ------------------------------------------------------------------------------------------
// 4a. Shortest-path centrality for one source (after search and sort).
// ------------------------------------------------------------------------------------------
// Per-phase cycle counters live in the warp's shared-memory row (lane 0 adds), not in registers.
__device__ __forceinline__ void phase_mark(long long *ph, int idx, long long &t) {
    const long long now = clock64();
    if (lane_id() == 0) ph[idx] += now - t;
    t = now;
}

// first threshold index k with c <= dk[k] (thresholds strictly increasing), K if none
__device__ __forceinline__ int first_k(const PrimalParams &p, float c) {
    int k = 0;
    while (k < p.k && !(c <= p.dk[k])) k++;
    return k;
}

// Dependency lanes of the backward sweep: the node at settle position i holds the lanes of the
// thresholds it lies within (k >= k0(i)), plain and beta-weighted interleaved, packed in settle
// order.  Positions are sorted by cost, so k0 steps up at the boundaries nk[k] (positions with cost
// <= d_k) and the offsets follow from them: lane (i, k, b) sits at lane_index(i) + 2 k + b.
// nk[] and cum[] (cum[k] = lanes held by the positions below nk[k - 1]) are the warp's shared rows.
__device__ __forceinline__ int lane_index(int i, int K, const int *nk, const int *cum) {
    int k0 = 0;
    while (k0 < K && i >= nk[k0]) k0++;
    const int lo = k0 ? nk[k0 - 1] : 0;
    return 2 * (cum[k0] + (i - lo) * (K - k0)) - 2 * k0;
}

// predecessor positions of the node at position i, in registers
template <int PM>
__device__ __forceinline__ int load_preds(const SlotPtrs &s, int i, int P, int *pl) {
    const int np = s.np[i];
#pragma unroll
    for (int r = 0; r < PM; r++) pl[r] = (r < np) ? s.pr[(size_t)i * P + r] : 0;
    return np;
}

// Phase barrier of the block-synchronous forms: GW warps (a whole 8-warp block: __syncthreads;
// 4: a named barrier per half block) meet at the end of each phase.  GW = 0: no barrier.
template <int GW>
__device__ __forceinline__ void phase_barrier() {
    if constexpr (GW == 8) {
        __syncthreads();
    } else if constexpr (GW > 0) {
        asm volatile("bar.sync %0, %1;" ::"r"(1 + (int)(threadIdx.x >> 5) / GW), "r"(GW * 32) : "memory");
    }
}

// With SYNC, every warp of the block runs each phase together (a block barrier ends each phase,
// and a warp without a source runs the phases with R = 0), so at any time a block's warps fetch one
// phase's code; there is no early return in that form.
// Trip weight of the pair (src, v) in the origin-destination rows, 0 when the pair has none.
__device__ __forceinline__ float od_weight(const PrimalParams &p, int src, int v) {
    int lo = __ldg(&p.od_ptr[src]);
    const int end = __ldg(&p.od_ptr[src + 1]);
    int hi = end;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(&p.od_dst[mid]) < v) lo = mid + 1;
        else hi = mid;
    }
    return (lo < end && __ldg(&p.od_dst[lo]) == v) ? __ldg(&p.od_w[lo]) : 0.0f;
}

// OD: betweenness only, seeded per pair by the origin-destination weights instead of the 0.5 / 1.0
// pair counts (rust/src/centrality.rs:2495-2507), source weight 1, written to rows 0 and 1.
template <int PM, int SYNC, bool OD = false>
CS_PHASE_INLINE __device__ void shortest_accumulate(const PrimalParams &p, const SlotPtrs &s, int src, int R, long long *ph,
                                    int *cnt, int *bw_pl, double *bw_fr) {
    const int lane = lane_id();
    bool failed = false;
    long long tph = clock64();
    const int K = p.k;
    const int P = p.P;
    const int N = p.g.n_bound;
    const float wt = OD ? 1.0f : __ldg(&p.src_wt[src]);
    const float cycles_wt = OD ? 0.0f : wt / __ldg(&p.g.node_w_dev[src]);
    const bool closeness = !OD && p.closeness;
    // cnt[0..K): nodes whose first qualifying threshold is k; cnt[MAXK..MAXK+K): same for edges;
    // cnt[2 MAXK..): nk, the positions with cost <= d_k; cnt[3 MAXK..): cum, lanes below nk[k - 1]
    for (int q = lane; q < 2 * MAXK; q += 32) cnt[q] = 0;
    int *nk = cnt + 2 * MAXK, *cum = cnt + 3 * MAXK;
    if (lane < K) {
        int lo = 0, hi = R;  // first position whose cost exceeds d_k
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (route_cost(s.sd[mid], p.speed) <= p.dk[lane]) lo = mid + 1;
            else hi = mid;
        }
        nk[lane] = lo;
    }
    __syncwarp();
    if (lane == 0) {
        int acc = 0, prev = 0;
        for (int k = 0; k < K; k++) {
            cum[k] = acc;
            acc += (nk[k] - prev) * (K - k);
            prev = nk[k];
        }
        cum[K] = acc;
    }
    __syncwarp();
    // --- one pass over out-edges in settle order, 32 nodes at a time: circuit-rank counts, the
    // predecessor replay and, with betweenness, sigma (f64 path counts, as the reference's
    // BrandesTraversalState.sigma) of the chunk: a node is ready once its in-chunk predecessors are
    // done.  The same pass zeroes each node's dependency lanes for the backward sweep.
    bool bad = false;
    double *sig = s.sig;
    double *dl = s.dl;  // dependency lanes, packed (lane_index)
    for (int base = 0; base < R; base += 32) {
        const int i = base + lane;
        const bool act = i < R;
        unsigned pm = 0u;
        Nb<PM> nb;
        if (act) {
            const int v = s.ord[i];
            const float dv = s.sd[i];
            const float cv = route_cost(dv, p.speed);
            const int k0v = first_k(p, cv);
            if (k0v < K) atomicAdd(&cnt[k0v], 1);
            load_nb<PM>(p, s, v, R, nb, bad);
            if (closeness) {
#pragma unroll
                for (int j = 0; j < PM; j++) {
                    if (nb.pos[j] < 0 || !__ldg(&p.g.out_cnt_dev[nb.beg + j])) continue;
                    const float ec = fmaxf(cv, route_cost(nb.d[j], p.speed));
                    const int k0e = first_k(p, ec);
                    if (k0e < K) atomicAdd(&cnt[MAXK + k0e], 1);
                }
            }
            if (p.betweenness) {
                if (i == 0) {
                    s.np[0] = 0;
                } else {
                    bool ok = true;
                    pm = replay_brandes<PM>(p, nb, i, dv, ok);
                    if (!ok) { bad = true; pm = 0u; }
                    int r = 0;
#pragma unroll
                    for (int j = 0; j < PM; j++)
                        if ((pm >> j) & 1u) s.pr[(size_t)i * P + r++] = nb.pos[j];
                    s.np[i] = (uint8_t)r;
                }
            }
        }
        if (!p.betweenness || failed) continue;  // uniform across the warp
        unsigned blk = 0u;  // in-chunk predecessors, as lane bits
#pragma unroll
        for (int j = 0; j < PM; j++)
            if (((pm >> j) & 1u) && nb.pos[j] >= base) blk |= 1u << (nb.pos[j] - base);
        unsigned done = __ballot_sync(FULL, !act);
        bool mine = !act;
        int guard = 0;
        while (done != FULL) {
            const bool ready = !mine && ((blk & ~done) == 0u);
            if (ready) {
                double sg = (i == 0) ? 1.0 : 0.0;
#pragma unroll
                for (int j = 0; j < PM; j++)
                    if ((pm >> j) & 1u) sg = __dadd_rn(sg, sig[nb.pos[j]]);
                sig[i] = sg;
                const int li0 = lane_index(i, K, nk, cum);
                for (int k = first_k(p, route_cost(s.sd[i], p.speed)); k < K; k++) {
                    dl[li0 + 2 * k] = 0.0;
                    dl[li0 + 2 * k + 1] = 0.0;
                }
                mine = true;
            }
            __syncwarp();
            done |= __ballot_sync(FULL, ready);
            if (++guard > 64) break;
        }
        if (done != FULL) {
            if (lane == 0) raise_err(p.hdr, CS_ERR_INTERNAL, 2);
            failed = true;
        }
    }
    if (__any_sync(FULL, bad)) {
        if (lane == 0) raise_err(p.hdr, CS_ERR_INTERNAL, 1);
    }
    __syncwarp();
    phase_barrier<SYNC>();
    phase_mark(ph, 2, tph);
    // --- closeness (rust/src/centrality.rs:1733-1780).  Density, farness and harmonic terms do not
    // depend on the threshold: they go once into the bucket of the first qualifying threshold and a
    // prefix over thresholds after the launch completes them.  Cycles and beta terms are per k.
    if (closeness) {
        // per-threshold circuit-rank weights, computed by lane 0 into the (now free) edge-count half
        // of the warp's shared counters
        float *rankw = (float *)(cnt + MAXK);
        if (lane == 0) {
            long long nc = 0, ec = 0;
            for (int k = 0; k < K; k++) {
                nc += cnt[k];
                ec += cnt[MAXK + k];
                const long long r = ec - nc + 1;
                const float rank = (nc == 0) ? 0.0f : (float)(r > 0 ? r : 0);
                rankw[k] = fmul(rank, cycles_wt);
                if (p.track_reach && nc > 1) atomicAdd(&p.reach[k], (unsigned)(nc - 1));
            }
        }
        __syncwarp();
        const double wt_d = f2d(wt);
        const size_t KN = (size_t)K * N;
        for (int i = 1 + lane; i < R; i += 32) {
            const int t = s.ord[i];
            const float c = route_cost(s.sd[i], p.speed);
            const int k0 = first_k(p, c);
            if (k0 >= K) continue;
            double *bk = p.bucket + (size_t)k0 * N + t;
            atomicAdd(bk, wt_d);
            atomicAdd(bk + KN, f2d(fmul(c, wt)));
            atomicAdd(bk + 2 * KN, f2d(fmul(__fdiv_rn(1.0f, c), wt)));
            for (int k = k0; k < K; k++) {
                double *row = p.out + (size_t)k * N + t;
                atomicAdd(row + 2 * KN, f2d(rankw[k]));
                atomicAdd(row + 4 * KN, f2d(fmul(expf(fmul(-p.beta[k], c)), wt)));
            }
        }
    }
    phase_barrier<SYNC>();
    phase_mark(ph, 3, tph);
    if constexpr (SYNC == 0) {
        if (!p.betweenness) return;
    }
    // in the block-synchronous form the flag can differ between a block's warps (batched jobs):
    // a warp without betweenness runs the remaining phases empty, so every warp meets the barriers
    const int Rb = (SYNC != 0 && !p.betweenness) ? 0 : R;
    // (sigma was built in the replay pass)
    phase_mark(ph, 4, tph);
    // --- backward Brandes sweep, all K thresholds in one pass (rust/src/centrality.rs:823-873,
    // 1782-1835), in the reference's f64: path counts, predecessor factors sigma_v / sigma_w, seeds
    // (pair count, and pair count * exp(-beta * cost) with the product and exp in f64) and
    // dependencies.
    __syncwarp();
    const bool unit_wt = (wt == 1.0f);
    const double wtd = (double)wt;
    const int nchunks = failed ? 0 : (Rb + 31) / 32;
    constexpr int BW = (PM < BW_COLS) ? PM : BW_COLS;  // predecessors kept in this lane's shared column
    for (int ch = nchunks - 1; ch >= 0; ch--) {
        const int base = ch * 32;
        const int i = base + lane;
        const bool act = i < Rb;
        int pl[PM];
        const int np = act ? load_preds<PM>(s, i, P, pl) : 0;
        unsigned pm = 0;
#pragma unroll
        for (int r = 0; r < PM; r++)
            if (r < np && pl[r] >= base) pm |= 1u << (pl[r] - base);
        bool mine = !act;
        unsigned done = __ballot_sync(FULL, mine);
        int guard = 0;
        while (done != FULL) {
            const unsigned blocked = __reduce_or_sync(FULL, mine ? 0u : pm);
            const bool ready = !mine && !((blocked >> lane) & 1u);
            if (ready) {
                const int v = s.ord[i];
                const float cost = route_cost(s.sd[i], p.speed);
                const double sw = sig[i];
                float pairf;
                if constexpr (OD) pairf = od_weight(p, src, v);
                else pairf = __ldg(&p.eligible[v]) ? 0.5f : 1.0f;
                const double pair = f2d(pairf);
                // predecessor rows and factors go to this lane's shared-memory column, so that the
                // push loop below is a plain (not unrolled) loop over the np predecessors
#pragma unroll
                for (int r = 0; r < BW; r++) {
                    if (r < np) {
                        const double sv = sig[pl[r]];
                        bw_pl[r * 32 + lane] = lane_index(pl[r], K, nk, cum);
                        bw_fr[r * 32 + lane] = (sv == sw) ? 1.0 : __ddiv_rn(sv, sw);
                    }
                }
                double *dli = dl + lane_index(i, K, nk, cum);
                const int k0 = first_k(p, cost);
                for (int k = k0; k < K; k++) {
                    if (sw == 0.0) break;
                    const double seed = (i == 0) ? 0.0 : pair;
                    const double seedb = (i == 0 || pairf == 0.0f) ? 0.0 : seed_exp(pairf, p.beta[k], cost);
                    const double dep = __dadd_rn(seed, __ldcg(&dli[2 * k]));
                    const double depb = __dadd_rn(seedb, __ldcg(&dli[2 * k + 1]));
                    if (dep == 0.0 && depb == 0.0) continue;
#pragma unroll 1
                    for (int r = 0; r < np; r++) {
                        int q;
                        double f;
                        if (r < BW) {
                            q = bw_pl[r * 32 + lane];
                            f = bw_fr[r * 32 + lane];
                        } else {  // beyond the shared column (high-degree graphs): from the scratch
                            const int qp = s.pr[(size_t)i * P + r];
                            const double sv = sig[qp];
                            f = (sv == sw) ? 1.0 : __ddiv_rn(sv, sw);
                            q = lane_index(qp, K, nk, cum);
                        }
                        if (f == 0.0) continue;
                        double *pd = dl + q;
                        atomicAdd(&pd[2 * k], f == 1.0 ? dep : __dmul_rn(f, dep));
                        atomicAdd(&pd[2 * k + 1], f == 1.0 ? depb : __dmul_rn(f, depb));
                    }
                    if (v == src) continue;
                    const double credit = __dadd_rn(dep, -seed);
                    const double creditb = __dadd_rn(depb, -seedb);
                    constexpr size_t row_b = OD ? 0 : 5;
                    if (credit > 0.0)
                        atomicAdd(p.out + (row_b * K + k) * N + v, unit_wt ? credit : __dmul_rn(credit, wtd));
                    if (creditb > 0.0)
                        atomicAdd(p.out + ((row_b + 1) * K + k) * N + v, unit_wt ? creditb : __dmul_rn(creditb, wtd));
                }
                mine = true;
            }
            __syncwarp();
            done |= __ballot_sync(FULL, ready);
            if (++guard > 64) break;
        }
        if (done != FULL) {
            if (lane == 0) raise_err(p.hdr, CS_ERR_INTERNAL, 3);
            break;
        }
    }
    phase_barrier<SYNC>();
    phase_mark(ph, 5, tph);
}

// Completes the bucketed closeness rows: out[m][k] += sum_{j<=k} bucket[m][j] for density,
// farness and harmonic (rows 0, 1, 3).
__global__ void bucket_prefix_kernel(const double *bucket, double *out, int K, int N) {
    const size_t KN = (size_t)K * N;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < N; t += gridDim.x * blockDim.x) {
        const int rows[3] = {0, 1, 3};
        for (int m = 0; m < 3; m++) {
            double acc = 0.0;
            for (int k = 0; k < K; k++) {
                acc += bucket[(size_t)m * KN + (size_t)k * N + t];
                out[(size_t)rows[m] * KN + (size_t)k * N + t] += acc;
            }
        }
    }
}

// Batched form: the same prefix for every shortest-path job with closeness (blockIdx.y strides the
// jobs), and the bucket is zeroed as it is read, so that buckets are zero between runs.
__global__ void batch_prefix_kernel(const cs_batch_job *jobs, int n_jobs) {
    for (int j = blockIdx.y; j < n_jobs; j += gridDim.y) {
        const cs_batch_job &jb = jobs[j];
        if ((jb.mode != MODE_SHORTEST && jb.mode != MODE_BOTH) || !jb.compute_closeness || jb.n_sources <= 0)
            continue;
        const int K = jb.k, N = jb.g.n_bound;
        const size_t KN = (size_t)K * N;
        double *bucket = jb.bucket_dev;
        double *out = jb.out_dev;
        for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < N; t += gridDim.x * blockDim.x) {
            const int rows[3] = {0, 1, 3};
            for (int m = 0; m < 3; m++) {
                double acc = 0.0;
                for (int k = 0; k < K; k++) {
                    const size_t o = (size_t)m * KN + (size_t)k * N + t;
                    acc += bucket[o];
                    bucket[o] = 0.0;
                    out[(size_t)rows[m] * KN + (size_t)k * N + t] += acc;
                }
            }
        }
    }
}

// ------------------------------------------------------------------------------------------
// 4b. Segment centrality for one source.
// ------------------------------------------------------------------------------------------
template <int PM>
CS_PHASE_INLINE __device__ void segment_accumulate(const PrimalParams &p, const SlotPtrs &s, int src, int R) {
    const int lane = lane_id();
    const int K = p.k;
    const int N = p.g.n_bound;
    double *const out = (p.mode == MODE_BOTH) ? p.out2 : p.out;  // segment rows
    bool bad = false;
    // single predecessor (strict <) with its last segment length; pred position in pr[i*P]
    for (int i = lane; i < R; i += 32) {
        if (i == 0) { s.pr[0] = -1; s.fa[0] = 0.0f; continue; }
        const int v = s.ord[i];
        Nb<PM> nb;
        load_nb<PM>(p, s, v, R, nb, bad);
        bool ok = true;
        const int q = replay_first_min<PM>(p, nb, i, s.sd[i], ok);
        if (!ok || q < 0) { bad = true; s.pr[(size_t)i * p.P] = -1; continue; }
        int pos = 0;
        float last = 0.0f;
#pragma unroll
        for (int j = 0; j < PM; j++)
            if (j == q) { pos = nb.pos[j]; last = __ldg(&p.g.out_seglen_dev[nb.beg + j]); }
        s.pr[(size_t)i * p.P] = pos;
        s.fa[i] = last;  // last segment length
    }
    if (__any_sync(FULL, bad)) {
        if (lane == 0) raise_err(p.hdr, CS_ERR_INTERNAL, 4);
        return;
    }
    __syncwarp();
    // origin segment length: inherited along the tree (settle order, chunked)
    for (int base = 0; base < R; base += 32) {
        const int i = base + lane;
        const bool act = i < R;
        const int pp = (act && i > 0) ? s.pr[(size_t)i * p.P] : -1;
        const unsigned pm = (pp >= base) ? (1u << (pp - base)) : 0u;
        bool mine = !act;
        if (act && i == 0) { s.fb[0] = 0.0f; mine = true; }
        unsigned done = __ballot_sync(FULL, mine);
        int guard = 0;
        while (done != FULL) {
            const bool ready = !mine && ((pm & ~done) == 0u);
            if (ready) {
                s.fb[i] = (pp == 0) ? s.fa[i] : s.fb[pp];
                mine = true;
            }
            __syncwarp();
            done |= __ballot_sync(FULL, ready);
            if (++guard > 64) break;
        }
        if (done != FULL) {
            if (lane == 0) raise_err(p.hdr, CS_ERR_INTERNAL, 5);
            return;
        }
    }
    // closeness integrals over visited edges (rust/src/centrality.rs:2201-2317), into the source
    // thresholds in groups of 4: per lane 12 f64 accumulators in registers and 4 unrolled copies of
    // the integral code (not 16 of each), one pass over the visited edges per group
    if (p.closeness) for (int kb = 0; kb < K; kb += 4) {
        double acc[12];
#pragma unroll
        for (int q = 0; q < 12; q++) acc[q] = 0.0;
        for (int i = lane; i < R; i += 32) {
            const int u = s.ord[i];
            const float au = route_cost(s.sd[i], p.speed);
            const int beg = __ldg(&p.g.in_ptr_dev[u]);
            const int end = __ldg(&p.g.in_ptr_dev[u + 1]);
            for (int e = beg; e < end; e++) {
                const int nb = __ldg(&p.g.in_nb_dev[e]);
                float bm;
                if (nb == u) {
                    bm = au;
                } else {
                    const uint32_t a = s.aux[nb];
                    if (a > (uint32_t)R) continue;  // cannot happen on clean scratch
                    if (a != 0u && (int)(a - 1) < i) continue;  // neighbour settled earlier
                    bm = (a != 0u) ? route_cost(s.sd[a - 1], p.speed) : __int_as_float(INF_BITS);
                }
                const bool n_nearer = au <= bm;
                const float A = n_nearer ? au : bm, Ai = A;
                const float B = n_nearer ? bm : au, Bi = B;
                const float elen = __ldg(&p.g.in_seglen_dev[e]);
                const float imp = __ldg(&p.g.in_segimp_dev[e]);
                const float C = __fdiv_rn(fadd(fadd(elen, A), B), 2.0f), D = C;
                const float Ci = fadd(Ai, fmul(__fadd_rn(C, -A), imp)), Di = Ci;
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int k = kb + q;
                    if (k >= K) break;
                    const float df = p.dk[k];
                    const float beta = p.beta[k], nbeta = -beta;
                    const float inb = (beta != 0.0f) ? __fdiv_rn(1.0f, nbeta) : 0.0f;
                    if (A < df) {
                        float cc = C, cci = Ci;
                        if (cc > df) { cc = df; cci = fadd(Ai, fmul(__fadd_rn(df, -A), imp)); }
                        acc[q] += (double)__fadd_rn(cc, -A);
                        const float sh = (Ai < 1.0f) ? logf(cci) : logf(fmaxf(__fdiv_rn(cci, Ai), 1.1920929e-07f));
                        acc[4 + q] += (double)sh;
                        const float bet = (beta == 0.0f) ? __fadd_rn(cci, -Ai)
                                                         : fmul(__fadd_rn(expf(fmul(nbeta, cci)), -expf(fmul(nbeta, Ai))), inb);
                        acc[8 + q] += (double)bet;
                    }
                    if (B == D) continue;
                    if (B <= df) {
                        float cd = D, cdi = Di;
                        if (cd > df) { cd = df; cdi = fadd(Bi, fmul(__fadd_rn(df, -B), imp)); }
                        acc[q] += (double)__fadd_rn(cd, -B);
                        const float sh = (Bi < 1.0f) ? logf(cdi) : logf(fmaxf(__fdiv_rn(cdi, Bi), 1.1920929e-07f));
                        acc[4 + q] += (double)sh;
                        const float bet = (beta == 0.0f) ? __fadd_rn(cdi, -Bi)
                                                         : fmul(__fadd_rn(expf(fmul(nbeta, cdi)), -expf(fmul(nbeta, Bi))), inb);
                        acc[8 + q] += (double)bet;
                    }
                }
            }
        }
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int k = kb + q;
            if (k >= K) break;
            const double a0 = warp_sum_d(acc[q]);
            const double a1 = warp_sum_d(acc[4 + q]);
            const double a2 = warp_sum_d(acc[8 + q]);
            if (lane == 0) {
                atomicAdd(out + ((size_t)0 * K + k) * N + src, a0);
                atomicAdd(out + ((size_t)1 * K + k) * N + src, a1);
                atomicAdd(out + ((size_t)2 * K + k) * N + src, a2);
            }
        }
    }
    if (!p.betweenness) return;
    // betweenness: subtree sums of per-target auc (rust/src/centrality.rs:2319-2401)
    double *acc = s.dl;  // [R][K]
    for (int i = lane; i < R; i += 32)
        for (int k = 0; k < K; k++) acc[(size_t)i * K + k] = 0.0;
    __syncwarp();
    const int nchunks = (R + 31) / 32;
    for (int ch = nchunks - 1; ch >= 0; ch--) {
        const int base = ch * 32;
        const int i = base + lane;
        const bool act = i < R;
        const int pp = (act && i > 0) ? s.pr[(size_t)i * p.P] : -1;
        const unsigned pm = (pp >= base) ? (1u << (pp - base)) : 0u;
        bool mine = !act;
        unsigned done = __ballot_sync(FULL, mine);
        int guard = 0;
        while (done != FULL) {
            const unsigned blocked = __reduce_or_sync(FULL, mine ? 0u : pm);
            const bool ready = !mine && !((blocked >> lane) & 1u);
            if (ready) {
                const int v = s.ord[i];
                const float sdist = route_cost(s.sd[i], p.speed);
                const float o_len = s.fb[i], l_len = s.fa[i];
                const float min_span = __fadd_rn(__fadd_rn(sdist, -o_len), -l_len);
                const float o_1 = min_span, o_2 = fadd(min_span, o_len);
                const float l_1 = min_span, l_2 = fadd(min_span, l_len);
                const bool own = (i > 0) && (v > src);
                for (int k = 0; k < K; k++) {
                    const double below = __ldcg(&acc[(size_t)i * K + k]);
                    double total = below;
                    if (own) {
                        const float df = p.dk[k];
                        const float beta = p.beta[k];
                        if (min_span <= df) {
                            const float o2s = fminf(o_2, df), l2s = fminf(l_2, df);
                            float auc;
                            if (beta == 0.0f) auc = fadd(__fadd_rn(o2s, -o_1), __fadd_rn(l2s, -l_1));
                            else {
                                const float nb = -beta, inb = __fdiv_rn(1.0f, nb);
                                auc = fadd(fmul(__fadd_rn(expf(fmul(nb, o2s)), -expf(fmul(nb, o_1))), inb),
                                           fmul(__fadd_rn(expf(fmul(nb, l2s)), -expf(fmul(nb, l_1))), inb));
                            }
                            if (isfinite(auc) && auc >= 0.0f) total += (double)auc;
                        }
                    }
                    if (i > 0 && v != src && below > 0.0) atomicAdd(out + ((size_t)3 * K + k) * N + v, below);
                    if (pp >= 0 && total != 0.0) atomicAdd(&acc[(size_t)pp * K + k], total);
                }
                mine = true;
            }
            __syncwarp();
            done |= __ballot_sync(FULL, ready);
            if (++guard > 64) break;
        }
        if (done != FULL) {
            if (lane == 0) raise_err(p.hdr, CS_ERR_INTERNAL, 6);
            return;
        }
    }
}

// ------------------------------------------------------------------------------------------
// 4c. Shortest-path tree rows (isochrone query).
// ------------------------------------------------------------------------------------------
template <int PM>
CS_PHASE_INLINE __device__ void tree_rows(const PrimalParams &p, const SlotPtrs &s, int qidx, int R) {
    const int lane = lane_id();
    if (R > p.row_cap) {
        if (lane == 0) p.t_count[qidx] = -R;  // rows too narrow: report the reach only
        return;
    }
    bool bad = false;
    for (int i = lane; i < R; i += 32) {
        const int v = s.ord[i];
        int pred = -1;
        if (i > 0) {
            Nb<PM> nb;
            load_nb<PM>(p, s, v, R, nb, bad);
            bool ok = true;
            const int q = replay_first_min<PM>(p, nb, i, s.sd[i], ok);
            if (!ok || q < 0) bad = true;
            else {
#pragma unroll
                for (int j = 0; j < PM; j++)
                    if (j == q) pred = s.ord[nb.pos[j]];
            }
        }
        const size_t o = (size_t)qidx * p.row_cap + i;
        p.t_node[o] = v;
        p.t_agg[o] = s.sd[i];
        p.t_pred[o] = pred;
    }
    if (__any_sync(FULL, bad) && lane == 0) raise_err(p.hdr, CS_ERR_INTERNAL, 7);
    if (lane == 0) p.t_count[qidx] = R;
}

// ------------------------------------------------------------------------------------------
// 4d. Accessibility of one source (rust/src/data.rs:513-602 aggregate_to_src_idx, :688-731).
//     Over the reached nodes (the search's distances are dijkstra_tree_shortest's), each assigned
//     entry's total distance (network + assignment, f32); an entry counts when it is the nearest
//     of its dedupe key (ties: the lower (node seconds, node, rank in the node's list), the
//     reference keeping the first one it meets), and adds to its class's rows.
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ void access_accumulate(const PrimalParams &p, const SlotPtrs &s, int src, int R) {
    const int lane = lane_id();
    const cs_data_map &dm = p.dm;
    const int K = p.k, N = p.g.n_bound;
    const float maxs = p.maxsec;
    const float max_walk = fmul(maxs, p.speed);
    for (int i = lane; i < R; i += 32) {
        const int v = s.rl[i];
        const float sec = __ldcg(&s.dist[v]);
        if (!(sec < maxs)) continue;
        const float net = fmul(sec, p.speed);
        const int a_end = __ldg(&dm.node_ptr_dev[v + 1]);
        for (int a = __ldg(&dm.node_ptr_dev[v]); a < a_end; a++) {
            const float tot = fadd(net, __ldg(&dm.assign_dist_dev[a]));
            if (!(tot <= max_walk)) continue;
            const int e = __ldg(&dm.assign_entry_dev[a]);
            const int grp = __ldg(&dm.entry_group_dev[e]);
            const int rank = __ldg(&dm.assign_rank_dev[a]);
            bool win = true;
            const int g_end = __ldg(&dm.group_ptr_dev[grp + 1]);
            for (int b = __ldg(&dm.group_ptr_dev[grp]); b < g_end && win; b++) {
                const int a2 = __ldg(&dm.group_assign_dev[b]);
                if (a2 == a) continue;
                const int v2 = __ldg(&dm.assign_node_dev[a2]);
                const float sec2 = __ldcg(&s.dist[v2]);  // +inf when not reached
                if (!(sec2 < maxs)) continue;
                const float tot2 = fadd(fmul(sec2, p.speed), __ldg(&dm.assign_dist_dev[a2]));
                if (!(tot2 <= max_walk)) continue;
                if (tot2 < tot) win = false;
                else if (tot2 == tot) {
                    const int r2 = __ldg(&dm.assign_rank_dev[a2]);
                    if (sec2 < sec || (sec2 == sec && (v2 < v || (v2 == v && r2 < rank)))) win = false;
                }
            }
            if (!win) continue;
            const int c = __ldg(&dm.entry_class_dev[e]);
            if (c < 0) continue;
            for (int k = 0; k < K; k++) {
                if (!(tot <= p.dk[k])) continue;
                const size_t o = ((size_t)c * K + k) * N + src;
                atomicAdd(&p.acc_unw[o], 1.0);
                // clipped_beta_wt (rust/src/common.rs:339-348)
                const float raw = expf(fmul(-p.beta[k], tot));
                atomicAdd(&p.acc_wt[o], f2d(__fdiv_rn(fminf(raw, p.mcw[k]), p.mcw[k])));
                if (p.dk[k] == p.max_dist) atomicMin(&p.acc_near[(size_t)c * N + src], __float_as_uint(tot));
            }
        }
    }
}

// ------------------------------------------------------------------------------------------
// Persistent kernel: each warp owns one scratch slot and pulls sources until the list is empty.
// ------------------------------------------------------------------------------------------
// One source on this warp's slot: search, sort, mode-specific accumulation, scratch reset.
// Returns false when the source overflowed the slot's capacity (recorded for the retry).
// MODE is the accumulation compiled in (a kernel per mode keeps each kernel's code, and so its
// instruction-cache footprint, to what that mode runs); -1 dispatches on p.mode at run time.
template <int PM, int MODE>
__device__ __forceinline__ bool run_source(const PrimalParams &p, const SlotPtrs &s, int li, int src, uint32_t *hist,
                                           int *cnt, int *bw_pl, double *bw_fr, long long *ph, long long &relaxed,
                                           long long &settled) {
    const int lane = lane_id();
    long long t0 = clock64();
    float dmax = 0.0f;
    const int R = warp_search(p, s, src, relaxed, dmax);
    phase_mark(ph, 0, t0);
    if (R < 0) {
        // Reach exceeded this slot's capacity: the reached list lost track of touched entries, so
        // reset the slot's whole dense state, record the source for the full-capacity retry and
        // carry on with the next source.
        for (int j = lane; j < p.g.n_bound; j += 32) {
            s.dist[j] = __int_as_float(INF_BITS);
            s.aux[j] = 0u;
        }
        if (lane == 0) {
            const unsigned f = atomicAdd(&p.hdr->n_failed, 1u);
            if (f < (unsigned)p.fail_cap) p.failed[f] = li;
            else raise_err(p.hdr, CS_ERR_CAPACITY, 8);
        }
        __syncwarp();
        return false;
    }
    if constexpr (MODE == MODE_ACCESS) {
        // no settle order needed: the reached list and the distances suffice
        access_accumulate(p, s, src, R);
        __syncwarp();
        for (int i = lane; i < R; i += 32) s.dist[s.rl[i]] = __int_as_float(INF_BITS);
        __syncwarp();
        settled += R;
        return true;
    }
    warp_sort(p, s, R, dmax, hist);
    __syncwarp();
    for (int i = lane; i < R; i += 32) s.aux[s.ord[i]] = (uint32_t)(i + 1);
    __syncwarp();
    phase_mark(ph, 1, t0);
    if constexpr (MODE == MODE_SHORTEST) {
        shortest_accumulate<PM, 0>(p, s, src, R, ph, cnt, bw_pl, bw_fr);
    } else if constexpr (MODE == MODE_SEGMENT) {
        segment_accumulate<PM>(p, s, src, R);
    } else if constexpr (MODE == MODE_TREE) {
        tree_rows<PM>(p, s, li, R);
    } else if constexpr (MODE == MODE_OD) {
        shortest_accumulate<PM, 0, true>(p, s, src, R, ph, cnt, bw_pl, bw_fr);
    } else {
        if (p.mode == MODE_SHORTEST) shortest_accumulate<PM, 0>(p, s, src, R, ph, cnt, bw_pl, bw_fr);
        else if (p.mode == MODE_SEGMENT) segment_accumulate<PM>(p, s, src, R);
        else if (p.mode == MODE_BOTH) {
            // one search and settle order serve both: shortest rows, then segment rows (its own
            // single-predecessor replay over the same positions)
            shortest_accumulate<PM, 0>(p, s, src, R, ph, cnt, bw_pl, bw_fr);
            __syncwarp();
            segment_accumulate<PM>(p, s, src, R);
        } else tree_rows<PM>(p, s, li, R);
    }
    __syncwarp();
    t0 = clock64();
    for (int i = lane; i < R; i += 32) {
        const int v = s.ord[i];
        s.dist[v] = __int_as_float(INF_BITS);
        s.aux[v] = 0u;
    }
    __syncwarp();
    phase_mark(ph, 6, t0);
    settled += R;
    return true;
}

__device__ __forceinline__ void flush_counters(const PrimalParams &p, long long *ph, long long relaxed,
                                               long long settled, long long done_src) {
    const long long rsum = warp_sum_ll(relaxed);
    __syncwarp();
    if (lane_id() == 0) {
        for (int q = 0; q < 8; q++) atomicAdd(&p.hdr->pad[q], (unsigned long long)ph[q]);
        atomicAdd(&p.hdr->edges_relaxed, (unsigned long long)rsum);
        atomicAdd(&p.hdr->nodes_settled, (unsigned long long)settled);
        atomicAdd(&p.hdr->sources_done, (unsigned long long)done_src);
    }
}

// ------------------------------------------------------------------------------------------
// Persistent kernel: each warp owns one scratch slot and pulls sources until the list is empty.
// ------------------------------------------------------------------------------------------
// Segment centrality with a block's warps in lockstep (as primal_sync_kernel for shortest paths):
// search | sort | accumulation + scratch reset, each phase closed by a block barrier that every warp
// meets (a warp without a source, or whose source overflowed, runs the phases empty).
template <int PM>
__device__ __forceinline__ bool run_segment_sync(const PrimalParams &p, const SlotPtrs &s, bool mine, int li, int src,
                                                 uint32_t *hist, long long *ph, long long &relaxed,
                                                 long long &settled) {
    const int lane = lane_id();
    long long t0 = clock64();
    float dmax = 0.0f;
    int R = 0;
    if (mine) R = warp_search(p, s, src, relaxed, dmax);
    phase_mark(ph, 0, t0);
    __syncthreads();
    const bool live = mine && R >= 0;
    if (mine && R < 0) {
        for (int j = lane; j < p.g.n_bound; j += 32) {
            s.dist[j] = __int_as_float(INF_BITS);
            s.aux[j] = 0u;
        }
        if (lane == 0) {
            const unsigned f = atomicAdd(&p.hdr->n_failed, 1u);
            if (f < (unsigned)p.fail_cap) p.failed[f] = li;
            else raise_err(p.hdr, CS_ERR_CAPACITY, 8);
        }
        __syncwarp();
    }
    if (live) {
        warp_sort(p, s, R, dmax, hist);
        __syncwarp();
        for (int i = lane; i < R; i += 32) s.aux[s.ord[i]] = (uint32_t)(i + 1);
        __syncwarp();
    }
    phase_mark(ph, 1, t0);
    __syncthreads();
    if (live) {
        segment_accumulate<PM>(p, s, src, R);
        __syncwarp();
        t0 = clock64();
        for (int i = lane; i < R; i += 32) {
            const int v = s.ord[i];
            s.dist[v] = __int_as_float(INF_BITS);
            s.aux[v] = 0u;
        }
        __syncwarp();
        phase_mark(ph, 6, t0);
        settled += R;
    }
    __syncthreads();
    return live;
}

template <int PM, int MINB>
__global__ void __launch_bounds__(256, MINB) segment_sync_kernel(const PrimalParams p) {
    __shared__ uint32_t hist_all[8][256];
    __shared__ long long ph_all[8][8];
    __shared__ unsigned long long blk_base;
    __shared__ unsigned blk_err;
    const int lane = lane_id();
    const int wib = threadIdx.x >> 5;
    const int slot0 = blockIdx.x * (blockDim.x >> 5);
    const int nw = min((int)(blockDim.x >> 5), p.n_slots - slot0);
    const bool has_slot = wib < nw;
    const SlotPtrs s = slot_ptrs(p.dense, p.dense_stride, p.compact, (size_t)p.cap, p.P, p.L,
                                 has_slot ? slot0 + wib : 0, p.g.n_bound);
    long long relaxed = 0, settled = 0, done_src = 0;
    long long *ph = ph_all[wib];
    if (lane < 8) ph[lane] = 0;
    __syncwarp();
    while (true) {
        if (threadIdx.x == 0) {
            blk_base = atomicAdd(p.rerun ? &p.hdr->work_next2 : &p.hdr->work_next, (unsigned long long)max(nw, 0));
            blk_err = __ldcg(&p.hdr->err);
        }
        __syncthreads();
        const unsigned long long b0 = blk_base;
        const unsigned berr = blk_err;
        __syncthreads();
        if (nw <= 0 || b0 >= (unsigned long long)p.n_src || berr != 0u) break;
        const unsigned long long idx = b0 + wib;
        const bool mine = has_slot && idx < (unsigned long long)p.n_src;
        const int li = mine ? (p.remap ? p.remap[idx] : (int)idx) : 0;
        const int src = mine ? p.src_list[li] : 0;
        if (run_segment_sync<PM>(p, s, mine, li, src, hist_all[wib], ph, relaxed, settled)) {
            done_src++;
            if (lane == 0) count_progress(p.hdr);
        }
    }
    if (has_slot) flush_counters(p, ph, relaxed, settled, done_src);
}

template <int PM, int MINB, int MODE>
__global__ void __launch_bounds__(256, MINB) primal_kernel(const PrimalParams p) {
    __shared__ uint32_t hist_all[8][256];
    __shared__ int cnt_all[8][4 * MAXK + 2];
    __shared__ long long ph_all[8][8];
    // backward sweep: each lane's predecessor rows and sigma fractions (column-major per warp)
    __shared__ int bw_pl_all[8][bw_cols(PM) * 32];
    __shared__ double bw_fr_all[8][bw_cols(PM) * 32];
    const int lane = lane_id();
    const int wib = threadIdx.x >> 5;
    const int slot = (int)((blockIdx.x * (blockDim.x >> 5)) + wib);
    if (slot >= p.n_slots) return;
    const SlotPtrs s = slot_ptrs(p.dense, p.dense_stride, p.compact, (size_t)p.cap, p.P, p.L, slot, p.g.n_bound);
    long long relaxed = 0, settled = 0, done_src = 0;
    long long *ph = ph_all[wib];
    if (lane < 8) ph[lane] = 0;
    __syncwarp();
    while (true) {
        unsigned long long idx = 0;
        if (lane == 0) idx = atomicAdd(p.rerun ? &p.hdr->work_next2 : &p.hdr->work_next, 1ull);
        idx = __shfl_sync(FULL, idx, 0);
        if (idx >= (unsigned long long)p.n_src) break;
        if (__ldcg(&p.hdr->err) != 0u) break;
        const int li = p.remap ? p.remap[idx] : (int)idx;
        if (run_source<PM, MODE>(p, s, li, p.src_list[li], hist_all[wib], cnt_all[wib], bw_pl_all[wib], bw_fr_all[wib],
                                 ph, relaxed, settled)) {
            done_src++;
            if (lane == 0) count_progress(p.hdr);
        }
    }
    flush_counters(p, ph, relaxed, settled, done_src);
}

// ------------------------------------------------------------------------------------------
// Shortest-path form with block-synchronous phases: a block claims one source per warp, and its
// warps run search, sort, replay, closeness, sigma, backward and reset together, a block barrier
// between phases.  At any time a block fetches one phase's code, so the SM's instruction caches
// hold the code of at most one phase per resident block.  Every warp reaches every barrier: a warp
// without a source (or whose source overflowed) runs the phases with R = 0.
// ------------------------------------------------------------------------------------------
template <int PM, int MINB, int WPB, int GW>
__global__ void __launch_bounds__(WPB * 32, MINB) primal_sync_kernel(const PrimalParams p) {
    __shared__ uint32_t hist_all[WPB][256];
    __shared__ int cnt_all[WPB][4 * MAXK + 2];
    __shared__ long long ph_all[WPB][8];
    __shared__ int bw_pl_all[WPB][bw_cols(PM) * 32];
    __shared__ double bw_fr_all[WPB][bw_cols(PM) * 32];
    __shared__ long long blk_base[WPB / GW];
    __shared__ unsigned blk_err[WPB / GW];
    const int lane = lane_id();
    const int wib = threadIdx.x >> 5;
    const int grp = wib / GW, gw = wib % GW;  // phase group of GW warps
    const int slot0 = blockIdx.x * (blockDim.x >> 5) + grp * GW;
    const int nw = min(GW, p.n_slots - slot0);  // warps of this group with a slot
    const bool has_slot = gw < nw;
    const SlotPtrs s = slot_ptrs(p.dense, p.dense_stride, p.compact, (size_t)p.cap, p.P, p.L,
                                 has_slot ? slot0 + gw : 0, p.g.n_bound);
    long long relaxed = 0, settled = 0, done_src = 0;
    long long *ph = ph_all[wib];
    if (lane < 8) ph[lane] = 0;
    __syncwarp();
    const long long n = p.n_src;
    while (true) {
        if (gw == 0 && lane == 0) {
            blk_base[grp] = (long long)atomicAdd(p.rerun ? &p.hdr->work_next2 : &p.hdr->work_next,
                                                 (unsigned long long)max(nw, 0));
            blk_err[grp] = __ldcg(&p.hdr->err);
        }
        phase_barrier<GW>();
        const long long base = blk_base[grp];
        const unsigned berr = blk_err[grp];
        phase_barrier<GW>();
        if (nw <= 0 || base >= n || berr != 0u) break;
        const long long idx = base + gw;
        const bool mine = has_slot && idx < n;
        const int li = mine ? (p.remap ? p.remap[idx] : (int)idx) : 0;
        const int src = mine ? p.src_list[li] : 0;
        long long t0 = clock64();
        int R = 0;
        float dmax = 0.0f;
        if (mine) R = warp_search(p, s, src, relaxed, dmax);
        phase_mark(ph, 0, t0);
        phase_barrier<GW>();
        const bool ok = mine && R >= 0;
        if (mine && R < 0) {
            for (int j = lane; j < p.g.n_bound; j += 32) {
                s.dist[j] = __int_as_float(INF_BITS);
                s.aux[j] = 0u;
            }
            if (lane == 0) {
                const unsigned f = atomicAdd(&p.hdr->n_failed, 1u);
                if (f < (unsigned)p.fail_cap) p.failed[f] = li;
                else raise_err(p.hdr, CS_ERR_CAPACITY, 8);
            }
        }
        if (ok) {
            warp_sort(p, s, R, dmax, hist_all[wib]);
            __syncwarp();
            for (int i = lane; i < R; i += 32) s.aux[s.ord[i]] = (uint32_t)(i + 1);
        }
        __syncwarp();
        phase_mark(ph, 1, t0);
        phase_barrier<GW>();
        shortest_accumulate<PM, GW>(p, s, src, ok ? R : 0, ph, cnt_all[wib], bw_pl_all[wib], bw_fr_all[wib]);
        __syncwarp();
        t0 = clock64();
        if (ok) {
            for (int i = lane; i < R; i += 32) {
                const int v = s.ord[i];
                s.dist[v] = __int_as_float(INF_BITS);
                s.aux[v] = 0u;
            }
            settled += R;
            done_src++;
            if (lane == 0) count_progress(p.hdr);
        }
        __syncwarp();
        phase_mark(ph, 6, t0);
        phase_barrier<GW>();
    }
    flush_counters(p, ph, relaxed, settled, done_src);
}

// ------------------------------------------------------------------------------------------
// Batched persistent kernel: one launch over the (job, source) items of many graphs, thresholds
// and modes.  Item i belongs to the job whose item_begin is the largest <= i.  Every warp's slot
// is sized for the largest graph, capacity and lane count of the batch.
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ int job_of(const cs_batch_job *jobs, int n_jobs, long long item) {
    int lo = 0, hi = n_jobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].item_begin <= item) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ void job_params(const PrimalParams &base, const cs_batch_job &j, PrimalParams &p) {
    p = base;
    p.g = j.g;
    p.k = j.k;
    uint32_t maxs = 0;
    for (int i = 0; i < MAXK; i++) {
        p.dk[i] = i < j.k ? (float)j.distances[i] : 0.0f;
        p.beta[i] = i < j.k ? j.betas[i] : 0.0f;
        if (i < j.k) maxs = max(maxs, j.seconds[i]);
    }
    p.maxsec = (float)maxs;
    p.speed = j.speed_m_s;
    p.tol = j.tolerance;
    p.delta = j.delta_seconds > 0.0f ? j.delta_seconds : fmaxf(1.0f, p.maxsec / 48.0f);
    p.closeness = j.compute_closeness;
    p.betweenness = j.compute_betweenness;
    p.track_reach = 0;
    p.src_list = j.sources_dev;
    p.n_src = j.n_sources;
    p.src_wt = j.src_wt_dev;
    p.eligible = j.eligible_dev;
    p.out = j.out_dev;
    p.bucket = j.bucket_dev;
    p.out2 = j.out2_dev;
    p.mode = j.mode;
}

// MODE: the accumulation compiled in (0 shortest, 1 segment), or -1 to dispatch on each job's
// mode; a launch covers items [item_lo, item_hi) (or, in a re-run, the listed items).
template <int PM, int MINB, int MODE>
__global__ void __launch_bounds__(256, MINB) batch_kernel(const PrimalParams base, const cs_batch_job *jobs,
                                                          int n_jobs, long long item_lo, long long item_hi) {
    __shared__ uint32_t hist_all[8][256];
    __shared__ int cnt_all[8][4 * MAXK + 2];
    __shared__ long long ph_all[8][8];
    // backward sweep: each lane's predecessor rows and sigma fractions (column-major per warp)
    __shared__ int bw_pl_all[8][bw_cols(PM) * 32];
    __shared__ double bw_fr_all[8][bw_cols(PM) * 32];
    const int lane = lane_id();
    const int wib = threadIdx.x >> 5;
    const int slot = (int)((blockIdx.x * (blockDim.x >> 5)) + wib);
    if (slot >= base.n_slots) return;
    // slot geometry from the batch maxima (base.g.n_bound = largest graph)
    const SlotPtrs s = slot_ptrs(base.dense, base.dense_stride, base.compact, (size_t)base.cap, base.P, base.L, slot,
                                 base.g.n_bound);
    long long relaxed = 0, settled = 0, done_src = 0;
    long long *ph = ph_all[wib];
    if (lane < 8) ph[lane] = 0;
    // the warp's job parameters live in shared memory: a local copy of the (large) parameter block
    // sits in the stack frame, and its loads then miss L1 under the kernel's global traffic
    __shared__ PrimalParams pj_all[8];
    PrimalParams &p = pj_all[wib];
    __syncwarp();
    int cur_job = -1;
    while (true) {
        unsigned long long idx = 0;
        if (lane == 0) idx = atomicAdd(base.rerun ? &base.hdr->work_next2 : &base.hdr->work_next, 1ull);
        idx = __shfl_sync(FULL, idx, 0);
        const long long n = base.rerun ? base.n_src : item_hi - item_lo;
        if ((long long)idx >= n) break;
        if (__ldcg(&base.hdr->err) != 0u) break;
        const long long item = base.remap ? (long long)base.remap[idx] : item_lo + (long long)idx;
        const int jb = job_of(jobs, n_jobs, item);
        if (jb != cur_job) {
            if (lane == 0) job_params(base, jobs[jb], p);
            __syncwarp();
            cur_job = jb;
        }
        const int li = (int)(item - jobs[jb].item_begin);
        // failures record the global item index
        if (run_source<PM, MODE>(p, s, (int)item, p.src_list[li], hist_all[wib], cnt_all[wib], bw_pl_all[wib],
                                 bw_fr_all[wib], ph, relaxed, settled)) {
            done_src++;
            if (lane == 0) count_progress(base.hdr);
        }
    }
    flush_counters(base, ph, relaxed, settled, done_src);
}

// Batched shortest-path items with block-synchronous phases (as primal_sync_kernel): a block
// claims one item per warp; each warp looks its item's job up.  Every warp reaches every barrier.
template <int PM, int MINB>
__global__ void __launch_bounds__(256, MINB) batch_sync_kernel(const PrimalParams base, const cs_batch_job *jobs,
                                                               int n_jobs, long long item_lo, long long item_hi) {
    __shared__ uint32_t hist_all[8][256];
    __shared__ int cnt_all[8][4 * MAXK + 2];
    __shared__ long long ph_all[8][8];
    __shared__ int bw_pl_all[8][bw_cols(PM) * 32];
    __shared__ double bw_fr_all[8][bw_cols(PM) * 32];
    __shared__ long long blk_base;
    __shared__ unsigned blk_err;
    const int lane = lane_id();
    const int wib = threadIdx.x >> 5;
    const int slot0 = blockIdx.x * (blockDim.x >> 5);
    const int nw = min((int)(blockDim.x >> 5), base.n_slots - slot0);
    const bool has_slot = wib < nw;
    const SlotPtrs s = slot_ptrs(base.dense, base.dense_stride, base.compact, (size_t)base.cap, base.P, base.L,
                                 has_slot ? slot0 + wib : 0, base.g.n_bound);
    long long relaxed = 0, settled = 0, done_src = 0;
    long long *ph = ph_all[wib];
    if (lane < 8) ph[lane] = 0;
    __syncwarp();
    const long long n = item_hi - item_lo;
    __shared__ PrimalParams pj_all[8];  // the warps' job parameters (as in batch_kernel)
    PrimalParams &p = pj_all[wib];
    int cur_job = -1;
    while (true) {
        if (threadIdx.x == 0) {
            blk_base = (long long)atomicAdd(&base.hdr->work_next, (unsigned long long)max(nw, 0));
            blk_err = __ldcg(&base.hdr->err);
        }
        __syncthreads();
        const long long b0 = blk_base;
        const unsigned berr = blk_err;
        __syncthreads();
        if (nw <= 0 || b0 >= n || berr != 0u) break;
        const long long idx = b0 + wib;
        const bool mine = has_slot && idx < n;
        int src = 0, li = 0;
        const long long item = item_lo + idx;
        if (mine) {
            const int jb = job_of(jobs, n_jobs, item);
            if (jb != cur_job) {
                if (lane == 0) job_params(base, jobs[jb], p);
                __syncwarp();
                cur_job = jb;
            }
            li = (int)(item - jobs[jb].item_begin);
            src = p.src_list[li];
        } else if (cur_job < 0) {
            if (lane == 0) job_params(base, jobs[0], p);  // an idle warp still runs the phases (R = 0)
            __syncwarp();
            cur_job = 0;
        }
        long long t0 = clock64();
        int R = 0;
        float dmax = 0.0f;
        if (mine) R = warp_search(p, s, src, relaxed, dmax);
        phase_mark(ph, 0, t0);
        __syncthreads();
        const bool ok = mine && R >= 0;
        if (mine && R < 0) {
            for (int j = lane; j < p.g.n_bound; j += 32) {
                s.dist[j] = __int_as_float(INF_BITS);
                s.aux[j] = 0u;
            }
            if (lane == 0) {
                const unsigned f = atomicAdd(&base.hdr->n_failed, 1u);
                if (f < (unsigned)base.fail_cap) base.failed[f] = (int)item;
                else raise_err(base.hdr, CS_ERR_CAPACITY, 8);
            }
        }
        if (ok) {
            warp_sort(p, s, R, dmax, hist_all[wib]);
            __syncwarp();
            for (int i = lane; i < R; i += 32) s.aux[s.ord[i]] = (uint32_t)(i + 1);
        }
        __syncwarp();
        phase_mark(ph, 1, t0);
        __syncthreads();
        // every warp of the block runs the phases with the same closeness / betweenness flags
        // only when its jobs agree on them; the barrier count must not depend on the job
        shortest_accumulate<PM, 8>(p, s, ok ? src : 0, ok ? R : 0, ph, cnt_all[wib], bw_pl_all[wib],
                                   bw_fr_all[wib]);
        __syncwarp();
        t0 = clock64();
        if (ok) {
            for (int i = lane; i < R; i += 32) {
                const int v = s.ord[i];
                s.dist[v] = __int_as_float(INF_BITS);
                s.aux[v] = 0u;
            }
            settled += R;
            done_src++;
            if (lane == 0) count_progress(p.hdr);
        }
        __syncwarp();
        phase_mark(ph, 6, t0);
        __syncthreads();
    }
    flush_counters(base, ph, relaxed, settled, done_src);
}

// Source-indexed plan on the device (prepare_source_sampling with source_indices): src_wt = node
// weight and eligible = 1 at each listed source, 0 elsewhere.  Pass 0 clears, pass 1 scatters.
__global__ void source_weights_kernel(const int32_t *sources, long long n, const float *node_w, int n_bound,
                                      float *src_wt, uint8_t *eligible, int pass) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (pass == 0) {
        for (; t < n_bound; t += stride) {
            src_wt[t] = 0.0f;
            eligible[t] = 0u;
        }
    } else {
        for (; t < n; t += stride) {
            const int s = sources[t];
            if (s < 0 || s >= n_bound) continue;
            src_wt[s] = node_w[s];
            eligible[s] = 1u;
        }
    }
}

__global__ void fill_dense_kernel(char *dense, size_t dense_stride, int n_bound, const int32_t *slots, int n_list,
                                  int all_slots) {
    // Resets dist (=inf) and aux (=0) of the listed slots (or of slots [0, all_slots)).
    const int n_sl = slots ? n_list : all_slots;
    const size_t per = (size_t)n_bound;
    const size_t total = per * (size_t)n_sl;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const int si = (int)(t / per);
        const size_t j = t % per;
        const int slot = slots ? slots[si] : si;
        char *d = dense + dense_stride * (size_t)slot;
        ((float *)d)[j] = __int_as_float(INF_BITS);
        ((uint32_t *)(d + al256(per * 4)))[j] = 0u;
    }
}

}  // namespace cs


// ==========================================================================================
// Host side (C-ABI).
// ==========================================================================================
namespace cs_host {
thread_local std::string g_last_error;
thread_local long long g_counters[4] = {0, 0, 0, 0};
thread_local long long g_phase[16] = {};
}

extern "C" void cs_set_error_internal(const char *msg) { cs_host::g_last_error = msg ? msg : ""; }

namespace cs_host {
thread_local long long g_retries[2] = {0, 0};
}
extern "C" void cs_set_retries_internal(long long overflowed, long long inexact) {
    cs_host::g_retries[0] = overflowed;
    cs_host::g_retries[1] = inexact;
}
// Phase cycle sums and diagnostics of the last call (the header's pad[0..15]); the dual host code
// sets them too.
extern "C" void cs_set_phase_internal(const unsigned long long *pad) {
    for (int i = 0; i < 16; i++) cs_host::g_phase[i] = (long long)pad[i];
}
// Device counters of the last call (sources done, edges relaxed, states settled, launches).
extern "C" void cs_set_counters_internal(long long sources, long long relaxed, long long settled, long long launches) {
    cs_host::g_counters[0] = sources;
    cs_host::g_counters[1] = relaxed;
    cs_host::g_counters[2] = settled;
    cs_host::g_counters[3] = launches;
}
extern "C" cs_status cs_last_retries(int64_t *overflowed, int64_t *inexact) {
    if (overflowed) *overflowed = cs_host::g_retries[0];
    if (inexact) *inexact = cs_host::g_retries[1];
    return CS_OK;
}

namespace {
using cs_host::g_counters;
using cs_host::g_phase;

cs_status fail(cs_status code, const std::string &msg) {
    cs_host::g_last_error = msg;
    return code;
}
cs_status cuda_fail(cudaError_t e, const char *what) {
    return fail(CS_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int sm_count() {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    return n;
}

struct Layout {
    size_t hdr_off, failed_off, failed2_off, bucket_off, dense_off, compact_off, compact_total, cta_off, total;
    size_t dense_stride;
    int fail_cap;
};

// sources that overflow their slot are listed for the in-call retry; beyond this many the call
// reports CS_ERR_CAPACITY (plan a larger cap)
int fail_capacity(int n_slots) { return std::max(n_slots, 1 << 18); }

// cta_blocks: blocks of the block-per-source kernel whose global scratch follows the per-warp regions.
Layout layout(int n_bound, int n_slots, int cap, int P, int L, int cta_blocks = 0) {
    Layout l;
    l.hdr_off = 0;
    l.failed_off = 256;
    l.fail_cap = fail_capacity(n_slots);
    l.failed2_off = cs::al256(l.failed_off + sizeof(int32_t) * (size_t)l.fail_cap);
    l.bucket_off = cs::al256(l.failed2_off + sizeof(int32_t) * (size_t)l.fail_cap);
    l.dense_off = cs::al256(l.bucket_off + sizeof(double) * 3 * (size_t)L * (size_t)n_bound);
    l.dense_stride = cs::al256((size_t)n_bound * 4) * 2;
    l.compact_off = l.dense_off + l.dense_stride * (size_t)n_slots;
    l.compact_total = cs::compact_bytes((size_t)cap, P, L) * (size_t)n_slots;
    // the in-call retry runs at cap = n_bound on the same compact region: keep room for one slot
    l.compact_total = std::max(l.compact_total, cs::compact_bytes((size_t)n_bound, P, L));
    l.cta_off = cs::al256(l.compact_off + l.compact_total);
    l.total = l.cta_off + cs::cta::scratch_bytes() * (size_t)std::max(0, cta_blocks);
    return l;
}

// Items that overflowed their slot's capacity run again at 4x the capacity (then 4x again, up to
// cap = full_n, where nothing can overflow), each level on as many slots as the compact region
// holds at that capacity; overflows of one level are listed for the next.  `run` launches one
// level: run(params, slots).  Leaves the last header in h.
template <typename Launch>
cs_status retry_chain(const cs::PrimalParams &p, const cs_plan *plan, const Layout &lay, char *base, int full_n, int P,
                      cs::WsHeader &h, cudaStream_t stream, bool poll, Launch run) {
    int32_t *listA = (int32_t *)(base + lay.failed_off);
    int32_t *listB = (int32_t *)(base + lay.failed2_off);
    const int32_t *list = listA;
    unsigned n_in = h.n_failed;
    int cap_l = (int)std::min<long long>(full_n, 4ll * std::max(plan->cap, 8));
    while (n_in > 0u) {
        if (n_in > (unsigned)lay.fail_cap) return fail(CS_ERR_CAPACITY, "more overflowed sources than the list holds");
        int32_t *out_l = (list == listA) ? listB : listA;
        cs::PrimalParams p2 = p;
        p2.cap = cap_l;
        p2.rerun = 1;
        p2.remap = list;
        p2.n_src = (int64_t)n_in;
        p2.failed = out_l;
        cudaError_t e = cudaMemsetAsync(&p.hdr->work_next2, 0, sizeof(unsigned long long), stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(&p.hdr->n_failed, 0, sizeof(unsigned), stream);
        if (e != cudaSuccess) return cuda_fail(e, "retry counter reset");
        const size_t per = cs::compact_bytes((size_t)cap_l, P, plan->lanes);
        int slots2 = (int)std::min<size_t>(lay.compact_total / per, (size_t)plan->n_slots);
        slots2 = std::max(1, std::min<int>(slots2, (int)n_in));
        cs_status st = run(p2, slots2);
        if (st != CS_OK) return st;
        e = cs::read_header(p.hdr, h, stream, poll);
        if (e != cudaSuccess) return cuda_fail(e, "retry kernel");
        if (h.err != 0u)
            return fail((cs_status)h.err, "device-side check failed in retry (code " + std::to_string(h.err) + ")");
        if (cap_l >= full_n && h.n_failed > 0u) return fail(CS_ERR_INTERNAL, "overflow at full capacity");
        n_in = h.n_failed;
        list = out_l;
        cap_l = (int)std::min<long long>(full_n, 4ll * cap_l);
    }
    return CS_OK;
}

int lanes_for(int mode, int k) {
    return (mode == cs::MODE_SHORTEST || mode == cs::MODE_BOTH || mode == cs::MODE_OD) ? 2 * k
                                                                                      : (mode == cs::MODE_SEGMENT ? k : 1);
}

cs_status validate_primal(const cs_primal_graph *g) {
    if (!g) return fail(CS_ERR_ARG, "graph is NULL");
    if (g->n_bound <= 0) return fail(CS_ERR_ARG, "NetworkStructure contains no nodes.");
    if (g->max_out_degree > CS_MAX_DEGREE)
        return fail(CS_ERR_ARG, "node out-degree " + std::to_string(g->max_out_degree) + " exceeds CS_MAX_DEGREE");
    return CS_OK;
}

// Register budget of the P <= 8 kernels: 4 resident 256-thread blocks per SM (64 registers), 3
// (80 registers) or 2 (128 registers).  A plan's variant field (2-4) or the environment variable
// CS_MIN_BLOCKS_PER_SM selects one for every launch.  Otherwise (variant 0) plans are sized for 4
// blocks, the most slots, and each launch picks by mode: 3 for shortest-path and OD centrality (on the
// 202,500-node lattice 4 blocks ran 395 ms per pass against 372 ms with 3, the spills of the
// dependency pass outweighing the extra warps), 4 for segments, trees and accessibility (segment
// centrality on the 250x250 curved lattice: 2.67M sources/s against 2.49M with 3).
int requested_variant(const cs_plan *plan) {
    if (plan && plan->variant >= 2 && plan->variant <= 4) return plan->variant;
    const char *e = getenv("CS_MIN_BLOCKS_PER_SM");
    return (e && e[0] >= '2' && e[0] <= '4') ? e[0] - '0' : 0;
}
// the budget a plan's slot count is sized for
int resolve_variant(const cs_plan *plan) {
    const int v = requested_variant(plan);
    return v ? v : 4;
}
// the budget one launch of a mode runs with
int launch_variant(const cs_plan *plan, int mode) {
    const int v = requested_variant(plan);
    if (v) return v;
    return (mode == cs::MODE_SHORTEST || mode == cs::MODE_OD) ? 3 : 4;
}

cudaError_t occupancy_blocks(int P, int variant, int *bpsm) {
    if (P > 8)
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bpsm, cs::primal_kernel<CS_MAX_DEGREE, 2, 0>, 256, 0);
    if (variant == 4) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bpsm, cs::primal_kernel<8, 4, 0>, 256, 0);
    if (variant == 3) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bpsm, cs::primal_kernel<8, 3, 0>, 256, 0);
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bpsm, cs::primal_kernel<8, 2, 0>, 256, 0);
}

// Block-synchronous phases for the shortest-path mode (CS_PHASE_SYNC=0 selects the per-warp form).
bool phase_sync() {
    const char *e = getenv("CS_PHASE_SYNC");
    return !(e && e[0] == '0');
}

// Block-per-source kernel for shortest-path and OD calls; CS_BLOCK_PER_SOURCE=0 in the environment
// leaves every source to the per-warp kernel (plans then hold no scratch for it).
bool block_kernel_enabled() {
    const char *e = getenv("CS_BLOCK_PER_SOURCE");
    return !(e && e[0] == '0');
}

// Schedule of one call: one block per source gives a source a whole SM (the lowest latency per
// source) and one warp per source keeps ~24 sources per SM in flight (the highest throughput).  Calls
// with at most CS_BLOCK_SOURCES_MAX sources (default: 4 per SM) take the block kernel, larger ones
// the per-warp kernel; CS_BLOCK_PER_SOURCE=1 forces the block kernel.  On the 202,500-node lattice
// at 5 km a call of 8-152 sources took 1.2 ms with blocks and 5.0-5.3 ms with warps, 608 sources
// 4.3 ms against 6.2 ms, and 1,216 sources 8.2 ms against 7.7 ms.
bool block_schedule(long long n_src) {
    const char *e = getenv("CS_BLOCK_PER_SOURCE");
    if (e && e[0] == '0') return false;
    if (e && e[0] == '1') return true;
    const char *m = getenv("CS_BLOCK_SOURCES_MAX");
    const long long cap = m ? atoll(m) : 4ll * std::max(1, sm_count());
    return n_src <= cap;
}

// Settle-order sort: distance buckets by default, CS_SORT=radix selects the LSD radix sort.
int radix_sort_choice() {
    const char *e = getenv("CS_SORT");
    return (e && strcmp(e, "radix") == 0) ? 1 : 0;
}

template <int MODE>
void launch_primal_mode(const cs::PrimalParams &p, int P, int minb, int blocks, cudaStream_t stream) {
    if (MODE == cs::MODE_SHORTEST && P <= 8 && phase_sync()) {
        // whole 8-warp blocks in lockstep: on the 202,500-node lattice 12- and 24-warp blocks ran no
        // faster and 4-warp groups (named barriers) 3% slower
        if (minb == 4) cs::primal_sync_kernel<8, 4, 8, 8><<<blocks, 256, 0, stream>>>(p);
        else if (minb == 3) cs::primal_sync_kernel<8, 3, 8, 8><<<blocks, 256, 0, stream>>>(p);
        else cs::primal_sync_kernel<8, 2, 8, 8><<<blocks, 256, 0, stream>>>(p);
        return;
    }
    if (MODE == cs::MODE_SEGMENT && P <= 8 && phase_sync()) {
        if (minb == 4) cs::segment_sync_kernel<8, 4><<<blocks, 256, 0, stream>>>(p);
        else if (minb == 3) cs::segment_sync_kernel<8, 3><<<blocks, 256, 0, stream>>>(p);
        else cs::segment_sync_kernel<8, 2><<<blocks, 256, 0, stream>>>(p);
        return;
    }
    if (P <= 8) {
        if (minb == 4) cs::primal_kernel<8, 4, MODE><<<blocks, 256, 0, stream>>>(p);
        else if (minb == 3) cs::primal_kernel<8, 3, MODE><<<blocks, 256, 0, stream>>>(p);
        else cs::primal_kernel<8, 2, MODE><<<blocks, 256, 0, stream>>>(p);
    } else {
        cs::primal_kernel<CS_MAX_DEGREE, 2, MODE><<<blocks, 256, 0, stream>>>(p);
    }
}

cs_status launch_primal(cs::PrimalParams &p, const cs_plan *plan, int n_slots, cudaStream_t stream) {
    const int tpb = 256;
    const int wpb = tpb / 32;
    const int minb = launch_variant(plan, p.mode);
    int blocks = (n_slots + wpb - 1) / wpb;
    if (p.P <= 8 && minb < resolve_variant(plan)) {
        // a tighter launch than the plan's slots were sized for: the blocks that are resident at once
        blocks = std::max(1, std::min(blocks, std::max(1, sm_count()) * minb));
        n_slots = std::min(n_slots, blocks * wpb);
    }
    p.n_slots = n_slots;
    if (p.mode == cs::MODE_SHORTEST) launch_primal_mode<cs::MODE_SHORTEST>(p, p.P, minb, blocks, stream);
    else if (p.mode == cs::MODE_SEGMENT) launch_primal_mode<cs::MODE_SEGMENT>(p, p.P, minb, blocks, stream);
    else if (p.mode == cs::MODE_OD) launch_primal_mode<cs::MODE_OD>(p, p.P, minb, blocks, stream);
    else if (p.mode == cs::MODE_ACCESS) launch_primal_mode<cs::MODE_ACCESS>(p, p.P, minb, blocks, stream);
    else launch_primal_mode<cs::MODE_TREE>(p, p.P, minb, blocks, stream);
    g_counters[3]++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "primal_kernel launch");
    return CS_OK;
}

template <int MODE>
void launch_batch_mode(const cs::PrimalParams &p, int minb, int blocks, const cs_batch_job *jobs_dev, int n_jobs,
                       long long lo, long long hi, cudaStream_t stream) {
    if (p.P <= 8) {
        if (minb == 4) cs::batch_kernel<8, 4, MODE><<<blocks, 256, 0, stream>>>(p, jobs_dev, n_jobs, lo, hi);
        else if (minb == 3) cs::batch_kernel<8, 3, MODE><<<blocks, 256, 0, stream>>>(p, jobs_dev, n_jobs, lo, hi);
        else cs::batch_kernel<8, 2, MODE><<<blocks, 256, 0, stream>>>(p, jobs_dev, n_jobs, lo, hi);
    } else {
        cs::batch_kernel<CS_MAX_DEGREE, 2, MODE><<<blocks, 256, 0, stream>>>(p, jobs_dev, n_jobs, lo, hi);
    }
}

// mode: the jobs' common mode (0 or 1) for a mode-specialised kernel, else -1
cs_status launch_batch(cs::PrimalParams &p, const cs_plan *plan, const cs_batch_job *jobs_dev, int n_jobs,
                       long long item_lo, long long item_hi, int n_slots, int mode, cudaStream_t stream) {
    // mixed-mode launches (and reruns) take the shortest-path budget
    const int minb = launch_variant(plan, mode == cs::MODE_SEGMENT ? cs::MODE_SEGMENT : cs::MODE_SHORTEST);
    int blocks = (n_slots + 7) / 8;
    if (p.P <= 8 && minb < resolve_variant(plan)) {
        blocks = std::max(1, std::min(blocks, std::max(1, sm_count()) * minb));
        n_slots = std::min(n_slots, blocks * 8);
    }
    p.n_slots = n_slots;
    if (mode == cs::MODE_SHORTEST && p.P <= 8 && !p.rerun && phase_sync()) {
        if (minb == 4) cs::batch_sync_kernel<8, 4><<<blocks, 256, 0, stream>>>(p, jobs_dev, n_jobs, item_lo, item_hi);
        else if (minb == 3) cs::batch_sync_kernel<8, 3><<<blocks, 256, 0, stream>>>(p, jobs_dev, n_jobs, item_lo, item_hi);
        else cs::batch_sync_kernel<8, 2><<<blocks, 256, 0, stream>>>(p, jobs_dev, n_jobs, item_lo, item_hi);
    } else if (mode == cs::MODE_SHORTEST)
        launch_batch_mode<cs::MODE_SHORTEST>(p, minb, blocks, jobs_dev, n_jobs, item_lo, item_hi, stream);
    else if (mode == cs::MODE_SEGMENT)
        launch_batch_mode<cs::MODE_SEGMENT>(p, minb, blocks, jobs_dev, n_jobs, item_lo, item_hi, stream);
    else
        launch_batch_mode<-1>(p, minb, blocks, jobs_dev, n_jobs, item_lo, item_hi, stream);
    g_counters[3]++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "batch_kernel launch");
    return CS_OK;
}

// Tabulates exp(-j / 256) for the beta-weighted seeds (cs_seed.cuh) on the call's stream.
cs_status launch_seed_table(cudaStream_t stream) {
    cs::seed_table_kernel<<<(cs::SEED_TAB + 255) / 256, 256, 0, stream>>>();
    g_counters[3]++;
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CS_OK : cuda_fail(e, "seed_table_kernel launch");
}

cs_status reset_dense(char *dense, size_t stride, int n_bound, int n_slots, cudaStream_t stream) {
    const size_t total = (size_t)n_bound * (size_t)n_slots;
    int blocks = (int)std::min<size_t>((total + 255) / 256, (size_t)sm_count() * 16);
    if (blocks < 1) blocks = 1;
    cs::fill_dense_kernel<<<blocks, 256, 0, stream>>>(dense, stride, n_bound, nullptr, 0, n_slots);
    g_counters[3]++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "fill_dense_kernel launch");
    return CS_OK;
}

cs_status run_primal(const cs_primal_graph *g, const cs_query *q, const cs_plan *plan, void *ws, size_t ws_bytes,
                     cs_outputs out, void *stream_v, int mode, int32_t row_cap, int32_t *t_count, int32_t *t_node,
                     float *t_agg, int32_t *t_pred, const int32_t *tree_src, int32_t n_tree, uint32_t tree_maxsec,
                     float tree_speed, bool poll = false, const int32_t *od_ptr = nullptr,
                     const int32_t *od_dst = nullptr, const float *od_w = nullptr) {
    cs_status st = validate_primal(g);
    if (st != CS_OK) return st;
    if (!plan || !ws) return fail(CS_ERR_ARG, "plan/workspace is NULL");
    const int P = std::max(1, g->max_out_degree);
    const int K = (mode == cs::MODE_TREE) ? 1 : q->k;
    if (K < 1 || K > CS_MAX_THRESHOLDS) return fail(CS_ERR_ARG, "threshold count out of range");
    const int L = lanes_for(mode, K);
    if (plan->lanes < L) return fail(CS_ERR_ARG, "plan was made for fewer thresholds");
    if (plan->n_bound > 0 && plan->n_bound != g->n_bound)
        return fail(CS_ERR_ARG, "plan was made for a graph of another node bound");
    const bool block = (mode == cs::MODE_SHORTEST || mode == cs::MODE_OD) && plan->cta_blocks > 0 &&
                       cs::cta::supported(P, K) && q && block_schedule(q->n_sources);
    Layout lay = layout(g->n_bound, plan->n_slots, plan->cap, P, plan->lanes, plan->cta_blocks);
    if (ws_bytes < lay.total) return fail(CS_ERR_ARG, "workspace too small for this plan");
    cudaStream_t stream = (cudaStream_t)stream_v;
    char *base = (char *)ws;
    cs::PrimalParams p;
    memset(&p, 0, sizeof(p));
    p.radix_sort = radix_sort_choice();
    p.g = *g;
    p.k = K;
    uint32_t maxs = 0;
    if (mode == cs::MODE_TREE) {
        maxs = tree_maxsec;
        p.speed = tree_speed;
        p.tol = cs::TIE_EPSILON;
        p.src_list = tree_src;
        p.n_src = n_tree;
    } else {
        if (!q) return fail(CS_ERR_ARG, "query is NULL");
        for (int i = 0; i < K; i++) {
            p.dk[i] = (float)q->distances[i];
            p.beta[i] = q->betas[i];
            maxs = std::max(maxs, q->seconds[i]);
        }
        p.speed = q->speed_m_s;
        p.tol = q->tolerance;
        p.closeness = q->compute_closeness;
        p.betweenness = q->compute_betweenness;
        p.track_reach = q->track_reach;
        p.src_list = q->sources_dev;
        p.n_src = q->n_sources;
        p.src_wt = q->src_wt_dev;
        p.eligible = q->eligible_dev;
        if (mode == cs::MODE_OD) {
            if (p.n_src > 0 && (!od_ptr || !od_dst || !od_w))
                return fail(CS_ERR_ARG, "origin-destination rows are NULL");
            p.closeness = 0;
            p.betweenness = 1;
            p.track_reach = 0;
            p.od_ptr = od_ptr;
            p.od_dst = od_dst;
            p.od_w = od_w;
        }
        if (p.track_reach && !out.reach_dev) return fail(CS_ERR_ARG, "reach_dev required when track_reach");
        if (!out.out_dev) return fail(CS_ERR_ARG, "out_dev is NULL");
    }
    if (!(p.speed > 0.0f) || !std::isfinite(p.speed)) return fail(CS_ERR_ARG, "speed_m_s must be finite and positive");
    p.maxsec = (float)maxs;
    p.delta = plan->delta_seconds > 0.0f ? plan->delta_seconds : std::max(1.0f, p.maxsec / 48.0f);
    p.out = out.out_dev;
    p.bucket = (double *)(base + lay.bucket_off);
    p.reach = out.reach_dev;
    p.hdr = (cs::WsHeader *)(base + lay.hdr_off);
    p.failed = (int32_t *)(base + lay.failed_off);
    p.fail_cap = lay.fail_cap;
    p.dense = base + lay.dense_off;
    p.dense_stride = lay.dense_stride;
    p.compact = base + lay.compact_off;
    p.cap = plan->cap;
    p.P = P;
    p.L = plan->lanes;
    p.mode = mode;
    p.row_cap = row_cap;
    p.t_count = t_count;
    p.t_node = t_node;
    p.t_agg = t_agg;
    p.t_pred = t_pred;
    g_counters[0] = g_counters[1] = g_counters[2] = g_counters[3] = 0;
    if (p.n_src <= 0) return CS_OK;
    cudaError_t e = cudaMemsetAsync(p.hdr, 0, sizeof(cs::WsHeader), stream);
    if (e != cudaSuccess) return cuda_fail(e, "workspace header reset");
    const bool bucketed = (mode == cs::MODE_SHORTEST) && p.closeness;
    if (bucketed) {
        e = cudaMemsetAsync(p.bucket, 0, sizeof(double) * 3 * (size_t)K * (size_t)g->n_bound, stream);
        if (e != cudaSuccess) return cuda_fail(e, "bucket reset");
    }
    if (p.betweenness && (mode == cs::MODE_SHORTEST || mode == cs::MODE_OD)) {
        st = launch_seed_table(stream);
        if (st != CS_OK) return st;
    }
    if (block) {
        // one block per source with its state on chip; the sources it lists (reach or queues beyond
        // its capacity) run through the per-warp kernel's capacity chain below
        e = cs::cta::launch_seed_table(stream);
        if (e != cudaSuccess) return cuda_fail(e, "seed table launch");
        cs::cta::Params c;
        memset(&c, 0, sizeof(c));
        c.n_bound = g->n_bound;
        c.in_ptr = g->in_ptr_dev;
        c.in_nb = g->in_nb_dev;
        c.in_w = g->in_w_dev;
        c.out_ptr = g->out_ptr_dev;
        c.out_to = g->out_to_dev;
        c.out_w = g->out_w_dev;
        c.out_cnt = g->out_cnt_dev;
        c.node_w = g->node_w_dev;
        c.k = K;
        for (int i = 0; i < K; i++) {
            c.dk[i] = p.dk[i];
            c.beta[i] = p.beta[i];
        }
        c.maxsec = p.maxsec;
        c.speed = p.speed;
        c.tol = p.tol;
        // the block kernel's rounds are paced by barriers: wider bands (fewer rounds, more
        // re-relaxations) suit it; CS_BLOCK_DELTA_SCALE overrides the width factor
        {
            const char *ev = getenv("CS_BLOCK_DELTA_SCALE");
            const float scale = ev ? (float)atof(ev) : 4.0f;
            c.delta = (scale > 0.0f) ? p.delta * scale : p.delta;
        }
        c.closeness = p.closeness;
        c.betweenness = p.betweenness;
        c.track_reach = p.track_reach;
        c.od = (mode == cs::MODE_OD) ? 1 : 0;
        c.src_list = p.src_list;
        c.n_src = p.n_src;
        c.src_wt = p.src_wt;
        c.eligible = p.eligible;
        c.od_ptr = p.od_ptr;
        c.od_dst = p.od_dst;
        c.od_w = p.od_w;
        c.out = p.out;
        c.bucket = p.bucket;
        c.reach = p.reach;
        c.hdr = p.hdr;
        c.failed = p.failed;
        c.fail_cap = p.fail_cap;
        c.scratch = base + lay.cta_off;
        c.scratch_stride = cs::cta::scratch_bytes();
        e = cs::cta::launch(c, plan->cta_blocks, stream);
        g_counters[3] += 2;
        if (e != cudaSuccess) return cuda_fail(e, "source_block_kernel launch");
    } else {
        st = launch_primal(p, plan, plan->n_slots, stream);
        if (st != CS_OK) return st;
    }
    cs::WsHeader h;
    e = cs::read_header(p.hdr, h, stream, poll);
    if (e != cudaSuccess) return cuda_fail(e, "centrality kernel");
    if (h.err != 0u)
        return fail((cs_status)h.err, "device-side check failed (code " + std::to_string(h.err) + " at " +
                                          std::to_string(h.err_where) + ")");
    long long done = (long long)h.sources_done, rel = (long long)h.edges_relaxed, set = (long long)h.nodes_settled;
    const long long n_over = h.n_failed;
    if (h.n_failed > 0u) {
        // Sources whose reach overflowed `cap` (their slots already reset themselves)
        st = retry_chain(p, plan, lay, base, g->n_bound, P, h, stream, poll,
                         [&](cs::PrimalParams &p2, int slots2) { return launch_primal(p2, plan, slots2, stream); });
        if (st != CS_OK) return st;
        done = (long long)h.sources_done;
        rel = (long long)h.edges_relaxed;
        set = (long long)h.nodes_settled;
    }
    if (bucketed) {
        int blocks = std::max(1, std::min((g->n_bound + 255) / 256, sm_count() * 8));
        cs::bucket_prefix_kernel<<<blocks, 256, 0, stream>>>(p.bucket, p.out, K, g->n_bound);
        g_counters[3]++;
        e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_fail(e, "bucket_prefix_kernel launch");
    }
    g_counters[0] = done;
    g_counters[1] = rel;
    g_counters[2] = set;
    for (int i = 0; i < 16; i++) cs_host::g_phase[i] = (long long)h.pad[i];
    cs_set_retries_internal(n_over, 0);
    return CS_OK;
}

cs_status plan_common(int n_bound, int P, int L, int cap, int max_slots, int64_t budget, cs_plan *plan,
                      bool block_kernel = false) {
    const int variant = resolve_variant(plan);
    if (!plan) return fail(CS_ERR_ARG, "plan is NULL");
    int sms = sm_count();
    if (sms <= 0) return fail(CS_ERR_CUDA, "no CUDA device");
    int bpsm = 0;
    cudaError_t e = occupancy_blocks(P, variant, &bpsm);
    if (e != cudaSuccess) return cuda_fail(e, "occupancy query");
    if (bpsm < 1) bpsm = 1;
    int slots = sms * bpsm * 8;
    if (max_slots > 0) slots = std::min(slots, max_slots);
    if (cap <= 0) cap = std::min(n_bound, 16384);
    cap = std::max(32, std::min(cap, n_bound));
    const int cta_blocks = block_kernel ? sms : 0;
    auto total_for = [&](int ns) { return layout(n_bound, ns, cap, P, L, cta_blocks).total; };
    if (budget > 0) {
        while (slots > 8 && (int64_t)total_for(slots) > budget) slots = (slots * 7) / 8;
    }
    slots = std::max(1, slots);
    plan->n_slots = slots;
    plan->cap = cap;
    plan->threads_per_block = 256;
    plan->blocks = (slots + 7) / 8;
    if (plan->delta_seconds != plan->delta_seconds) plan->delta_seconds = 0.0f;
    plan->lanes = L;
    plan->variant = requested_variant(plan);  // 0: each launch picks its budget by mode
    plan->max_degree = P;
    plan->n_bound = n_bound;
    plan->cta_blocks = cta_blocks;
    plan->workspace_bytes = total_for(slots);
    return CS_OK;
}

}  // namespace

extern "C" {

size_t cs_last_error(char *buf, size_t len) {
    const std::string &m = cs_host::g_last_error;
    const size_t n = m.size();
    if (buf && len) {
        const size_t c = std::min(n, len - 1);
        memcpy(buf, m.data(), c);
        buf[c] = 0;
    }
    return n;
}

int32_t cs_device_sm_count(void) { return sm_count(); }

cs_status cs_last_phase_cycles(int64_t *cycles, int32_t n) {
    if (!cycles || n < 0) return fail(CS_ERR_ARG, "cycles is NULL");
    for (int i = 0; i < n && i < 16; i++) cycles[i] = cs_host::g_phase[i];
    return CS_OK;
}

cs_status cs_last_counters(int64_t *sources, int64_t *edges_relaxed, int64_t *nodes_settled, int64_t *launches) {
    if (sources) *sources = g_counters[0];
    if (edges_relaxed) *edges_relaxed = g_counters[1];
    if (nodes_settled) *nodes_settled = g_counters[2];
    if (launches) *launches = g_counters[3];
    return CS_OK;
}

cs_status cs_plan_primal(const cs_primal_graph *g, int32_t mode, int32_t k, int32_t cap, int32_t max_slots,
                         int64_t mem_budget_bytes, cs_plan *plan) {
    cs_status st = validate_primal(g);
    if (st != CS_OK) return st;
    if (mode < 0 || mode > 2) return fail(CS_ERR_ARG, "unknown mode");
    if (mode != cs::MODE_TREE && (k < 1 || k > CS_MAX_THRESHOLDS)) return fail(CS_ERR_ARG, "threshold count out of range");
    const int P = std::max(1, g->max_out_degree);
    const float keep_delta = plan ? plan->delta_seconds : 0.0f;
    if (plan) plan->delta_seconds = keep_delta;
    const bool block = mode == cs::MODE_SHORTEST && block_kernel_enabled() && cs::cta::supported(P, k);
    return plan_common(g->n_bound, P, lanes_for(mode, mode == cs::MODE_TREE ? 1 : k), cap, max_slots,
                       mem_budget_bytes, plan, block);
}

cs_status cs_workspace_init(const cs_plan *plan, int32_t n_bound, void *workspace_dev, size_t workspace_bytes,
                            void *stream) {
    if (!plan || !workspace_dev) return fail(CS_ERR_ARG, "plan/workspace is NULL");
    if (workspace_bytes < plan->workspace_bytes) return fail(CS_ERR_ARG, "workspace smaller than plan");
    if (plan->lanes < 1) return fail(CS_ERR_ARG, "plan has no lanes");
    // the dense region's offset depends only on (n_bound, n_slots, lanes): same as every call
    Layout lay = layout(n_bound, plan->n_slots, plan->cap, 1, plan->lanes);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(workspace_dev, 0, 256, s);
    if (e != cudaSuccess) return cuda_fail(e, "workspace init");
    return reset_dense((char *)workspace_dev + lay.dense_off, lay.dense_stride, n_bound, plan->n_slots, s);
}

cs_status cs_centrality_shortest(const cs_primal_graph *g, const cs_query *q, const cs_plan *plan,
                                 void *workspace_dev, size_t workspace_bytes, cs_outputs out, void *stream) {
    return run_primal(g, q, plan, workspace_dev, workspace_bytes, out, stream, cs::MODE_SHORTEST, 0, nullptr, nullptr,
                      nullptr, nullptr, nullptr, 0, 0, 0.0f, true);
}

cs_status cs_betweenness_od_shortest(const cs_primal_graph *g, const cs_query *q, const int32_t *od_ptr_dev,
                                     const int32_t *od_dst_dev, const float *od_w_dev, const cs_plan *plan,
                                     void *workspace_dev, size_t workspace_bytes, cs_outputs out, void *stream) {
    return run_primal(g, q, plan, workspace_dev, workspace_bytes, out, stream, cs::MODE_OD, 0, nullptr, nullptr,
                      nullptr, nullptr, nullptr, 0, 0, 0.0f, true, od_ptr_dev, od_dst_dev, od_w_dev);
}

cs_status cs_segment_centrality(const cs_primal_graph *g, const cs_query *q, const cs_plan *plan,
                                void *workspace_dev, size_t workspace_bytes, cs_outputs out, void *stream) {
    return run_primal(g, q, plan, workspace_dev, workspace_bytes, out, stream, cs::MODE_SEGMENT, 0, nullptr, nullptr,
                      nullptr, nullptr, nullptr, 0, 0, 0.0f, true);
}

cs_status cs_tree_shortest(const cs_primal_graph *g, int32_t n_queries, const int32_t *src_dev, uint32_t max_seconds,
                           float speed_m_s, const cs_plan *plan, void *workspace_dev, size_t workspace_bytes,
                           int32_t row_cap, int32_t *count_dev, int32_t *node_dev, float *agg_seconds_dev,
                           int32_t *pred_dev, void *stream) {
    if (!count_dev || !node_dev || !agg_seconds_dev || !pred_dev || row_cap <= 0)
        return fail(CS_ERR_ARG, "tree outputs missing");
    cs_outputs o{nullptr, nullptr};
    return run_primal(g, nullptr, plan, workspace_dev, workspace_bytes, o, stream, cs::MODE_TREE, row_cap, count_dev,
                      node_dev, agg_seconds_dev, pred_dev, src_dev, n_queries, max_seconds, speed_m_s, true);
}

cs_status cs_accessibility(const cs_primal_graph *g, const cs_data_map *dm, const cs_query *q,
                           const float *max_curve_wts, int32_t n_classes, const cs_plan *plan, void *workspace_dev,
                           size_t workspace_bytes, double *unweighted_dev, double *weighted_dev,
                           uint32_t *nearest_dev, void *stream) {
    cs_status st = validate_primal(g);
    if (st != CS_OK) return st;
    if (!dm || !q || !max_curve_wts || !plan || !workspace_dev) return fail(CS_ERR_ARG, "accessibility: NULL argument");
    if (q->k < 1 || q->k > CS_MAX_THRESHOLDS) return fail(CS_ERR_ARG, "threshold count out of range");
    if (n_classes < 0) return fail(CS_ERR_ARG, "accessibility: negative class count");
    if (q->n_sources > 0 && (!dm->node_ptr_dev || !dm->assign_entry_dev || !dm->assign_dist_dev ||
                             !dm->assign_node_dev || !dm->assign_rank_dev || !dm->entry_group_dev ||
                             !dm->entry_class_dev || !dm->group_ptr_dev || !dm->group_assign_dev))
        return fail(CS_ERR_ARG, "accessibility: data map array is NULL");
    if (n_classes > 0 && q->n_sources > 0 && (!unweighted_dev || !weighted_dev || !nearest_dev))
        return fail(CS_ERR_ARG, "accessibility: output is NULL");
    for (int i = 0; i < q->k; i++)
        if (!(max_curve_wts[i] > 0.0f && max_curve_wts[i] <= 1.0f))
            return fail(CS_ERR_ARG, "Max curve weight must be in the range [0, 1].");
    const int P = std::max(1, g->max_out_degree);
    Layout lay = layout(g->n_bound, plan->n_slots, plan->cap, P, plan->lanes, plan->cta_blocks);
    if (workspace_bytes < lay.total) return fail(CS_ERR_ARG, "workspace too small for this plan");
    if (plan->n_bound > 0 && plan->n_bound != g->n_bound)
        return fail(CS_ERR_ARG, "plan was made for a graph of another node bound");
    cudaStream_t stream_c = (cudaStream_t)stream;
    char *base = (char *)workspace_dev;
    cs::PrimalParams p;
    memset(&p, 0, sizeof(p));
    p.g = *g;
    p.k = q->k;
    uint32_t maxs = 0, maxd = 0;
    for (int i = 0; i < q->k; i++) {
        p.dk[i] = (float)q->distances[i];
        p.beta[i] = q->betas[i];
        p.mcw[i] = max_curve_wts[i];
        maxs = std::max(maxs, q->seconds[i]);
        maxd = std::max(maxd, q->distances[i]);
    }
    p.max_dist = (float)maxd;
    p.speed = q->speed_m_s;
    if (!(p.speed > 0.0f) || !std::isfinite(p.speed)) return fail(CS_ERR_ARG, "speed_m_s must be finite and positive");
    p.tol = cs::TIE_EPSILON;
    p.maxsec = (float)maxs;
    p.delta = plan->delta_seconds > 0.0f ? plan->delta_seconds : std::max(1.0f, p.maxsec / 48.0f);
    p.src_list = q->sources_dev;
    p.n_src = q->n_sources;
    p.dm = *dm;
    p.acc_unw = unweighted_dev;
    p.acc_wt = weighted_dev;
    p.acc_near = nearest_dev;
    p.hdr = (cs::WsHeader *)(base + lay.hdr_off);
    p.failed = (int32_t *)(base + lay.failed_off);
    p.fail_cap = lay.fail_cap;
    p.dense = base + lay.dense_off;
    p.dense_stride = lay.dense_stride;
    p.compact = base + lay.compact_off;
    p.cap = plan->cap;
    p.P = P;
    p.L = plan->lanes;
    p.mode = cs::MODE_ACCESS;
    p.radix_sort = radix_sort_choice();
    g_counters[0] = g_counters[1] = g_counters[2] = g_counters[3] = 0;
    if (p.n_src <= 0 || n_classes == 0) return CS_OK;
    cudaError_t e = cudaMemsetAsync(p.hdr, 0, sizeof(cs::WsHeader), stream_c);
    if (e != cudaSuccess) return cuda_fail(e, "workspace header reset");
    st = launch_primal(p, plan, plan->n_slots, stream_c);
    if (st != CS_OK) return st;
    cs::WsHeader h;
    e = cs::read_header(p.hdr, h, stream_c, true);
    if (e != cudaSuccess) return cuda_fail(e, "accessibility kernel");
    if (h.err != 0u) return fail((cs_status)h.err, "device-side check failed (code " + std::to_string(h.err) + ")");
    if (h.n_failed > 0u) {
        st = retry_chain(p, plan, lay, base, g->n_bound, P, h, stream_c, true,
                         [&](cs::PrimalParams &p2, int slots2) { return launch_primal(p2, plan, slots2, stream_c); });
        if (st != CS_OK) return st;
    }
    g_counters[0] = (long long)h.sources_done;
    g_counters[1] = (long long)h.edges_relaxed;
    g_counters[2] = (long long)h.nodes_settled;
    return CS_OK;
}

}  // extern "C"

// ==========================================================================================
// Allocation-free entry point (cs_centrality_shortest_noalloc).
//
// Some callers cannot allocate device memory at the time they want centralities: code running
// inside a host application that owns every device allocation through its own pool, plugins whose
// memory budget is fixed when the process starts, or code paths where an allocation could fail or
// block.  For them this entry point draws its scratch from one static device array that the CUDA
// module reserves when it is loaded, so the call itself allocates nothing.
//
// Limits and rules:
//  - The array holds 64 MiB; every GPU that loads this library keeps it until the process exits.
//  - One search needs 8 bytes per node of dense state plus its per-node arrays for the whole
//    graph (the capacity is node_bound, so no search can overflow).  Graphs whose single search
//    does not fit are rejected with CS_ERR_ARG and a message naming the sizes.
//  - All calls share the array and it keeps the previous call's contents; each call therefore
//    re-initialises the state that must start clean.  Calls that overlap on the GPU (two streams,
//    two host threads) race on the array: issue them one after another.
//  - Every call looks up the array's device address with cudaGetSymbolAddress while the
//    caller's device and context are current, so the address always belongs to the context the
//    call runs in (a context the host application created itself, or one re-created after
//    cudaDeviceReset).  The lookup allocates nothing.
//  - With lazy module loading (the CUDA default since 12.2) this file's device code, and with it
//    the 64 MiB array, is loaded on the first use of any of its kernels or of the array on a
//    device: if this entry point is that first use, the reservation happens inside the call.
//    Callers that must not see it there make one call (of any entry point) while setting up,
//    before the device's memory is handed to their pool and before any stream capture.
// ==========================================================================================
namespace {
constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;
}  // namespace

static __device__ __align__(256) unsigned char cs_noalloc_scratch[kNoAllocScratchBytes];

namespace {
cs_status noalloc_scratch_address(void **out) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, cs_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(static scratch)");
    if (!p) return fail(CS_ERR_CUDA, "static scratch has no device address");
    *out = p;
    return CS_OK;
}
}  // namespace

extern "C" cs_status cs_centrality_shortest_noalloc(const cs_primal_graph *g, const cs_query *q, cs_outputs out,
                                                    void *stream) {
    cs_status st = validate_primal(g);
    if (st != CS_OK) return st;
    if (!q) return fail(CS_ERR_ARG, "query is NULL");
    if (q->k < 1 || q->k > CS_MAX_THRESHOLDS) return fail(CS_ERR_ARG, "threshold count out of range");
    const int P = std::max(1, g->max_out_degree);
    const int L = lanes_for(cs::MODE_SHORTEST, q->k);
    const int cap = g->n_bound;  // a search can never overflow: no retry pass is needed
    const size_t one = layout(g->n_bound, 1, cap, P, L).total;
    if (one > kNoAllocScratchBytes)
        return fail(CS_ERR_ARG, "graph too large for the allocation-free path: one search needs " +
                                    std::to_string(one) + " bytes of scratch, the static array holds " +
                                    std::to_string(kNoAllocScratchBytes) + " bytes");
    int sms = sm_count();
    if (sms <= 0) return fail(CS_ERR_CUDA, "no CUDA device");
    int bpsm = 0;
    cudaError_t e = occupancy_blocks(P, launch_variant(nullptr, cs::MODE_SHORTEST), &bpsm);
    if (e != cudaSuccess) return cuda_fail(e, "occupancy query");
    int slots = std::max(1, sms * std::max(1, bpsm) * 8);
    while (slots > 1 && layout(g->n_bound, slots, cap, P, L).total > kNoAllocScratchBytes) {
        const int next = (slots * 7) / 8;
        slots = next < slots ? next : slots - 1;
    }
    void *ws = nullptr;
    st = noalloc_scratch_address(&ws);
    if (st != CS_OK) return st;
    cs_plan plan;
    memset(&plan, 0, sizeof(plan));
    plan.n_slots = slots;
    plan.cap = cap;
    plan.threads_per_block = 256;
    plan.blocks = (slots + 7) / 8;
    plan.delta_seconds = 0.0f;
    plan.lanes = L;
    plan.variant = launch_variant(nullptr, cs::MODE_SHORTEST);
    plan.max_degree = P;
    const Layout lay = layout(g->n_bound, slots, cap, P, L);
    plan.workspace_bytes = lay.total;
    cudaStream_t s = (cudaStream_t)stream;
    // The array keeps whatever the previous call left there (another graph's dense state or
    // compact scratch, or the remains of a call that failed midway), and this call's regions sit
    // at offsets set by its own node bound and threshold count.  Put every region that must start
    // clean into its clean state: the header, the dense per-slot state and the [3][K][n_bound]
    // closeness bucket.  The compact per-source arrays are written before they are read.
    e = cudaMemsetAsync(ws, 0, 256, s);
    if (e != cudaSuccess) return cuda_fail(e, "static scratch header reset");
    e = cudaMemsetAsync((char *)ws + lay.bucket_off, 0, sizeof(double) * 3 * (size_t)q->k * (size_t)g->n_bound, s);
    if (e != cudaSuccess) return cuda_fail(e, "static scratch bucket reset");
    st = reset_dense((char *)ws + lay.dense_off, lay.dense_stride, g->n_bound, slots, s);
    if (st != CS_OK) return st;
    return run_primal(g, q, &plan, ws, kNoAllocScratchBytes, out, stream, cs::MODE_SHORTEST, 0, nullptr, nullptr,
                      nullptr, nullptr, nullptr, 0, 0, 0.0f);
}

// ==========================================================================================
// Batched persistent form (cs_batch_*).
// ==========================================================================================
namespace {
struct BatchShape {
    int max_n, P, L;
};

cs_status batch_shape(const cs_batch_job *jobs, int n_jobs, BatchShape &b) {
    if (!jobs || n_jobs <= 0) return fail(CS_ERR_ARG, "empty batch");
    b.max_n = 1;
    b.P = 1;
    b.L = 1;
    for (int j = 0; j < n_jobs; j++) {
        cs_status st = validate_primal(&jobs[j].g);
        if (st != CS_OK) return st;
        if (jobs[j].mode != cs::MODE_SHORTEST && jobs[j].mode != cs::MODE_SEGMENT && jobs[j].mode != cs::MODE_BOTH)
            return fail(CS_ERR_ARG, "batch job mode must be 0 (shortest), 1 (segment) or 3 (both)");
        if (jobs[j].mode == cs::MODE_BOTH && !jobs[j].out2_dev) return fail(CS_ERR_ARG, "mode 3 job without out2_dev");
        if (jobs[j].k < 1 || jobs[j].k > CS_MAX_THRESHOLDS) return fail(CS_ERR_ARG, "threshold count out of range");
        if (!(jobs[j].speed_m_s > 0.0f)) return fail(CS_ERR_ARG, "speed_m_s must be finite and positive");
        if (!jobs[j].out_dev) return fail(CS_ERR_ARG, "job without out_dev");
        if ((jobs[j].mode == cs::MODE_SHORTEST || jobs[j].mode == cs::MODE_BOTH) && jobs[j].compute_closeness &&
            !jobs[j].bucket_dev)
            return fail(CS_ERR_ARG, "shortest job with closeness needs bucket_dev");
        b.max_n = std::max(b.max_n, jobs[j].g.n_bound);
        b.P = std::max(b.P, jobs[j].g.max_out_degree);
        b.L = std::max(b.L, lanes_for(jobs[j].mode, jobs[j].k));
    }
    return CS_OK;
}
}  // namespace

extern "C" {

cs_status cs_batch_prepare(cs_batch_job *jobs_host, int32_t n_jobs, int64_t *n_items) {
    if (!jobs_host || n_jobs <= 0 || !n_items) return fail(CS_ERR_ARG, "empty batch");
    int64_t acc = 0;
    for (int j = 0; j < n_jobs; j++) {
        jobs_host[j].item_begin = acc;
        acc += std::max(0, jobs_host[j].n_sources);
    }
    *n_items = acc;
    return CS_OK;
}

cs_status cs_batch_plan(const cs_batch_job *jobs_host, int32_t n_jobs, int32_t cap, int32_t max_slots,
                        int64_t mem_budget_bytes, cs_plan *plan) {
    BatchShape b;
    cs_status st = batch_shape(jobs_host, n_jobs, b);
    if (st != CS_OK) return st;
    return plan_common(b.max_n, b.P, b.L, cap, max_slots, mem_budget_bytes, plan);
}

cs_status cs_batch_run(const cs_batch_job *jobs_host, const cs_batch_job *jobs_dev, int32_t n_jobs, const cs_plan *plan,
                       void *ws, size_t ws_bytes, int32_t flags, void *stream_v) {
    BatchShape b;
    cs_status st = batch_shape(jobs_host, n_jobs, b);
    if (st != CS_OK) return st;
    if (!plan || !ws || !jobs_dev) return fail(CS_ERR_ARG, "plan/workspace/jobs_dev is NULL");
    if (plan->lanes < b.L) return fail(CS_ERR_ARG, "plan was made for fewer lanes");
    const int P = std::max(1, plan->max_degree);
    if (P < b.P) return fail(CS_ERR_ARG, "plan was made for a smaller degree");
    // slot geometry is the plan's, so one workspace serves batches of any graphs up to its size
    const int geo_n = plan->n_bound > 0 ? plan->n_bound : b.max_n;
    if (geo_n < b.max_n) return fail(CS_ERR_ARG, "plan was made for a smaller graph");
    const Layout lay = layout(geo_n, plan->n_slots, plan->cap, P, plan->lanes);
    if (ws_bytes < lay.total) return fail(CS_ERR_ARG, "workspace too small for this plan");
    long long n_items = 0;
    for (int j = 0; j < n_jobs; j++) {
        if (jobs_host[j].item_begin != n_items) return fail(CS_ERR_ARG, "jobs not prepared (cs_batch_prepare)");
        n_items += std::max(0, jobs_host[j].n_sources);
    }
    cudaStream_t stream = (cudaStream_t)stream_v;
    char *base = (char *)ws;
    cs::PrimalParams p;
    memset(&p, 0, sizeof(p));
    p.radix_sort = radix_sort_choice();
    p.g.n_bound = geo_n;  // slot geometry only; each job brings its own graph
    p.hdr = (cs::WsHeader *)(base + lay.hdr_off);
    p.failed = (int32_t *)(base + lay.failed_off);
    p.fail_cap = lay.fail_cap;
    p.dense = base + lay.dense_off;
    p.dense_stride = lay.dense_stride;
    p.compact = base + lay.compact_off;
    p.cap = plan->cap;
    p.P = P;
    p.L = plan->lanes;
    g_counters[0] = g_counters[1] = g_counters[2] = g_counters[3] = 0;
    cudaError_t e = cudaMemsetAsync(p.hdr, 0, sizeof(cs::WsHeader), stream);
    if (e != cudaSuccess) return cuda_fail(e, "batch reset");
    if (n_items == 0) return CS_OK;
    // consecutive jobs of one mode run as one launch of that mode's kernel (a smaller instruction
    // footprint than the all-mode kernel); more than four such runs use the all-mode kernel once
    struct Run {
        long long lo, hi;
        int mode;
    };
    std::vector<Run> runs;
    for (int j = 0; j < n_jobs; j++) {
        const int m = (jobs_host[j].mode == cs::MODE_SHORTEST || jobs_host[j].mode == cs::MODE_SEGMENT)
                          ? jobs_host[j].mode : -1;
        const long long lo = jobs_host[j].item_begin, hi = lo + std::max(0, jobs_host[j].n_sources);
        if (!runs.empty() && runs.back().mode == m) runs.back().hi = hi;
        else runs.push_back({lo, hi, m});
    }
    if (runs.size() > 4) runs.assign(1, Run{0, n_items, -1});
    st = launch_seed_table(stream);
    if (st != CS_OK) return st;
    for (const Run &r : runs) {
        if (r.hi <= r.lo) continue;
        e = cudaMemsetAsync(&p.hdr->work_next, 0, sizeof(unsigned long long), stream);
        if (e != cudaSuccess) return cuda_fail(e, "batch counter reset");
        st = launch_batch(p, plan, jobs_dev, n_jobs, r.lo, r.hi, plan->n_slots, r.mode, stream);
        if (st != CS_OK) return st;
    }
    if (!(flags & CS_BATCH_ASYNC)) {
        cs::WsHeader h;
        e = cs::read_header(p.hdr, h, stream, true);
        if (e != cudaSuccess) return cuda_fail(e, "batch kernel");
        if (h.err != 0u) return fail((cs_status)h.err, "device-side check failed (code " + std::to_string(h.err) + ")");
        const long long n_over = h.n_failed;
        if (h.n_failed > 0u) {
            st = retry_chain(p, plan, lay, base, b.max_n, P, h, stream, true, [&](cs::PrimalParams &p2, int slots2) {
                return launch_batch(p2, plan, jobs_dev, n_jobs, 0, n_items, slots2, -1, stream);
            });
            if (st != CS_OK) return st;
        }
        cs_set_retries_internal(n_over, 0);
        g_counters[0] = (long long)h.sources_done;
        g_counters[1] = (long long)h.edges_relaxed;
        g_counters[2] = (long long)h.nodes_settled;
        for (int i = 0; i < 16; i++) g_phase[i] = (long long)h.pad[i];
    }
    int max_n = 0, n_pref = 0;
    for (int j = 0; j < n_jobs; j++) {
        const cs_batch_job &jb = jobs_host[j];
        if ((jb.mode == cs::MODE_SHORTEST || jb.mode == cs::MODE_BOTH) && jb.compute_closeness && jb.n_sources > 0) {
            max_n = std::max(max_n, jb.g.n_bound);
            n_pref++;
        }
    }
    if (n_pref > 0) {
        const int sms = std::max(1, sm_count());
        const int gy = std::min(n_pref, 65535);
        const int gx = std::max(1, std::min((max_n + 255) / 256, std::max(1, sms * 8 / gy)));
        cs::batch_prefix_kernel<<<dim3(gx, gy), 256, 0, stream>>>(jobs_dev, n_jobs);
        g_counters[3]++;
        e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_fail(e, "batch_prefix_kernel launch");
    }
    return CS_OK;
}

cs_status cs_batch_status(void *ws, int64_t *n_overflowed, int64_t *sources_done, void *stream) {
    if (!ws) return fail(CS_ERR_ARG, "workspace is NULL");
    cs::WsHeader h;
    cudaError_t e = cs::read_header((const cs::WsHeader *)ws, h, (cudaStream_t)stream, true);
    if (e != cudaSuccess) return cuda_fail(e, "batch status");
    if (n_overflowed) *n_overflowed = (int64_t)h.n_failed;
    if (sources_done) *sources_done = (int64_t)h.sources_done;
    g_counters[0] = (long long)h.sources_done;
    g_counters[1] = (long long)h.edges_relaxed;
    g_counters[2] = (long long)h.nodes_settled;
    if (h.err != 0u) return fail((cs_status)h.err, "device-side check failed (code " + std::to_string(h.err) + ")");
    return CS_OK;
}

cs_status cs_batch_failed(void *ws, const cs_plan *plan, int32_t *items_host, int32_t max_items, int64_t *n_failed,
                          void *stream) {
    if (!ws || !plan || !n_failed) return fail(CS_ERR_ARG, "workspace/plan/n_failed is NULL");
    cs::WsHeader h;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cs::read_header((const cs::WsHeader *)ws, h, st, true);
    if (e != cudaSuccess) return cuda_fail(e, "batch failed list");
    const Layout lay = layout(std::max(1, plan->n_bound), plan->n_slots, plan->cap, 1, plan->lanes);
    const int64_t nf = (int64_t)h.n_failed;
    *n_failed = nf;
    if (nf > (int64_t)lay.fail_cap) return fail(CS_ERR_CAPACITY, "more overflowed items than the failed list holds");
    const int64_t c = std::min<int64_t>(nf, std::max(0, max_items));
    if (c > 0 && items_host) {
        e = cudaMemcpyAsync(items_host, (char *)ws + lay.failed_off, sizeof(int32_t) * (size_t)c, cudaMemcpyDeviceToHost,
                            st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return cuda_fail(e, "batch failed list");
    }
    return CS_OK;
}

}  // extern "C"

extern "C" cs_status cs_source_weights(const int32_t *sources_dev, int64_t n_sources, const float *node_w_dev,
                                        int32_t n_bound, float *src_wt_dev, uint8_t *eligible_dev, void *stream) {
    if (n_bound <= 0 || !node_w_dev || !src_wt_dev || !eligible_dev || (n_sources > 0 && !sources_dev))
        return fail(CS_ERR_ARG, "source weights: bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    const int sms = std::max(1, sm_count());
    const int b0 = std::max(1, std::min((n_bound + 255) / 256, sms * 4));
    cs::source_weights_kernel<<<b0, 256, 0, st>>>(sources_dev, n_sources, node_w_dev, n_bound, src_wt_dev, eligible_dev,
                                                  0);
    if (n_sources > 0) {
        const int b1 = (int)std::max<long long>(1, std::min<long long>((n_sources + 255) / 256, sms * 4));
        cs::source_weights_kernel<<<b1, 256, 0, st>>>(sources_dev, n_sources, node_w_dev, n_bound, src_wt_dev,
                                                      eligible_dev, 1);
    }
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CS_OK : cuda_fail(e, "source_weights_kernel launch");
}

namespace cs {
__global__ void seed_check_kernel(const float *w, const float *beta, const float *cost, double *out, long long n) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        out[t] = seed_exp(w[t], beta[t], cost[t]);
}
}  // namespace cs

extern "C" cs_status cs_debug_seed_exp(const float *w_dev, const float *beta_dev, const float *cost_dev,
                                       double *out_dev, int64_t n, void *stream) {
    if (n < 0 || (n > 0 && (!w_dev || !beta_dev || !cost_dev || !out_dev))) return fail(CS_ERR_ARG, "seed check: bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    cs_status rc = launch_seed_table(st);
    if (rc != CS_OK) return rc;
    if (n == 0) return CS_OK;
    const int blocks = (int)std::min<long long>((n + 255) / 256, 4096);
    cs::seed_check_kernel<<<blocks, 256, 0, st>>>(w_dev, beta_dev, cost_dev, out_dev, n);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CS_OK : cuda_fail(e, "seed_check_kernel launch");
}

// Live progress: the completed-source count the kernels keep in the workspace header, copied on a
// stream of its own (so it does not wait for the call's kernels) into pinned memory of this thread.
extern "C" cs_status cs_workspace_progress(const void *workspace_dev, int64_t *sources_done) {
    if (!workspace_dev || !sources_done) return fail(CS_ERR_ARG, "workspace/sources_done is NULL");
    thread_local unsigned long long *pinned = nullptr;
    thread_local cudaStream_t side = nullptr;
    cudaError_t e = cudaSuccess;
    if (!pinned) e = cudaHostAlloc((void **)&pinned, sizeof(unsigned long long), cudaHostAllocDefault);
    if (e == cudaSuccess && !side) e = cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail(e, "progress buffer");
    const cs::WsHeader *h = (const cs::WsHeader *)workspace_dev;
    e = cudaMemcpyAsync(pinned, &h->pad[cs::PROGRESS_SLOT], sizeof(unsigned long long), cudaMemcpyDeviceToHost, side);
    if (e == cudaSuccess) e = cudaStreamSynchronize(side);
    if (e != cudaSuccess) return cuda_fail(e, "progress read");
    *sources_done = (int64_t)*pinned;
    return CS_OK;
}

extern "C" cs_status cs_abi_sizes(int32_t *out, int32_t n) {
    // sizes of the public structs, for bindings to check their layouts against
    const int32_t v[7] = {(int32_t)sizeof(cs_primal_graph), (int32_t)sizeof(cs_dual_graph), (int32_t)sizeof(cs_query),
                          (int32_t)sizeof(cs_plan),         (int32_t)sizeof(cs_outputs),    (int32_t)sizeof(cs_batch_job),
                          (int32_t)sizeof(cs_dual_batch_job)};
    if (!out) return fail(CS_ERR_ARG, "out is NULL");
    for (int i = 0; i < n && i < 7; i++) out[i] = v[i];
    return CS_OK;
}
