// cs_dual.cu -- GB300 kernels for simplest-path (angular) centrality on the dual graph.
//
// Reference behaviour (cityseer-api v4.24.0):
//   centrality_simplest          rust/src/centrality.rs:1880-2132
//   dijkstra_brandes_angular     rust/src/centrality.rs:577-775 (doubled states, endpoint slots)
//   dual_node_endpoint_slots     rust/src/centrality.rs:533-566
//   best_angular_target_states   rust/src/centrality.rs:793-821
//   brandes_backprop_with_beta   rust/src/centrality.rs:823-873
//   dijkstra_tree_angular        rust/src/centrality.rs:1202-1332
//
// A state is (dual node, entry slot): index 2*node + slot.  The route cost is the summed angular
// change plus 1e-6 * length; the search is cut off on the summed travel seconds, which travel with
// each state's chosen route.  Per source, one warp:
//  A. Label-correcting search over states: atomicMin on a packed (route, seconds) 64-bit key gives
//     the lexicographic least fixpoint, route first.
//  B. Warp radix sort of the reached states by route: the reference's settle order.
//  C. Replay, in route order, of every state's candidate offers through the reference's tie rules:
//     final route, seconds, predecessors and sigma, each checked bit for bit against A.  The tie
//     window can make the reference keep seconds that differ from the lexicographic minimum; a
//     source where any state disagrees is redone by an exact sequential heap Dijkstra (the same
//     BinaryHeap order as the reference) and replayed again.
//  D. Per node: the best route / seconds over offers to both of its states (the reference's
//     best_route_cost / best_agg_seconds), closeness into target rows.
//  E. One backward Brandes sweep over states carrying every threshold.
#include <cstdio>
#include <cstring>
#include <string>
#include <algorithm>
#include <cmath>

#include "cs_common.cuh"
#include "cs_sort.cuh"

extern "C" void cs_set_error_internal(const char *msg);
extern "C" void cs_set_retries_internal(long long overflowed, long long inexact);
extern "C" void cs_set_phase_internal(const unsigned long long *pad);
extern "C" void cs_set_counters_internal(long long sources, long long relaxed, long long settled, long long launches);

namespace csd {
using namespace cs;

constexpr unsigned long long KEY_INF = 0xffffffffffffffffull;
// The key of a reached state whose every offer was withdrawn (a NaN route, above every real key and
// below KEY_INF): it offers nothing, a new offer replaces it, and it is not reached a second time.
constexpr unsigned long long KEY_WITHDRAWN = KEY_INF - 2ull;
constexpr int DPM = 8;  // max incoming / outgoing dual edges per state handled in registers

__host__ __device__ inline size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

struct DSlot {
    unsigned long long *key;  // [2N] packed (route bits << 32 | seconds bits)
    uint32_t *aux;            // [2N] settle position + 1 (0: unreached); bit 31 = settled (exact mode)
    int32_t *rl;              // [cap] reached states, discovery order
    ulonglong2 *qa, *qb, *qf;  // [2 cap] (state, key) queue entries
    uint32_t *kb;
    int32_t *vb;
    uint32_t *rk;  // [cap] sorted route bits
    int32_t *ord;  // [cap] sorted states
    float *rB, *sB, *nbR, *nbS;  // [cap] replayed route and seconds; node best route/seconds
    double *sig;  // [cap] path counts (f64, as the reference's sigma)
    uint8_t *np;
    int32_t *pr;  // [cap * DPM]
    double *dl;   // [cap * K] dependencies (f64, as the reference's delta)
    int32_t *hp;  // exact-mode heap: [2 cap] (route bits, state) pairs interleaved
    uint32_t *lsec;  // widened pass: [2N] least arrival seconds (f32 bits; all ones = none), else null
};

__host__ __device__ inline size_t compact_bytes_d(size_t cap, int K) {
    size_t b = 0;
    b += 4 * al256(cap * 4);        // rl kb vb ord
    b += 3 * al256(cap * 32);       // qa qb qf
    b += 5 * al256(cap * 4);        // rk rB sB nbR nbS
    b += al256(cap * 8);            // sig
    b += al256(cap);                // np
    b += al256(cap * 4 * DPM);      // pr
    b += al256(cap * 8 * (size_t)K);  // dl
    b += al256(cap * 16);           // hp
    return b;
}

__host__ __device__ inline DSlot dslot(char *dense, size_t dense_stride, char *compact, size_t cap, int K, int slot,
                                       int n_bound) {
    DSlot s;
    char *d = dense + dense_stride * (size_t)slot;
    s.key = (unsigned long long *)d;
    s.aux = (uint32_t *)(d + al256((size_t)n_bound * 16));
    char *c = compact + compact_bytes_d(cap, K) * (size_t)slot;
    size_t o = 0;
    s.rl = (int32_t *)(c + o); o += al256(cap * 4);
    s.kb = (uint32_t *)(c + o); o += al256(cap * 4);
    s.vb = (int32_t *)(c + o); o += al256(cap * 4);
    s.ord = (int32_t *)(c + o); o += al256(cap * 4);
    s.qa = (ulonglong2 *)(c + o); o += al256(cap * 32);
    s.qb = (ulonglong2 *)(c + o); o += al256(cap * 32);
    s.qf = (ulonglong2 *)(c + o); o += al256(cap * 32);
    s.rk = (uint32_t *)(c + o); o += al256(cap * 4);
    s.rB = (float *)(c + o); o += al256(cap * 4);
    s.sB = (float *)(c + o); o += al256(cap * 4);
    s.sig = (double *)(c + o); o += al256(cap * 8);
    s.nbR = (float *)(c + o); o += al256(cap * 4);
    s.nbS = (float *)(c + o); o += al256(cap * 4);
    s.np = (uint8_t *)(c + o); o += al256(cap);
    s.pr = (int32_t *)(c + o); o += al256(cap * 4 * DPM);
    s.dl = (double *)(c + o); o += al256(cap * 8 * (size_t)K);
    s.hp = (int32_t *)(c + o); o += al256(cap * 16);
    s.lsec = nullptr;
    return s;
}

enum DMode { DMODE_CENTRALITY = 0, DMODE_TREE = 1 };

struct DualParams {
    cs_dual_graph g;
    int32_t k;
    float sk[MAXK];  // seconds thresholds as f32
    float maxsec;
    float tol;
    float asu, fso;
    float delta;     // band width in route (degrees)
    int32_t closeness, betweenness, track_reach;
    const int32_t *src_list;
    int64_t n_src;
    const float *src_wt;
    const uint8_t *eligible;
    double *out;     // [4][K][N]
    double *bucket;  // [3][K][N]
    uint32_t *reach;
    WsHeader *hdr;
    int32_t *failed;
    int32_t fail_cap;
    int32_t *inexact;     // sources whose replay disagreed with the search
    int32_t inexact_cap;
    char *dense;
    size_t dense_stride;
    char *compact;
    int32_t cap;
    int32_t n_slots;
    int32_t pass;  // 0 = label-correcting pass, 1 = larger-capacity retry, 2 = exact heap pass,
                   // 3 = widened label-correcting pass (sources whose replay disagreed)
    int32_t lsec_slot_off;  // pass 3: slot i keeps its lsec array in slot i + this one's dense key array
    int32_t geo_n; // node bound the workspace's slot geometry was planned for (>= g.n_bound)
    const int32_t *remap;
    int32_t mode;
    int32_t fail_final;  // an overflow at this capacity is an error (capacity = every state)
    int32_t replay_rounds;  // replay / re-sort rounds before a source falls back to the exact search
    int32_t force_exact;
    int32_t row_cap;
    int32_t *t_count, *t_node, *t_pred;
    float *t_simpl, *t_agg;
};

__device__ __forceinline__ float hi_f(unsigned long long k) { return __uint_as_float((unsigned)(k >> 32)); }
__device__ __forceinline__ float lo_f(unsigned long long k) { return __uint_as_float((unsigned)(k & 0xffffffffull)); }
__device__ __forceinline__ unsigned long long pack(float r, float s) {
    return ((unsigned long long)__float_as_uint(r) << 32) | (unsigned long long)__float_as_uint(s);
}
// route candidate exactly as rust/src/centrality.rs:665-667 evaluates it
__device__ __forceinline__ float cand_route(float r, float ang, float len) {
    return __fadd_rn(__fadd_rn(r, ang), __fmul_rn(ANGULAR_TIE_BREAK, len));
}

// Per-phase cycle counters (the warp's shared-memory row; lane 0 adds): 0 search, 1 sort, 2 replay,
// 3 node best + closeness, 4 backward sweep, 5 scratch reset, 6 exact heap search; 7 counts replay
// rounds.
__device__ __forceinline__ void dphase(long long *ph, int idx, long long &t) {
    const long long now = clock64();
    if (lane_id() == 0) ph[idx] += now - t;
    t = now;
}

// ------------------------------------------------------------------------------------------
// A. Label-correcting search over states.  Returns R or -1 on overflow.
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ void dpush(bool first, int route, int V, unsigned long long key, int &R, int &nn, int &nf,
                                      int cap, int qcap, const DSlot &s, ulonglong2 *nxt, unsigned lt) {
    const unsigned mf = __ballot_sync(FULL, first);
    const unsigned mn = __ballot_sync(FULL, route == 1);
    const unsigned mr = __ballot_sync(FULL, route == 2);
    // a first touch's entry carries the state's discovery index + 1 in its upper half (else 0)
    unsigned long long x = (unsigned long long)(uint32_t)V;
    if (first) {
        const int q = R + __popc(mf & lt);
        if (q < cap) {
            s.rl[q] = V;
            s.aux[V] = (uint32_t)(q + 1);  // discovery index during the search (the sort rewrites it)
            ((unsigned long long *)s.sig)[q] = KEY_INF;  // the key V last relaxed with (none yet)
            x |= (unsigned long long)(q + 1) << 32;
        }
    }
    if (route == 1) {
        const int q = nn + __popc(mn & lt);
        if (q < qcap) nxt[q] = make_ulonglong2(x, key);
    }
    if (route == 2) {
        const int q = nf + __popc(mr & lt);
        if (q < qcap) s.qf[q] = make_ulonglong2(x, key);
    }
    R += __popc(mf);
    nn += __popc(mn);
    nf += __popc(mr);
}

// A state's key recomputed from its offerers' current keys (the lexicographic least in-cutoff offer;
// KEY_INF when none remains).
__device__ __noinline__ unsigned long long dual_rekey(const DualParams &p, const DSlot &s, int V) {
    const int v = V >> 1, sv = V & 1;
    const int beg = __ldg(&p.g.rptr_dev[v]), end = __ldg(&p.g.rptr_dev[v + 1]);
    const uint4 *re = (const uint4 *)p.g.rev_pack_dev;
    unsigned long long best = KEY_INF;
    for (int k = beg; k < end; k++) {
        const uint4 ed = __ldg(&re[k]);
        if ((int)(ed.x >> 31) != sv) continue;
        const unsigned long long kU = __ldcg(&s.key[ed.x & 0x7fffffffu]);
        if (kU == KEY_INF) continue;
        const float cs_ = __fadd_rn(lo_f(kU), __uint_as_float(ed.y));
        if (!(cs_ <= p.maxsec)) continue;
        const unsigned long long o = pack(cand_route(hi_f(kU), __uint_as_float(ed.z), __uint_as_float(ed.w)), cs_);
        best = o < best ? o : best;
    }
    return best;
}

__device__ int dual_search(const DualParams &p, const DSlot &s, int src, long long &relaxed) {
    const float maxsec_ = p.maxsec, delta_ = p.delta;  // in registers (p may live in shared memory)
    const int lane = lane_id();
    const unsigned lt = lanemask_lt();
    const int cap = p.cap, qcap = 2 * cap;
    // The key each reached state last relaxed with (by discovery index, in the sigma array, free until
    // the replay): when a state relaxes again with a key whose offer along an edge is now cut or worse,
    // a target whose key still equals the old offer holds a withdrawn offer, and its key is recomputed
    // from its offerers' current keys (raised, if nothing better remains) and relaxed again, so that
    // the withdrawal reaches its own targets.  A per-source budget bounds the withdrawals; past it the
    // search only lowers keys (and terminates), and the replay rounds settle what is left.
    unsigned long long *lastk = (unsigned long long *)s.sig;
    if (lane == 0) {
        s.key[2 * src] = 0ull;
        s.key[2 * src + 1] = 0ull;
        s.rl[0] = 2 * src;
        s.rl[1] = 2 * src + 1;
        s.aux[2 * src] = 1u;
        s.aux[2 * src + 1] = 2u;
        lastk[0] = KEY_INF;
        lastk[1] = KEY_INF;
        s.qa[0] = make_ulonglong2((unsigned long long)(2 * src), 0ull);
        s.qa[1] = make_ulonglong2((unsigned long long)(2 * src + 1), 0ull);
    }
    __syncwarp();
    int R = 2, nnear = 2, nfar = 0;
    ulonglong2 *cur = s.qa, *nxt = s.qb;
    float T = delta_;
    float fmn = __int_as_float(INF_BITS);  // this lane's smallest route queued far since the last split
    int withdrawals = 0;                   // warp-uniform
    const int max_withdrawals = cap;
    bool overflow = false;
    while (true) {
        while (nnear > 0) {
            int nnext = 0;
            for (int base = 0; base < nnear; base += 32) {
                const int i = base + lane;
                ulonglong2 ent = make_ulonglong2(0ull, KEY_INF);
                if (i < nnear) ent = cur[i];
                const int S = (int)(uint32_t)ent.x;
                const uint32_t qi = (uint32_t)(ent.x >> 32);  // discovery index + 1 of a first touch's entry
                const unsigned long long kS = (i < nnear) ? __ldcg(&s.key[S]) : KEY_INF;
                const bool live = (i < nnear) && kS == ent.y;
                // a first touch's entry knows the state's discovery index; later entries look it up
                const uint32_t aS = (live && qi == 0u) ? __ldcg(&s.aux[S]) : qi;
                const int u = S >> 1, e = S & 1;
                const int beg = live ? __ldg(&p.g.ptr_dev[u]) : 0;
                const int deg = live ? __ldg(&p.g.ptr_dev[u + 1]) - beg : 0;
                const bool track = live && aS != 0u && aS <= (uint32_t)cap;
                const unsigned long long lk = track ? __ldcg(&lastk[aS - 1]) : KEY_INF;
                relaxed += deg;
                const float rU = hi_f(kS), sU = lo_f(kS);
                const float rL = hi_f(lk), sL = lo_f(lk);
                // withdrawals only from a state relaxing again (it has a last key), within the budget
                const bool again = lk != KEY_INF && withdrawals < max_withdrawals;
                int tried = 0;
                const int maxdeg = warp_max_i(deg);
                const uint4 *fe = (const uint4 *)p.g.fwd_pack_dev;
                // four edges at a time: their records load together, then their atomics issue together
                for (int j0 = 0; j0 < maxdeg; j0 += 4) {
                    int Vq[4];
                    float crq[4];
                    unsigned long long nkq[4], oq[4];
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        const uint4 ed = (j0 + q < deg) ? __ldg(&fe[beg + j0 + q]) : make_uint4(0u, 0u, 0u, 0u);
                        const float cs_ = __fadd_rn(sU, __uint_as_float(ed.y));
                        const bool ok = j0 + q < deg && (int)(ed.x >> 31) == 1 - e && cs_ <= maxsec_;
                        Vq[q] = (int)(ed.x & 0x7fffffffu);
                        crq[q] = cand_route(rU, __uint_as_float(ed.z), __uint_as_float(ed.w));
                        nkq[q] = ok ? pack(crq[q], cs_) : KEY_INF;
                    }
#pragma unroll
                    for (int q = 0; q < 4; q++) oq[q] = nkq[q] != KEY_INF ? atomicMin(&s.key[Vq[q]], nkq[q]) : KEY_INF;
#pragma unroll
                    for (int q = 0; q < 4; q++) {
                        const bool imp = nkq[q] < oq[q];
                        const bool first = imp && oq[q] == KEY_INF;
                        unsigned long long pk = nkq[q];
                        int route = imp ? (crq[q] < T ? 1 : 2) : 0;
                        if (again && !imp && j0 + q < deg) {
                            // the offer this edge carried at the state's last relaxation (record re-read)
                            const uint4 ed = __ldg(&fe[beg + j0 + q]);
                            const float ocs = __fadd_rn(sL, __uint_as_float(ed.y));
                            if ((int)(ed.x >> 31) == 1 - e && ocs <= maxsec_) {
                                const unsigned long long ok =
                                    pack(cand_route(rL, __uint_as_float(ed.z), __uint_as_float(ed.w)), ocs);
                                // withdrawn: cut now, or worse than before, and still the target's key
                                if ((nkq[q] == KEY_INF || nkq[q] > ok) && __ldcg(&s.key[Vq[q]]) == ok) {
                                    tried++;
                                    unsigned long long kn = dual_rekey(p, s, Vq[q]);
                                    if (kn == KEY_INF) kn = KEY_WITHDRAWN;  // reached before: not a first touch again
                                    if (kn != ok && atomicCAS(&s.key[Vq[q]], ok, kn) == ok) {
                                        pk = kn;
                                        route = (kn == KEY_WITHDRAWN || hi_f(kn) < T) ? 1 : 2;
                                    }
                                }
                            }
                        }
                        if (route == 2) fmn = fminf(fmn, hi_f(pk));
                        dpush(first, route, Vq[q], pk, R, nnext, nfar, cap, qcap, s, nxt, lt);
                    }
                }
                withdrawals += (int)__reduce_add_sync(FULL, (unsigned)tried);
                if (track) lastk[aS - 1] = kS;
            }
            __syncwarp();
            if (R > cap || nnext > qcap || nfar > qcap) { overflow = true; break; }
            ulonglong2 *t = cur; cur = nxt; nxt = t;
            nnear = nnext;
        }
        if (overflow) break;
        if (nfar == 0) break;
        // next band from the smallest queued far route (lane minima over the pushes and the entries
        // the last split kept); one streaming pass by the queued routes, dead entries dropped when
        // their band runs
        const float mn = warp_min_f(fmn);
        T = fmaxf(__fadd_rn(mn, delta_), __int_as_float(__float_as_int(mn) + 1));
        fmn = __int_as_float(INF_BITS);
        int nn = 0, nf2 = 0;
        for (int base = 0; base < nfar; base += 32) {
            const int i = base + lane;
            const bool act = i < nfar;
            const ulonglong2 ent = act ? s.qf[i] : make_ulonglong2(0ull, KEY_INF);
            const float r = hi_f(ent.y);
            const bool tonear = act && r < T;
            const bool keep = act && !tonear;
            if (keep) fmn = fminf(fmn, r);
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
    if (overflow) return -1;
    return R;
}

// ------------------------------------------------------------------------------------------
// A (widened, pass 3).  The search of A plus, per state, the least arrival seconds over every path
// inside the cutoff (s.lsec, f32 bits, route-independent), and every state with such a path joins
// the reached set.  The reference's seconds for a state are the seconds of one of its paths, so this
// set contains every state the reference reaches, including those reached only through seconds
// that its tie window lowered below the search key's.  States reached only through lsec keep
// KEY_INF (they sort last); the replay gives each its route (+inf when the reference does not reach
// it) and the replay rounds settle the order.
// Queue entries: x = state | lsec part << 32 (NO_LSEC: none), y = key part (NO_KEY: none).  An entry
// is live while either part equals the state's current value; a live entry relaxes both the key and
// the lsec offers from the state's current values.  Entries with only an lsec part skip the bands.
// ------------------------------------------------------------------------------------------
constexpr uint32_t NO_LSEC = 0xffffffffu;
constexpr unsigned long long NO_KEY = KEY_INF - 1ull;  // a NaN route: never a key

__device__ int dual_search_wide(const DualParams &p, const DSlot &s, int src, long long &relaxed) {
    const float maxsec_ = p.maxsec, delta_ = p.delta;  // in registers (p may live in shared memory)
    const int lane = lane_id();
    const unsigned lt = lanemask_lt();
    const int cap = p.cap, qcap = 2 * cap;
    if (lane == 0) {
        s.key[2 * src] = 0ull;
        s.key[2 * src + 1] = 0ull;
        s.lsec[2 * src] = 0u;
        s.lsec[2 * src + 1] = 0u;
        s.rl[0] = 2 * src;
        s.rl[1] = 2 * src + 1;
        s.qa[0] = make_ulonglong2((unsigned long long)(2 * src), 0ull);
        s.qa[1] = make_ulonglong2((unsigned long long)(2 * src + 1), 0ull);
    }
    __syncwarp();
    int R = 2, nnear = 2, nfar = 0;
    ulonglong2 *cur = s.qa, *nxt = s.qb;
    float T = delta_;
    float fmn = __int_as_float(INF_BITS);
    bool overflow = false;
    while (true) {
        while (nnear > 0) {
            int nnext = 0;
            for (int base = 0; base < nnear; base += 32) {
                const int i = base + lane;
                const bool act = i < nnear;
                const ulonglong2 ent = act ? cur[i] : make_ulonglong2(0ull, NO_KEY);
                const int S = (int)(uint32_t)ent.x;
                const uint32_t nl = (uint32_t)(ent.x >> 32);
                const unsigned long long kS = act ? __ldcg(&s.key[S]) : KEY_INF;
                const uint32_t lS = act ? __ldcg(&s.lsec[S]) : NO_LSEC;
                const bool live = act && ((ent.y != NO_KEY && kS == ent.y) || (nl != NO_LSEC && lS == nl));
                const int u = S >> 1, e = S & 1;
                const int beg = live ? __ldg(&p.g.ptr_dev[u]) : 0;
                const int deg = live ? __ldg(&p.g.ptr_dev[u + 1]) - beg : 0;
                relaxed += deg;
                const bool has_key = kS != KEY_INF;
                const float rU = hi_f(kS), sU = lo_f(kS), lU = __uint_as_float(lS);
                const int maxdeg = warp_max_i(deg);
                for (int j = 0; j < maxdeg; j++) {
                    int V = 0;
                    unsigned long long nk = KEY_INF;
                    uint32_t lb = NO_LSEC;
                    bool impk = false, impl = false, first = false;
                    float cr = 0.0f;
                    if (j < deg) {
                        const uint4 ed = __ldg((const uint4 *)p.g.fwd_pack_dev + beg + j);
                        if ((int)(ed.x >> 31) == 1 - e) {
                            const float w = __uint_as_float(ed.y);
                            const float cs_ = has_key ? __fadd_rn(sU, w) : __int_as_float(INF_BITS);
                            // a key's path is a path too: lsec stays <= the key's seconds
                            const float ls_ = fminf(__fadd_rn(lU, w), cs_);
                            if (ls_ <= maxsec_) {
                                V = (int)(ed.x & 0x7fffffffu);
                                lb = __float_as_uint(ls_);
                                const uint32_t ol = atomicMin(&s.lsec[V], lb);
                                impl = lb < ol;
                                first = impl && ol == NO_LSEC;
                                if (cs_ <= maxsec_) {
                                    cr = cand_route(rU, __uint_as_float(ed.z), __uint_as_float(ed.w));
                                    nk = pack(cr, cs_);
                                    const unsigned long long o = atomicMin(&s.key[V], nk);
                                    impk = nk < o;
                                }
                            }
                        }
                    }
                    const int route = impk ? (cr < T ? 1 : 2) : (impl ? 1 : 0);
                    if (route == 2) fmn = fminf(fmn, cr);
                    const ulonglong2 ne = make_ulonglong2(
                        (unsigned long long)(uint32_t)V | ((unsigned long long)(impl ? lb : NO_LSEC) << 32),
                        impk ? nk : NO_KEY);
                    const unsigned mf = __ballot_sync(FULL, first);
                    const unsigned mn = __ballot_sync(FULL, route == 1);
                    const unsigned mr = __ballot_sync(FULL, route == 2);
                    if (first) {
                        const int q = R + __popc(mf & lt);
                        if (q < cap) s.rl[q] = V;
                    }
                    if (route == 1) {
                        const int q = nnext + __popc(mn & lt);
                        if (q < qcap) nxt[q] = ne;
                    }
                    if (route == 2) {
                        const int q = nfar + __popc(mr & lt);
                        if (q < qcap) s.qf[q] = ne;
                    }
                    R += __popc(mf);
                    nnext += __popc(mn);
                    nfar += __popc(mr);
                }
            }
            __syncwarp();
            if (R > cap || nnext > qcap || nfar > qcap) { overflow = true; break; }
            ulonglong2 *t = cur; cur = nxt; nxt = t;
            nnear = nnext;
        }
        if (overflow) break;
        if (nfar == 0) break;
        // as in dual_search: far entries always carry a key part (lsec-only entries go near)
        const float mn = warp_min_f(fmn);
        T = fmaxf(__fadd_rn(mn, delta_), __int_as_float(__float_as_int(mn) + 1));
        fmn = __int_as_float(INF_BITS);
        int nn = 0, nf2 = 0;
        for (int base = 0; base < nfar; base += 32) {
            const int i = base + lane;
            const bool act = i < nfar;
            const ulonglong2 ent = act ? s.qf[i] : make_ulonglong2(0ull, NO_KEY);
            const float r = hi_f(ent.y);
            const bool tonear = act && r < T;
            const bool keep = act && !tonear;
            if (keep) fmn = fminf(fmn, r);
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
    if (overflow) return -1;
    return R;
}

// ------------------------------------------------------------------------------------------
// A'. Exact sequential Dijkstra (lane 0) with the reference's BinaryHeap order
//     (rust/src/centrality.rs:357-386, 598-705).  Writes key[] and the settle order into ord/rk.
//     Returns R or -1 on overflow.
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ bool hle(const int32_t *h, int a, int b) {
    // a <= b under Ord for NodeDistance: other.metric.total_cmp(self.metric) (metrics >= 0 here)
    return h[2 * a] >= h[2 * b];
}
__device__ __forceinline__ void hswap(int32_t *h, int a, int b) {
    const int32_t m = h[2 * a], st = h[2 * a + 1];
    h[2 * a] = h[2 * b];
    h[2 * a + 1] = h[2 * b + 1];
    h[2 * b] = m;
    h[2 * b + 1] = st;
}
__device__ void heap_sift_up(int32_t *h, int start, int pos) {
    while (pos > start) {
        const int parent = (pos - 1) / 2;
        if (hle(h, pos, parent)) break;
        hswap(h, pos, parent);
        pos = parent;
    }
}

__device__ int dual_exact_search(const DualParams &p, const DSlot &s, int src) {
    const int lane = lane_id();
    int R = -1;
    if (lane == 0) {
        const int cap = p.cap, hcap = 2 * cap;
        int32_t *h = s.hp;
        int len = 0;
        bool overflow = false;
        s.key[2 * src] = 0ull;
        s.key[2 * src + 1] = 0ull;
        for (int sl = 0; sl < 2; sl++) {
            h[2 * len] = 0;
            h[2 * len + 1] = 2 * src + sl;
            len++;
            heap_sift_up(h, 0, len - 1);
        }
        const float one_plus = 1.0f + TIE_EPSILON;
        int n = 0;
        while (len > 0 && !overflow) {
            // pop: swap last into the root, sift down to the bottom, then up (Rust BinaryHeap)
            len--;
            const int32_t s_top = h[1];
            if (len > 0) {
                const int32_t m_last = h[2 * len], s_last = h[2 * len + 1];
                h[0] = m_last;
                h[1] = s_last;
                int pos = 0, child = 1;
                const int end = len;
                while (end >= 2 && child <= end - 2) {
                    child += hle(h, child, child + 1) ? 1 : 0;
                    h[2 * pos] = h[2 * child];
                    h[2 * pos + 1] = h[2 * child + 1];
                    pos = child;
                    child = 2 * pos + 1;
                }
                if (child == end - 1) {
                    h[2 * pos] = h[2 * child];
                    h[2 * pos + 1] = h[2 * child + 1];
                    pos = child;
                }
                h[2 * pos] = m_last;
                h[2 * pos + 1] = s_last;
                heap_sift_up(h, 0, pos);
            }
            const int S = s_top;
            if (s.aux[S] & 0x80000000u) continue;
            if (n >= cap) { overflow = true; break; }
            s.aux[S] = 0x80000000u;
            const unsigned long long kS = s.key[S];
            s.ord[n] = S;
            s.rk[n] = (uint32_t)(kS >> 32);
            n++;
            const int u = S >> 1, e = S & 1;
            const float rU = hi_f(kS), sU = lo_f(kS);
            const int beg = __ldg(&p.g.ptr_dev[u]), end2 = __ldg(&p.g.ptr_dev[u + 1]);
            for (int ej = beg; ej < end2; ej++) {
                if (__ldg(&p.g.exit_slot_dev[ej]) != 1 - e) continue;
                const float cs_ = __fadd_rn(sU, __ldg(&p.g.w_dev[ej]));
                if (cs_ > p.maxsec) continue;
                const int V = 2 * __ldg(&p.g.to_dev[ej]) + __ldg(&p.g.entry_slot_dev[ej]);
                if (s.aux[V] & 0x80000000u) continue;
                const float cr = cand_route(rU, __ldg(&p.g.ang_dev[ej]), __ldg(&p.g.len_dev[ej]));
                const unsigned long long kV = s.key[V];
                const float curR = (kV == KEY_INF) ? __int_as_float(INF_BITS) : hi_f(kV);
                const float curS = (kV == KEY_INF) ? __int_as_float(INF_BITS) : lo_f(kV);
                if (cr < curR) {
                    s.key[V] = pack(cr, cs_);
                    if (len >= hcap) { overflow = true; break; }
                    h[2 * len] = (int32_t)__float_as_uint(cr);
                    h[2 * len + 1] = V;
                    len++;
                    heap_sift_up(h, 0, len - 1);
                } else if (cr <= __fmul_rn(curR, one_plus) && cs_ < curS) {
                    s.key[V] = pack(curR, cs_);
                }
            }
        }
        // clear the settled marks (positions are written after the sort step is skipped)
        for (int i = 0; i < n; i++) s.aux[s.ord[i]] = 0u;
        R = overflow ? -1 : n;
    }
    R = __shfl_sync(FULL, R, 0);
    return R;
}

// ------------------------------------------------------------------------------------------
// C. Replay in route order.
// ------------------------------------------------------------------------------------------
struct DOff {
    int pos[DPM];
    float cr[DPM];
    float cs[DPM];
    unsigned valid;  // offers settled before the target
};

__device__ __forceinline__ int dnext(const DOff &o, unsigned todo) {
    int best = -1, bp = 0x7fffffff;
#pragma unroll
    for (int j = 0; j < DPM; j++)
        if (((todo >> j) & 1u) && o.pos[j] < bp) { bp = o.pos[j]; best = j; }
    return best;
}

__device__ __forceinline__ bool dpos_in(const DOff &o, unsigned mask, int pos) {
    bool has = false;
#pragma unroll
    for (int j = 0; j < DPM; j++) has |= ((mask >> j) & 1u) && o.pos[j] == pos;
    return has;
}

// Reference state machine (rust/src/centrality.rs:658-693) over offers in settle order; returns the
// predecessor mask and writes the replayed route and seconds.
__device__ __forceinline__ unsigned dreplay(const DualParams &p, const DOff &o, float &route, float &secs) {
    const float one_plus = 1.0f + TIE_EPSILON, one_minus = 1.0f - TIE_EPSILON;
    float cur = __int_as_float(INF_BITS), sc = __int_as_float(INF_BITS);
    unsigned pm = 0u, t = o.valid;
    while (t) {
        const int j = dnext(o, t);
        t &= ~(1u << j);
        float crj = 0.0f, csj = 0.0f;
        int pj = 0;
#pragma unroll
        for (int q = 0; q < DPM; q++)
            if (q == j) { crj = o.cr[q]; csj = o.cs[q]; pj = o.pos[q]; }
        if (csj > p.maxsec) continue;
        const bool improved = crj < cur;
        const bool tied = crj <= __fmul_rn(cur, one_plus);
        if (improved) {
            if (crj < __fmul_rn(cur, one_minus)) pm = 0u;
            pm |= 1u << j;
            cur = crj;
            sc = csj;
        } else if (tied && !dpos_in(o, pm, pj)) {
            if (csj < sc) sc = csj;
            pm |= 1u << j;
        }
    }
    route = cur;
    secs = sc;
    if (p.tol > TIE_EPSILON) {
        const float lim = __fmul_rn(cur, 1.0f + p.tol);
        pm = 0u;
        t = o.valid;
        while (t) {
            const int j = dnext(o, t);
            t &= ~(1u << j);
            float crj = 0.0f;
            int pj = 0;
#pragma unroll
            for (int q = 0; q < DPM; q++)
                if (q == j) { crj = o.cr[q]; pj = o.pos[q]; }
            if (crj <= lim && !dpos_in(o, pm, pj)) pm |= 1u << j;
        }
    }
    return pm;
}

// The replay keeps each state's offers (position, or -1; route; seconds) for the node-level best,
// in the search queues' space (free once the search is done): 8 positions in qa, 8 routes in qb,
// 8 seconds in qf per settle position.
__device__ __forceinline__ void store_doffers(const DSlot &s, int i, const DOff &o) {
    int4 *op = (int4 *)s.qa + 2 * (size_t)i;
    float4 *cp = (float4 *)s.qb + 2 * (size_t)i;
    float4 *sp = (float4 *)s.qf + 2 * (size_t)i;
    int q[DPM];
#pragma unroll
    for (int j = 0; j < DPM; j++) q[j] = ((o.valid >> j) & 1u) ? o.pos[j] : -1;
    op[0] = make_int4(q[0], q[1], q[2], q[3]);
    op[1] = make_int4(q[4], q[5], q[6], q[7]);
    cp[0] = make_float4(o.cr[0], o.cr[1], o.cr[2], o.cr[3]);
    cp[1] = make_float4(o.cr[4], o.cr[5], o.cr[6], o.cr[7]);
    sp[0] = make_float4(o.cs[0], o.cs[1], o.cs[2], o.cs[3]);
    sp[1] = make_float4(o.cs[4], o.cs[5], o.cs[6], o.cs[7]);
}

__device__ __forceinline__ void load_doffers(const DSlot &s, int i, DOff &o) {
    const int4 *op = (const int4 *)s.qa + 2 * (size_t)i;
    const float4 *cp = (const float4 *)s.qb + 2 * (size_t)i;
    const float4 *sp = (const float4 *)s.qf + 2 * (size_t)i;
    const int4 a = __ldcg(op), b = __ldcg(op + 1);
    const float4 c = __ldcg(cp), d = __ldcg(cp + 1), e = __ldcg(sp), f = __ldcg(sp + 1);
    const int q[DPM] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
    const float cr[DPM] = {c.x, c.y, c.z, c.w, d.x, d.y, d.z, d.w};
    const float cs[DPM] = {e.x, e.y, e.z, e.w, f.x, f.y, f.z, f.w};
    o.valid = 0u;
#pragma unroll
    for (int j = 0; j < DPM; j++) {
        o.pos[j] = q[j];
        o.cr[j] = cr[j];
        o.cs[j] = cs[j];
        if (q[j] >= 0) o.valid |= 1u << j;
    }
}

// Node-level best route / seconds (rust/src/centrality.rs:695-703) over offers to both states of
// the node, in the global settle order of the offering states.  Positions of the states: i0/i1
// (-1 when unreached).
__device__ __forceinline__ void node_best(const DualParams &p, const DSlot &s, int v, int src, int i0, int i1, int R,
                                          float &best, float &bsecs, bool &bad) {
    DOff o0, o1;
    o0.valid = 0u;
    o1.valid = 0u;
    if (i0 >= 0) load_doffers(s, i0, o0);
    if (i1 >= 0) load_doffers(s, i1, o1);
    const float one_plus = 1.0f + TIE_EPSILON, one_minus = 1.0f - TIE_EPSILON;
    best = (v == src) ? 0.0f : __int_as_float(INF_BITS);
    bsecs = best;
    unsigned t0 = o0.valid, t1 = o1.valid;
    while (t0 | t1) {
        const int j0 = t0 ? dnext(o0, t0) : -1;
        const int j1 = t1 ? dnext(o1, t1) : -1;
        int p0 = 0x7fffffff, p1 = 0x7fffffff;
        float c0 = 0.0f, s0 = 0.0f, c1 = 0.0f, s1 = 0.0f;
#pragma unroll
        for (int q = 0; q < DPM; q++) {
            if (q == j0) { p0 = o0.pos[q]; c0 = o0.cr[q]; s0 = o0.cs[q]; }
            if (q == j1) { p1 = o1.pos[q]; c1 = o1.cr[q]; s1 = o1.cs[q]; }
        }
        // equal offering positions: the offering state relaxes its out-edges in list order; the
        // two target slots are reached through different edges, so either order is one offer each
        const bool take0 = j0 >= 0 && (j1 < 0 || p0 <= p1);
        float cr, cs_;
        if (take0) { cr = c0; cs_ = s0; t0 &= ~(1u << j0); }
        else { cr = c1; cs_ = s1; t1 &= ~(1u << j1); }
        if (cs_ > p.maxsec) continue;
        if (cr < __fmul_rn(best, one_minus)) {
            best = cr;
            bsecs = cs_;
        } else if (cr <= __fmul_rn(best, one_plus)) {
            bsecs = fminf(bsecs, cs_);
        }
    }
}

__device__ __forceinline__ int first_ks(const DualParams &p, float secs) {
    int k = 0;
    while (k < p.k && !(secs <= p.sk[k])) k++;
    return k;
}

// Replay + sigma in route order.  Returns false (and sets mismatch) when the replay disagrees with
// the search's keys.
// Returns 0 when the replay is exact, 1 when some replayed route differs from the search's key and
// the replayed routes are out of order (the keys are then rewritten with the replayed values, so
// that sorting them again gives the next settle-order estimate), 2 when the replayed seconds would
// reach a state the search did not.
// check_reach: run the reach check even when every replayed value equals its key (the keys were
// rewritten by an earlier round, and the search never relaxed from the rewritten seconds).
__device__ int dual_replay(const DualParams &p, const DSlot &s, int src, int R, bool &bad, bool rewrite,
                           bool check_reach, int start, int &first_change) {
    const int lane = lane_id();
    bool mismatch = false;
    int change = R;  // this lane's lowest position a rewritten key can move a state to or from
    // The replay recomputes every state's (route, seconds) from its offers in settle order, as the
    // reference's heap search does.  Routes must equal the search's (then the settle order is the
    // reference's).  Seconds may differ where near-tied offers arrived in another order: the
    // reference's seconds are then never larger, so the replay is exact as long as no state the
    // search left unreached is offered within the cutoff by the replayed seconds (checked below).
    bool secs_diff = false;
    for (int base = start; base < R; base += 32) {
        const int i = base + lane;
        const bool act = i < R;
        const int V = act ? s.ord[i] : 0;
        const bool is_src = act && (V >> 1) == src;
        // The state's offers from reached states settled before it: positions and dual edges, found
        // once; the offer values need the offerers' replayed route and seconds, final once the
        // in-chunk offerers (pm) are done.
        DOff o;
        o.valid = 0u;
        unsigned pm = 0u;
        const uint4 *re = (const uint4 *)p.g.rev_pack_dev;
        int rbeg = 0;  // the state's incoming records: re[rbeg + j]
        if (act && !is_src) {
            const int v = V >> 1, sv = V & 1;
            rbeg = __ldg(&p.g.rptr_dev[v]);
            const int deg = min(__ldg(&p.g.rptr_dev[v + 1]) - rbeg, DPM);
            uint32_t aa[DPM];
#pragma unroll
            for (int j = 0; j < DPM; j++) {
                aa[j] = 0u;
                const unsigned x = (j < deg) ? __ldg(&re[rbeg + j]).x : 0u;
                if (j < deg && (int)(x >> 31) == sv) aa[j] = s.aux[x & 0x7fffffffu];
            }
#pragma unroll
            for (int j = 0; j < DPM; j++) {
                o.pos[j] = -1;
                if (aa[j] > (uint32_t)R) bad = true;
                if (aa[j] != 0u && aa[j] <= (uint32_t)R && (int)aa[j] - 1 < i) {
                    const int pu = (int)aa[j] - 1;
                    o.pos[j] = pu;
                    o.valid |= 1u << j;
                    if (pu >= base) pm |= 1u << (pu - base);
                }
            }
        } else {
#pragma unroll
            for (int j = 0; j < DPM; j++) {
                o.pos[j] = -1;
                o.cr[j] = 0.0f;
                o.cs[j] = 0.0f;
            }
        }
        bool mine = !act;
        unsigned done = __ballot_sync(FULL, mine);
        int guard = 0;
        while (done != FULL) {
            const bool ready = !mine && ((pm & ~done) == 0u);
            if (ready) {
                float route, secs;
                double sg;
                int np = 0;
                if (is_src) {
                    route = 0.0f;
                    secs = 0.0f;
                    sg = 1.0;
                } else {
#pragma unroll
                    for (int j = 0; j < DPM; j++) {
                        o.cr[j] = 0.0f;
                        o.cs[j] = 0.0f;
                        if ((o.valid >> j) & 1u) {
                            const int pu = o.pos[j];
                            const uint4 ed = __ldg(&re[rbeg + j]);
                            o.cr[j] = cand_route(__ldcg(&s.rB[pu]), __uint_as_float(ed.z), __uint_as_float(ed.w));
                            o.cs[j] = __fadd_rn(__ldcg(&s.sB[pu]), __uint_as_float(ed.y));
                        }
                    }
                const unsigned pmask = dreplay(p, o, route, secs);
                    sg = 0.0;
#pragma unroll
                    for (int j = 0; j < DPM; j++) {
                        if ((pmask >> j) & 1u) {
                            s.pr[(size_t)i * DPM + np] = o.pos[j];
                            sg = __dadd_rn(sg, s.sig[o.pos[j]]);
                            np++;
                        }
                    }
                }
                s.rB[i] = route;
                s.sB[i] = secs;
                s.sig[i] = sg;
                s.np[i] = (uint8_t)np;
                store_doffers(s, i, o);
                const unsigned long long k = __ldcg(&s.key[V]);
                // a widened-pass state without a key that the replay leaves unreached agrees
                const bool both_unreached = (k == KEY_INF || k == KEY_WITHDRAWN) && route == __int_as_float(INF_BITS);
                if (both_unreached) {
                } else if (__float_as_uint(route) != (unsigned)(k >> 32)) {
                    mismatch = true;
                    // diagnostics: replayed route below / above the key, or unreached
                    const int slot9 = route == __int_as_float(INF_BITS) ? 11 : (route < hi_f(k) ? 9 : 10);
                    atomicAdd(&p.hdr->pad[slot9], 1ull);
                    if (rewrite) {
                        s.key[V] = pack(route, secs);
                        // the rewritten state leaves position i for one at or after the first sorted
                        // key not below its new route (s.rk holds the sorted keys)
                        const uint32_t nb = __float_as_uint(route);
                        int lo = 0, hi = min(i, R);
                        while (lo < hi) {
                            const int mid = (lo + hi) >> 1;
                            if (__ldcg(&s.rk[mid]) < nb) lo = mid + 1;
                            else hi = mid;
                        }
                        change = min(change, lo);
                    }
                } else if (__float_as_uint(secs) != (unsigned)(k & 0xffffffffull)) {
                    secs_diff = true;
                }
                mine = true;
            }
            __syncwarp();
            done |= __ballot_sync(FULL, ready);
            if (++guard > 64) break;
        }
        if (done != FULL) {
            if (lane == 0) raise_err(p.hdr, CS_ERR_INTERNAL, 21);
            return 2;
        }
    }
    const bool any_mismatch = __any_sync(FULL, mismatch);
    first_change = -warp_max_i(-change);
    __syncwarp();
    if (any_mismatch) {
        // The keys only order the states: the replay ran in the reference's settle order, and is
        // therefore its result, whenever the finite replayed routes are non-decreasing in that order
        // (states the replay leaves unreached offer nothing and are inert wherever they sit).
        // Otherwise the rewritten keys give the next order.
        bool disorder = false;
        float run = -1.0f;  // largest finite route of the earlier chunks (routes are >= 0)
        for (int base = 0; base < R; base += 32) {
            const int i = base + lane;
            const float r = i < R ? __ldcg(&s.rB[i]) : -1.0f;
            const float rf = (r == __int_as_float(INF_BITS)) ? -1.0f : r;
            float m = rf;  // inclusive running max over the chunk
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const float t = __shfl_up_sync(FULL, m, o);
                if (lane >= o) m = fmaxf(m, t);
            }
            float before = __shfl_up_sync(FULL, m, 1);
            before = fmaxf(lane == 0 ? -1.0f : before, run);
            if (rf >= 0.0f && rf < before) disorder = true;
            run = fmaxf(run, __shfl_sync(FULL, m, 31));
        }
        if (__any_sync(FULL, disorder)) {
            if (lane == 0) atomicAdd(&p.hdr->pad[12], 1ull);
            return 1;
        }
    }
    if (!check_reach && !any_mismatch && !__any_sync(FULL, secs_diff)) return 0;
    __syncwarp();
    // reach check with the replayed seconds: every in-cutoff offer must land on a reached state.
    // After mismatches (in this round or, for the states ahead of start, an earlier one), a state the
    // replay left unreached may only have been positioned before its offerers: an in-cutoff offer to
    // it means the order was wrong (another round).
    bool escape = false, stale = false;
    for (int i = lane; i < R; i += 32) {
        const int U = s.ord[i];
        const int u = U >> 1, e = U & 1;
        const float sU = s.sB[i];
        const int beg = __ldg(&p.g.ptr_dev[u]), end = __ldg(&p.g.ptr_dev[u + 1]);
        for (int ej = beg; ej < end; ej++) {
            const uint4 ed = __ldg((const uint4 *)p.g.fwd_pack_dev + ej);
            if ((int)(ed.x >> 31) != 1 - e) continue;
            if (__fadd_rn(sU, __uint_as_float(ed.y)) > p.maxsec) continue;
            const int V = (int)(ed.x & 0x7fffffffu);
            const uint32_t a = s.aux[V];
            if (a == 0u) escape = true;
            else if ((any_mismatch || check_reach) && __ldcg(&s.rB[a - 1]) == __int_as_float(INF_BITS)) stale = true;
        }
    }
    if (__any_sync(FULL, stale)) {
        if (lane == 0) atomicAdd(&p.hdr->pad[13], 1ull);
        return 1;
    }
    if (__any_sync(FULL, escape)) {
        if (lane == 0) atomicAdd(&p.hdr->pad[14], 1ull);
        return 2;
    }
    return 0;
}

// ------------------------------------------------------------------------------------------
// D + E. Node best, closeness, backward sweep.
// ------------------------------------------------------------------------------------------
__device__ void dual_accumulate(const DualParams &p, const DSlot &s, int src, int R, int *cnt, bool &bad, long long *ph) {
    long long tph = clock64();
    const int lane = lane_id();
    const int K = p.k;
    const int N = p.g.n_bound;
    const float wt = __ldg(&p.src_wt[src]);
    for (int q = lane; q < MAXK; q += 32) cnt[q] = 0;
    __syncwarp();
    // node best (the lane of the lower-positioned state of each node) + closeness
    const size_t KN = (size_t)K * N;
    const double wt_d = f2d(wt);
    // per position, for the backward sweep: the sibling state's position + 1 and the node's
    // eligibility in the top bit (the sort's key scratch is free by now)
    uint32_t *info = s.kb;
    for (int i = lane; i < R; i += 32) {
        const int V = s.ord[i];
        const int v = V >> 1;
        const uint32_t as = s.aux[V ^ 1];
        const int isib = (as != 0u && as <= (uint32_t)R) ? (int)as - 1 : -1;
        info[i] = (uint32_t)(isib + 1) | (__ldg(&p.eligible[v]) ? 0x80000000u : 0u);
        if (isib >= 0 && isib < i) continue;
        const int i0 = (V & 1) ? isib : i;
        const int i1 = (V & 1) ? i : isib;
        float best, bsecs;
        node_best(p, s, v, src, i0, i1, R, best, bsecs, bad);
        s.nbR[i] = best;
        s.nbS[i] = bsecs;
        if (isib >= 0) {
            s.nbR[isib] = best;
            s.nbS[isib] = bsecs;
        }
        if (!p.closeness || v == src) continue;
        if (!isfinite(best) || !isfinite(bsecs)) continue;
        const int k0 = first_ks(p, bsecs);
        if (k0 >= K) continue;
        atomicAdd(&cnt[k0], 1);
        const float ratio = __fdiv_rn(best, p.asu);
        const float far_ang = __fadd_rn(p.fso, ratio);
        const float harm_ang = __fadd_rn(1.0f, ratio);
        double *bk = p.bucket + (size_t)k0 * N + v;
        atomicAdd(bk, wt_d);
        atomicAdd(bk + KN, f2d(__fmul_rn(far_ang, wt)));
        atomicAdd(bk + 2 * KN, f2d(__fmul_rn(__fdiv_rn(1.0f, harm_ang), wt)));
    }
    __syncwarp();
    if (p.closeness && p.track_reach && lane == 0) {
        int run = 0;
        for (int k = 0; k < K; k++) {
            run += cnt[k];
            if (run > 0) atomicAdd(&p.reach[k], (unsigned)run);
        }
    }
    dphase(ph, 3, tph);
    if (!p.betweenness) return;
    // backward sweep over states, K lanes (rust/src/centrality.rs:2036-2096)
    double *dl = s.dl;
    for (int i = lane; i < R; i += 32)
        for (int q = 0; q < K; q++) dl[(size_t)i * K + q] = 0.0;
    __syncwarp();
    const bool unit_wt = (wt == 1.0f);
    const double wtd = (double)wt;
    const float one_tol = 1.0f + p.tol;
    const int nchunks = (R + 31) / 32;
    for (int ch = nchunks - 1; ch >= 0; ch--) {
        const int base = ch * 32;
        const int i = base + lane;
        const bool act = i < R;
        const int np = act ? s.np[i] : 0;
        int pl[DPM];
        unsigned pm = 0u;
#pragma unroll
        for (int r = 0; r < DPM; r++) {
            pl[r] = (r < np) ? s.pr[(size_t)i * DPM + r] : 0;
            if (r < np && pl[r] >= base) pm |= 1u << (pl[r] - base);
        }
        bool mine = !act;
        unsigned done = __ballot_sync(FULL, mine);
        int guard = 0;
        while (done != FULL) {
            const unsigned blocked = __reduce_or_sync(FULL, mine ? 0u : pm);
            const bool ready = !mine && !((blocked >> lane) & 1u);
            if (ready) {
                const int V = s.ord[i];
                const int v = V >> 1;
                const double sw = s.sig[i];
                const float secs = s.sB[i];
                const float route = s.rB[i];
                const float best = s.nbR[i], bsecs = s.nbS[i];
                // sibling state for the seed split, and the pair weight
                const uint32_t inf = __ldcg(&info[i]);
                const int isib = (int)(inf & 0x7fffffffu) - 1;
                const double sig_sib = isib >= 0 ? s.sig[isib] : 0.0;
                const float secs_sib = isib >= 0 ? s.sB[isib] : 0.0f;
                const float route_sib = isib >= 0 ? s.rB[isib] : 0.0f;
                const double pair = (inf >> 31) ? 0.5 : 1.0;
                // predecessor factors sigma_v / sigma_w in f64 (1 exactly when the counts agree)
                double fr[DPM];
#pragma unroll
                for (int r = 0; r < DPM; r++) {
                    fr[r] = 0.0;
                    if (r < np) {
                        const double sv = s.sig[pl[r]];
                        fr[r] = (sv == sw) ? 1.0 : __ddiv_rn(sv, sw);
                    }
                }
                double *dli = dl + (size_t)i * K;
                for (int k = 0; k < K; k++) {
                    const float thr = p.sk[k];
                    if (!(secs <= thr)) continue;  // include_state: agg_seconds <= threshold
                    if (sw == 0.0) continue;
                    double seed = 0.0;
                    if (v != src && isfinite(best) && isfinite(bsecs) && bsecs <= thr) {
                        const bool me = sw != 0.0 && secs <= thr && route <= __fmul_rn(best, one_tol);
                        const bool sib = isib >= 0 && sig_sib != 0.0 && secs_sib <= thr &&
                                         route_sib <= __fmul_rn(best, one_tol);
                        if (me) {
                            // the seed splits the pair count over the best states by sigma
                            // (rust/src/centrality.rs:2066-2077), in f64
                            const double tot = sib ? __dadd_rn(sw, sig_sib) : sw;
                            seed = (tot == sw) ? pair : __dmul_rn(pair, __ddiv_rn(sw, tot));
                        }
                    }
                    const double dep = __dadd_rn(seed, __ldcg(&dli[k]));
                    if (dep == 0.0) continue;
#pragma unroll
                    for (int r = 0; r < DPM; r++) {
                        if (r >= np || fr[r] == 0.0) continue;
                        atomicAdd(&dl[(size_t)pl[r] * K + k], fr[r] == 1.0 ? dep : __dmul_rn(fr[r], dep));
                    }
                    if (v == src) continue;
                    const double credit = __dadd_rn(dep, -seed);
                    if (credit > 0.0)
                        atomicAdd(p.out + ((size_t)3 * K + k) * N + v, unit_wt ? credit : __dmul_rn(credit, wtd));
                }
                mine = true;
            }
            __syncwarp();
            done |= __ballot_sync(FULL, ready);
            if (++guard > 64) break;
        }
        if (done != FULL) {
            if (lane == 0) raise_err(p.hdr, CS_ERR_INTERNAL, 22);
            return;
        }
    }
    dphase(ph, 4, tph);
}

// ------------------------------------------------------------------------------------------
// Persistent kernel.
// ------------------------------------------------------------------------------------------
// One source on this warp's slot: search, settle order, replay, accumulation, scratch reset.
// Returns true when the source was accumulated; false when it was listed (overflow or a replay
// that disagreed) for a later pass.  li is what the lists record.
__device__ __forceinline__ bool run_dual_source(const DualParams &p, const DSlot &s, int li, int src, uint32_t *hist,
                                                int *cnt, long long *ph, long long &relaxed, long long &settled) {
    const int lane = lane_id();
    long long tph = clock64();
    const int N2 = 2 * p.g.n_bound;
    const bool exact = (p.pass == 2) || p.force_exact;
    const bool wide = s.lsec != nullptr;
    int R;
    if (exact) {
        R = dual_exact_search(p, s, src);
    } else if (wide) {
        R = dual_search_wide(p, s, src, relaxed);
    } else {
        R = dual_search(p, s, src, relaxed);
    }
    dphase(ph, exact ? 6 : 0, tph);
    if (R < 0) {
        for (int j = lane; j < N2; j += 32) {
            s.key[j] = KEY_INF;
            s.aux[j] = 0u;
            if (wide) s.lsec[j] = NO_LSEC;
        }
        if (lane == 0) {
            if (p.fail_final) {
                raise_err(p.hdr, CS_ERR_CAPACITY, 27);  // full-capacity passes must not overflow
            } else {
                const unsigned f = atomicAdd(&p.hdr->n_failed, 1u);
                if (f < (unsigned)p.fail_cap) p.failed[f] = li;
                else raise_err(p.hdr, CS_ERR_CAPACITY, 23);
            }
        }
        __syncwarp();
        return false;
    }
    // Replay in settle order.  A search key can hold a route from an offer its offering state
    // later withdrew (that state improved its route but its new seconds crossed the cutoff), so
    // the first order is an estimate: replay, re-sort by the replayed routes, and replay again
    // until the order is consistent (the reference's), else fall back to the exact search.
    bool bad = false;
    int rr = 1;
    // the widened set's keyless states that the reference reaches take one more round to sort
    const int rounds = exact ? 1 : max(1, p.replay_rounds) + (wide ? 4 : 0);
    int rounds_run = 0;
    int32_t *prev = (int32_t *)s.nbR;  // the previous round's order (nbR is free until the accumulation)
    int first_change = 0;
    auto key_of = [&](int S) { return (uint32_t)(__ldcg(&s.key[S]) >> 32); };
    for (int it = 0; it < rounds && rr == 1; it++) {
        rounds_run++;
        int start = 0;
        if (!exact) {
            if (it == 0) {
                warp_radix_sort(R, s.rl, key_of, s.kb, s.vb, s.rk, s.ord, hist);
            } else {
                // Only the keys the last round rewrote changed, and no state ahead of first_change
                // moves: the suffix from there is sorted again (from its current order, which holds
                // the same states), the prefix keeps its order and sorted keys.
                const int p0 = max(0, min(first_change, R));
                for (int i = p0 + lane; i < R; i += 32) prev[i] = s.ord[i];
                __syncwarp();
                if (p0 < R) warp_radix_sort(R - p0, s.ord + p0, key_of, s.kb, s.vb, s.rk + p0, s.ord + p0, hist);
            }
            __syncwarp();
            if (it > 0) {
                // the states ahead of the first moved one keep their place, offers and replayed
                // values: the next round replays from that one's chunk on
                const int p0 = max(0, min(first_change, R));
                start = R;
                for (int base = p0 & ~31; base < R; base += 32) {
                    const int i = base + lane;
                    const unsigned moved = __ballot_sync(FULL, i >= p0 && i < R && __ldcg(&s.ord[i]) != prev[i]);
                    if (moved) {
                        start = base + __ffs(moved) - 1;
                        break;
                    }
                }
                start &= ~31;
                if (lane == 0) ph[15] += start;
            }
        }
        for (int i = start + lane; i < R; i += 32) s.aux[s.ord[i]] = (uint32_t)(i + 1);
        __syncwarp();
        dphase(ph, 1, tph);
        // after a round that rewrote keys, lower rewritten seconds may reach states the search cut
        rr = dual_replay(p, s, src, R, bad, !exact, it > 0, start, first_change);
        __syncwarp();
        dphase(ph, 2, tph);
    }
    if (lane == 0) ph[7] += rounds_run;
    const bool ok = rr == 0;
    if (ok) {
        dual_accumulate(p, s, src, R, cnt, bad, ph);
        tph = clock64();
    } else if (lane == 0) {
        if (exact) raise_err(p.hdr, CS_ERR_INTERNAL, 24);  // the exact pass must replay cleanly
        else {
            const unsigned f = atomicAdd(&p.hdr->n_inexact, 1u);
            if (f < (unsigned)p.inexact_cap) p.inexact[f] = li;
            else raise_err(p.hdr, CS_ERR_CAPACITY, 25);
        }
    }
    if (__any_sync(FULL, bad) && lane == 0) raise_err(p.hdr, CS_ERR_INTERNAL, 26);
    __syncwarp();
    for (int i = lane; i < R; i += 32) {
        const int S = s.ord[i];
        s.key[S] = KEY_INF;
        s.aux[S] = 0u;
        if (wide) s.lsec[S] = NO_LSEC;
    }
    __syncwarp();
    dphase(ph, 5, tph);
    settled += R;
    return ok;
}

// The same per-source work with the block's warps in lockstep: search, then sort + replay rounds,
// then accumulation + scratch reset, each phase closed by a block barrier that every warp meets
// (a warp without a source, or whose source overflowed, runs the phases empty), so that the SM
// fetches one phase's code at a time.  Returns true when the source was accumulated.
__device__ __forceinline__ bool run_dual_source_sync(const DualParams &p, const DSlot &s, bool mine, int li,
                                                     int src, uint32_t *hist, int *cnt, long long *ph,
                                                     long long &relaxed, long long &settled) {
    const int lane = lane_id();
    long long tph = clock64();
    const int N2 = 2 * p.g.n_bound;
    const bool exact = (p.pass == 2) || p.force_exact;
    const bool wide = s.lsec != nullptr;
    int R = 0;
    if (mine) {
        if (exact) R = dual_exact_search(p, s, src);
        else if (wide) R = dual_search_wide(p, s, src, relaxed);
        else R = dual_search(p, s, src, relaxed);
    }
    dphase(ph, exact ? 6 : 0, tph);
    __syncthreads();
    const bool live = mine && R >= 0;
    if (mine && R < 0) {
        for (int j = lane; j < N2; j += 32) {
            s.key[j] = KEY_INF;
            s.aux[j] = 0u;
            if (wide) s.lsec[j] = NO_LSEC;
        }
        if (lane == 0) {
            if (p.fail_final) {
                raise_err(p.hdr, CS_ERR_CAPACITY, 27);
            } else {
                const unsigned f = atomicAdd(&p.hdr->n_failed, 1u);
                if (f < (unsigned)p.fail_cap) p.failed[f] = li;
                else raise_err(p.hdr, CS_ERR_CAPACITY, 23);
            }
        }
        __syncwarp();
    }
    bool bad = false;
    int rr = 1;
    if (live) {
        const int rounds = exact ? 1 : max(1, p.replay_rounds) + (wide ? 4 : 0);
        int rounds_run = 0;
        int32_t *prev = (int32_t *)s.nbR;
        int first_change = 0;
        auto key_of = [&](int S) { return (uint32_t)(__ldcg(&s.key[S]) >> 32); };
        for (int it = 0; it < rounds && rr == 1; it++) {
            rounds_run++;
            int start = 0;
            if (!exact) {
                if (it == 0) {
                    warp_radix_sort(R, s.rl, key_of, s.kb, s.vb, s.rk, s.ord, hist);
                } else {
                    const int p0 = max(0, min(first_change, R));
                    for (int i = p0 + lane; i < R; i += 32) prev[i] = s.ord[i];
                    __syncwarp();
                    if (p0 < R) warp_radix_sort(R - p0, s.ord + p0, key_of, s.kb, s.vb, s.rk + p0, s.ord + p0, hist);
                }
                __syncwarp();
                if (it > 0) {
                    const int p0 = max(0, min(first_change, R));
                    start = R;
                    for (int base = p0 & ~31; base < R; base += 32) {
                        const int i = base + lane;
                        const unsigned moved = __ballot_sync(FULL, i >= p0 && i < R && __ldcg(&s.ord[i]) != prev[i]);
                        if (moved) {
                            start = base + __ffs(moved) - 1;
                            break;
                        }
                    }
                    start &= ~31;
                    if (lane == 0) ph[15] += start;
                }
            }
            for (int i = start + lane; i < R; i += 32) s.aux[s.ord[i]] = (uint32_t)(i + 1);
            __syncwarp();
            dphase(ph, 1, tph);
            rr = dual_replay(p, s, src, R, bad, !exact, it > 0, start, first_change);
            __syncwarp();
            dphase(ph, 2, tph);
        }
        if (lane == 0) ph[7] += rounds_run;
    }
    __syncthreads();
    tph = clock64();
    const bool ok = live && rr == 0;
    if (live) {
        if (ok) {
            dual_accumulate(p, s, src, R, cnt, bad, ph);
            tph = clock64();
        } else if (lane == 0) {
            if (exact) raise_err(p.hdr, CS_ERR_INTERNAL, 24);
            else {
                const unsigned f = atomicAdd(&p.hdr->n_inexact, 1u);
                if (f < (unsigned)p.inexact_cap) p.inexact[f] = li;
                else raise_err(p.hdr, CS_ERR_CAPACITY, 25);
            }
        }
        if (__any_sync(FULL, bad) && lane == 0) raise_err(p.hdr, CS_ERR_INTERNAL, 26);
        __syncwarp();
        for (int i = lane; i < R; i += 32) {
            const int S = s.ord[i];
            s.key[S] = KEY_INF;
            s.aux[S] = 0u;
            if (wide) s.lsec[S] = NO_LSEC;
        }
        __syncwarp();
        dphase(ph, 5, tph);
        settled += R;
    }
    __syncthreads();
    return ok;
}

__device__ __forceinline__ void flush_dual_counters(const DualParams &p, const long long *ph, long long relaxed,
                                                    long long settled, long long done_src) {
    const long long rsum = warp_sum_ll(relaxed);
    __syncwarp();
    if (lane_id() == 0) {
        for (int q = 0; q < 8; q++) atomicAdd(&p.hdr->pad[q], (unsigned long long)ph[q]);
        atomicAdd(&p.hdr->pad[15], (unsigned long long)ph[15]);
        atomicAdd(&p.hdr->edges_relaxed, (unsigned long long)rsum);
        atomicAdd(&p.hdr->nodes_settled, (unsigned long long)settled);
        atomicAdd(&p.hdr->sources_done, (unsigned long long)done_src);
    }
}

// dual_kernel with the block's warps in lockstep (run_dual_source_sync): a block claims one source per
// warp at a time; every warp of the block stays in the loop until the block's sources run out.
template <int MINB>
__global__ void __launch_bounds__(256, MINB) dual_sync_kernel(const DualParams p) {
    __shared__ uint32_t hist_all[8][256];
    __shared__ int cnt_all[8][MAXK];
    __shared__ long long ph_all[8][16];
    __shared__ unsigned long long blk_base;
    __shared__ unsigned blk_err;
    const int lane = lane_id();
    const int wib = threadIdx.x >> 5;
    const int slot0 = blockIdx.x * (blockDim.x >> 5);
    const int nw = min((int)(blockDim.x >> 5), p.n_slots - slot0);
    const bool has_slot = wib < nw;
    const int slot = has_slot ? slot0 + wib : 0;
    DSlot s = dslot(p.dense, p.dense_stride, p.compact, (size_t)p.cap, p.k, slot, p.geo_n);
    if (p.pass == 3) s.lsec = (uint32_t *)(p.dense + p.dense_stride * (size_t)(slot + p.lsec_slot_off));
    long long *ph = ph_all[wib];
    if (lane < 16) ph[lane] = 0;
    __syncwarp();
    long long relaxed = 0, settled = 0, done_src = 0;
    while (true) {
        if (threadIdx.x == 0) {
            blk_base = atomicAdd(p.pass ? &p.hdr->work_next2 : &p.hdr->work_next, (unsigned long long)max(nw, 0));
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
        if (run_dual_source_sync(p, s, mine, li, src, hist_all[wib], cnt_all[wib], ph, relaxed, settled)) {
            done_src++;
            if (lane == 0) count_progress(p.hdr);
        }
    }
    if (has_slot) flush_dual_counters(p, ph, relaxed, settled, done_src);
}

template <int MINB>
__global__ void __launch_bounds__(256, MINB) dual_kernel(const DualParams p) {
    __shared__ uint32_t hist_all[8][256];
    __shared__ int cnt_all[8][MAXK];
    __shared__ long long ph_all[8][16];
    const int lane = lane_id();
    const int wib = threadIdx.x >> 5;
    const int slot = (int)((blockIdx.x * (blockDim.x >> 5)) + wib);
    if (slot >= p.n_slots) return;
    long long *ph = ph_all[wib];
    if (lane < 16) ph[lane] = 0;
    __syncwarp();
    DSlot s = dslot(p.dense, p.dense_stride, p.compact, (size_t)p.cap, p.k, slot, p.geo_n);
    if (p.pass == 3) s.lsec = (uint32_t *)(p.dense + p.dense_stride * (size_t)(slot + p.lsec_slot_off));
    long long relaxed = 0, settled = 0, done_src = 0;
    while (true) {
        unsigned long long idx = 0;
        if (lane == 0) idx = atomicAdd(p.pass ? &p.hdr->work_next2 : &p.hdr->work_next, 1ull);
        idx = __shfl_sync(FULL, idx, 0);
        if (idx >= (unsigned long long)p.n_src) break;
        if (__ldcg(&p.hdr->err) != 0u) break;
        const int li = p.remap ? p.remap[idx] : (int)idx;
        if (run_dual_source(p, s, li, p.src_list[li], hist_all[wib], cnt_all[wib], ph, relaxed, settled)) {
            done_src++;
            if (lane_id() == 0) count_progress(p.hdr);
        }
    }
    flush_dual_counters(p, ph, relaxed, settled, done_src);
}

// Batched form: the (job, source) items of many simplest-path queries (graphs, thresholds, source
// subsets) in one persistent launch.  Slot geometry comes from the base parameters (largest graph,
// threshold count and capacity of the batch); an item's job is the one whose item_begin is the
// largest <= the item.  Lists record global item indices.
__device__ __forceinline__ int djob_of(const cs_dual_batch_job *jobs, int n_jobs, long long item) {
    int lo = 0, hi = n_jobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].item_begin <= item) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ void djob_params(const DualParams &base, const cs_dual_batch_job &j, DualParams &p) {
    p = base;
    p.g = j.g;
    p.k = j.k;
    uint32_t maxs = 0;
    for (int i = 0; i < MAXK; i++) {
        p.sk[i] = i < j.k ? (float)j.seconds[i] : 0.0f;
        if (i < j.k) maxs = max(maxs, j.seconds[i]);
    }
    p.maxsec = (float)maxs;
    p.tol = j.tolerance;
    p.asu = j.angular_scaling_unit;
    p.fso = j.farness_scaling_offset;
    p.closeness = j.compute_closeness;
    p.betweenness = j.compute_betweenness;
    p.track_reach = 0;
    p.reach = nullptr;
    p.src_list = j.sources_dev;
    p.n_src = j.n_sources;
    p.src_wt = j.src_wt_dev;
    p.eligible = j.eligible_dev;
    p.out = j.out_dev;
    p.bucket = j.bucket_dev;
}

template <int MINB>
__global__ void __launch_bounds__(256, MINB) dual_batch_kernel(const DualParams base, const cs_dual_batch_job *jobs,
                                                            int n_jobs, long long n_items) {
    __shared__ uint32_t hist_all[8][256];
    __shared__ int cnt_all[8][MAXK];
    __shared__ long long ph_all[8][16];
    const int lane = lane_id();
    const int wib = threadIdx.x >> 5;
    const int slot = (int)((blockIdx.x * (blockDim.x >> 5)) + wib);
    if (slot >= base.n_slots) return;
    long long *ph = ph_all[wib];
    if (lane < 16) ph[lane] = 0;
    __syncwarp();
    DSlot s = dslot(base.dense, base.dense_stride, base.compact, (size_t)base.cap, base.k, slot, base.geo_n);
    if (base.pass == 3)
        s.lsec = (uint32_t *)(base.dense + base.dense_stride * (size_t)(slot + base.lsec_slot_off));
    long long relaxed = 0, settled = 0, done_src = 0;
    // the warp's job parameters in shared memory (a local copy would sit in the stack frame)
    __shared__ DualParams pj_all[8];
    DualParams &p = pj_all[wib];
    int cur_job = -1;
    while (true) {
        unsigned long long idx = 0;
        if (lane == 0) idx = atomicAdd(base.pass ? &base.hdr->work_next2 : &base.hdr->work_next, 1ull);
        idx = __shfl_sync(FULL, idx, 0);
        const long long n = base.pass ? base.n_src : n_items;
        if ((long long)idx >= n) break;
        if (__ldcg(&base.hdr->err) != 0u) break;
        const long long item = base.remap ? (long long)base.remap[idx] : (long long)idx;
        const int jb = djob_of(jobs, n_jobs, item);
        if (jb != cur_job) {
            if (lane == 0) djob_params(base, jobs[jb], p);
            __syncwarp();
            cur_job = jb;
        }
        const int li = (int)(item - jobs[jb].item_begin);
        if (run_dual_source(p, s, (int)item, p.src_list[li], hist_all[wib], cnt_all[wib], ph, relaxed, settled))
            done_src++;
    }
    flush_dual_counters(base, ph, relaxed, settled, done_src);
}

// Closeness prefixes of every job with closeness (blockIdx.y strides the jobs); the bucket is
// zeroed as it is read, so buckets are zero between runs.
__global__ void dual_batch_prefix(const cs_dual_batch_job *jobs, int n_jobs) {
    for (int j = blockIdx.y; j < n_jobs; j += gridDim.y) {
        const cs_dual_batch_job &jb = jobs[j];
        if (!jb.compute_closeness || jb.n_sources <= 0) continue;
        const int K = jb.k, N = jb.g.n_bound;
        const size_t KN = (size_t)K * N;
        for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < N; t += gridDim.x * blockDim.x) {
            for (int m = 0; m < 3; m++) {
                double acc = 0.0;
                for (int k = 0; k < K; k++) {
                    const size_t o = (size_t)m * KN + (size_t)k * N + t;
                    acc += jb.bucket_dev[o];
                    jb.bucket_dev[o] = 0.0;
                    jb.out_dev[o] += acc;
                }
            }
        }
    }
}

// ------------------------------------------------------------------------------------------
// Simplest-path trees: dijkstra_tree_angular (rust/src/centrality.rs:1202-1332), one query per
// warp, run by lane 0 in the reference's exact heap order (Rust BinaryHeap restated by
// heap_sift_up / tree_heap_pop).  This search is heap-order dependent by construction: it accepts
// tied offers within an absolute epsilon, updates already-visited states, and keeps a node-level
// best with its own epsilon rule, so it is replayed sequentially rather than label-corrected.
// Per slot: dense state records [2N] and node positions [N] (zero = untouched), compact rows
// (node, simpl_dist, agg_seconds, pred) in first-reach order and the heap.
// ------------------------------------------------------------------------------------------
struct DTreeState {
    float route, simpl, agg;
    uint32_t flags;  // 1: touched, 2: visited
};
struct DTreeRow {
    int32_t node;
    float simpl, agg;
    int32_t pred;
};
struct DTreeParams {
    cs_dual_graph g;
    const int32_t *src;
    const int32_t *remap;  // retry pass: query indices to run
    long long n_items;
    float maxsec;
    char *dense;
    size_t dense_stride;
    int geo_n;
    char *compact;
    size_t compact_stride;
    int cap, hcap;
    int32_t row_cap;
    int32_t *t_count, *t_node, *t_pred;
    float *t_simpl, *t_agg;
    int32_t *failed;
    int fail_cap;
    int final_pass;
    int n_slots;
    WsHeader *hdr;
};

// pop of a Rust BinaryHeap (sift_down_to_bottom, then sift_up): returns the top state
__device__ __forceinline__ int32_t tree_heap_pop(int32_t *h, int &len) {
    len--;
    const int32_t s_top = h[1];
    if (len > 0) {
        const int32_t m_last = h[2 * len], s_last = h[2 * len + 1];
        int pos = 0, child = 1;
        const int end = len;
        while (end >= 2 && child <= end - 2) {
            child += hle(h, child, child + 1) ? 1 : 0;
            h[2 * pos] = h[2 * child];
            h[2 * pos + 1] = h[2 * child + 1];
            pos = child;
            child = 2 * pos + 1;
        }
        if (child == end - 1) {
            h[2 * pos] = h[2 * child];
            h[2 * pos + 1] = h[2 * child + 1];
            pos = child;
        }
        h[2 * pos] = m_last;
        h[2 * pos + 1] = s_last;
        heap_sift_up(h, 0, pos);
    }
    return s_top;
}

// Returns the number of reached nodes, or -1 when the rows or the heap overflowed.
__device__ int dual_tree_search(const DTreeParams &p, DTreeState *S, uint32_t *pos, DTreeRow *rows, int32_t *h,
                                int src) {
    const float eps = TIE_EPSILON;
    int n = 0, len = 0;
    pos[src] = 1u;
    rows[0] = DTreeRow{src, 0.0f, 0.0f, -1};
    n = 1;
    for (int sl = 0; sl < 2; sl++) {
        const int st = 2 * src + sl;
        S[st] = DTreeState{0.0f, 0.0f, 0.0f, 1u};
        h[2 * len] = 0;
        h[2 * len + 1] = st;
        len++;
        heap_sift_up(h, 0, len - 1);
    }
    while (len > 0) {
        const int st = tree_heap_pop(h, len);
        if (S[st].flags & 2u) continue;
        S[st].flags |= 2u;
        const int cur = st >> 1, entry = st & 1;
        const DTreeState cs0 = S[st];
        const int beg = __ldg(&p.g.ptr_dev[cur]), end = __ldg(&p.g.ptr_dev[cur + 1]);
        for (int e = beg; e < end; e++) {
            if (__ldg(&p.g.exit_slot_dev[e]) != 1 - entry) continue;
            const int nx = __ldg(&p.g.to_dev[e]);
            const int nst = 2 * nx + __ldg(&p.g.entry_slot_dev[e]);
            const float csec = __fadd_rn(cs0.agg, __ldg(&p.g.w_dev[e]));
            if (csec > p.maxsec) continue;
            const float csimpl = __fadd_rn(cs0.simpl, __ldg(&p.g.ang_dev[e]));
            const float cm = __fadd_rn(csimpl, __fmul_rn(ANGULAR_TIE_BREAK, __ldg(&p.g.len_dev[e])));
            const DTreeState nxs = S[nst];
            const bool touched = (nxs.flags & 1u) != 0u;
            const float nroute = touched ? nxs.route : __int_as_float(INF_BITS);
            const float nagg = touched ? nxs.agg : __int_as_float(INF_BITS);
            const bool improved = __fadd_rn(cm, eps) < nroute;
            const bool tied = fabsf(__fadd_rn(cm, -nroute)) <= eps;
            if (!(improved || (tied && csec < nagg && st != nst))) continue;
            S[nst] = DTreeState{cm, csimpl, csec, 1u | (nxs.flags & 2u)};
            if (len >= p.hcap) return -1;
            h[2 * len] = (int32_t)__float_as_uint(cm);
            h[2 * len + 1] = nst;
            len++;
            heap_sift_up(h, 0, len - 1);
            uint32_t ps = pos[nx];
            if (ps == 0u) {
                if (n >= p.cap) return -1;
                pos[nx] = (uint32_t)(n + 1);
                rows[n] = DTreeRow{nx, csimpl, csec, cur};
                n++;
                continue;
            }
            DTreeRow &r = rows[ps - 1];
            const bool node_improved = __fadd_rn(csimpl, eps) < r.simpl;
            const bool node_tied = fabsf(__fadd_rn(csimpl, -r.simpl)) <= eps;
            if (node_improved || (node_tied && csec < r.agg)) r = DTreeRow{nx, csimpl, csec, cur};
        }
    }
    return n;
}

__global__ void __launch_bounds__(256) dual_tree_kernel(const DTreeParams p) {
    const int lane = lane_id();
    const int slot = (int)(blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5));
    if (slot >= p.n_slots) return;
    char *d = p.dense + p.dense_stride * (size_t)slot;
    DTreeState *S = (DTreeState *)d;
    uint32_t *pos = (uint32_t *)(d + al256((size_t)p.geo_n * 2 * sizeof(DTreeState)));
    char *c = p.compact + p.compact_stride * (size_t)slot;
    DTreeRow *rows = (DTreeRow *)c;
    int32_t *h = (int32_t *)(c + al256((size_t)p.cap * sizeof(DTreeRow)));
    while (true) {
        unsigned long long idx = 0;
        if (lane == 0) idx = atomicAdd(p.remap ? &p.hdr->work_next2 : &p.hdr->work_next, 1ull);
        idx = __shfl_sync(FULL, idx, 0);
        if ((long long)idx >= p.n_items) break;
        const int q = p.remap ? p.remap[idx] : (int)idx;
        const int src = p.src[q];
        int n = 0;
        if (lane == 0) n = dual_tree_search(p, S, pos, rows, h, src);
        n = __shfl_sync(FULL, n, 0);
        __syncwarp();
        if (n < 0) {
            // rows or heap overflowed: the touched entries are not all listed, so clear the slot
            for (size_t j = lane; j < (size_t)p.g.n_bound * 2; j += 32) S[j] = DTreeState{0.0f, 0.0f, 0.0f, 0u};
            for (int j = lane; j < p.g.n_bound; j += 32) pos[j] = 0u;
            if (lane == 0) {
                if (p.final_pass) {
                    raise_err(p.hdr, CS_ERR_CAPACITY, 30);
                } else {
                    const unsigned f = atomicAdd(&p.hdr->n_failed, 1u);
                    if (f < (unsigned)p.fail_cap) p.failed[f] = q;
                    else raise_err(p.hdr, CS_ERR_CAPACITY, 31);
                }
            }
            __syncwarp();
            continue;
        }
        const bool fits = n <= p.row_cap;
        for (int i = lane; i < n; i += 32) {
            const DTreeRow r = rows[i];
            if (fits) {
                const size_t o = (size_t)q * p.row_cap + i;
                p.t_node[o] = r.node;
                p.t_simpl[o] = r.simpl;
                p.t_agg[o] = r.agg;
                p.t_pred[o] = r.pred;
            }
            S[2 * r.node] = DTreeState{0.0f, 0.0f, 0.0f, 0u};
            S[2 * r.node + 1] = DTreeState{0.0f, 0.0f, 0.0f, 0u};
            pos[r.node] = 0u;
        }
        if (lane == 0) p.t_count[q] = fits ? n : -n;
        __syncwarp();
    }
}

// Packed edge records (one 128-bit load per edge in the searches and the replay).
__global__ void dual_pack_kernel(const cs_dual_graph g, uint4 *fwd, uint4 *rev) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < g.n_edges; e += gridDim.x * blockDim.x) {
        const unsigned ex = g.exit_slot_dev[e], en = g.entry_slot_dev[e];
        fwd[e] = make_uint4((unsigned)(2 * g.to_dev[e]) + en | (ex << 31), __float_as_uint(g.w_dev[e]),
                            __float_as_uint(g.ang_dev[e]), __float_as_uint(g.len_dev[e]));
        const int id = g.rid_dev[e];
        const unsigned rex = g.exit_slot_dev[id], ren = g.entry_slot_dev[id];
        rev[e] = make_uint4((unsigned)(2 * g.rfrom_dev[e]) + (1u - rex) | (ren << 31), __float_as_uint(g.w_dev[id]),
                            __float_as_uint(g.ang_dev[id]), __float_as_uint(g.len_dev[id]));
    }
}

__global__ void fill_dual_dense(char *dense, size_t stride, int n_bound, int n_slots) {
    const size_t per = 2 * (size_t)n_bound;
    const size_t total = per * (size_t)n_slots;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const int slot = (int)(t / per);
        const size_t j = t % per;
        char *d = dense + stride * (size_t)slot;
        ((unsigned long long *)d)[j] = KEY_INF;
        ((uint32_t *)(d + al256((size_t)n_bound * 16)))[j] = 0u;
    }
}

__global__ void dual_bucket_prefix(const double *bucket, double *out, int K, int N) {
    const size_t KN = (size_t)K * N;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < N; t += gridDim.x * blockDim.x) {
        for (int m = 0; m < 3; m++) {
            double acc = 0.0;
            for (int k = 0; k < K; k++) {
                acc += bucket[(size_t)m * KN + (size_t)k * N + t];
                out[(size_t)m * KN + (size_t)k * N + t] += acc;
            }
        }
    }
}

}  // namespace csd

// ==========================================================================================
// Host side (C-ABI).
// ==========================================================================================
namespace {
thread_local std::string d_err;

cs_status dfail(cs_status code, const std::string &msg) {
    cs_set_error_internal(msg.c_str());
    return code;
}
cs_status dcuda(cudaError_t e, const char *what) {
    return dfail(CS_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
int dsm_count() {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    return n;
}

struct DLayout {
    size_t failed_off, failed2_off, inexact_off, inexact2_off, bucket_off, dense_off, compact_off, compact_total, total,
        dense_stride;
    int fail_cap;
};

DLayout dlayout(int n_bound, int n_slots, int cap, int K) {
    DLayout l;
    l.fail_cap = std::max(n_slots, 1 << 18);
    l.failed_off = 256;
    l.failed2_off = csd::al256(l.failed_off + 4 * (size_t)l.fail_cap);
    l.inexact_off = csd::al256(l.failed2_off + 4 * (size_t)l.fail_cap);
    l.inexact2_off = csd::al256(l.inexact_off + 4 * (size_t)l.fail_cap);
    l.bucket_off = csd::al256(l.inexact2_off + 4 * (size_t)l.fail_cap);
    l.dense_off = csd::al256(l.bucket_off + sizeof(double) * 3 * (size_t)K * (size_t)n_bound);
    l.dense_stride = csd::al256((size_t)n_bound * 16) + csd::al256((size_t)n_bound * 8);
    l.compact_off = l.dense_off + l.dense_stride * (size_t)n_slots;
    l.compact_total = std::max(csd::compact_bytes_d((size_t)cap, K) * (size_t)n_slots,
                               csd::compact_bytes_d(2 * (size_t)n_bound, K));
    l.total = l.compact_off + l.compact_total;
    return l;
}

// Tree workspace: header, failed list, per-slot dense (state records + node positions), per-slot
// compact (rows + heap of 4 x cap entries; the full-size retry uses cap = N with 8 x N entries).
struct TLayout {
    size_t failed_off, dense_off, dense_stride, compact_off, compact_total, total;
    int fail_cap;
};
size_t tcompact_bytes_h(size_t cap, size_t hcap) {
    return csd::al256(cap * sizeof(csd::DTreeRow)) + csd::al256(hcap * 8);
}
size_t tcompact_bytes(size_t cap) { return tcompact_bytes_h(cap, 4 * cap); }
TLayout tlayout(int n_bound, int n_slots, int cap) {
    TLayout l;
    l.fail_cap = std::max(n_slots, 1 << 16);
    l.failed_off = 256;
    l.dense_off = csd::al256(l.failed_off + 4 * (size_t)l.fail_cap);
    l.dense_stride = csd::al256((size_t)n_bound * 2 * sizeof(csd::DTreeState)) + csd::al256((size_t)n_bound * 4);
    l.compact_off = l.dense_off + l.dense_stride * (size_t)n_slots;
    l.compact_total = std::max(tcompact_bytes((size_t)cap) * (size_t)n_slots,
                               tcompact_bytes_h((size_t)n_bound, 8 * (size_t)n_bound));
    l.total = l.compact_off + l.compact_total;
    return l;
}

cs_status dvalidate(const cs_dual_graph *g) {
    if (!g) return dfail(CS_ERR_ARG, "graph is NULL");
    if (g->n_bound <= 0) return dfail(CS_ERR_ARG, "NetworkStructure contains no nodes.");
    if (g->max_out_degree > csd::DPM)
        return dfail(CS_ERR_ARG, "a dual node has more than 8 incoming or outgoing dual edges (intersections of "
                                 "degree above 5); not supported by the simplest-path kernels");
    return CS_OK;
}

// The centrality kernels read the packed edge records.
cs_status dvalidate_packed(const cs_dual_graph *g) {
    if (g->n_bound >= (1 << 30)) return dfail(CS_ERR_ARG, "dual graph too large (2^30 nodes or more)");
    if (g->n_edges > 0 && (!g->fwd_pack_dev || !g->rev_pack_dev))
        return dfail(CS_ERR_ARG, "dual graph without packed edge records (cs_dual_pack)");
    if (((uintptr_t)g->fwd_pack_dev | (uintptr_t)g->rev_pack_dev) & 15u)
        return dfail(CS_ERR_ARG, "packed edge records must be 16-byte aligned");
    return CS_OK;
}

cs_status dreset(char *dense, size_t stride, int n_bound, int n_slots, cudaStream_t s) {
    const size_t total = 2 * (size_t)n_bound * (size_t)n_slots;
    int blocks = (int)std::min<size_t>((total + 255) / 256, (size_t)std::max(1, dsm_count()) * 16);
    csd::fill_dual_dense<<<std::max(1, blocks), 256, 0, s>>>(dense, stride, n_bound, n_slots);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CS_OK : dcuda(e, "fill_dual_dense launch");
}

// Replay / re-sort rounds per source (CS_DUAL_REPLAY_ROUNDS overrides the default of 4).
int replay_rounds() {
    const char *e = getenv("CS_DUAL_REPLAY_ROUNDS");
    const int r = e ? atoi(e) : 0;
    return (r >= 1 && r <= 64) ? r : 4;
}

// Sources whose replay disagreed first run the widened search (pass 3) and only those that still
// disagree run the exact heap search.  CS_DUAL_WIDE=0 sends them straight to the exact search;
// CS_DUAL_WIDE=1 runs every source through the widened search (a check of that pass).
int dual_wide_mode() {
    const char *e = getenv("CS_DUAL_WIDE");
    if (e && e[0] == '0') return 0;
    if (e && e[0] == '1') return 2;
    return 1;
}

// Resident 256-thread blocks per SM the dual kernels are compiled for: 4 (32 warps per SM, 64
// registers).  On the 124,500-node curved dual the memory latency the extra warps hide outweighs their
// register spills: 224k sources/s at 2 km against 211k with 3 blocks (30.9k and 30.4k at 5 km); 3
// blocks had beaten 2 by 5% and 8%.  CS_DUAL_MINB=2 or 3 selects the other builds.
int dual_minb() {
    const char *e = getenv("CS_DUAL_MINB");
    return (e && e[0] == '2') ? 2 : ((e && e[0] == '3') ? 3 : 4);
}

// Lockstep phases for the simplest-path kernel (default; CS_DUAL_SYNC=0 leaves each warp on its own
// source).  On the 124,500-node curved dual: 270k sources/s at 2 km against 227k, 31.7k against
// 30.6k at 5 km, with the SMs fetching one phase's code at a time.
bool dual_sync() {
    const char *e = getenv("CS_DUAL_SYNC");
    return !(e && e[0] == '0');
}

cs_status dlaunch(csd::DualParams &p, int n_slots, cudaStream_t s) {
    p.n_slots = n_slots;
    if (dual_sync()) {
        if (dual_minb() == 4) csd::dual_sync_kernel<4><<<(n_slots + 7) / 8, 256, 0, s>>>(p);
        else if (dual_minb() == 3) csd::dual_sync_kernel<3><<<(n_slots + 7) / 8, 256, 0, s>>>(p);
        else csd::dual_sync_kernel<2><<<(n_slots + 7) / 8, 256, 0, s>>>(p);
    } else if (dual_minb() == 4) csd::dual_kernel<4><<<(n_slots + 7) / 8, 256, 0, s>>>(p);
    else if (dual_minb() == 3) csd::dual_kernel<3><<<(n_slots + 7) / 8, 256, 0, s>>>(p);
    else csd::dual_kernel<2><<<(n_slots + 7) / 8, 256, 0, s>>>(p);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CS_OK : dcuda(e, "dual_kernel launch");
}

cs_status dsync_header(cs::WsHeader *hd, cs::WsHeader &h, cudaStream_t s) {
    cudaError_t e = cs::read_header(hd, h, s, true);
    if (e != cudaSuccess) return dcuda(e, "dual kernel");
    if (h.err != 0u)
        return dfail((cs_status)h.err, "device-side check failed (code " + std::to_string(h.err) + " at " +
                                           std::to_string(h.err_where) + ")");
    return CS_OK;
}

// The passes of one call after its parameters are set.  The first pass runs every source on every
// slot.  Sources that overflowed their slot run again at 4x the capacity (then 4x again, up to every
// state), each level on as many slots as the workspace's compact region holds at that capacity.
// Sources whose replay disagreed then run the widened search (pass 3, on half the slots: each keeps
// its lsec array in the key array of a partner slot), and those that still disagree the exact heap
// search, both starting at the plan's capacity.  wide_mode 2 runs every source through pass 3 in
// place of the first pass.  launch(params, slots) starts one pass.  n_exact: sources the exact
// search redid.
template <class Launch>
cs_status dual_passes(const csd::DualParams &p, const DLayout &lay, const cs_plan *plan, int K, int N2, long long n_all,
                      int wide_mode, Launch launch, cudaStream_t s, long long &n_over, long long &n_exact) {
    char *base = (char *)p.hdr;
    int32_t *listA = p.failed;
    int32_t *listB = (int32_t *)(base + lay.failed2_off);
    int32_t *inexact2 = (int32_t *)(base + lay.inexact2_off);
    const int half = plan->n_slots / 2;
    if (half < 1) wide_mode = 0;
    cs::WsHeader h;
    memset(&h, 0, sizeof(h));
    auto chain = [&](int pass, const int32_t *in, long long n_in, int cap0) -> cs_status {
        int cap_l = std::min(N2, cap0);
        const int32_t *list = in;
        while (n_in > 0) {
            const bool final = cap_l >= N2;
            int32_t *out_l = (list == listA) ? listB : listA;
            csd::DualParams p2 = p;
            p2.pass = pass;
            p2.cap = cap_l;
            p2.remap = list;
            p2.n_src = list ? std::min<long long>(n_in, lay.fail_cap) : n_in;
            p2.failed = out_l;
            p2.fail_final = final ? 1 : 0;
            if (pass == 3) {
                p2.inexact = inexact2;
                p2.lsec_slot_off = half;
            }
            cudaError_t e2 = cudaMemsetAsync(&p.hdr->work_next2, 0, sizeof(unsigned long long), s);
            if (e2 == cudaSuccess) e2 = cudaMemsetAsync(&p.hdr->n_failed, 0, sizeof(unsigned), s);
            if (e2 != cudaSuccess) return dcuda(e2, "retry counter reset");
            const size_t per = csd::compact_bytes_d((size_t)cap_l, K);
            long long slots2 = std::min<long long>((long long)(lay.compact_total / per), plan->n_slots);
            if (pass == 3) slots2 = std::min<long long>(slots2, half);
            slots2 = std::max<long long>(1, std::min<long long>(slots2, p2.n_src));
            cs_status st2 = launch(p2, (int)slots2);
            if (st2 != CS_OK) return st2;
            cs::WsHeader h2;
            st2 = dsync_header(p.hdr, h2, s);
            if (st2 != CS_OK) return st2;
            h.n_inexact = h2.n_inexact;  // retries may list more disagreeing sources
            n_in = final ? 0 : (long long)h2.n_failed;
            list = out_l;
            cap_l = (int)std::min<long long>(N2, 4ll * cap_l);
        }
        return CS_OK;
    };
    cs_status st;
    n_over = 0;
    if (wide_mode == 2) {
        st = chain(3, nullptr, n_all, plan->cap);
        if (st != CS_OK) return st;
    } else {
        csd::DualParams p0 = p;
        st = launch(p0, plan->n_slots);
        if (st != CS_OK) return st;
        st = dsync_header(p.hdr, h, s);
        if (st != CS_OK) return st;
        n_over = h.n_failed;
        if (h.n_failed > 0u) {
            st = chain(1, listA, h.n_failed, 4 * std::max(plan->cap, 16));
            if (st != CS_OK) return st;
        }
    }
    const int32_t *ex = (wide_mode == 2) ? inexact2 : p.inexact;
    long long n_ex = std::min<long long>(h.n_inexact, lay.fail_cap);
    if (wide_mode == 1 && n_ex > 0) {
        cudaError_t e = cudaMemsetAsync(&p.hdr->n_inexact, 0, sizeof(unsigned), s);
        if (e != cudaSuccess) return dcuda(e, "retry counter reset");
        h.n_inexact = 0;
        st = chain(3, p.inexact, n_ex, plan->cap);
        if (st != CS_OK) return st;
        ex = inexact2;
        n_ex = std::min<long long>(h.n_inexact, lay.fail_cap);
    }
    n_exact = n_ex;
    if (n_ex > 0) return chain(2, ex, n_ex, plan->cap);
    return CS_OK;
}
}  // namespace

extern "C" {

cs_status cs_dual_pack(const cs_dual_graph *g, void *fwd_pack_dev, void *rev_pack_dev, void *stream) {
    cs_status st = dvalidate(g);
    if (st != CS_OK) return st;
    if (g->n_bound >= (1 << 30)) return dfail(CS_ERR_ARG, "dual graph too large (2^30 nodes or more)");
    if (g->n_edges <= 0) return CS_OK;
    if (!fwd_pack_dev || !rev_pack_dev) return dfail(CS_ERR_ARG, "packed record arrays are NULL");
    if (((uintptr_t)fwd_pack_dev | (uintptr_t)rev_pack_dev) & 15u)
        return dfail(CS_ERR_ARG, "packed edge records must be 16-byte aligned");
    const int blocks = std::max(1, std::min((g->n_edges + 255) / 256, std::max(1, dsm_count()) * 8));
    csd::dual_pack_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(*g, (uint4 *)fwd_pack_dev, (uint4 *)rev_pack_dev);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CS_OK : dcuda(e, "dual_pack_kernel launch");
}

cs_status cs_plan_dual(const cs_dual_graph *g, int32_t mode, int32_t k, int32_t cap, int32_t max_slots,
                       int64_t mem_budget_bytes, cs_plan *plan) {
    cs_status st = dvalidate(g);
    if (st != CS_OK) return st;
    if (!plan) return dfail(CS_ERR_ARG, "plan is NULL");
    if (mode != 0) return dfail(CS_ERR_ARG, "unknown dual mode");
    if (k < 1 || k > CS_MAX_THRESHOLDS) return dfail(CS_ERR_ARG, "threshold count out of range");
    const int sms = dsm_count();
    if (sms <= 0) return dfail(CS_ERR_CUDA, "no CUDA device");
    int bpsm = 0;
    const int mb = dual_minb();
    cudaError_t e = mb == 4   ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bpsm, csd::dual_kernel<4>, 256, 0)
                    : mb == 3 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bpsm, csd::dual_kernel<3>, 256, 0)
                              : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bpsm, csd::dual_kernel<2>, 256, 0);
    if (e != cudaSuccess) return dcuda(e, "occupancy query");
    int slots = sms * std::max(1, bpsm) * 8;
    if (max_slots > 0) slots = std::min(slots, max_slots);
    const int n2 = 2 * g->n_bound;
    if (cap <= 0) cap = std::min(n2, 16384);
    cap = std::max(64, std::min(cap, n2));
    if (mem_budget_bytes > 0)
        while (slots > 8 && (int64_t)dlayout(g->n_bound, slots, cap, k).total > mem_budget_bytes) slots = slots * 7 / 8;
    plan->n_slots = std::max(1, slots);
    plan->cap = cap;
    plan->threads_per_block = 256;
    plan->blocks = (plan->n_slots + 7) / 8;
    if (!(plan->delta_seconds > 0.0f)) plan->delta_seconds = 30.0f;  // band width in route degrees
    plan->lanes = k;
    plan->n_bound = g->n_bound;
    plan->workspace_bytes = dlayout(g->n_bound, plan->n_slots, cap, k).total;
    return CS_OK;
}

cs_status cs_centrality_simplest(const cs_dual_graph *g, const cs_query *q, const cs_plan *plan, void *ws,
                                 size_t ws_bytes, cs_outputs out, void *stream_v) {
    cs_status st = dvalidate(g);
    if (st == CS_OK) st = dvalidate_packed(g);
    if (st != CS_OK) return st;
    if (!q || !plan || !ws) return dfail(CS_ERR_ARG, "query/plan/workspace is NULL");
    const int K = q->k;
    if (K < 1 || K > CS_MAX_THRESHOLDS) return dfail(CS_ERR_ARG, "threshold count out of range");
    if (plan->lanes < K) return dfail(CS_ERR_ARG, "plan was made for fewer thresholds");
    // slot geometry is the plan's: one workspace serves every dual graph up to its node bound
    const int geo_n = plan->n_bound > 0 ? plan->n_bound : g->n_bound;
    if (geo_n < g->n_bound) return dfail(CS_ERR_ARG, "plan was made for a smaller graph");
    const DLayout lay = dlayout(geo_n, plan->n_slots, plan->cap, plan->lanes);
    if (ws_bytes < lay.total) return dfail(CS_ERR_ARG, "workspace too small for this plan");
    if (!out.out_dev) return dfail(CS_ERR_ARG, "out_dev is NULL");
    if (q->track_reach && !out.reach_dev) return dfail(CS_ERR_ARG, "reach_dev required when track_reach");
    if (!(q->speed_m_s > 0.0f)) return dfail(CS_ERR_ARG, "speed_m_s must be finite and positive");
    cudaStream_t s = (cudaStream_t)stream_v;
    char *base = (char *)ws;
    csd::DualParams p;
    memset(&p, 0, sizeof(p));
    p.g = *g;
    p.geo_n = geo_n;
    p.k = K;
    uint32_t maxs = 0;
    for (int i = 0; i < K; i++) {
        p.sk[i] = (float)q->seconds[i];
        maxs = std::max(maxs, q->seconds[i]);
    }
    p.maxsec = (float)maxs;
    p.tol = q->tolerance;
    p.asu = q->angular_scaling_unit;
    p.fso = q->farness_scaling_offset;
    p.delta = plan->delta_seconds > 0.0f ? plan->delta_seconds : 30.0f;
    p.closeness = q->compute_closeness;
    p.betweenness = q->compute_betweenness;
    p.track_reach = q->track_reach;
    p.src_list = q->sources_dev;
    p.n_src = q->n_sources;
    p.src_wt = q->src_wt_dev;
    p.eligible = q->eligible_dev;
    p.out = out.out_dev;
    p.reach = out.reach_dev;
    p.hdr = (cs::WsHeader *)base;
    p.failed = (int32_t *)(base + lay.failed_off);
    p.fail_cap = lay.fail_cap;
    p.inexact = (int32_t *)(base + lay.inexact_off);
    p.inexact_cap = lay.fail_cap;
    p.bucket = (double *)(base + lay.bucket_off);
    p.dense = base + lay.dense_off;
    p.dense_stride = lay.dense_stride;
    p.compact = base + lay.compact_off;
    p.cap = plan->cap;
    const char *fe = getenv("CS_DUAL_FORCE_EXACT");
    p.force_exact = (fe && fe[0] == '1') ? 1 : 0;
    p.replay_rounds = replay_rounds();
    if (p.n_src <= 0) return CS_OK;
    cudaError_t e = cudaMemsetAsync(p.hdr, 0, sizeof(cs::WsHeader), s);
    if (e == cudaSuccess && p.closeness)
        e = cudaMemsetAsync(p.bucket, 0, sizeof(double) * 3 * (size_t)K * (size_t)g->n_bound, s);
    if (e != cudaSuccess) return dcuda(e, "workspace reset");
    long long n_over = 0, n_exact = 0, n_launch = 0;
    st = dual_passes(
        p, lay, plan, K, 2 * g->n_bound, p.n_src, dual_wide_mode(),
        [&](csd::DualParams &pp, int slots) {
            n_launch++;
            return dlaunch(pp, slots, s);
        },
        s, n_over, n_exact);
    if (st != CS_OK) return st;
    cs::WsHeader hf;
    st = dsync_header(p.hdr, hf, s);
    if (st != CS_OK) return st;
    cs_set_phase_internal(hf.pad);
    cs_set_counters_internal((long long)hf.sources_done, (long long)hf.edges_relaxed, (long long)hf.nodes_settled,
                             n_launch + (p.closeness ? 1 : 0));
    cs_set_retries_internal(n_over, n_exact);
    if (p.closeness) {
        int blocks = std::max(1, std::min((g->n_bound + 255) / 256, dsm_count() * 8));
        csd::dual_bucket_prefix<<<blocks, 256, 0, s>>>(p.bucket, p.out, K, g->n_bound);
        e = cudaGetLastError();
        if (e != cudaSuccess) return dcuda(e, "dual_bucket_prefix launch");
    }
    return CS_OK;
}

cs_status cs_dual_workspace_init(const cs_plan *plan, int32_t n_bound, void *ws, size_t ws_bytes, void *stream) {
    if (!plan || !ws) return dfail(CS_ERR_ARG, "plan/workspace is NULL");
    if (ws_bytes < plan->workspace_bytes) return dfail(CS_ERR_ARG, "workspace smaller than plan");
    const DLayout lay = dlayout(n_bound, plan->n_slots, plan->cap, plan->lanes);
    cudaError_t e = cudaMemsetAsync(ws, 0, 256, (cudaStream_t)stream);
    if (e != cudaSuccess) return dcuda(e, "workspace init");
    return dreset((char *)ws + lay.dense_off, lay.dense_stride, n_bound, plan->n_slots, (cudaStream_t)stream);
}

// ------------------------------------------------------------------------------------------
// Batched simplest-path form.
// ------------------------------------------------------------------------------------------
}  // extern "C"
namespace {
struct DBatchShape {
    int max_n, max_k;
};

cs_status dbatch_shape(const cs_dual_batch_job *jobs, int n_jobs, DBatchShape &b) {
    if (!jobs || n_jobs <= 0) return dfail(CS_ERR_ARG, "empty batch");
    b.max_n = 1;
    b.max_k = 1;
    for (int j = 0; j < n_jobs; j++) {
        cs_status st = dvalidate(&jobs[j].g);
        if (st == CS_OK) st = dvalidate_packed(&jobs[j].g);
        if (st != CS_OK) return st;
        if (jobs[j].k < 1 || jobs[j].k > CS_MAX_THRESHOLDS) return dfail(CS_ERR_ARG, "threshold count out of range");
        if (!jobs[j].out_dev) return dfail(CS_ERR_ARG, "job without out_dev");
        if (jobs[j].compute_closeness && !jobs[j].bucket_dev)
            return dfail(CS_ERR_ARG, "job with closeness needs bucket_dev");
        b.max_n = std::max(b.max_n, jobs[j].g.n_bound);
        b.max_k = std::max(b.max_k, jobs[j].k);
    }
    return CS_OK;
}

cs_status dbatch_launch(csd::DualParams &p, const cs_dual_batch_job *jobs_dev, int n_jobs, long long n_items, int slots,
                        cudaStream_t s) {
    p.n_slots = slots;
    if (dual_minb() == 4) csd::dual_batch_kernel<4><<<(slots + 7) / 8, 256, 0, s>>>(p, jobs_dev, n_jobs, n_items);
    else if (dual_minb() == 3) csd::dual_batch_kernel<3><<<(slots + 7) / 8, 256, 0, s>>>(p, jobs_dev, n_jobs, n_items);
    else csd::dual_batch_kernel<2><<<(slots + 7) / 8, 256, 0, s>>>(p, jobs_dev, n_jobs, n_items);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? CS_OK : dcuda(e, "dual_batch_kernel launch");
}
}  // namespace
extern "C" {

cs_status cs_dual_batch_prepare(cs_dual_batch_job *jobs_host, int32_t n_jobs, int64_t *n_items) {
    if (!jobs_host || n_jobs <= 0 || !n_items) return dfail(CS_ERR_ARG, "empty batch");
    int64_t acc = 0;
    for (int j = 0; j < n_jobs; j++) {
        jobs_host[j].item_begin = acc;
        acc += std::max(0, jobs_host[j].n_sources);
    }
    *n_items = acc;
    return CS_OK;
}

cs_status cs_dual_batch_plan(const cs_dual_batch_job *jobs_host, int32_t n_jobs, int32_t cap, int32_t max_slots,
                             int64_t mem_budget_bytes, cs_plan *plan) {
    DBatchShape b;
    cs_status st = dbatch_shape(jobs_host, n_jobs, b);
    if (st != CS_OK) return st;
    // the largest job graph with the largest threshold count sizes the slots
    int big = 0;
    for (int j = 1; j < n_jobs; j++)
        if (jobs_host[j].g.n_bound > jobs_host[big].g.n_bound) big = j;
    return cs_plan_dual(&jobs_host[big].g, 0, b.max_k, cap, max_slots, mem_budget_bytes, plan);
}

cs_status cs_dual_batch_run(const cs_dual_batch_job *jobs_host, const cs_dual_batch_job *jobs_dev, int32_t n_jobs,
                            const cs_plan *plan, void *ws, size_t ws_bytes, int32_t flags, void *stream_v) {
    DBatchShape b;
    cs_status st = dbatch_shape(jobs_host, n_jobs, b);
    if (st != CS_OK) return st;
    if (!plan || !ws || !jobs_dev) return dfail(CS_ERR_ARG, "plan/workspace/jobs_dev is NULL");
    if (plan->lanes < b.max_k) return dfail(CS_ERR_ARG, "plan was made for fewer thresholds");
    const int geo_n = plan->n_bound > 0 ? plan->n_bound : b.max_n;
    if (geo_n < b.max_n) return dfail(CS_ERR_ARG, "plan was made for a smaller graph");
    const int L = plan->lanes;
    const DLayout lay = dlayout(geo_n, plan->n_slots, plan->cap, L);
    if (ws_bytes < lay.total) return dfail(CS_ERR_ARG, "workspace too small for this plan");
    long long n_items = 0;
    for (int j = 0; j < n_jobs; j++) {
        if (jobs_host[j].item_begin != n_items) return dfail(CS_ERR_ARG, "jobs not prepared (cs_dual_batch_prepare)");
        n_items += std::max(0, jobs_host[j].n_sources);
    }
    cudaStream_t s = (cudaStream_t)stream_v;
    char *base = (char *)ws;
    csd::DualParams p;
    memset(&p, 0, sizeof(p));
    p.g.n_bound = geo_n;
    p.geo_n = geo_n;
    p.k = L;  // slot geometry; each job brings its own k
    p.replay_rounds = replay_rounds();
    p.delta = plan->delta_seconds > 0.0f ? plan->delta_seconds : 30.0f;
    p.hdr = (cs::WsHeader *)base;
    p.failed = (int32_t *)(base + lay.failed_off);
    p.fail_cap = lay.fail_cap;
    p.inexact = (int32_t *)(base + lay.inexact_off);
    p.inexact_cap = lay.fail_cap;
    p.dense = base + lay.dense_off;
    p.dense_stride = lay.dense_stride;
    p.compact = base + lay.compact_off;
    p.cap = plan->cap;
    cudaError_t e = cudaMemsetAsync(p.hdr, 0, sizeof(cs::WsHeader), s);
    if (e != cudaSuccess) return dcuda(e, "batch reset");
    auto launch = [&](csd::DualParams &pp, int slots) {
        return dbatch_launch(pp, jobs_dev, n_jobs, n_items, slots, s);
    };
    if (n_items > 0 && (flags & CS_BATCH_ASYNC)) {
        // one pass; the caller re-runs listed items (cs_dual_batch_failed)
        st = launch(p, plan->n_slots);
        if (st != CS_OK) return st;
    } else if (n_items > 0) {
        // overflowed items at growing capacities, then items whose replay disagreed through the
        // widened and the exact search (as cs_centrality_simplest)
        long long n_over = 0, n_exact = 0;
        st = dual_passes(p, lay, plan, L, 2 * b.max_n, n_items, dual_wide_mode(), launch, s, n_over, n_exact);
        if (st != CS_OK) return st;
        cs_set_retries_internal(n_over, n_exact);
    }
    int max_n = 0, n_pref = 0;
    for (int j = 0; j < n_jobs; j++)
        if (jobs_host[j].compute_closeness && jobs_host[j].n_sources > 0) {
            max_n = std::max(max_n, jobs_host[j].g.n_bound);
            n_pref++;
        }
    if (n_pref > 0) {
        const int gy = std::min(n_pref, 65535);
        const int gx = std::max(1, std::min((max_n + 255) / 256, std::max(1, dsm_count() * 8 / gy)));
        csd::dual_batch_prefix<<<dim3(gx, gy), 256, 0, s>>>(jobs_dev, n_jobs);
        e = cudaGetLastError();
        if (e != cudaSuccess) return dcuda(e, "dual_batch_prefix launch");
    }
    return CS_OK;
}

cs_status cs_dual_batch_failed(void *ws, const cs_plan *plan, int32_t *items_host, int32_t max_items, int64_t *n_items,
                               void *stream) {
    // overflowed items first, then items whose replay disagreed
    if (!ws || !plan || !n_items) return dfail(CS_ERR_ARG, "workspace/plan/n_items is NULL");
    cs::WsHeader h;
    cudaStream_t st = (cudaStream_t)stream;
    cs_status rc = dsync_header((cs::WsHeader *)ws, h, st);
    if (rc != CS_OK) return rc;
    const DLayout lay = dlayout(std::max(1, plan->n_bound), plan->n_slots, plan->cap, plan->lanes);
    if (h.n_failed > (unsigned)lay.fail_cap || h.n_inexact > (unsigned)lay.fail_cap)
        return dfail(CS_ERR_CAPACITY, "more listed items than the lists hold");
    *n_items = (int64_t)h.n_failed + (int64_t)h.n_inexact;
    const int64_t c1 = std::min<int64_t>(h.n_failed, std::max(0, max_items));
    const int64_t c2 = std::min<int64_t>(h.n_inexact, std::max<int64_t>(0, max_items - c1));
    cudaError_t e = cudaSuccess;
    if (c1 > 0 && items_host)
        e = cudaMemcpyAsync(items_host, (char *)ws + lay.failed_off, 4 * (size_t)c1, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && c2 > 0 && items_host)
        e = cudaMemcpyAsync(items_host + c1, (char *)ws + lay.inexact_off, 4 * (size_t)c2, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? CS_OK : dcuda(e, "dual batch lists");
}

cs_status cs_plan_dual_tree(const cs_dual_graph *g, int32_t cap, int32_t max_slots, int64_t mem_budget_bytes,
                            cs_plan *plan) {
    cs_status st = dvalidate(g);
    if (st != CS_OK) return st;
    if (!plan) return dfail(CS_ERR_ARG, "plan is NULL");
    const int sms = dsm_count();
    if (sms <= 0) return dfail(CS_ERR_CUDA, "no CUDA device");
    int slots = sms * 8;
    if (max_slots > 0) slots = std::min(slots, max_slots);
    if (cap <= 0) cap = std::min(g->n_bound, 16384);
    cap = std::max(64, std::min(cap, g->n_bound));
    if (mem_budget_bytes > 0)
        while (slots > 8 && (int64_t)tlayout(g->n_bound, slots, cap).total > mem_budget_bytes) slots = slots * 7 / 8;
    plan->n_slots = std::max(1, slots);
    plan->cap = cap;
    plan->threads_per_block = 256;
    plan->blocks = (plan->n_slots + 7) / 8;
    plan->lanes = 1;
    plan->n_bound = g->n_bound;
    plan->workspace_bytes = tlayout(g->n_bound, plan->n_slots, cap).total;
    return CS_OK;
}

cs_status cs_dual_tree_workspace_init(const cs_plan *plan, void *ws, size_t ws_bytes, void *stream) {
    if (!plan || !ws) return dfail(CS_ERR_ARG, "plan/workspace is NULL");
    if (ws_bytes < plan->workspace_bytes) return dfail(CS_ERR_ARG, "workspace smaller than plan");
    const TLayout lay = tlayout(plan->n_bound, plan->n_slots, plan->cap);
    cudaError_t e = cudaMemsetAsync(ws, 0, lay.compact_off, (cudaStream_t)stream);  // header, lists, dense
    return e == cudaSuccess ? CS_OK : dcuda(e, "tree workspace init");
}

cs_status cs_tree_simplest(const cs_dual_graph *g, int32_t n_queries, const int32_t *src_dev, uint32_t max_seconds,
                           float speed_m_s, const cs_plan *plan, void *ws, size_t ws_bytes, int32_t row_cap,
                           int32_t *count_dev, int32_t *node_dev, float *simpl_dev, float *agg_seconds_dev,
                           int32_t *pred_dev, void *stream_v) {
    cs_status st = dvalidate(g);
    if (st != CS_OK) return st;
    if (!plan || !ws) return dfail(CS_ERR_ARG, "plan/workspace is NULL");
    if (n_queries < 0 || (n_queries > 0 && !src_dev)) return dfail(CS_ERR_ARG, "bad query list");
    if (!count_dev || !node_dev || !simpl_dev || !agg_seconds_dev || !pred_dev || row_cap <= 0)
        return dfail(CS_ERR_ARG, "tree outputs missing");
    if (!(speed_m_s > 0.0f)) return dfail(CS_ERR_ARG, "speed_m_s must be finite and positive");
    const int geo_n = plan->n_bound > 0 ? plan->n_bound : g->n_bound;
    if (geo_n < g->n_bound) return dfail(CS_ERR_ARG, "plan was made for a smaller graph");
    const TLayout lay = tlayout(geo_n, plan->n_slots, plan->cap);
    if (ws_bytes < lay.total) return dfail(CS_ERR_ARG, "workspace too small for this plan");
    if (n_queries == 0) return CS_OK;
    cudaStream_t s = (cudaStream_t)stream_v;
    char *base = (char *)ws;
    csd::DTreeParams p;
    memset(&p, 0, sizeof(p));
    p.g = *g;
    p.src = src_dev;
    p.n_items = n_queries;
    p.maxsec = (float)max_seconds;
    p.dense = base + lay.dense_off;
    p.dense_stride = lay.dense_stride;
    p.geo_n = geo_n;
    p.compact = base + lay.compact_off;
    p.compact_stride = tcompact_bytes(plan->cap);
    p.cap = plan->cap;
    p.hcap = 4 * plan->cap;
    p.row_cap = row_cap;
    p.t_count = count_dev;
    p.t_node = node_dev;
    p.t_pred = pred_dev;
    p.t_simpl = simpl_dev;
    p.t_agg = agg_seconds_dev;
    p.failed = (int32_t *)(base + lay.failed_off);
    p.fail_cap = lay.fail_cap;
    p.hdr = (cs::WsHeader *)base;
    p.n_slots = std::max(1, std::min(plan->n_slots, n_queries));
    cudaError_t e = cudaMemsetAsync(p.hdr, 0, sizeof(cs::WsHeader), s);
    if (e != cudaSuccess) return dcuda(e, "tree header reset");
    csd::dual_tree_kernel<<<(p.n_slots + 7) / 8, 256, 0, s>>>(p);
    e = cudaGetLastError();
    if (e != cudaSuccess) return dcuda(e, "dual_tree_kernel launch");
    cs::WsHeader h;
    st = dsync_header(p.hdr, h, s);
    if (st != CS_OK) return st;
    if (h.n_failed > 0u) {
        // queries whose rows or heap overflowed: again with every node's row and a larger heap, on as
        // many slots as the compact region holds at that size
        csd::DTreeParams p2 = p;
        p2.cap = g->n_bound;
        p2.hcap = 8 * g->n_bound;
        p2.compact_stride = tcompact_bytes_h(p2.cap, p2.hcap);
        p2.remap = p.failed;
        p2.n_items = std::min<unsigned>(h.n_failed, (unsigned)lay.fail_cap);
        p2.final_pass = 1;
        p2.n_slots = (int)std::max<size_t>(1, std::min<size_t>(lay.compact_total / p2.compact_stride,
                                                                 (size_t)std::min<long long>(p2.n_items, p.n_slots)));
        if (lay.compact_total < p2.compact_stride)
            return dfail(CS_ERR_CAPACITY, "tree workspace cannot hold one full-size search");
        csd::dual_tree_kernel<<<(p2.n_slots + 7) / 8, 256, 0, s>>>(p2);
        e = cudaGetLastError();
        if (e != cudaSuccess) return dcuda(e, "dual_tree_kernel launch");
        st = dsync_header(p.hdr, h, s);
        if (st != CS_OK) return st;
    }
    return CS_OK;
}

}  // extern "C"
