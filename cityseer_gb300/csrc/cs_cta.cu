// cs_cta.cu -- shortest-path node centrality and OD-weighted betweenness with one thread block per
// source, the source's search state in shared memory.
//
// Reference behaviour (cityseer-api v4.24.0):
//   centrality_shortest        rust/src/centrality.rs:1624-1874
//   dijkstra_brandes_shortest  rust/src/centrality.rs:1344-1494
//   circuit_ranks_from_traversal rust/src/centrality.rs:470-526
//   brandes_backprop_with_beta rust/src/centrality.rs:823-873
//   betweenness_od_shortest    rust/src/centrality.rs:2419-2540
//
// One persistent block of 1024 threads per SM takes sources from the work counter.  Per source:
//  1. Search: banded label-correcting search ("near-far" delta-stepping) over reversed edges.  The
//     reached set is an open-addressing hash table in shared memory (node -> f32 distance bits,
//     atomicMin), the near / next / far queues hold (slot, distance) entries in shared memory, so a
//     relaxation costs one global read of the edge and shared-memory atomics.  The least fixpoint
//     of fl(d[u] + w) is unique, so the distances equal the reference's heap Dijkstra's bit for bit.
//  2. Settle order: distance-bucket sort of the hash slots in shared memory (1024 buckets quadratic
//     in distance / the search's last band end, then a rank sort inside each bucket by (distance,
//     node), the source first).  The table's value becomes the settle position.
//  3. Replay: for every reached node, in parallel, the candidate offers the heap Dijkstra makes to
//     it in settle order (its reached out-neighbours, looked up in the hash table), through Phase 1
//     (rust/src/centrality.rs:1413-1437) and Phase 2 (:1447-1483): the multi-predecessor lists.  The
//     same pass counts the circuit ranks' nodes and edges per threshold and builds the path counts
//     (sigma) in settle order: warps take consecutive chunks of 32 positions, a chunk waits for the
//     chunks holding its predecessors (shared-memory flags), and a lane waits for its in-chunk
//     predecessors (warp ballot).  Path counts are integers; they are kept as u32 in shared memory
//     and a source whose counts would pass 2^32 - 1 goes to the per-warp kernel, which carries them
//     in f64.
//  4. Closeness: f64 reductions of the f32 terms into the target rows (density, farness and
//     harmonic into the bucket of the first qualifying threshold, cycles and beta per threshold).
//  5. Backward Brandes sweep per threshold k over the positions within d_k, descending: the
//     dependencies live in shared memory as f64 (plain and beta-weighted), pushed to predecessors
//     with shared-memory f64 atomics; a chunk waits for the chunks holding its successors.  Seeds,
//     factors sigma_v / sigma_w, dependencies and credits are f64 as in the reference; the beta
//     seed's exp is evaluated to ~1e-14 on the f32 pipe (cs_seed.cuh).
// Sources that do not fit (reach above RMAX, a queue or a sort bucket overflowing, path counts past
// 2^32 - 1) are listed before they write any output, and the host runs them through the per-warp
// kernel of cs_primal.cu.
#include <algorithm>

#include "cs_cta.cuh"
#include "cs_seed.cuh"

namespace cs {
namespace cta {

constexpr uint32_t EMPTY = 0xffffffffu;
constexpr uint32_t HMASK = HSIZE - 1;
constexpr long long SPIN_LIMIT = 1ll << 26;  // bounded waits on other warps' flags

// ---- shared memory layout (bytes) ----
constexpr size_t OFF_HKEY = 0;                            // u32[HSIZE]
constexpr size_t OFF_HVAL = OFF_HKEY + 4ull * HSIZE;      // u32[HSIZE]: distance bits, then position
constexpr size_t OFF_B = OFF_HVAL + 4ull * HSIZE;         // queues during the search
constexpr size_t SZ_Q = 8ull * QCAP;
constexpr size_t OFF_SD = OFF_B;                          // f32[RMAX] settle distances (after the sort)
constexpr size_t OFF_SIG = OFF_B + 4ull * RMAX;           // u32[RMAX]: sort slots, then path counts
constexpr size_t OFF_S = OFF_B + 3 * SZ_Q;                // small region
constexpr size_t OFF_HIST = OFF_S;                        // u32[NBK]
constexpr size_t OFF_WSUM = OFF_HIST + 4ull * NBK;        // u32[NW] scan partials
constexpr size_t OFF_CNT = OFF_WSUM + 4ull * NW;          // i32[2 MAXK]
constexpr size_t OFF_RANKW = OFF_CNT + 8ull * MAXK;       // f32[MAXK]
constexpr size_t OFF_VARS = OFF_RANKW + 4ull * MAXK;      // block variables
constexpr size_t SMEM = OFF_VARS + 256;
// the backward sweep's dependencies and pending-successor counts overlay the hash table and the
// settle distances
constexpr size_t OFF_DPLAIN = 0;                          // f64[RMAX]
constexpr size_t OFF_DBETA = 8ull * RMAX;                 // f64[RMAX]
constexpr size_t OFF_SCNT = 16ull * RMAX;                 // u8[RMAX], updated as u32 words
static_assert(3 * SZ_Q >= 8ull * RMAX, "sort buffers exceed the queue region");
static_assert(OFF_SCNT + RMAX <= OFF_SIG, "backward arrays overlap the path counts");
static_assert(RMAX % 32 == 0 && RMAX < 65536, "positions are u16 in the predecessor lists");
static_assert(SMEM <= 232448, "shared memory beyond the per-block limit");

struct Vars {
    int R;           // reached nodes
    int nnear, nnext, nfar;
    int fail;        // 0 ok, else the reason the source goes to the per-warp kernel
    int err;         // device-side error (CS_ERR_*), ends the launch
    float band_end;  // upper end of the current band
    int bandmin;     // min live far distance (float bits)
    int src;
    int li;
    long long idx;
    unsigned herr;
};

enum Fail { F_NONE = 0, F_REACH = 1, F_QUEUE = 2, F_BUCKET = 3, F_SIGMA = 4 };

__device__ __forceinline__ uint32_t hslot(uint32_t v) { return (v * 0x9E3779B1u) >> (32 - HBITS); }

__device__ __forceinline__ uint32_t vload(const uint32_t *a) { return *(const volatile uint32_t *)a; }

// Inserts v (or finds it) and lowers its distance to cbits.  Returns the slot (-1: table full) and
// the previous distance bits in old.
__device__ __forceinline__ int hash_upsert_min(uint32_t *hkey, uint32_t *hval, uint32_t v, uint32_t cbits,
                                               uint32_t &old) {
    uint32_t s = hslot(v);
    for (int probe = 0; probe < HSIZE; probe++) {
        uint32_t k = vload(&hkey[s]);
        if (k == EMPTY) k = atomicCAS(&hkey[s], EMPTY, v);
        if (k == EMPTY || k == v) {
            old = atomicMin(&hval[s], cbits);
            return (int)s;
        }
        s = (s + 1) & HMASK;
    }
    return -1;
}

// Slot of v, or -1 when v is not in the table.
__device__ __forceinline__ int hash_find(const uint32_t *hkey, uint32_t v) {
    uint32_t s = hslot(v);
    for (int probe = 0; probe < HSIZE; probe++) {
        const uint32_t k = hkey[s];
        if (k == v) return (int)s;
        if (k == EMPTY) return -1;
        s = (s + 1) & HMASK;
    }
    return -1;
}

__device__ __forceinline__ float route_cost(float secs, float speed) { return __fmul_rn(secs, speed); }

__device__ __forceinline__ int first_k(const Params &p, float c) {
    int k = 0;
    while (k < p.k && !(c <= p.dk[k])) k++;
    return k;
}

__device__ __forceinline__ float od_weight(const Params &p, int src, int v) {
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

// Appends (slot, dist bits) to a queue with one shared atomic per warp.  Returns false on overflow.
__device__ __forceinline__ void queue_push(bool want, uint2 *q, int *count, uint2 ent, int &fail_flag) {
    const unsigned m = __ballot_sync(FULL, want);
    if (!m) return;
    const int lane = lane_id();
    const int leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(count, __popc(m));
    base = __shfl_sync(FULL, base, leader);
    if (want) {
        const int at = base + __popc(m & lanemask_lt());
        if (at < QCAP) q[at] = ent;
        else fail_flag = 1;
    }
}

// ------------------------------------------------------------------------------------------
// 1. Search.  Returns with v.R (reached count) or v.fail set; every thread sees the same outcome.
// ------------------------------------------------------------------------------------------
__device__ void search(const Params &p, char *sm, Vars &v, long long &relaxed) {
    uint32_t *hkey = (uint32_t *)(sm + OFF_HKEY);
    uint32_t *hval = (uint32_t *)(sm + OFF_HVAL);
    uint2 *qa = (uint2 *)(sm + OFF_B);
    uint2 *qb = (uint2 *)(sm + OFF_B + SZ_Q);
    uint2 *qf = (uint2 *)(sm + OFF_B + 2 * SZ_Q);
    const int tid = threadIdx.x;
    // clear the table
    uint4 *hk4 = (uint4 *)hkey;
    uint4 *hv4 = (uint4 *)hval;
    for (int i = tid; i < HSIZE / 4; i += TPB) {
        hk4[i] = make_uint4(EMPTY, EMPTY, EMPTY, EMPTY);
        hv4[i] = make_uint4(INF_BITS, INF_BITS, INF_BITS, INF_BITS);
    }
    __syncthreads();
    if (tid == 0) {
        uint32_t old;
        const int s0 = hash_upsert_min(hkey, hval, (uint32_t)v.src, 0u, old);
        qa[0] = make_uint2((uint32_t)s0, 0u);
        v.R = 1;
        v.nnear = 1;
        v.nnext = 0;
        v.nfar = 0;
        v.band_end = p.delta;
    }
    __syncthreads();
    // queue roles (all threads agree): ic current near, in next near, iff far
    uint2 *const Q[3] = {qa, qb, qf};
    int ic = 0, in = 1, iff = 2;
    int qfail = 0;
    while (true) {
        // near phase: relax the current band until no distance in it improves
        while (true) {
            const int nnear = v.nnear;
            const float T = v.band_end;
            uint2 *cur = Q[ic], *nxt = Q[in], *far = Q[iff];
            for (int base = 0; base < nnear; base += TPB) {
                const int e = base + tid;
                const bool act = e < nnear;
                const uint2 ent = act ? cur[e] : make_uint2(0u, 0u);
                const bool live = act && vload(&hval[ent.x]) == ent.y;
                const uint32_t u = live ? hkey[ent.x] : 0u;
                const float du = __uint_as_float(ent.y);
                int beg = 0, end = 0;
                if (live) {
                    beg = __ldg(&p.in_ptr[u]);
                    end = __ldg(&p.in_ptr[u + 1]);
                }
                relaxed += end - beg;
                const int deg = end - beg;
                const int maxdeg = warp_max_i(deg);
                // the node's first PMAX edges are loaded together, then relaxed
                int nbs[PMAX];
                float cs[PMAX];
#pragma unroll
                for (int j = 0; j < PMAX; j++) {
                    nbs[j] = (int)u;
                    cs[j] = 0.0f;
                    if (j < deg) {
                        nbs[j] = __ldg(&p.in_nb[beg + j]);
                        cs[j] = __fadd_rn(du, __ldg(&p.in_w[beg + j]));
                    }
                }
                for (int j = 0; j < maxdeg; j++) {
                    int nb = (int)u;
                    float c = 0.0f;
                    if (j < PMAX) {
#pragma unroll
                        for (int q = 0; q < PMAX; q++)
                            if (q == j) {
                                nb = nbs[q];
                                c = cs[q];
                            }
                    } else if (j < deg) {  // high in-degree: one at a time
                        nb = __ldg(&p.in_nb[beg + j]);
                        c = __fadd_rn(du, __ldg(&p.in_w[beg + j]));
                    }
                    bool push_near = false, push_far = false;
                    uint2 out = make_uint2(0u, 0u);
                    if (j < deg && (uint32_t)nb != u && c <= p.maxsec) {
                        uint32_t old;
                        const uint32_t cb = __float_as_uint(c);
                        const int sl = hash_upsert_min(hkey, hval, (uint32_t)nb, cb, old);
                        if (sl < 0) {
                            qfail = 1;
                        } else if (cb < old) {
                            if (old == (uint32_t)INF_BITS) atomicAdd(&v.R, 1);
                            out = make_uint2((uint32_t)sl, cb);
                            push_near = c < T;
                            push_far = !push_near;
                        }
                    }
                    queue_push(push_near, nxt, &v.nnext, out, qfail);
                    queue_push(push_far, far, &v.nfar, out, qfail);
                }
            }
            if (qfail) atomicCAS(&v.fail, 0, F_QUEUE);
            __syncthreads();
            if (tid == 0) {
                if (v.R > RMAX && v.fail == 0) v.fail = F_REACH;
                if ((v.nnext > QCAP || v.nfar > QCAP) && v.fail == 0) v.fail = F_QUEUE;
                v.nnear = v.nnext;
                v.nnext = 0;
            }
            __syncthreads();
            if (v.fail) return;
            const int t = ic;
            ic = in;
            in = t;
            if (v.nnear == 0) break;
        }
        // next band: from the smallest live pending distance
        const int nfar = v.nfar;
        if (nfar == 0) break;
        const uint2 *far = Q[iff];
        if (tid == 0) v.bandmin = INF_BITS;
        __syncthreads();
        float mn = __int_as_float(INF_BITS);
        for (int e = tid; e < nfar; e += TPB) {
            const uint2 ent = far[e];
            if (vload(&hval[ent.x]) == ent.y) mn = fminf(mn, __uint_as_float(ent.y));
        }
        mn = warp_min_f(mn);
        if (lane_id() == 0) atomicMin(&v.bandmin, __float_as_int(mn));
        __syncthreads();
        const int bmin_bits = v.bandmin;
        const float bmin = __int_as_float(bmin_bits);
        // [bmin, bmin + delta), strictly above bmin even when delta is below its ulp
        const float T = (bmin_bits == INF_BITS) ? v.band_end
                                                : fmaxf(__fadd_rn(bmin, p.delta), __int_as_float(bmin_bits + 1));
        __syncthreads();
        if (tid == 0) {
            v.band_end = T;
            v.nnear = 0;
            v.nfar = 0;
        }
        __syncthreads();
        // split the far list: below T into the (empty) near queue, the rest into the free queue,
        // which then becomes the far list
        uint2 *nearq = Q[ic], *keep = Q[in];
        for (int base = 0; base < nfar; base += TPB) {
            const int e = base + tid;
            const bool act = e < nfar;
            const uint2 ent = act ? far[e] : make_uint2(0u, 0u);
            const bool live = act && vload(&hval[ent.x]) == ent.y;
            const bool tonear = live && __uint_as_float(ent.y) < T;
            queue_push(tonear, nearq, &v.nnear, ent, qfail);
            queue_push(live && !tonear, keep, &v.nfar, ent, qfail);
        }
        if (qfail) atomicCAS(&v.fail, 0, F_QUEUE);
        __syncthreads();
        if (v.fail) return;
        const int t = iff;
        iff = in;
        in = t;
        if (v.nnear == 0) break;  // every pending entry was stale
    }
    __syncthreads();
    if (tid == 0 && v.R > RMAX && v.fail == 0) v.fail = F_REACH;
    __syncthreads();
}

// ------------------------------------------------------------------------------------------
// 2. Settle order: bucket sort of the hash slots by distance, ranks inside each bucket.
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long sort_key(const uint32_t *hkey, const uint32_t *hval, uint32_t slot,
                                                       uint32_t src) {
    const uint32_t node = hkey[slot];
    return ((unsigned long long)hval[slot] << 32) | (node == src ? 0u : node + 1u);
}

__device__ void settle_order(const Params &p, char *sm, Vars &v, float *sd_g, uint32_t *ord_g) {
    uint32_t *hkey = (uint32_t *)(sm + OFF_HKEY);
    uint32_t *hval = (uint32_t *)(sm + OFF_HVAL);
    uint32_t *hist = (uint32_t *)(sm + OFF_HIST);
    uint32_t *slots = (uint32_t *)(sm + OFF_SIG);
    float *sd = (float *)(sm + OFF_SD);
    const int tid = threadIdx.x, lane = lane_id(), warp = tid >> 5;
    const int R = v.R;
    const float dmax = fminf(v.band_end, p.maxsec);
    const float inv = dmax > 0.0f ? __fdiv_rn(1.0f, dmax) : 0.0f;
    for (int b = tid; b < NBK; b += TPB) hist[b] = 0u;
    __syncthreads();
    auto bucket_of = [&](uint32_t dbits) {
        const float q = fminf(__fmul_rn(__uint_as_float(dbits), inv), 1.0f);
        return min(NBK - 1, (int)__fmul_rn(__fmul_rn(q, q), (float)NBK));
    };
    for (int s = tid; s < HSIZE; s += TPB)
        if (hkey[s] != EMPTY) atomicAdd(&hist[bucket_of(hval[s])], 1u);
    __syncthreads();
    // exclusive scan of the bucket counts (one bucket per thread)
    {
        const uint32_t c = (tid < NBK) ? hist[tid] : 0u;
        uint32_t inc = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(FULL, inc, o);
            if (lane >= o) inc += t;
        }
        uint32_t *wsum = (uint32_t *)(sm + OFF_WSUM);
        if (lane == 31) wsum[warp] = inc;
        __syncthreads();
        if (warp == 0) {
            uint32_t x = (lane < NW) ? wsum[lane] : 0u;
            uint32_t y = x;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(FULL, y, o);
                if (lane >= o) y += t;
            }
            if (lane < NW) wsum[lane] = y - x;
        }
        __syncthreads();
        if (tid < NBK) hist[tid] = wsum[warp] + inc - c;
        __syncthreads();
    }
    for (int s = tid; s < HSIZE; s += TPB)
        if (hkey[s] != EMPTY) slots[atomicAdd(&hist[bucket_of(hval[s])], 1u)] = (uint32_t)s;
    __syncthreads();
    // hist[b] is now the end of bucket b; rank inside each bucket by (distance, source first, node)
    const uint32_t src = (uint32_t)v.src;
    for (int b = warp; b < NBK; b += NW) {
        const int lo = b ? (int)hist[b - 1] : 0, hi = (int)hist[b];
        const int n = hi - lo;
        if (n <= 1) continue;
        if (n > BKMAX) {
            if (lane == 0) atomicCAS(&v.fail, 0, F_BUCKET);
            continue;
        }
        if (n <= 32) {
            const uint32_t my_slot = (lane < n) ? slots[lo + lane] : 0u;
            const unsigned long long key = (lane < n) ? sort_key(hkey, hval, my_slot, src) : ~0ull;
            int rank = 0;
            for (int m = 0; m < n; m++) rank += __shfl_sync(FULL, key, m) < key;
            __syncwarp();
            if (lane < n) slots[lo + rank] = my_slot;
        } else {
            // ranks by counting over the bucket, written to the (not yet used) settle-distance
            // region, then copied back
            uint32_t *tmp = (uint32_t *)(sm + OFF_SD);
            for (int e = lo + lane; e < hi; e += 32) {
                const uint32_t sl = slots[e];
                const unsigned long long key = sort_key(hkey, hval, sl, src);
                int rank = 0;
                for (int m = lo; m < hi; m++) rank += sort_key(hkey, hval, slots[m], src) < key;
                tmp[lo + rank] = sl;
            }
            __syncwarp();
            for (int e = lo + lane; e < hi; e += 32) slots[e] = tmp[e];
        }
        __syncwarp();
    }
    __syncthreads();
    if (v.fail) return;
    // settle distances and order; the table's value becomes the settle position
    for (int i = tid; i < R; i += TPB) {
        const uint32_t s = slots[i];
        const uint32_t d = hval[s];
        sd[i] = __uint_as_float(d);
        sd_g[i] = __uint_as_float(d);
        ord_g[i] = hkey[s];
        hval[s] = (uint32_t)i;
    }
    __syncthreads();
}

// ------------------------------------------------------------------------------------------
// 3. Replay: predecessors (Phase 1 / Phase 2), circuit-rank counts, path counts.
// ------------------------------------------------------------------------------------------
// Reached out-neighbours of the node at position i: slot j holds out-CSR edge beg + j.
struct Nb {
    int pos[PMAX];
    float d[PMAX];
    int beg, deg;
};

__device__ __forceinline__ void load_nb(const Params &p, const uint32_t *hkey, const uint32_t *hval, const float *sd,
                                        int vtx, Nb &nb) {
    nb.beg = __ldg(&p.out_ptr[vtx]);
    nb.deg = min(__ldg(&p.out_ptr[vtx + 1]) - nb.beg, PMAX);
#pragma unroll
    for (int j = 0; j < PMAX; j++) {
        nb.pos[j] = -1;
        nb.d[j] = 0.0f;
        if (j < nb.deg) {
            const int u = __ldg(&p.out_to[nb.beg + j]);
            if (u != vtx) {
                const int s = hash_find(hkey, (uint32_t)u);
                if (s >= 0) {
                    nb.pos[j] = (int)hval[s];
                    nb.d[j] = sd[nb.pos[j]];
                }
            }
        }
    }
}

// Phase-1 (+ Phase-2) predecessor replay (rust/src/centrality.rs:1413-1437, 1444-1483): offers in
// settle order of the offering node, parallel edges in list order.  Returns the predecessor slots;
// ok = false if the replayed distance differs from the searched one.
__device__ __forceinline__ unsigned replay_preds(const Params &p, const Nb &nb, int i, float dv, bool &ok) {
    const float one_plus = 1.0f + TIE_EPSILON, one_minus = 1.0f - TIE_EPSILON;
    float c[PMAX];
    unsigned todo = 0u;
#pragma unroll
    for (int j = 0; j < PMAX; j++) {
        const bool off = nb.pos[j] >= 0 && nb.pos[j] < i;
        c[j] = off ? __fadd_rn(nb.d[j], __ldg(&p.out_w[nb.beg + j])) : 0.0f;
        if (off) todo |= 1u << j;
    }
    auto next = [&](unsigned t, int &bp, float &bc) {
        int best = -1;
        bp = 0x7fffffff;
        bc = 0.0f;
#pragma unroll
        for (int j = 0; j < PMAX; j++)
            if (((t >> j) & 1u) && nb.pos[j] < bp) {
                bp = nb.pos[j];
                best = j;
                bc = c[j];
            }
        return best;
    };
    auto has_pos = [&](unsigned mask, int pos) {
        bool h = false;
#pragma unroll
        for (int j = 0; j < PMAX; j++) h |= ((mask >> j) & 1u) && nb.pos[j] == pos;
        return h;
    };
    unsigned t = todo, pm = 0u;
    float cur = __int_as_float(INF_BITS);
    while (t) {
        int bp;
        float bc;
        const int best = next(t, bp, bc);
        t &= ~(1u << best);
        if (bc > p.maxsec) continue;
        if (bc < cur) {
            if (bc < __fmul_rn(cur, one_minus)) pm = 0u;
            pm |= 1u << best;
            cur = bc;
        } else if (bc <= __fmul_rn(cur, one_plus) && !has_pos(pm, bp)) {
            pm |= 1u << best;
        }
    }
    ok = __float_as_int(cur) == __float_as_int(dv);
    if (p.tol > TIE_EPSILON) {
        const float lim = __fmul_rn(dv, 1.0f + p.tol);
        pm = 0u;
        t = todo;
        while (t) {
            int bp;
            float bc;
            const int best = next(t, bp, bc);
            t &= ~(1u << best);
            if (bc <= lim && !has_pos(pm, bp)) pm |= 1u << best;
        }
    }
    return pm;
}

// Waits (bounded) until another thread has written a non-zero value at a; returns it (0: gave up,
// after raising CS_ERR_TIMEOUT).
__device__ __forceinline__ uint32_t wait_nonzero(const uint32_t *a, Vars &v) {
    long long spins = 0;
    uint32_t x;
    while ((x = vload(a)) == 0u) {
        if (++spins > SPIN_LIMIT) {
            atomicCAS(&v.err, 0, CS_ERR_TIMEOUT);
            return 0u;
        }
        __nanosleep(20);
    }
    __threadfence_block();
    return x;
}

__device__ void replay(const Params &p, char *sm, Vars &v, const uint32_t *ord_g, uint16_t *pr_g, uint8_t *np_g) {
    const uint32_t *hkey = (const uint32_t *)(sm + OFF_HKEY);
    const uint32_t *hval = (const uint32_t *)(sm + OFF_HVAL);
    const float *sd = (const float *)(sm + OFF_SD);
    uint32_t *sig = (uint32_t *)(sm + OFF_SIG);
    int *cnt = (int *)(sm + OFF_CNT);
    const int tid = threadIdx.x, lane = lane_id(), warp = tid >> 5;
    const int R = v.R;
    const int nch = (R + 31) / 32;
    // a path count is at least 1 once written: 0 marks "not yet"
    for (int i = tid; i < R; i += TPB) sig[i] = 0u;
    for (int q = tid; q < 2 * MAXK; q += TPB) cnt[q] = 0;
    __syncthreads();
    const int K = p.k;
    const bool betw = p.betweenness != 0;
    bool bad = false;
    for (int ch = warp; ch < nch; ch += NW) {
        const int base = ch * 32;
        const int i = base + lane;
        const bool act = i < R;
        unsigned pm = 0u;
        Nb nb;
        nb.deg = 0;
        if (act) {
            const int vtx = (int)ord_g[i];
            const float dv = sd[i];
            const float cv = route_cost(dv, p.speed);
            const int k0v = first_k(p, cv);
            if (k0v < K) atomicAdd(&cnt[k0v], 1);
            load_nb(p, hkey, hval, sd, vtx, nb);
            if (p.closeness) {
#pragma unroll
                for (int j = 0; j < PMAX; j++) {
                    if (nb.pos[j] < 0 || !__ldg(&p.out_cnt[nb.beg + j])) continue;
                    const float ec = fmaxf(cv, route_cost(nb.d[j], p.speed));
                    const int k0e = first_k(p, ec);
                    if (k0e < K) atomicAdd(&cnt[MAXK + k0e], 1);
                }
            }
            if (betw && i > 0) {
                bool ok = true;
                pm = replay_preds(p, nb, i, dv, ok);
                if (!ok) {
                    bad = true;
                    pm = 0u;
                }
                int r = 0;
#pragma unroll
                for (int j = 0; j < PMAX; j++) {
                    if ((pm >> j) & 1u) pr_g[(size_t)i * PMAX + r++] = (uint16_t)nb.pos[j];
                }
                np_g[i] = (uint8_t)r;
            } else if (act) {
                np_g[i] = 0;
            }
        }
        if (!betw) continue;
        // path counts: wait for the predecessors in earlier chunks (their counts become non-zero),
        // then resolve the in-chunk ones in ballot rounds
#pragma unroll
        for (int j = 0; j < PMAX; j++)
            if (((pm >> j) & 1u) && nb.pos[j] < base) {
                if (!wait_nonzero(&sig[nb.pos[j]], v)) pm = 0u;
            }
        __syncwarp();
        unsigned blk = 0u;
#pragma unroll
        for (int j = 0; j < PMAX; j++)
            if (((pm >> j) & 1u) && nb.pos[j] >= base) blk |= 1u << (nb.pos[j] - base);
        bool mine = !act;
        unsigned fin = __ballot_sync(FULL, mine);
        int guard = 0;
        while (fin != FULL) {
            const bool ready = !mine && ((blk & ~fin) == 0u);
            if (ready) {
                unsigned long long sg = (i == 0) ? 1ull : 0ull;
#pragma unroll
                for (int j = 0; j < PMAX; j++)
                    if ((pm >> j) & 1u) sg += sig[nb.pos[j]];
                if (sg > 0xffffffffull) {
                    atomicCAS(&v.fail, 0, F_SIGMA);
                    sg = 0xffffffffull;
                }
                *(volatile uint32_t *)&sig[i] = (uint32_t)sg;
                mine = true;
            }
            __syncwarp();
            fin |= __ballot_sync(FULL, ready);
            if (++guard > 64) break;
        }
        if (fin != FULL) bad = true;
        __syncwarp();
    }
    if (bad) atomicCAS(&v.err, 0, CS_ERR_INTERNAL);
    __syncthreads();
}

// ------------------------------------------------------------------------------------------
// 4. Closeness (rust/src/centrality.rs:1733-1780) and the circuit-rank weights.
// ------------------------------------------------------------------------------------------
__device__ void closeness(const Params &p, char *sm, Vars &v, const uint32_t *ord_g) {
    const float *sd = (const float *)(sm + OFF_SD);
    int *cnt = (int *)(sm + OFF_CNT);
    float *rankw = (float *)(sm + OFF_RANKW);
    const int tid = threadIdx.x;
    const int K = p.k, N = p.n_bound, R = v.R;
    const int src = v.src;
    const float wt = __ldg(&p.src_wt[src]);
    if (tid == 0) {
        const float cycles_wt = __fdiv_rn(wt, __ldg(&p.node_w[src]));
        long long nc = 0, ec = 0;
        for (int k = 0; k < K; k++) {
            nc += cnt[k];
            ec += cnt[MAXK + k];
            const long long r = ec - nc + 1;
            const float rank = (nc == 0) ? 0.0f : (float)(r > 0 ? r : 0);
            rankw[k] = __fmul_rn(rank, cycles_wt);
            if (p.track_reach && nc > 1) atomicAdd(&p.reach[k], (unsigned)(nc - 1));
        }
    }
    __syncthreads();
    const double wt_d = f2d(wt);
    const size_t KN = (size_t)K * N;
    for (int i = 1 + tid; i < R; i += TPB) {
        const int t = (int)ord_g[i];
        const float c = route_cost(sd[i], p.speed);
        const int k0 = first_k(p, c);
        if (k0 >= K) continue;
        double *bk = p.bucket + (size_t)k0 * N + t;
        atomicAdd(bk, wt_d);
        atomicAdd(bk + KN, f2d(__fmul_rn(c, wt)));
        atomicAdd(bk + 2 * KN, f2d(__fmul_rn(__fdiv_rn(1.0f, c), wt)));
        for (int k = k0; k < K; k++) {
            double *row = p.out + (size_t)k * N + t;
            atomicAdd(row + 2 * KN, f2d(rankw[k]));
            atomicAdd(row + 4 * KN, f2d(__fmul_rn(expf(__fmul_rn(-p.beta[k], c)), wt)));
        }
    }
}

// ------------------------------------------------------------------------------------------
// 5. Backward Brandes sweep, one threshold at a time over the positions within it.  A node waits
//    for its pending-successor count (successors within the sweep that have not pushed yet) to
//    reach zero, then pushes its dependency to its predecessors and decrements theirs.
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t scnt_get(const uint32_t *w, int i) {
    return (vload(&w[i >> 2]) >> ((i & 3) * 8)) & 0xffu;
}

__device__ void backward(const Params &p, char *sm, Vars &v, const uint32_t *ord_g, const float *sd_g,
                         const uint16_t *pr_g, const uint8_t *np_g) {
    const uint32_t *sig = (const uint32_t *)(sm + OFF_SIG);
    const int *cnt = (const int *)(sm + OFF_CNT);
    double *dpl = (double *)(sm + OFF_DPLAIN);
    double *dbe = (double *)(sm + OFF_DBETA);
    uint32_t *scnt = (uint32_t *)(sm + OFF_SCNT);
    const int tid = threadIdx.x, lane = lane_id(), warp = tid >> 5;
    const int K = p.k, N = p.n_bound;
    const int src = v.src;
    const float wt = p.od ? 1.0f : __ldg(&p.src_wt[src]);
    const bool unit_wt = (wt == 1.0f);
    const double wtd = f2d(wt);
    const size_t row_b = p.od ? 0 : 5;
    int n_k = 0;
    for (int k = 0; k < K; k++) {
        n_k += cnt[k];  // positions with route cost <= d_k (a prefix of the settle order)
        const int nk = n_k;
        const int nch = (nk + 31) / 32;
        for (int i = tid; i < nk; i += TPB) {
            dpl[i] = 0.0;
            dbe[i] = 0.0;
        }
        for (int w = tid; w < (nk + 3) / 4; w += TPB) scnt[w] = 0u;
        __syncthreads();
        // successors of each node within this sweep (a predecessor's position is below its node's)
        for (int i = tid; i < nk; i += TPB) {
            const int np = np_g[i];
            for (int r = 0; r < np; r++) {
                const int q = pr_g[(size_t)i * PMAX + r];
                const uint32_t old = atomicAdd(&scnt[q >> 2], 1u << ((q & 3) * 8));
                // a byte counter holds 255 successors; street graphs have a handful
                if (((old >> ((q & 3) * 8)) & 0xffu) == 0xffu) atomicCAS(&v.err, 0, CS_ERR_INTERNAL);
            }
        }
        __syncthreads();
        const float beta = p.beta[k];
        for (int ch = nch - 1 - warp; ch >= 0; ch -= NW) {
            const int i = ch * 32 + lane;
            if (i < nk) {
                // predecessors and seeds first, then the wait
                const int np = np_g[i];
                int pl[PMAX];
#pragma unroll
                for (int r = 0; r < PMAX; r++) pl[r] = (r < np) ? (int)pr_g[(size_t)i * PMAX + r] : 0;
                const int vtx = (int)ord_g[i];
                double seed = 0.0, seedb = 0.0;
                if (i > 0) {
                    const float cost = route_cost(sd_g[i], p.speed);
                    const float pairf = p.od ? od_weight(p, src, vtx) : (__ldg(&p.eligible[vtx]) ? 0.5f : 1.0f);
                    seed = f2d(pairf);
                    seedb = (pairf == 0.0f) ? 0.0 : seed_exp(pairf, beta, cost);
                }
                long long spins = 0;
                while (scnt_get(scnt, i) != 0u) {
                    if (++spins > SPIN_LIMIT) {
                        atomicCAS(&v.err, 0, CS_ERR_TIMEOUT);
                        break;
                    }
                    __nanosleep(20);
                }
                __threadfence_block();
                const double sw = (double)sig[i];
                const double dep = __dadd_rn(seed, dpl[i]);
                const double depb = __dadd_rn(seedb, dbe[i]);
                const bool push = sw != 0.0 && (dep != 0.0 || depb != 0.0);
                for (int r = 0; r < np; r++) {
                    const int q = pl[r];
                    const double sv = (double)sig[q];
                    if (push && sv != 0.0) {
                        if (sv == sw) {
                            atomicAdd(&dpl[q], dep);
                            atomicAdd(&dbe[q], depb);
                        } else {
                            const double f = __ddiv_rn(sv, sw);
                            atomicAdd(&dpl[q], __dmul_rn(f, dep));
                            atomicAdd(&dbe[q], __dmul_rn(f, depb));
                        }
                    }
                }
                __threadfence_block();
                for (int r = 0; r < np; r++) atomicSub(&scnt[pl[r] >> 2], 1u << ((pl[r] & 3) * 8));
                if (push && vtx != src) {
                    const double credit = __dadd_rn(dep, -seed);
                    const double creditb = __dadd_rn(depb, -seedb);
                    if (credit > 0.0)
                        atomicAdd(p.out + (row_b * K + k) * N + vtx, unit_wt ? credit : __dmul_rn(credit, wtd));
                    if (creditb > 0.0)
                        atomicAdd(p.out + ((row_b + 1) * K + k) * N + vtx,
                                  unit_wt ? creditb : __dmul_rn(creditb, wtd));
                }
            }
            __syncwarp();
        }
        __syncthreads();
        if (v.err) return;
    }
}

// ------------------------------------------------------------------------------------------
// Persistent kernel.
// ------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(TPB, 1) source_block_kernel(const Params p) {
    extern __shared__ __align__(16) char sm[];
    Vars &v = *(Vars *)(sm + OFF_VARS);
    const int tid = threadIdx.x;
    char *scr = p.scratch + p.scratch_stride * blockIdx.x;
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    uint32_t *ord_g = (uint32_t *)scr;
    float *sd_g = (float *)(scr + al(4ull * RMAX));
    uint16_t *pr_g = (uint16_t *)(scr + 2 * al(4ull * RMAX));
    uint8_t *np_g = (uint8_t *)(scr + 2 * al(4ull * RMAX) + al(2ull * PMAX * RMAX));
    long long relaxed = 0, settled = 0, done_src = 0;
    long long ph[6] = {0, 0, 0, 0, 0, 0};
    if (tid == 0) v.err = 0;
    while (true) {
        if (tid == 0) {
            v.idx = (long long)atomicAdd(&p.hdr->work_next, 1ull);
            v.herr = __ldcg(&p.hdr->err);
            v.fail = 0;
            if (v.idx < p.n_src) {
                v.li = (int)v.idx;
                v.src = __ldg(&p.src_list[v.li]);
            }
        }
        __syncthreads();
        if (v.idx >= p.n_src || v.herr != 0u || v.err) break;
        long long t0 = clock64(), t1;
        search(p, sm, v, relaxed);
        t1 = clock64();
        ph[0] += t1 - t0;
        t0 = t1;
        if (!v.fail) settle_order(p, sm, v, sd_g, ord_g);
        t1 = clock64();
        ph[1] += t1 - t0;
        t0 = t1;
        if (!v.fail) replay(p, sm, v, ord_g, pr_g, np_g);
        t1 = clock64();
        ph[2] += t1 - t0;
        t0 = t1;
        if (v.err) break;
        if (v.fail) {
            // nothing was written for this source: the per-warp kernel redoes it
            if (tid == 0) {
                const unsigned f = atomicAdd(&p.hdr->n_failed, 1u);
                if (f < (unsigned)p.fail_cap) p.failed[f] = v.li;
                else raise_err(p.hdr, CS_ERR_CAPACITY, 40);
            }
            __syncthreads();
            continue;
        }
        if (p.closeness) closeness(p, sm, v, ord_g);
        __syncthreads();
        t1 = clock64();
        ph[3] += t1 - t0;
        t0 = t1;
        if (p.betweenness) backward(p, sm, v, ord_g, sd_g, pr_g, np_g);
        t1 = clock64();
        ph[5] += t1 - t0;
        settled += v.R;
        done_src++;
        if (tid == 0) count_progress(p.hdr);
        __syncthreads();
        if (v.err) break;
    }
    if (v.err && tid == 0) raise_err(p.hdr, (unsigned)v.err, 41);
    const long long rsum = warp_sum_ll(relaxed);
    if (lane_id() == 0) atomicAdd(&p.hdr->edges_relaxed, (unsigned long long)rsum);
    if (tid == 0) {
        atomicAdd(&p.hdr->nodes_settled, (unsigned long long)settled);
        atomicAdd(&p.hdr->sources_done, (unsigned long long)done_src);
        // phase cycles, summed per block: 0 search, 1 sort, 2 replay, 3 closeness, 5 backward
        for (int q = 0; q < 6; q++) atomicAdd(&p.hdr->pad[q], (unsigned long long)ph[q]);
    }
}

size_t smem_bytes() { return SMEM; }

bool supported(int max_out_degree, int k) { return max_out_degree <= PMAX && k >= 1 && k <= MAXK; }

cudaError_t launch(const Params &p, int blocks, cudaStream_t stream) {
    static_assert(sizeof(Vars) <= 256, "block variables exceed their region");
    cudaError_t e = cudaFuncSetAttribute(source_block_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM);
    if (e != cudaSuccess) return e;
    source_block_kernel<<<blocks, TPB, SMEM, stream>>>(p);
    return cudaGetLastError();
}

// Tabulates exp(-j / 256) for this translation unit's seeds (cs_seed.cuh).
cudaError_t launch_seed_table(cudaStream_t stream) {
    seed_table_kernel<<<(SEED_TAB + 255) / 256, 256, 0, stream>>>();
    return cudaGetLastError();
}

}  // namespace cta
}  // namespace cs
