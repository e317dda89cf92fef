// cs_sort.cuh -- warp-cooperative stable sorts of a search's reached set over global memory: an LSD
// radix sort (4 passes of 8 bits) and a distance-bucket sort (3 passes).
#pragma once
#include "cs_common.cuh"

namespace cs {

// Sorts the R values vin0[0..R) by key_of(value) (u32, ascending, stable).  Passes ping-pong
// through (kb, vb); the sorted keys land in kout and the values in vout.  hist: 256 u32 of this
// warp's shared memory.
template <class KeyOf>
__device__ __forceinline__ void warp_radix_sort(int R, const int32_t *vin0, KeyOf key_of, uint32_t *kb, int32_t *vb,
                                                uint32_t *kout_final, int32_t *vout_final, uint32_t *hist) {
    const int lane = lane_id();
    const unsigned lt = lanemask_lt();
    for (int pass = 0; pass < 4; pass++) {
        const int shift = pass * 8;
        for (int b = lane; b < 256; b += 32) hist[b] = 0;
        __syncwarp();
        const uint32_t *kin = (pass == 0) ? nullptr : ((pass & 1) ? kb : kout_final);
        const int32_t *vin = (pass == 0) ? vin0 : ((pass & 1) ? vb : vout_final);
        uint32_t *kout = (pass & 1) ? kout_final : kb;
        int32_t *vout = (pass & 1) ? vout_final : vb;
#pragma unroll 4
        for (int i = lane; i < R; i += 32) {
            const uint32_t key = (pass == 0) ? key_of(vin[i]) : kin[i];
            atomicAdd(&hist[(key >> shift) & 255u], 1u);
        }
        __syncwarp();
        // exclusive scan of 256 bins: each lane owns 8 consecutive bins
        uint32_t loc[8];
        uint32_t tot = 0;
#pragma unroll
        for (int q = 0; q < 8; q++) { loc[q] = hist[lane * 8 + q]; tot += loc[q]; }
        uint32_t inc = tot;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(FULL, inc, o);
            if (lane >= o) inc += t;
        }
        uint32_t run = inc - tot;
        __syncwarp();
#pragma unroll
        for (int q = 0; q < 8; q++) { hist[lane * 8 + q] = run; run += loc[q]; }
        __syncwarp();
        // software-pipelined: the next chunk's key/value loads are in flight while this one scatters
        int32_t val_n = 0;
        uint32_t key_n = 0;
        if (lane < R) {
            val_n = vin[lane];
            key_n = (pass == 0) ? key_of(val_n) : kin[lane];
        }
        for (int base = 0; base < R; base += 32) {
            const int i = base + lane;
            const bool act = i < R;
            const uint32_t key = key_n;
            const int32_t val = val_n;
            const int inext = i + 32;
            if (inext < R) {
                val_n = vin[inext];
                key_n = (pass == 0) ? key_of(val_n) : kin[inext];
            }
            const uint32_t dg = act ? ((key >> shift) & 255u) : (256u + (uint32_t)lane);
            const unsigned peers = __match_any_sync(FULL, dg);
            const int rank = __popc(peers & lt);
            const int leader = __ffs(peers) - 1;
            uint32_t off = 0;
            if (act) off = hist[dg];
            __syncwarp();
            if (act) {
                kout[off + rank] = key;
                vout[off + rank] = val;
            }
            if (act && lane == leader) hist[dg] = off + __popc(peers);
            __syncwarp();
        }
        __syncwarp();
    }
}

// Bucket of a key (the bits of a non-negative float distance at most dmax; inv = 1 / dmax): 512
// buckets, quadratic in distance / dmax so that a search disk, whose reach grows with the square of
// the distance, fills them about evenly.  Monotone non-decreasing in the key, so that bucket order
// followed by key order within each bucket is key order.
__device__ __forceinline__ int dist_bucket(uint32_t key, float inv) {
    const float t = fminf(__fmul_rn(__uint_as_float(key), inv), 1.0f);
    return min(511, (int)__fmul_rn(__fmul_rn(t, t), 512.0f));
}

// Same result as warp_radix_sort (ascending, stable) for keys that are non-negative float bits at
// most dmax, in three passes over the data instead of eight: bucket counts, a stable scatter into
// the 512 distance buckets, then runs of whole buckets (at most 32 keys, or one bucket of at most
// 64) ranked in registers by (key, position) and written back in place.  The bucket counters are
// 16-bit halves of the 256 words of hist.  Falls back to warp_radix_sort when a bucket holds more
// than 64 keys or R >= 65536.  Keys go to kout, values to vout; kb holds the keys between passes.
template <class KeyOf>
__device__ __forceinline__ void warp_bucket_sort(int R, float dmax, const int32_t *vin0, KeyOf key_of, uint32_t *kb,
                                                 int32_t *vb, uint32_t *kout, int32_t *vout, uint32_t *hist) {
    if (R >= 65536) {
        warp_radix_sort(R, vin0, key_of, kb, vb, kout, vout, hist);
        return;
    }
    const int lane = lane_id();
    const unsigned lt = lanemask_lt();
    const float inv = (dmax > 0.0f) ? __fdiv_rn(1.0f, dmax) : 0.0f;
    for (int b = lane; b < 256; b += 32) hist[b] = 0;
    __syncwarp();
#pragma unroll 4
    for (int i = lane; i < R; i += 32) {
        const uint32_t key = key_of(vin0[i]);
        kb[i] = key;
        const int b = dist_bucket(key, inv);
        atomicAdd(&hist[b >> 1], 1u << ((b & 1) * 16));
    }
    __syncwarp();
    // exclusive scan of the 512 counts; lane owns words lane * 8 .. lane * 8 + 7 (bins lane * 16 ..)
    uint32_t w[8];
    uint32_t tot = 0, mx = 0;
#pragma unroll
    for (int q = 0; q < 8; q++) {
        w[q] = hist[lane * 8 + q];
        const uint32_t lo = w[q] & 0xFFFFu, hi = w[q] >> 16;
        tot += lo + hi;
        mx = max(mx, max(lo, hi));
    }
    uint32_t inc = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(FULL, inc, o);
        if (lane >= o) inc += t;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(FULL, mx, o));
    if (mx > 64u) {
        __syncwarp();
        warp_radix_sort(R, vin0, key_of, kb, vb, kout, vout, hist);
        return;
    }
    uint32_t run = inc - tot;
    __syncwarp();
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const uint32_t lo = w[q] & 0xFFFFu, hi = w[q] >> 16;
        hist[lane * 8 + q] = run | ((run + lo) << 16);
        run += lo + hi;
    }
    __syncwarp();
    // stable scatter into bucket order (software-pipelined like warp_radix_sort's passes); afterwards
    // each bucket's counter holds its end offset
    int32_t val_n = 0;
    uint32_t key_n = 0;
    if (lane < R) {
        val_n = vin0[lane];
        key_n = kb[lane];
    }
    for (int base = 0; base < R; base += 32) {
        const int i = base + lane;
        const bool act = i < R;
        const uint32_t key = key_n;
        const int32_t val = val_n;
        const int inext = i + 32;
        if (inext < R) {
            val_n = vin0[inext];
            key_n = kb[inext];
        }
        const int b = act ? dist_bucket(key, inv) : (512 + lane);
        const unsigned peers = __match_any_sync(FULL, b);
        const int rank = __popc(peers & lt);
        const int leader = __ffs(peers) - 1;
        uint32_t off = 0;
        if (act) off = (hist[b >> 1] >> ((b & 1) * 16)) & 0xFFFFu;
        __syncwarp();
        if (act) {
            kout[off + rank] = key;
            vout[off + rank] = val;
        }
        if (act && lane == leader) atomicAdd(&hist[b >> 1], (uint32_t)__popc(peers) << ((b & 1) * 16));
        __syncwarp();
    }
    __syncwarp();
    // runs of whole buckets: [w0, start of the bucket of element w0 + 32), ranked by (key, position)
    int w0 = 0;
    while (w0 < R) {
        const int i = w0 + lane;
        uint32_t k = 0xFFFFFFFFu;
        int32_t v = 0;
        if (i < R) {
            k = kout[i];
            v = vout[i];
        }
        const int bnext = (w0 + 32 < R) ? dist_bucket(kout[w0 + 32], inv) : (1 << 20);
        const int b = (i < R) ? dist_bucket(k, inv) : (1 << 21);
        const int n = __popc(__ballot_sync(FULL, b < bnext));  // a prefix of the lanes
        if (n > 0) {
            int r = 0;
            for (int j = 0; j < n; j++) {
                const uint32_t a = __shfl_sync(FULL, k, j);
                r += (a < k) || (a == k && j < lane);
            }
            __syncwarp();
            if (lane < n) {
                kout[w0 + r] = k;
                vout[w0 + r] = v;
            }
            __syncwarp();
            w0 += n;
        } else {
            // the bucket starting at w0 holds 33..64 keys: two per lane
            const int b0 = __shfl_sync(FULL, b, 0);
            const int end = (int)((hist[b0 >> 1] >> ((b0 & 1) * 16)) & 0xFFFFu);
            const int i1 = i + 32;
            uint32_t k1 = 0xFFFFFFFFu;
            int32_t v1 = 0;
            if (i1 < end) {
                k1 = kout[i1];
                v1 = vout[i1];
            }
            int r0 = 0, r1 = 0;
            for (int j = 0; j < 32; j++) {
                const uint32_t a = __shfl_sync(FULL, k, j);
                r0 += (a < k) || (a == k && j < lane);
                r1 += (a <= k1);
            }
            const int n1 = end - w0 - 32;
            for (int j = 0; j < n1; j++) {
                const uint32_t a = __shfl_sync(FULL, k1, j);
                r0 += (a < k);
                r1 += (a < k1) || (a == k1 && j < lane);
            }
            __syncwarp();
            kout[w0 + r0] = k;
            vout[w0 + r0] = v;
            if (i1 < end) {
                kout[w0 + r1] = k1;
                vout[w0 + r1] = v1;
            }
            __syncwarp();
            w0 = end;
        }
    }
    __syncwarp();
}

}  // namespace cs
