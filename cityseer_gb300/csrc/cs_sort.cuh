// cs_sort.cuh -- warp-cooperative stable LSD radix sort (4 passes of 8 bits) over global memory.
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

}  // namespace cs
