// cs_common.cuh -- shared device helpers for the cityseer_gb300 kernels (sm_103a).
#pragma once
#include <chrono>
#include <cstdint>
#include <thread>
#include <cuda_runtime.h>

#include "../../include/cityseer_gb300.h"

namespace cs {

constexpr unsigned FULL = 0xffffffffu;
constexpr int INF_BITS = 0x7f800000;
constexpr uint32_t NEAR_BIT = 1u << 30;
constexpr uint32_t FAR_BIT = 1u << 31;
// TIE_EPSILON and the f32 constants (1 + eps), (1 - eps) exactly as rust/src/centrality.rs:28,
// 671-674 evaluates them (f32 arithmetic).
constexpr float TIE_EPSILON = 1e-4f;
constexpr float ANGULAR_TIE_BREAK = 1e-6f;
constexpr int MAXK = CS_MAX_THRESHOLDS;
constexpr int MAXDEG = CS_MAX_DEGREE;

// Shared workspace header (first 256 bytes of every workspace).
struct WsHeader {
    unsigned long long work_next;     // persistent work counter
    unsigned long long work_next2;    // second-phase counter (retries)
    unsigned int n_failed;            // sources that overflowed their slot's capacity
    unsigned int err;                 // first device-side error code (CS_ERR_*)
    unsigned int err_where;           // diagnostic: where the error was raised
    unsigned int n_inexact;         // sources whose parallel replay disagreed (redone exactly)
    unsigned long long sources_done;
    unsigned long long edges_relaxed;
    unsigned long long nodes_settled;
    unsigned long long pad[24];
};
static_assert(sizeof(WsHeader) <= 256, "header too large");

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}
__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }

__device__ __forceinline__ int warp_max_i(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(FULL, v, o));
    return v;
}
__device__ __forceinline__ float warp_min_f(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(FULL, v, o));
    return v;
}
__device__ __forceinline__ long long warp_sum_ll(long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    return v;
}
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    return v;
}

// f32 -> f64 by integer ops: keeps the conversion off GB300's narrow FP64 pipe.  Exact for
// every finite f32; zeros, subnormals, infinities and NaN take the hardware conversion.
__device__ __forceinline__ double f2d(float x) {
    const uint32_t b = __float_as_uint(x);
    const uint32_t e = (b >> 23) & 0xffu;
    if (e == 0u || e == 0xffu) return (double)x;
    const uint32_t hi = (b & 0x80000000u) | ((e + 896u) << 20) | ((b & 0x7fffffu) >> 3);
    const uint32_t lo = b << 29;
    return __hiloint2double((int)hi, (int)lo);
}

// Sources completed so far in the current call, counted as they finish (read on a side stream by
// cs_workspace_progress while the kernels run): the header's pad[PROGRESS_SLOT].
constexpr int PROGRESS_SLOT = 8;
__device__ __forceinline__ void count_progress(WsHeader *h) { atomicAdd(&h->pad[PROGRESS_SLOT], 1ull); }

__device__ __forceinline__ void raise_err(WsHeader *h, unsigned code, unsigned where) {
    if (atomicCAS(&h->err, 0u, code) == 0u) h->err_where = where;
}

// Reads a workspace header after the work queued on `s`.  With poll, waits for the stream by
// querying it between short sleeps first: a device->host copy into pageable memory issued while
// long kernels are still queued holds driver resources until they finish, which stalls other host
// threads' CUDA calls (allocations, event creation) for that long.
inline cudaError_t read_header(const WsHeader *dev, WsHeader &h, cudaStream_t s, bool poll) {
    cudaError_t e;
    if (poll) {
        while ((e = cudaStreamQuery(s)) == cudaErrorNotReady) std::this_thread::sleep_for(std::chrono::microseconds(20));
        if (e != cudaSuccess) return e;
    }
    e = cudaMemcpyAsync(&h, dev, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return e;
}

}  // namespace cs
