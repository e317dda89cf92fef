// cs_cta.cuh -- host/device interface of the block-per-source shortest-path kernel (cs_cta.cu).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "cs_common.cuh"

namespace cs {
namespace cta {

// One thread block per source; the source's reached set lives in a shared-memory hash table.
constexpr int TPB = 1024;       // threads per block
constexpr int NW = TPB / 32;    // warps per block
constexpr int HBITS = 14;
constexpr int HSIZE = 1 << HBITS;  // hash slots (node -> distance, then node -> settle position)
constexpr int RMAX = 9984;      // reached nodes per source held on chip (more: the per-warp kernel)
constexpr int NCH = RMAX / 32;  // chunks of 32 settle positions
constexpr int QCAP = 3328;      // entries per search queue (near, next, far)
constexpr int NBK = 1024;       // distance buckets of the settle-order sort
constexpr int BKMAX = 512;      // largest bucket sorted on chip
constexpr int PMAX = 8;         // predecessors per node (the graph's maximum out-degree)

// Launch parameters (filled by the host side of cs_primal.cu).
struct Params {
    // graph (primal CSR, cs_primal_graph)
    int32_t n_bound;
    const int32_t *in_ptr, *in_nb;
    const float *in_w;
    const int32_t *out_ptr, *out_to;
    const float *out_w;
    const uint8_t *out_cnt;
    const float *node_w;
    // query
    int32_t k;
    float dk[MAXK];
    float beta[MAXK];
    float maxsec, speed, tol, delta;
    int32_t closeness, betweenness, track_reach, od;
    const int32_t *src_list;
    int64_t n_src;
    const float *src_wt;
    const uint8_t *eligible;
    const int32_t *od_ptr, *od_dst;
    const float *od_w;
    // outputs: rows [7][K][n_bound] (OD: [2][K][n_bound]), closeness bucket [3][K][n_bound]
    double *out, *bucket;
    uint32_t *reach;
    // workspace
    WsHeader *hdr;
    int32_t *failed;  // sources (indices into src_list) left to the per-warp kernel
    int32_t fail_cap;
    char *scratch;    // per-block global scratch, scratch_stride bytes each
    size_t scratch_stride;
};

// Global scratch of one block: settle order (node ids), settle distances, predecessor positions
// and counts, all indexed by settle position.
inline size_t scratch_bytes() {
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    return al(4ull * RMAX) + al(4ull * RMAX) + al(2ull * PMAX * RMAX) + al(1ull * RMAX);
}

// Dynamic shared memory of the kernel.
size_t smem_bytes();
// True when the kernel can serve this graph and query (maximum out-degree, threshold count).
bool supported(int max_out_degree, int k);
// Launches `blocks` persistent blocks on `stream`; returns the launch error.
cudaError_t launch(const Params &p, int blocks, cudaStream_t stream);
// Tabulates the seed exponentials of this kernel (cs_seed.cuh) on `stream`.
cudaError_t launch_seed_table(cudaStream_t stream);

}  // namespace cta
}  // namespace cs
