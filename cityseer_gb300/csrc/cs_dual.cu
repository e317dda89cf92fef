// cs_dual.cu -- simplest-path (angular) centrality on the dual graph.  Placeholder entry points;
// the kernels land in a later revision of this file.
#include <cstdint>
#include "cs_common.cuh"

extern "C" void cs_set_error_internal(const char *msg);

extern "C" {
cs_status cs_plan_dual(const cs_dual_graph *, int32_t, int32_t, int32_t, int32_t, int64_t, cs_plan *) {
    cs_set_error_internal("simplest-path kernels are not built yet");
    return CS_ERR_ARG;
}
cs_status cs_centrality_simplest(const cs_dual_graph *, const cs_query *, const cs_plan *, void *, size_t, cs_outputs,
                                 void *) {
    cs_set_error_internal("simplest-path kernels are not built yet");
    return CS_ERR_ARG;
}
cs_status cs_tree_simplest(const cs_dual_graph *, int32_t, const int32_t *, uint32_t, float, const cs_plan *, void *,
                           size_t, int32_t, int32_t *, int32_t *, float *, float *, int32_t *, void *) {
    cs_set_error_internal("simplest-path kernels are not built yet");
    return CS_ERR_ARG;
}
}
