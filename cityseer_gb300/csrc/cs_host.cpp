// cs_host.cpp -- host-side (CPU) parts of the C-ABI that must reproduce the reference's f32
// arithmetic bit for bit: threshold conversions (rust/src/common.rs:99-270) and per-edge travel
// seconds with the Tobler slope penalty (rust/src/centrality.rs:961-1007).
// Compiled with -ffp-contract=off so that no a*b+c is fused into an FMA (Rust never fuses).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>

#include "../../include/cityseer_gb300.h"

extern "C" void cs_set_error_internal(const char *msg);

namespace {
const float MIN_THRESH_WT = 0.01831563888873418f;  // rust/src/common.rs:10

cs_status arg_err(const char *msg) {
    cs_set_error_internal(msg);
    return CS_ERR_ARG;
}

// betas_from_distances (common.rs:134-165)
cs_status betas_from_distances(const uint32_t *d, int k, float mtw, float *betas) {
    if (k <= 0) return arg_err("Input 'distances' cannot be empty.");
    for (int i = 1; i < k; i++)
        if (d[i] <= d[i - 1]) return arg_err("Distances must be unique and sorted in strictly increasing order.");
    for (int i = 0; i < k; i++) {
        if (d[i] == 0) return arg_err("Distances must be positive integers.");
        const float beta = -std::log(mtw) / (float)d[i];
        betas[i] = std::round(beta * 100000.0f) / 100000.0f;
    }
    return CS_OK;
}
// distances_from_betas (common.rs:99-131)
cs_status distances_from_betas(const float *b, int k, float mtw, uint32_t *d) {
    if (k <= 0) return arg_err("Input 'betas' cannot be empty.");
    for (int i = 1; i < k; i++)
        if (b[i] >= b[i - 1]) return arg_err("Betas must be unique and sorted in strictly decreasing order.");
    for (int i = 0; i < k; i++) {
        if (b[i] <= 0.0f) return arg_err("Beta values must be greater than zero.");
        const float dist = std::round(std::log(mtw) / -b[i]);
        if (dist <= 0.0f) return arg_err("Derived distance must be positive. Check beta values.");
        d[i] = (uint32_t)dist;
    }
    return CS_OK;
}
// seconds_from_distances (common.rs:203-237)
cs_status seconds_from_distances(const uint32_t *d, int k, float speed, uint32_t *s) {
    if (k <= 0) return arg_err("Input 'distances' cannot be empty.");
    if (speed <= 0.0f) return arg_err("Speed must be positive.");
    for (int i = 1; i < k; i++)
        if (d[i] <= d[i - 1]) return arg_err("Distances must be unique and sorted in strictly increasing order.");
    for (int i = 0; i < k; i++) {
        if (d[i] == 0) return arg_err("Distances must be positive integers.");
        const float t = std::round((float)d[i] / speed);
        if (t <= 0.0f) return arg_err("Derived time must be positive. Check distance and speed values.");
        s[i] = (uint32_t)t;
    }
    return CS_OK;
}
// distances_from_seconds (common.rs:167-201)
cs_status distances_from_seconds(const uint32_t *s, int k, float speed, uint32_t *d) {
    if (k <= 0) return arg_err("Input 'seconds' cannot be empty.");
    if (speed <= 0.0f) return arg_err("Speed must be positive.");
    for (int i = 1; i < k; i++)
        if (s[i] <= s[i - 1]) return arg_err("Times must be unique and sorted in strictly increasing order.");
    for (int i = 0; i < k; i++) {
        if (s[i] == 0) return arg_err("Time values must be positive integers.");
        const float dist = std::round((float)s[i] * speed);
        if (dist <= 0.0f) return arg_err("Derived distance must be positive. Check time and speed values.");
        d[i] = (uint32_t)dist;
    }
    return CS_OK;
}
// Rust `f32 as u32`: saturating, NaN -> 0.
uint32_t sat_u32(float x) {
    if (!(x > 0.0f)) return 0u;
    if (x >= 4294967295.0f) return 4294967295u;
    return (uint32_t)x;
}
}  // namespace

extern "C" {

cs_status cs_pair_distances_betas_time(float speed_m_s, int32_t mode, int32_t k, const uint32_t *distances,
                                       const float *betas, const float *minutes, float min_threshold_wt,
                                       uint32_t *out_distances, float *out_betas, uint32_t *out_seconds) {
    const float mtw = min_threshold_wt < 0.0f ? MIN_THRESH_WT : min_threshold_wt;
    if (!out_distances || !out_betas || !out_seconds) return arg_err("output arrays are NULL");
    cs_status st;
    switch (mode) {
    case 0:
        if (!distances) return arg_err("distances is NULL");
        st = betas_from_distances(distances, k, mtw, out_betas);
        if (st) return st;
        st = seconds_from_distances(distances, k, speed_m_s, out_seconds);
        if (st) return st;
        std::memcpy(out_distances, distances, sizeof(uint32_t) * (size_t)k);
        return CS_OK;
    case 1:
        if (!betas) return arg_err("betas is NULL");
        st = distances_from_betas(betas, k, mtw, out_distances);
        if (st) return st;
        st = seconds_from_distances(out_distances, k, speed_m_s, out_seconds);
        if (st) return st;
        std::memcpy(out_betas, betas, sizeof(float) * (size_t)k);
        return CS_OK;
    case 2:
        if (!minutes) return arg_err("minutes is NULL");
        for (int i = 0; i < k; i++) out_seconds[i] = sat_u32(std::round(minutes[i] * 60.0f));
        st = distances_from_seconds(out_seconds, k, speed_m_s, out_distances);
        if (st) return st;
        return betas_from_distances(out_distances, k, mtw, out_betas);
    default:
        return arg_err(
            "Please provide exactly one of the following arguments: 'distances', 'betas', or 'minutes'.");
    }
}

cs_status cs_edge_travel_seconds(int64_t n_edges, const int32_t *src, const int32_t *dst, const float *length,
                                 const float *imp_factor, const float *seconds, const uint8_t *has_z,
                                 const double *z, float speed_m_s, int32_t use_impedance, float *out) {
    if (n_edges < 0 || !src || !dst || !length || !imp_factor || !seconds || !out) return arg_err("NULL edge array");
    if (!std::isfinite(speed_m_s) || speed_m_s <= 0.0f) return arg_err("speed_m_s must be finite and positive");
    const float FLAT_FACTOR = 0.839457f;
    for (int64_t e = 0; e < n_edges; e++) {
        if (!std::isnan(seconds[e])) {
            out[e] = seconds[e];
            continue;
        }
        const float len = length[e];
        float slope_pen = 1.0f;
        if (len > 0.0f && has_z && z && has_z[src[e]] && has_z[dst[e]]) {
            const float slope = (float)(z[dst[e]] - z[src[e]]) / len;
            const float slope_factor = std::exp(-3.5f * std::fabs(slope + 0.05f));
            slope_pen = FLAT_FACTOR / slope_factor;
        }
        const float imp = use_impedance ? imp_factor[e] : 1.0f;
        out[e] = (len * imp * slope_pen) / speed_m_s;
    }
    return CS_OK;
}

}  // extern "C"
