// isp_tone.cpp - the reference's RGB tone curves (tone::process_tone) as per-sample tables, and
// the device entry point that maps an RGB frame through such a table.
//
// GAMMA, S_CURVE, LEVELS and CURVES_3POINT compute every output sample from that sample's value
// alone, with the same function for R, G and B (src/tone/gamma.cpp:22-32, s_curve.cpp:21-39,
// levels.cpp:40-57, curves_3point.cpp:64-101 of the reference).  A table over every value the
// frame's storage can hold (256 for u8, 65536 for u16) therefore reproduces the reference's output
// exactly when each entry is evaluated with the reference's float expression, in its order, with
// the same libm calls (this file is compiled with -ffp-contract=off, as the oracle pins the
// reference).  SHADOWS_HIGHLIGHTS mixes the channels through a luminance (shadows_highlights.cpp:
// 30-73), so it has no such table and is not served here.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "isp_context.h"

using namespace imop;

namespace {

inline int clamp_val(int v, int max_val) { return std::max(0, std::min(v, max_val)); }

// tone::detail::safe_max_val (src/tone/common.hpp:16-20)
inline int tone_max_val(int bd) {
    if (bd <= 0) return 255;
    if (bd >= 16) return 65535;
    return (1 << bd) - 1;
}

// src/tone/gamma.cpp:18-32
void gamma_table(int bd, const ImopToneParams& p, uint16_t* t, int n) {
    const int max_val = tone_max_val(bd);
    const float mv = static_cast<float>(max_val);
    const float g = std::max(0.1f, std::min(10.0f, p.gamma));
    const float inv_gamma = 1.0f / g;
    for (int val = 0; val < n; val++) {
        const float norm = static_cast<float>(val) / mv;
        const float corrected = std::pow(norm, inv_gamma);
        t[val] = (uint16_t)clamp_val(static_cast<int>(corrected * mv + 0.5f), max_val);
    }
}

// src/tone/s_curve.cpp:13-39
void s_curve_table(int bd, const ImopToneParams& p, uint16_t* t, int n) {
    const int max_val = tone_max_val(bd);
    const float mv = static_cast<float>(max_val);
    const float contrast = std::max(-1.0f, std::min(2.0f, p.contrast));
    const float shadows = std::max(-1.0f, std::min(1.0f, p.shadows));
    const float highlights = std::max(-1.0f, std::min(1.0f, p.highlights));
    const float k = 1.0f + contrast * 4.0f;
    const float denom = 2.0f * std::tanh(k * 0.5f);
    for (int val = 0; val < n; val++) {
        const float norm = static_cast<float>(val) / mv;
        float sc = 0.5f + std::tanh(k * (norm - 0.5f)) / denom;
        const float shadow_weight = (1.0f - norm) * (1.0f - norm);
        sc += shadows * shadow_weight * 0.15f;
        const float highlight_weight = norm * norm;
        sc += highlights * highlight_weight * 0.15f;
        t[val] = (uint16_t)clamp_val(static_cast<int>(sc * mv + 0.5f), max_val);
    }
}

// src/tone/levels.cpp:18-57
void levels_table(int bd, const ImopToneParams& p, uint16_t* t, int n) {
    const int max_val = tone_max_val(bd);
    const float mv = static_cast<float>(max_val);
    const float black = std::max(0.0f, std::min(0.99f, p.black_point));
    float white = std::max(0.01f, std::min(1.0f, p.white_point));
    const float mid = std::max(0.01f, std::min(0.99f, p.mid_point));
    if (white <= black) white = black + 0.01f;
    const float range = white - black;
    const float mid_norm = (mid - black) / range;
    float gamma;
    if (mid_norm > 0.0f && mid_norm < 1.0f) gamma = std::log(0.5f) / std::log(mid_norm);
    else gamma = 1.0f;
    for (int val = 0; val < n; val++) {
        const float norm = static_cast<float>(val) / mv;
        float stretched = (norm - black) / range;
        stretched = std::max(0.0f, std::min(1.0f, stretched));
        const float corrected = std::pow(stretched, 1.0f / gamma);
        t[val] = (uint16_t)clamp_val(static_cast<int>(corrected * mv + 0.5f), max_val);
    }
}

// src/tone/curves_3point.cpp:24-101: two quadratic Bezier segments sampled into 256 floats, then
// a linear interpolation of that table per sample
void curves_table(int bd, const ImopToneParams& p, uint16_t* t, int n) {
    const int max_val = tone_max_val(bd);
    const float mv = static_cast<float>(max_val);
    const float shadows = std::max(-1.0f, std::min(1.0f, p.shadows));
    const float contrast = std::max(-1.0f, std::min(2.0f, p.contrast));
    const float highlights = std::max(-1.0f, std::min(1.0f, p.highlights));
    const float y0 = std::max(0.0f, std::min(1.0f, shadows * 0.1f));
    const float y1 = std::max(0.0f, std::min(1.0f, 0.5f + contrast * 0.15f));
    const float y2 = std::max(0.0f, std::min(1.0f, 1.0f + highlights * 0.1f));
    const float q0y = 0.5f * (y0 + y1);
    const float q1y = 0.5f * (y1 + y2);
    // the y coordinate of B(t) = (1-t)^2 a + 2 (1-t) t b + t^2 c
    auto bezier_y = [](float s, float ay, float by, float cy) {
        const float s1 = 1.0f - s;
        return s1 * s1 * ay + 2.0f * s1 * s * by + s * s * cy;
    };
    float curve[256];
    for (int i = 0; i < 256; i++) {
        const float norm = static_cast<float>(i) / 255.0f;
        float r;
        if (norm <= 0.5f) r = bezier_y(norm * 2.0f, y0, q0y, y1);
        else r = bezier_y((norm - 0.5f) * 2.0f, y1, q1y, y2);
        curve[i] = std::max(0.0f, std::min(1.0f, r));
    }
    for (int val = 0; val < n; val++) {
        float norm, frac;
        int idx;
        if (bd <= 8) {
            idx = val;
            frac = 0.0f;
            if (idx > 254) { idx = 254; frac = 1.0f; }
        } else {
            norm = static_cast<float>(val) / mv;
            const float fi = norm * 255.0f;
            idx = static_cast<int>(fi);
            frac = fi - static_cast<float>(idx);
            if (idx > 254) { idx = 254; frac = 1.0f; }
        }
        norm = curve[idx] * (1.0f - frac) + curve[idx + 1] * frac;
        t[val] = (uint16_t)clamp_val(static_cast<int>(norm * mv + 0.5f), max_val);
    }
}

}  // namespace

extern "C" {

size_t imop_tone_table_entries(int bit_depth) { return bit_depth <= 8 ? 256u : 65536u; }

int imop_tone_table(int algorithm, int bit_depth, const ImopToneParams* params, uint16_t* table, size_t entries) {
    if (!params || !table) return set_error(IMOP_ERR_NULL_INPUT, "null tone parameters or table");
    if (bit_depth < 1 || bit_depth > 16) return set_error(IMOP_ERR_INVALID_BIT_DEPTH, "bit depth must be 1..16");
    const size_t n = imop_tone_table_entries(bit_depth);
    if (entries < n) return set_error(IMOP_ERR_INVALID_ARGUMENT, "tone table smaller than the sample range");
    switch (algorithm) {
        case IMOP_TONE_CURVE_GAMMA: gamma_table(bit_depth, *params, table, (int)n); break;
        case IMOP_TONE_CURVE_S_CURVE: s_curve_table(bit_depth, *params, table, (int)n); break;
        case IMOP_TONE_CURVE_LEVELS: levels_table(bit_depth, *params, table, (int)n); break;
        case IMOP_TONE_CURVE_3POINT: curves_table(bit_depth, *params, table, (int)n); break;
        default: return set_error(IMOP_ERR_UNSUPPORTED, "tone curve has no per-sample table");
    }
    return IMOP_OK;
}

int imop_op_rgb_table(imop_isp_t ctx, int width, int height, int bit_depth, const uint16_t* table, const void* in,
                      void* out) {
    if (!ctx) return set_error(IMOP_ERR_NULL_INPUT, "ctx is null");
    if (!table || !in || !out) return set_error(IMOP_ERR_NULL_INPUT, "null table or frame pointer");
    if (width <= 0 || height <= 0) return set_error(IMOP_ERR_INVALID_DIMENSIONS, "invalid dimensions");
    if (bit_depth < 1 || bit_depth > 16) return set_error(IMOP_ERR_INVALID_BIT_DEPTH, "bit depth must be 1..16");
    if (!device_ready()) return set_error(IMOP_ERR_NO_DEVICE, "no CUDA device");
    const size_t n = (size_t)width * height * 3;
    const int bps = bit_depth <= 8 ? 1 : 2;
    const size_t tab_bytes = imop_tone_table_entries(bit_depth) * sizeof(uint16_t);
    cudaError_t e;
    if ((e = ctx->d_in.ensure(n * bps)) || (e = ctx->op_tone.ensure(tab_bytes)))
        return cuda_fail(e, "alloc tone buffers");
    if ((e = cudaMemcpy(ctx->op_tone.ptr, table, tab_bytes, cudaMemcpyHostToDevice)) ||
        (e = cudaMemcpy(ctx->d_in.ptr, in, n * bps, cudaMemcpyHostToDevice)) ||
        (e = launch_table_map((const uint8_t*)ctx->d_in.ptr, (uint8_t*)ctx->d_in.ptr, n, bps,
                              (const uint16_t*)ctx->op_tone.ptr, 0)) ||
        (e = cudaMemcpy(out, ctx->d_in.ptr, n * bps, cudaMemcpyDeviceToHost)))
        return cuda_fail(e, "tone table stage");
    return IMOP_OK;
}

}  // extern "C"
