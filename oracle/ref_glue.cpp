// ref_glue.cpp - TEST INFRASTRUCTURE ONLY.
//
// extern "C" wrappers around the reference's own CPU functions, linked with the reference's
// CPU sources compiled in place (oracle/Makefile, target _ref/libimop_ref.so).  The tests use
// these wrappers to pin the C restatement (isp_oracle.c) stage by stage.  Nothing here is
// part of the product; nothing here copies reference code - it only calls it.
//
// Build workarounds (the reference's CPU-only link is incomplete):
//  * the per-module has_cuda()/process_*_cuda() symbols normally come from
//    src/gpu_dispatch.cpp, whose non-CUDA branch (:575-592) defines only has_cuda(); this file
//    defines all of them, the *_cuda ones returning InternalError so the dispatchers take the
//    CPU path;
//  * AMAZE's FloatBufferPool::get resizes the outer vector while earlier references are alive
//    (src/algorithms/common.hpp:16-23 with amaze.cpp:152-154); reserving 11 slots once per
//    thread before the first call keeps those references valid.

#include <cstdint>
#include <cstring>
#include <vector>

#include "black_level/algorithms.hpp"
#include "ccm/algorithms.hpp"
#include "defect_correct/algorithms.hpp"
#include "imop/algorithms.hpp"
#include "imop/analyzer.hpp"
#include "color_calibration/algorithms.hpp"
#include "lut/algorithms.hpp"
#include "tone/algorithms.hpp"
#include "jpeg_codec/algorithms.hpp"
#include "imop/pixel_utils.hpp"
#include "lens_shading/algorithms.hpp"
#include "white_balance/algorithms.hpp"
#include "algorithms/common.hpp"

namespace black_level {
bool has_cuda() { return false; }
BlackLevelError process_black_level_cuda(uint8_t*, int, int, BayerPattern, BlackLevelAlgorithm, int,
                                         const BlackLevelParams&) {
    return BlackLevelError::InternalError;
}
}  // namespace black_level
namespace defect_correct {
bool has_cuda() { return false; }
DefectCorrectError process_defect_correct_cuda(uint8_t*, int, int, BayerPattern, DefectCorrectAlgorithm,
                                               int, const DefectCorrectParams&) {
    return DefectCorrectError::InternalError;
}
}  // namespace defect_correct
namespace lens_shading {
bool has_cuda() { return false; }
LensShadingError process_lens_shading_cuda(uint8_t*, int, int, BayerPattern, LensShadingAlgorithm, int,
                                           const LensShadingParams&) {
    return LensShadingError::InternalError;
}
}  // namespace lens_shading
namespace white_balance {
bool has_cuda() { return false; }
WhiteBalanceError process_white_balance_cuda(const uint8_t*, uint8_t*, int, int, int, int, float, float,
                                             float) {
    return WhiteBalanceError::InternalError;
}
}  // namespace white_balance
namespace tone {
bool has_cuda() { return false; }
ToneError process_tone_cuda(const uint8_t*, uint8_t*, int, int, int, ToneAlgorithm, int, const ToneParams&) {
    return ToneError::InternalError;
}
}  // namespace tone
namespace ccm {
bool has_cuda() { return false; }
CCMError process_ccm_cuda(const uint8_t*, uint8_t*, int, int, int, int, const float*) {
    return CCMError::InternalError;
}
}  // namespace ccm

namespace {

void reserve_pool() {
    static thread_local bool done = false;
    if (!done) {
        imop::detail::thread_local_pool().get(1, 10);
        done = true;
    }
}

// u16 plane <-> the reference's storage (u8 for bd <= 8, u16 otherwise)
std::vector<uint8_t> to_store(const uint16_t* d, size_t n, int bd) {
    std::vector<uint8_t> s(bd <= 8 ? n : 2 * n);
    if (bd <= 8) {
        for (size_t i = 0; i < n; i++) s[i] = static_cast<uint8_t>(d[i]);
    } else {
        std::memcpy(s.data(), d, 2 * n);
    }
    return s;
}
void from_store(const std::vector<uint8_t>& s, uint16_t* d, size_t n, int bd) {
    if (bd <= 8) {
        for (size_t i = 0; i < n; i++) d[i] = s[i];
    } else {
        std::memcpy(d, s.data(), 2 * n);
    }
}

}  // namespace

extern "C" {

int ref_get_packed_raw(const uint8_t* data, int x, int y, int w, int h, int bd) {
    return imop::pixel::get_packed_raw(data, x, y, w, bd, 0, h);
}

int ref_get_raw(const uint8_t* data, int x, int y, int w, int h, int bd, int packed) {
    return imop::pixel::get_raw(data, x, y, w, bd, packed != 0, 0, h);
}

int ref_black_level(uint16_t* d, int w, int h, int pattern, int bd, int mode, const float off[4]) {
    size_t n = static_cast<size_t>(w) * h;
    auto s = to_store(d, n, bd);
    black_level::BlackLevelParams p;
    p.r_offset = off[0]; p.gr_offset = off[1]; p.gb_offset = off[2]; p.b_offset = off[3];
    auto e = black_level::process_black_level(s.data(), w, h, static_cast<imop::BayerPattern>(pattern),
                                              static_cast<black_level::BlackLevelAlgorithm>(mode), bd, p);
    from_store(s, d, n, bd);
    return static_cast<int>(e);
}

int ref_dpc(uint16_t* d, int w, int h, int pattern, int bd, int mode, float threshold,
            const int* map_xy, int map_count) {
    size_t n = static_cast<size_t>(w) * h;
    auto s = to_store(d, n, bd);
    std::vector<defect_correct::DefectPoint> pts(static_cast<size_t>(map_count > 0 ? map_count : 0));
    for (int i = 0; i < map_count; i++) pts[i] = {map_xy[2 * i], map_xy[2 * i + 1]};
    defect_correct::DefectCorrectParams p;
    p.threshold = threshold;
    p.map = pts.empty() ? nullptr : pts.data();
    p.map_count = map_count;
    auto e = defect_correct::process_defect_correct(s.data(), w, h, static_cast<imop::BayerPattern>(pattern),
                                                    static_cast<defect_correct::DefectCorrectAlgorithm>(mode),
                                                    bd, p);
    from_store(s, d, n, bd);
    return static_cast<int>(e);
}

int ref_lsc_poly(uint16_t* d, int w, int h, int pattern, int bd, const float coef[12], float cx, float cy) {
    size_t n = static_cast<size_t>(w) * h;
    auto s = to_store(d, n, bd);
    lens_shading::LensShadingParams p;
    p.r_coef = {coef[0], coef[1], coef[2]};
    p.gr_coef = {coef[3], coef[4], coef[5]};
    p.gb_coef = {coef[6], coef[7], coef[8]};
    p.b_coef = {coef[9], coef[10], coef[11]};
    p.center_x = cx;
    p.center_y = cy;
    auto e = lens_shading::process_lens_shading(s.data(), w, h, static_cast<imop::BayerPattern>(pattern),
                                                lens_shading::LensShadingAlgorithm::POLYNOMIAL, bd, p);
    from_store(s, d, n, bd);
    return static_cast<int>(e);
}

// flat field given as the reference's storage (u8 / u16 bytes)
int ref_lsc_flat_field(uint16_t* d, int w, int h, int pattern, int bd, const uint8_t* ff, int ffw, int ffh) {
    size_t n = static_cast<size_t>(w) * h;
    auto s = to_store(d, n, bd);
    lens_shading::LensShadingParams p;
    p.flat_field = ff;
    p.flat_field_width = ffw;
    p.flat_field_height = ffh;
    auto e = lens_shading::process_lens_shading(s.data(), w, h, static_cast<imop::BayerPattern>(pattern),
                                                lens_shading::LensShadingAlgorithm::FLAT_FIELD, bd, p);
    from_store(s, d, n, bd);
    return static_cast<int>(e);
}

// Bayer u16 plane -> RGB u16 x 3 through imop::demosaic_cpu on a zeroed output buffer.
int ref_demosaic(const uint16_t* bay, uint16_t* rgb, int w, int h, int pattern, int algo, int bd) {
    reserve_pool();
    size_t n = static_cast<size_t>(w) * h;
    auto s = to_store(bay, n, bd);
    std::vector<uint8_t> out(n * 3 * (bd <= 8 ? 1 : 2), 0);
    auto e = imop::demosaic_cpu(s.data(), out.data(), w, h, static_cast<imop::BayerPattern>(pattern),
                                static_cast<imop::DemosaicAlgorithm>(algo), bd, false);
    if (bd <= 8) {
        for (size_t i = 0; i < n * 3; i++) rgb[i] = out[i];
    } else {
        std::memcpy(rgb, out.data(), n * 6);
    }
    return static_cast<int>(e);
}

// Packed / unpacked input straight into imop::demosaic_cpu (the reference's own unpack).
int ref_demosaic_raw(const uint8_t* in, uint16_t* rgb, int w, int h, int pattern, int algo, int bd,
                     int packed) {
    reserve_pool();
    size_t n = static_cast<size_t>(w) * h;
    std::vector<uint8_t> out(n * 3 * (bd <= 8 ? 1 : 2), 0);
    auto e = imop::demosaic_cpu(in, out.data(), w, h, static_cast<imop::BayerPattern>(pattern),
                                static_cast<imop::DemosaicAlgorithm>(algo), bd, packed != 0);
    if (bd <= 8) {
        for (size_t i = 0; i < n * 3; i++) rgb[i] = out[i];
    } else {
        std::memcpy(rgb, out.data(), n * 6);
    }
    return static_cast<int>(e);
}

int ref_wb_rgb(uint16_t* rgb, int w, int h, int bd, const float gain[3]) {
    size_t n = static_cast<size_t>(w) * h * 3;
    auto s = to_store(rgb, n, bd);
    std::vector<uint8_t> out(s.size());
    white_balance::WBCoefficients g;
    g.r_gain = gain[0]; g.g_gain = gain[1]; g.b_gain = gain[2];
    auto e = white_balance::process_white_balance(s.data(), out.data(), w, h, 3,
                                                  white_balance::WhiteBalanceAlgorithm::MANUAL, bd, 6.0f, g);
    from_store(out, rgb, n, bd);
    return static_cast<int>(e);
}

int ref_ccm(uint16_t* rgb, int w, int h, int bd, const float m[9]) {
    size_t n = static_cast<size_t>(w) * h * 3;
    auto s = to_store(rgb, n, bd);
    std::vector<uint8_t> out(s.size());
    ccm::CCMatrix3x3 mat;
    for (int i = 0; i < 9; i++) mat.m[i] = m[i];
    auto e = ccm::process_ccm(s.data(), out.data(), w, h, 3, ccm::CCMAlgorithm::LINEAR_3X3, bd, &mat);
    from_store(out, rgb, n, bd);
    return static_cast<int>(e);
}

// analyzer: detected depth and sizes; info = {depth, w, h, pixels, max, min, is16, packed, n_dims}
int ref_detect_bit_depth(const uint8_t* d, size_t n) { return imop::detect_bit_depth(d, n); }
int ref_suggest_dimensions(size_t n, int* out, int cap) {
    const auto v = imop::suggest_dimensions(n);
    for (size_t k = 0; k < v.size() && (int)k < cap; k++) {
        out[2 * k] = v[k].first;
        out[2 * k + 1] = v[k].second;
    }
    return (int)v.size();
}
int ref_analyze_data(const uint8_t* d, size_t n, int* info, int* dims, int cap) {
    const imop::DataInfo a = imop::analyze_data(d, n);
    const int v[9] = {a.detected_bit_depth, a.suggested_width, a.suggested_height, a.pixel_count, a.max_value,
                      a.min_value, a.is_likely_16bit ? 1 : 0, a.is_packed ? 1 : 0, (int)a.possible_dimensions.size()};
    for (int k = 0; k < 9; k++) info[k] = v[k];
    for (size_t k = 0; k < a.possible_dimensions.size() && (int)k < cap; k++) {
        dims[2 * k] = a.possible_dimensions[k].first;
        dims[2 * k + 1] = a.possible_dimensions[k].second;
    }
    return 0;
}
int ref_guess_pattern(const uint8_t* d, int w, int h, int bd, int packed) {
    return (int)imop::guess_pattern(d, w, h, bd, packed != 0);
}

// colour calibration: m receives rows x cols floats; returns the error code
int ref_solve_ccm(const float* measured, const float* reference, int n, int type, float* m, int* rows, int* cols) {
    color_calibration::SolveCCMParams p;
    p.measured = reinterpret_cast<const color_calibration::PatchColor*>(measured);
    p.reference = reinterpret_cast<const color_calibration::PatchColor*>(reference);
    p.patch_count = n;
    p.matrix_type = static_cast<color_calibration::MatrixType>(type);
    color_calibration::SolvedMatrix r;
    const int e = (int)color_calibration::process_solve_ccm(p, &r);
    if (e == 0) {
        std::memcpy(m, r.m, sizeof(r.m));
        *rows = r.rows;
        *cols = r.cols;
    }
    return e;
}

// ---- the reference's per-module calls on frames in the reference's own storage (no conversion
// copies), the form the timed CPU baseline composes: u8 samples for bd <= 8, u16 otherwise
// pixel::get_packed_raw (include/imop/pixel_utils.hpp:58-118) of every pixel of a packed frame
void ref_unpack_packed(const uint8_t* raw, size_t nbytes, uint16_t* out, int w, int h, int bd) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++)
            out[(size_t)y * w + x] = (uint16_t)imop::pixel::get_packed_raw(raw, x, y, w, bd, nbytes, h);
}
int ref_black_level_store(uint8_t* data, int w, int h, int pattern, int bd, const float off[4]) {
    black_level::BlackLevelParams p;
    p.r_offset = off[0]; p.gr_offset = off[1]; p.gb_offset = off[2]; p.b_offset = off[3];
    return (int)black_level::process_black_level(data, w, h, static_cast<imop::BayerPattern>(pattern),
                                                 black_level::BlackLevelAlgorithm::PER_CHANNEL, bd, p);
}
int ref_dpc_adaptive_store(uint8_t* data, int w, int h, int pattern, int bd, float threshold) {
    defect_correct::DefectCorrectParams p;
    p.threshold = threshold;
    return (int)defect_correct::process_defect_correct(data, w, h, static_cast<imop::BayerPattern>(pattern),
                                                       defect_correct::DefectCorrectAlgorithm::ADAPTIVE, bd, p);
}
int ref_demosaic_store(const uint8_t* bay, uint8_t* rgb, int w, int h, int pattern, int algo, int bd) {
    reserve_pool();
    return (int)imop::demosaic_cpu(bay, rgb, w, h, static_cast<imop::BayerPattern>(pattern),
                                   static_cast<imop::DemosaicAlgorithm>(algo), bd, false);
}
int ref_ccm_store(const uint8_t* in, uint8_t* out, int w, int h, int bd, const float m[9]) {
    ccm::CCMatrix3x3 mat;
    for (int i = 0; i < 9; i++) mat.m[i] = m[i];
    return (int)ccm::process_ccm(in, out, w, h, 3, ccm::CCMAlgorithm::LINEAR_3X3, bd, &mat);
}

// tone::process_tone on interleaved RGB in its storage (u8 for bd <= 8, u16 otherwise), in -> out;
// p = gamma, contrast, shadows, highlights, black_point, white_point, mid_point
int ref_tone(const uint16_t* rgb, uint16_t* out, int w, int h, int bd, int algo, const float p[7]) {
    tone::ToneParams tp;
    tp.gamma = p[0]; tp.contrast = p[1]; tp.shadows = p[2]; tp.highlights = p[3];
    tp.black_point = p[4]; tp.white_point = p[5]; tp.mid_point = p[6];
    const size_t n = (size_t)w * h * 3;
    std::vector<uint8_t> in = to_store(rgb, n, bd), o(in.size());
    const int e = (int)tone::process_tone(in.data(), o.data(), w, h, 3, static_cast<tone::ToneAlgorithm>(algo), bd, tp);
    if (e == 0) from_store(o, out, n, bd);
    return e;
}

// 3D LUT on interleaved RGB in its storage (u8 for bd <= 8, u16 otherwise), in place
int ref_apply_lut(uint16_t* rgb, int w, int h, int bd, const float* lut, int size) {
    lut::LUT3D L;
    L.size = size;
    L.data.assign(lut, lut + (size_t)size * size * size * 3);
    const size_t n = (size_t)w * h * 3;
    std::vector<uint8_t> in = to_store(rgb, n, bd), out(in.size());
    const int e = (int)lut::apply_lut(L, in.data(), out.data(), w, h, bd);
    if (e == 0) from_store(out, rgb, n, bd);
    return e;
}

// jpeg_codec::process_encode_baseline / process_decode_baseline (src/jpeg_codec/encode_baseline.cpp,
// decode_baseline.cpp); *size in = capacity (0: the reference's default), out = bytes written
int ref_jpeg_encode(const uint8_t* rgb, int w, int h, int bd, int quality, int subsample, uint8_t* out,
                    size_t* size) {
    jpeg_codec::JpegParams p;
    p.quality = quality;
    p.chroma_subsample = subsample;
    return (int)jpeg_codec::process_encode_baseline(rgb, out, size, w, h, 3, bd, p);
}
int ref_jpeg_decode(const uint8_t* jpg, size_t n, uint8_t* rgb, int* w, int* h, int* c) {
    return (int)jpeg_codec::process_decode_baseline(jpg, n, rgb, w, h, c);
}

}  // extern "C"
