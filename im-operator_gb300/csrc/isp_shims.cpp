// isp_shims.cpp - the reference's GPU glue symbols (include/imop_ref_shims.hpp) on this library.
//
// Each shim runs on a per-thread context, as the reference's glue keeps per-thread workspaces
// (src/gpu_dispatch.cpp:45, src/algorithms/cuda_dispatch.cpp:51), and is synchronous with host
// buffers in and out.  Statuses 0..6 carry over numerically; anything this path does not serve
// returns InternalError, which sends the reference's dispatcher to its CPU code.

#include <cuda_runtime.h>

#include <atomic>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/imop_isp.h"
#include "../../include/imop_ref_shims.hpp"

namespace {

struct ThreadCtx {
    imop_isp_t ctx = nullptr;
    ~ThreadCtx() {
        if (ctx) imop_isp_destroy(ctx);
    }
};
thread_local ThreadCtx t_ctx;

imop_isp_t thread_ctx() {
    if (!t_ctx.ctx && imop_isp_create(&t_ctx.ctx) != IMOP_OK) t_ctx.ctx = nullptr;
    return t_ctx.ctx;
}

// status of this library -> the reference's enum (equal values 0..6, InternalError beyond)
template <class E>
E as_status(int rc) {
    return (rc >= 0 && rc <= 6) ? static_cast<E>(rc) : E::InternalError;
}

// calls that ran on the device and returned Ok (imop_shim_calls_served)
std::atomic<long long> g_served{0};

// as_status, counting a call that the device served
template <class E>
E served(int rc) {
    if (rc == 0) g_served.fetch_add(1, std::memory_order_relaxed);
    return as_status<E>(rc);
}

ImopIspParams base_params(int w, int h, int bd, int pattern) {
    ImopIspParams p;
    imop_isp_params_default(&p, w, h, bd, 0);
    p.pattern = pattern;
    p.out_format = IMOP_OUT_NATIVE;
    return p;
}

int demosaic_code(imop::DemosaicAlgorithm a) {
    switch (a) {
        case imop::DemosaicAlgorithm::HQLI: return IMOP_DEMOSAIC_HQLI;
        case imop::DemosaicAlgorithm::MG: return IMOP_DEMOSAIC_MG;
        case imop::DemosaicAlgorithm::AMAZE: return IMOP_DEMOSAIC_AMAZE;
        default: return -1;
    }
}

}  // namespace

namespace imop {

bool has_cuda() { return imop_has_cuda() == 1; }

const char* cuda_device_name() {
    static thread_local char name[256] = {0};
    cudaDeviceProp prop;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return "";
    std::snprintf(name, sizeof(name), "%s", prop.name);
    return name;
}

void cuda_synchronize() { cudaDeviceSynchronize(); }

DemosaicError demosaic_cuda(const uint8_t* bayer_data, uint8_t* rgb_data, int width, int height, BayerPattern pattern,
                            DemosaicAlgorithm algorithm, int bit_depth, bool is_packed) {
    if (!bayer_data || !rgb_data) return DemosaicError::NullInput;
    const int code = demosaic_code(algorithm);
    imop_isp_t ctx = thread_ctx();
    if (code < 0 || !ctx) return DemosaicError::InternalError;
    ImopIspParams p = base_params(width, height, bit_depth, static_cast<int>(pattern));
    p.packed = is_packed ? 1 : 0;
    p.demosaic = code;
    int rc = imop_isp_set_params(ctx, &p);
    if (rc == IMOP_OK)
        rc = imop_isp_run_host(ctx, bayer_data, imop_isp_input_bytes(&p), rgb_data, imop_isp_output_bytes(&p));
    return served<DemosaicError>(rc);
}

DemosaicError demosaic_cuda_batch(const uint8_t* const* bayer_data_array, uint8_t* const* rgb_data_array,
                                  int num_frames, int width, int height, BayerPattern pattern,
                                  DemosaicAlgorithm algorithm, int bit_depth) {
    if (num_frames <= 0) return DemosaicError::Ok;
    if (!bayer_data_array || !rgb_data_array) return DemosaicError::NullInput;
    const int code = demosaic_code(algorithm);
    imop_isp_t ctx = thread_ctx();
    if (code < 0 || !ctx) return DemosaicError::InternalError;
    ImopIspParams p = base_params(width, height, bit_depth, static_cast<int>(pattern));
    p.demosaic = code;
    std::vector<ImopFrameDesc> frames((size_t)num_frames);
    for (int i = 0; i < num_frames; i++) {
        if (!bayer_data_array[i] || !rgb_data_array[i]) return DemosaicError::NullInput;
        frames[i].params = &p;
        frames[i].in = bayer_data_array[i];
        frames[i].out = rgb_data_array[i];
    }
    return served<DemosaicError>(imop_isp_run_host_batch(ctx, frames.data(), num_frames));
}

}  // namespace imop

namespace black_level {

bool has_cuda() { return imop::has_cuda(); }

BlackLevelError process_black_level_cuda(uint8_t* data, int width, int height, BayerPattern pattern,
                                         BlackLevelAlgorithm algorithm, int bit_depth, const BlackLevelParams& params) {
    if (!data) return BlackLevelError::NullInput;
    imop_isp_t ctx = thread_ctx();
    if (!ctx) return BlackLevelError::InternalError;
    ImopIspParams p = base_params(width, height, bit_depth, static_cast<int>(pattern));
    // process_global uses r_offset for every pixel (src/black_level/global.cpp:14)
    p.bl_mode = algorithm == BlackLevelAlgorithm::GLOBAL ? IMOP_BL_GLOBAL : IMOP_BL_PER_CHANNEL;
    p.bl_offset[0] = params.r_offset;
    p.bl_offset[1] = params.gr_offset;
    p.bl_offset[2] = params.gb_offset;
    p.bl_offset[3] = params.b_offset;
    return served<BlackLevelError>(imop_op_bayer_stage(ctx, &p, IMOP_STAGE_BLACK_LEVEL, data));
}

}  // namespace black_level

namespace defect_correct {

bool has_cuda() { return imop::has_cuda(); }

DefectCorrectError process_defect_correct_cuda(uint8_t* data, int width, int height, BayerPattern pattern,
                                               DefectCorrectAlgorithm algorithm, int bit_depth,
                                               const DefectCorrectParams& params) {
    if (!data) return DefectCorrectError::NullInput;
    imop_isp_t ctx = thread_ctx();
    if (!ctx) return DefectCorrectError::InternalError;
    static_assert(sizeof(DefectPoint) == sizeof(ImopDefectPoint), "defect point layout");
    ImopIspParams p = base_params(width, height, bit_depth, static_cast<int>(pattern));
    p.dpc_mode = algorithm == DefectCorrectAlgorithm::MAP_BASED ? IMOP_DPC_MAP_BASED : IMOP_DPC_ADAPTIVE;
    p.dpc_threshold = params.threshold;
    p.dpc_map = reinterpret_cast<const ImopDefectPoint*>(params.map);
    p.dpc_map_count = params.map ? params.map_count : 0;
    return served<DefectCorrectError>(imop_op_bayer_stage(ctx, &p, IMOP_STAGE_DEFECT, data));
}

}  // namespace defect_correct

namespace lens_shading {

bool has_cuda() { return imop::has_cuda(); }

LensShadingError process_lens_shading_cuda(uint8_t* data, int width, int height, BayerPattern pattern,
                                           LensShadingAlgorithm algorithm, int bit_depth,
                                           const LensShadingParams& params) {
    if (!data) return LensShadingError::NullInput;
    imop_isp_t ctx = thread_ctx();
    if (!ctx) return LensShadingError::InternalError;
    ImopIspParams p = base_params(width, height, bit_depth, static_cast<int>(pattern));
    if (algorithm == LensShadingAlgorithm::FLAT_FIELD) {
        p.lsc_mode = IMOP_LSC_FLAT_FIELD;
        p.lsc_flat_field = params.flat_field;
        p.lsc_flat_w = params.flat_field_width;
        p.lsc_flat_h = params.flat_field_height;
    } else {
        p.lsc_mode = IMOP_LSC_POLYNOMIAL;
        const ShadingPolynomial* c[4] = {&params.r_coef, &params.gr_coef, &params.gb_coef, &params.b_coef};
        for (int k = 0; k < 4; k++) {
            p.lsc_poly[k][0] = c[k]->a2;
            p.lsc_poly[k][1] = c[k]->a4;
            p.lsc_poly[k][2] = c[k]->a6;
        }
        p.lsc_center[0] = params.center_x;
        p.lsc_center[1] = params.center_y;
    }
    return served<LensShadingError>(imop_op_bayer_stage(ctx, &p, IMOP_STAGE_LENS_SHADING, data));
}

}  // namespace lens_shading

namespace white_balance {

bool has_cuda() { return imop::has_cuda(); }

WhiteBalanceError process_white_balance_cuda(const uint8_t* input, uint8_t* output, int width, int height, int channels,
                                             int bit_depth, float r_gain, float g_gain, float b_gain) {
    if (!input || !output) return WhiteBalanceError::NullInput;
    if (channels != 3) return WhiteBalanceError::InternalError;
    imop_isp_t ctx = thread_ctx();
    if (!ctx) return WhiteBalanceError::InternalError;
    ImopIspParams p = base_params(width, height, bit_depth, IMOP_RGGB);
    p.wb_gain[0] = r_gain;
    p.wb_gain[1] = g_gain;
    p.wb_gain[2] = b_gain;
    return served<WhiteBalanceError>(imop_op_rgb_stage(ctx, &p, IMOP_STAGE_WHITE_BALANCE, input, output));
}

}  // namespace white_balance

namespace ccm {

bool has_cuda() { return imop::has_cuda(); }

CCMError process_ccm_cuda(const uint8_t* input, uint8_t* output, int width, int height, int channels, int bit_depth,
                          const float* matrix) {
    if (!input || !output) return CCMError::NullInput;
    if (channels != 3 || !matrix) return CCMError::InternalError;
    imop_isp_t ctx = thread_ctx();
    if (!ctx) return CCMError::InternalError;
    ImopIspParams p = base_params(width, height, bit_depth, IMOP_RGGB);
    std::memcpy(p.ccm, matrix, sizeof(p.ccm));
    return served<CCMError>(imop_op_rgb_stage(ctx, &p, IMOP_STAGE_CCM, input, output));
}

}  // namespace ccm

namespace tone {

bool has_cuda() { return imop::has_cuda(); }

// GAMMA, S_CURVE, LEVELS and CURVES_3POINT: a per-sample table of the reference's expression
// (imop_tone_table), applied to the frame on the device.  SHADOWS_HIGHLIGHTS couples the channels
// and returns InternalError, so the dispatcher runs the reference's CPU code for it.
ToneError process_tone_cuda(const uint8_t* input, uint8_t* output, int width, int height, int channels,
                            ToneAlgorithm algorithm, int bit_depth, const ToneParams& params) {
    if (!input || !output) return ToneError::NullInput;
    if (channels != 3 || algorithm == ToneAlgorithm::SHADOWS_HIGHLIGHTS) return ToneError::InternalError;
    imop_isp_t ctx = thread_ctx();
    if (!ctx) return ToneError::InternalError;
    static_assert(sizeof(ToneParams) == sizeof(ImopToneParams), "tone parameter layout");
    ImopToneParams tp;
    std::memcpy(&tp, &params, sizeof(tp));
    thread_local std::vector<uint16_t> table;
    table.resize(imop_tone_table_entries(bit_depth));
    int rc = imop_tone_table(static_cast<int>(algorithm), bit_depth, &tp, table.data(), table.size());
    if (rc == IMOP_OK) rc = imop_op_rgb_table(ctx, width, height, bit_depth, table.data(), input, output);
    return served<ToneError>(rc);
}

}  // namespace tone

namespace lut {

bool has_cuda() { return imop::has_cuda(); }

// CUSTOM_3D (src/lut/dispatch.cpp:84-88): the trilinear 3D LUT of lut::apply_lut on the device
LUTError process_lut_cuda(const uint8_t* input, uint8_t* output, int width, int height, int channels, int bit_depth,
                          const LUT3D& lut_data) {
    if (!input || !output) return LUTError::NullInput;
    const size_t n = (size_t)lut_data.size * lut_data.size * lut_data.size * 3;
    if (channels != 3 || lut_data.size < 2 || lut_data.size > 65 || lut_data.data.size() != n)
        return LUTError::InternalError;
    imop_isp_t ctx = thread_ctx();
    if (!ctx) return LUTError::InternalError;
    ImopIspParams p = base_params(width, height, bit_depth, IMOP_RGGB);
    p.lut3d = lut_data.data.data();
    p.lut3d_size = lut_data.size;
    return served<LUTError>(imop_op_rgb_stage(ctx, &p, IMOP_STAGE_LUT3D, input, output));
}

}  // namespace lut

// ---- jpeg_codec: the glue of src/jpeg_codec/cuda_dispatch.cpp ----------------------------------
namespace jpeg_codec {

// the reference's CPU decoder, when the caller links it (weak: absent -> null)
JpegError process_decode_baseline(const uint8_t*, size_t, uint8_t*, int*, int*, int*) __attribute__((weak));

namespace {
struct JpegThreadCtx {
    imop_jpeg_t ctx = nullptr;
    ~JpegThreadCtx() {
        if (ctx) imop_jpeg_destroy(ctx);
    }
};
thread_local JpegThreadCtx t_jpeg;
}  // namespace

bool has_cuda() { return imop::has_cuda(); }
const char* cuda_device_name() { return imop::cuda_device_name(); }
void cuda_synchronize() { cudaDeviceSynchronize(); }

// src/jpeg_codec/cuda_dispatch.cpp:121-240: CudaNotAvailable without a device, then the
// reference's validation (channels taken as 3), then the encode; the status values are equal
JpegError process_encode_cuda(const uint8_t* input, uint8_t* output, size_t* output_size, int width, int height,
                              int channels, int bit_depth, const JpegParams& params) {
    (void)channels;
    if (!has_cuda()) return JpegError::CudaNotAvailable;
    if (!t_jpeg.ctx && imop_jpeg_create(&t_jpeg.ctx) != IMOP_JPEG_OK) {
        t_jpeg.ctx = nullptr;
        return JpegError::InternalError;
    }
    const int rc = imop_jpeg_encode_host(t_jpeg.ctx, input, width, height, bit_depth, params.quality,
                                         params.chroma_subsample, output, output_size);
    if (rc == IMOP_JPEG_OK) g_served.fetch_add(1, std::memory_order_relaxed);
    return (rc >= 0 && rc <= 12) ? static_cast<JpegError>(rc) : JpegError::InternalError;
}

// src/jpeg_codec/cuda_dispatch.cpp:246-255
JpegError process_decode_cuda(const uint8_t* input, size_t input_size, uint8_t* output, int* width, int* height,
                              int* channels) {
    if (!has_cuda()) return JpegError::CudaNotAvailable;
    if (!input || !output || !width || !height || !channels) return JpegError::NullInput;
    if (input_size < 2 || input[0] != 0xFF || input[1] != 0xD8) return JpegError::InvalidJpegData;
    if (!&process_decode_baseline) return JpegError::InternalError;
    return process_decode_baseline(input, input_size, output, width, height, channels);
}

}  // namespace jpeg_codec

extern "C" long long imop_shim_calls_served(void) { return g_served.load(std::memory_order_relaxed); }

// ---- modules off this path: CPU fallback ------------------------------------------------------
namespace denoise {
bool has_cuda() { return false; }
DenoiseError process_denoise_cuda(const uint8_t*, uint8_t*, int, int, int, DenoiseAlgorithm, int, float) {
    return DenoiseError::InternalError;
}
}  // namespace denoise

namespace sharpen {
bool has_cuda() { return false; }
SharpenError process_sharpen_cuda(const uint8_t*, uint8_t*, int, int, int, SharpenAlgorithm, int, const SharpenParams&) {
    return SharpenError::InternalError;
}
}  // namespace sharpen

namespace local_contrast {
bool has_cuda() { return false; }
LocalContrastError process_local_contrast_cuda(const uint8_t*, uint8_t*, int, int, int, int, const LocalContrastParams&) {
    return LocalContrastError::InternalError;
}
}  // namespace local_contrast

namespace saturation {
bool has_cuda() { return false; }
SaturationError process_saturation_cuda(const uint8_t*, uint8_t*, int, int, int, int, float, float) {
    return SaturationError::InternalError;
}
}  // namespace saturation

namespace color_temp {
bool has_cuda() { return false; }
ColorTempError process_color_temp_cuda(const uint8_t*, uint8_t*, int, int, int, int, float, float, float) {
    return ColorTempError::InternalError;
}
}  // namespace color_temp

namespace highlight_reconstruct {
bool has_cuda() { return false; }
HighlightReconstructError process_highlight_reconstruct_cuda(const uint8_t*, uint8_t*, int, int, int,
                                                             HighlightReconstructAlgorithm, int,
                                                             const HighlightReconstructParams&) {
    return HighlightReconstructError::InternalError;
}
}  // namespace highlight_reconstruct
