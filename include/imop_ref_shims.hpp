/*
 * imop_ref_shims.hpp - C++ entry points with the names, namespaces and signatures of the
 * reference's GPU glue, so that its CPU dispatchers link against this library unchanged.
 *
 * Linking libimop_isp.so in place of src/algorithms/cuda_dispatch.cpp and src/gpu_dispatch.cpp
 * of im-operator puts the GB300 path behind the reference's own dispatchers: each dispatcher
 * calls <module>::has_cuda() and then <module>::process_<module>_cuda(); a non-Ok status makes it
 * run its CPU path.  Enumerations and structures below repeat the reference's (names, enumerator
 * order, member order and types), because the mangled symbol names and the argument layouts
 * depend on them; the reference file each one follows is named beside it.  A translation unit
 * uses either these declarations or the reference's headers, not both.
 *
 * Served on the GPU: demosaic HQLI / MG / AMAZE (packed input of any depth included), black level,
 * adaptive and map-based defect correction, polynomial and flat-field lens shading, manual white
 * balance, 3x3 CCM, custom 3D LUTs, the GAMMA / S_CURVE / LEVELS / CURVES_3POINT tone curves (a
 * per-sample table of the reference's expression, mapped on the device), baseline JPEG encode.
 * tone::process_tone_cuda returns InternalError for SHADOWS_HIGHLIGHTS, whose luminance couples
 * the channels, so the reference runs that curve on its CPU; the other modules of the same glue file
 * (denoise, sharpen, local contrast, saturation, colour temperature, highlight reconstruction)
 * report no CUDA and stay on the CPU.
 */
#ifndef IMOP_REF_SHIMS_HPP
#define IMOP_REF_SHIMS_HPP

#include <cstddef>
#include <cstdint>
#include <vector>

namespace imop {
enum class BayerPattern { RGGB, BGGR, GRBG, GBRG };                                   // include/imop/types.hpp:12-17
enum class DemosaicAlgorithm { SUPER_FAST, HQLI, MG, L7, DFPD, AHD, AMAZE, RCD, PRISM };  // include/imop/types.hpp:19-29
enum class DemosaicError {                                                            // include/imop/types.hpp:31-39
    Ok = 0, NullInput, InvalidDimensions, InvalidBitDepth, InvalidPattern, ImageTooSmall, InternalError
};
// include/imop/algorithms.hpp:69-84, defined by src/algorithms/cuda_dispatch.cpp:28-209
bool has_cuda();
const char* cuda_device_name();
void cuda_synchronize();
DemosaicError demosaic_cuda(const uint8_t* bayer_data, uint8_t* rgb_data, int width, int height, BayerPattern pattern,
                            DemosaicAlgorithm algorithm, int bit_depth = 8, bool is_packed = false);
DemosaicError demosaic_cuda_batch(const uint8_t* const* bayer_data_array, uint8_t* const* rgb_data_array,
                                  int num_frames, int width, int height, BayerPattern pattern,
                                  DemosaicAlgorithm algorithm, int bit_depth = 8);
}  // namespace imop

namespace black_level {
using imop::BayerPattern;
enum class BlackLevelAlgorithm { PER_CHANNEL, GLOBAL };                               // include/black_level/types.hpp:8-11
enum class BlackLevelError {                                                          // include/black_level/types.hpp:13-21
    Ok = 0, NullInput, InvalidDimensions, InvalidBitDepth, InvalidChannels, ImageTooSmall, InternalError
};
struct BlackLevelParams {                                                             // include/black_level/types.hpp:41-46
    float r_offset = 0.0f, gr_offset = 0.0f, gb_offset = 0.0f, b_offset = 0.0f;
};
bool has_cuda();                                                                      // include/black_level/algorithms.hpp:40-46
BlackLevelError process_black_level_cuda(uint8_t* data, int width, int height, BayerPattern pattern,
                                         BlackLevelAlgorithm algorithm, int bit_depth, const BlackLevelParams& params);
}  // namespace black_level

namespace defect_correct {
using imop::BayerPattern;
enum class DefectCorrectAlgorithm { ADAPTIVE, MAP_BASED };                            // include/defect_correct/types.hpp:8-11
enum class DefectCorrectError {                                                       // include/defect_correct/types.hpp:13-21
    Ok = 0, NullInput, InvalidDimensions, InvalidBitDepth, InvalidChannels, ImageTooSmall, InternalError
};
struct DefectPoint { int x, y; };                                                     // include/defect_correct/types.hpp:41-43
struct DefectCorrectParams {                                                          // include/defect_correct/types.hpp:45-49
    float threshold = 0.3f;
    const DefectPoint* map = nullptr;
    int map_count = 0;
};
bool has_cuda();                                                                      // include/defect_correct/algorithms.hpp:40-46
DefectCorrectError process_defect_correct_cuda(uint8_t* data, int width, int height, BayerPattern pattern,
                                               DefectCorrectAlgorithm algorithm, int bit_depth,
                                               const DefectCorrectParams& params);
}  // namespace defect_correct

namespace lens_shading {
using imop::BayerPattern;
enum class LensShadingAlgorithm { POLYNOMIAL, FLAT_FIELD };                           // include/lens_shading/types.hpp:8-11
enum class LensShadingError {                                                         // include/lens_shading/types.hpp:13-21
    Ok = 0, NullInput, InvalidDimensions, InvalidBitDepth, InvalidChannels, ImageTooSmall, InternalError
};
struct ShadingPolynomial { float a2 = 0.0f, a4 = 0.0f, a6 = 0.0f; };                  // include/lens_shading/types.hpp:37-41
struct LensShadingParams {                                                            // include/lens_shading/types.hpp:43-60
    ShadingPolynomial r_coef, gr_coef, gb_coef, b_coef;
    float center_x = 0.5f, center_y = 0.5f;
    const uint8_t* flat_field = nullptr;
    int flat_field_width = 0, flat_field_height = 0;
};
bool has_cuda();                                                                      // include/lens_shading/algorithms.hpp:40-46
LensShadingError process_lens_shading_cuda(uint8_t* data, int width, int height, BayerPattern pattern,
                                           LensShadingAlgorithm algorithm, int bit_depth,
                                           const LensShadingParams& params);
}  // namespace lens_shading

namespace white_balance {
enum class WhiteBalanceError {                                                        // include/white_balance/types.hpp
    Ok = 0, NullInput, InvalidDimensions, InvalidBitDepth, InvalidChannels, ImageTooSmall, InternalError
};
bool has_cuda();                                                                      // include/white_balance/algorithms.hpp:59-62
WhiteBalanceError process_white_balance_cuda(const uint8_t* input, uint8_t* output, int width, int height, int channels,
                                             int bit_depth, float r_gain, float g_gain, float b_gain);
}  // namespace white_balance

namespace ccm {
enum class CCMError {                                                                 // include/ccm/types.hpp
    Ok = 0, NullInput, InvalidDimensions, InvalidBitDepth, InvalidChannels, ImageTooSmall, InternalError
};
bool has_cuda();                                                                      // include/ccm/algorithms.hpp:62-65
CCMError process_ccm_cuda(const uint8_t* input, uint8_t* output, int width, int height, int channels, int bit_depth,
                          const float* matrix);
}  // namespace ccm

namespace tone {
enum class ToneAlgorithm { GAMMA, S_CURVE, LEVELS, CURVES_3POINT, SHADOWS_HIGHLIGHTS };  // include/tone/types.hpp
enum class ToneError { Ok = 0, NullInput, InvalidDimensions, InvalidBitDepth, InvalidChannels, ImageTooSmall, InternalError };
struct ToneParams {                                                                   // include/tone/types.hpp:50-58
    float gamma = 1.0f, contrast = 0.0f, shadows = 0.0f, highlights = 0.0f;
    float black_point = 0.0f, white_point = 1.0f, mid_point = 0.5f;
};
bool has_cuda();                                                                      // include/tone/algorithms.hpp:47-51
ToneError process_tone_cuda(const uint8_t* input, uint8_t* output, int width, int height, int channels,
                            ToneAlgorithm algorithm, int bit_depth, const ToneParams& params);
}  // namespace tone

namespace lut {
enum class LUTError {                                                                 // include/lut/types.hpp
    Ok = 0, NullInput, InvalidDimensions, InvalidBitDepth, InvalidChannels, LUTSizeMismatch, FileNotFound,
    FileParseError, ImageTooSmall, InternalError
};
struct LUT3D {                                                                        // include/lut/types.hpp
    int size = 0;
    std::vector<float> data;
};
bool has_cuda();                                                                      // include/lut/algorithms.hpp:89-92
LUTError process_lut_cuda(const uint8_t* input, uint8_t* output, int width, int height, int channels, int bit_depth,
                          const LUT3D& lut_data);
}  // namespace lut

namespace jpeg_codec {
// the GPU glue of src/jpeg_codec/cuda_dispatch.cpp (a translation unit of its own)
enum class JpegError {                                                                // include/jpeg_codec/types.hpp:15-29
    Ok = 0, NullInput, NullOutput, InvalidDimensions, InvalidBitDepth, InvalidChannels, InvalidQuality,
    ImageTooSmall, EncodeFailed, DecodeFailed, InvalidJpegData, CudaNotAvailable, InternalError
};
struct JpegParams {                                                                   // include/jpeg_codec/types.hpp:66-71
    int quality = 90;
    bool progressive = false;
    bool optimize = true;
    int chroma_subsample = 1;
};
bool has_cuda();                                                                      // include/jpeg_codec/algorithms.hpp
const char* cuda_device_name();
void cuda_synchronize();
// The baseline encoder on the device: the bytes of process_encode_baseline for every
// subsampling (0 = 4:4:4, 1 = 4:2:0, 2 = 4:2:2).
JpegError process_encode_cuda(const uint8_t* input, uint8_t* output, size_t* output_size, int width, int height,
                              int channels, int bit_depth, const JpegParams& params);
// Checks as the reference's, then the reference's own CPU decoder when it is linked in
// (src/jpeg_codec/decode_baseline.cpp); InternalError when it is not.
JpegError process_decode_cuda(const uint8_t* input, size_t input_size, uint8_t* output, int* width, int* height,
                              int* channels);
JpegError process_decode_baseline(const uint8_t* input, size_t input_size, uint8_t* output, int* width,
                                  int* height, int* channels);
}  // namespace jpeg_codec

// Modules off this path whose GPU glue lives in the same reference translation unit
// (src/gpu_dispatch.cpp:50-415, 490-520): has_cuda() is false and the *_cuda entry returns
// InternalError, so their dispatchers run the reference's CPU code.  Parameter types that only
// appear by reference are declared opaque; the error enumerations repeat the reference's.
#define IMOP_SHIM_ERROR_ENUM(Name) \
    enum class Name { Ok = 0, NullInput, InvalidDimensions, InvalidBitDepth, InvalidChannels, ImageTooSmall, InternalError }

namespace denoise {                                                                   // include/denoise/algorithms.hpp:52-55
enum class DenoiseAlgorithm : int;
IMOP_SHIM_ERROR_ENUM(DenoiseError);
bool has_cuda();
DenoiseError process_denoise_cuda(const uint8_t* input, uint8_t* output, int width, int height, int channels,
                                  DenoiseAlgorithm algorithm, int bit_depth, float strength);
}  // namespace denoise

namespace sharpen {                                                                   // include/sharpen/algorithms.hpp:44-48
enum class SharpenAlgorithm : int;
IMOP_SHIM_ERROR_ENUM(SharpenError);
struct SharpenParams;
bool has_cuda();
SharpenError process_sharpen_cuda(const uint8_t* input, uint8_t* output, int width, int height, int channels,
                                  SharpenAlgorithm algorithm, int bit_depth, const SharpenParams& params);
}  // namespace sharpen

namespace local_contrast {                                                            // include/local_contrast/algorithms.hpp:32-35
IMOP_SHIM_ERROR_ENUM(LocalContrastError);
struct LocalContrastParams;
bool has_cuda();
LocalContrastError process_local_contrast_cuda(const uint8_t* input, uint8_t* output, int width, int height,
                                               int channels, int bit_depth, const LocalContrastParams& params);
}  // namespace local_contrast

namespace saturation {                                                                // include/saturation/algorithms.hpp:44-47
IMOP_SHIM_ERROR_ENUM(SaturationError);
bool has_cuda();
SaturationError process_saturation_cuda(const uint8_t* input, uint8_t* output, int width, int height, int channels,
                                        int bit_depth, float sat, float vib);
}  // namespace saturation

namespace color_temp {                                                                // include/color_temp/algorithms.hpp:75-78
IMOP_SHIM_ERROR_ENUM(ColorTempError);
bool has_cuda();
ColorTempError process_color_temp_cuda(const uint8_t* input, uint8_t* output, int width, int height, int channels,
                                       int bit_depth, float r_mult, float g_mult, float b_mult);
}  // namespace color_temp

namespace highlight_reconstruct {                                                     // include/highlight_reconstruct/algorithms.hpp:35-40
enum class HighlightReconstructAlgorithm : int;
IMOP_SHIM_ERROR_ENUM(HighlightReconstructError);
struct HighlightReconstructParams;
bool has_cuda();
HighlightReconstructError process_highlight_reconstruct_cuda(const uint8_t* input, uint8_t* output, int width,
                                                             int height, int channels,
                                                             HighlightReconstructAlgorithm algorithm, int bit_depth,
                                                             const HighlightReconstructParams& params);
}  // namespace highlight_reconstruct

#undef IMOP_SHIM_ERROR_ENUM

#endif  /* IMOP_REF_SHIMS_HPP */
