// Link probe: takes the address of every GPU-glue entry point as the reference's own headers
// declare it (include/<module>/algorithms.hpp, include/imop/algorithms.hpp,
// include/jpeg_codec/algorithms.hpp), so linking this
// against libimop_isp.so proves that the library defines each symbol with the reference's
// mangled name.  Built by `make -C oracle shimlink` where the reference tree exists.
#include "denoise/algorithms.hpp"
#include "sharpen/algorithms.hpp"
#include "local_contrast/algorithms.hpp"
#include "saturation/algorithms.hpp"
#include "color_temp/algorithms.hpp"
#include "highlight_reconstruct/algorithms.hpp"
#include "black_level/algorithms.hpp"
#include "defect_correct/algorithms.hpp"
#include "lens_shading/algorithms.hpp"
#include "white_balance/algorithms.hpp"
#include "ccm/algorithms.hpp"
#include "tone/algorithms.hpp"
#include "lut/algorithms.hpp"
#include "imop/algorithms.hpp"
#include "jpeg_codec/algorithms.hpp"
void* refs[] = {
 (void*)&denoise::process_denoise_cuda, (void*)&denoise::has_cuda,
 (void*)&sharpen::process_sharpen_cuda, (void*)&sharpen::has_cuda,
 (void*)&local_contrast::process_local_contrast_cuda, (void*)&saturation::process_saturation_cuda,
 (void*)&color_temp::process_color_temp_cuda, (void*)&highlight_reconstruct::process_highlight_reconstruct_cuda,
 (void*)&black_level::process_black_level_cuda, (void*)&defect_correct::process_defect_correct_cuda,
 (void*)&lens_shading::process_lens_shading_cuda, (void*)&white_balance::process_white_balance_cuda,
 (void*)&ccm::process_ccm_cuda, (void*)&tone::process_tone_cuda, (void*)&lut::process_lut_cuda,
 (void*)&imop::demosaic_cuda, (void*)&imop::demosaic_cuda_batch, (void*)&imop::has_cuda,
 (void*)&imop::cuda_device_name, (void*)&imop::cuda_synchronize,
 (void*)&local_contrast::has_cuda, (void*)&saturation::has_cuda, (void*)&color_temp::has_cuda,
 (void*)&highlight_reconstruct::has_cuda, (void*)&black_level::has_cuda, (void*)&tone::has_cuda, (void*)&lut::has_cuda,
 (void*)&ccm::has_cuda, (void*)&white_balance::has_cuda, (void*)&lens_shading::has_cuda, (void*)&defect_correct::has_cuda,
 (void*)&jpeg_codec::process_encode_cuda, (void*)&jpeg_codec::process_decode_cuda, (void*)&jpeg_codec::has_cuda,
 (void*)&jpeg_codec::cuda_device_name, (void*)&jpeg_codec::cuda_synchronize};
int main() { return refs[0] == nullptr; }
