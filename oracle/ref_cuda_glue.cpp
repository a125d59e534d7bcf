// ref_cuda_glue.cpp - TEST AND MEASUREMENT INFRASTRUCTURE ONLY: C entry points into the
// reference's own GPU path (its src/gpu_dispatch.cpp and src/algorithms/cuda_dispatch.cpp,
// compiled from the reference's sources by `make -C oracle refcuda`), so the timed reference arm
// can run the calls the reference's dispatchers make on a CUDA host.  Timing only: the reference's
// GPU kernels do not reproduce its CPU results (its adaptive defect kernel, for one, takes the
// relative threshold as an absolute one), so nothing compares their bytes.
//
// Served: black_level::process_black_level_cuda (src/gpu_dispatch.cpp:421-448),
// defect_correct::process_defect_correct_cuda (:529-575), imop::demosaic_cuda
// (src/algorithms/cuda_dispatch.cpp:68-141).  Not served: ccm::process_ccm_cuda and the other
// stages the reference runs through kern_gpu_pipeline, whose parameter buffer is never allocated
// on the path they take (GpuWorkspace::ensure(w, h, bd, 0), src/gpu_dispatch.cpp:322 and
// src/gpu_ops_kernels.cu:10-23), so the kernel would read through a null pointer.
#include <cstdint>

#include "black_level/algorithms.hpp"
#include "defect_correct/algorithms.hpp"
#include "imop/algorithms.hpp"

extern "C" {

__attribute__((visibility("default"))) int refcuda_has_cuda() { return imop::has_cuda() ? 1 : 0; }

__attribute__((visibility("default"))) int refcuda_black_level(uint8_t* data, int w, int h, int pattern, int bd,
                                                               const float* off4) {
    black_level::BlackLevelParams p;
    p.r_offset = off4[0];
    p.gr_offset = off4[1];
    p.gb_offset = off4[2];
    p.b_offset = off4[3];
    return (int)black_level::process_black_level_cuda(data, w, h, static_cast<imop::BayerPattern>(pattern),
                                                       black_level::BlackLevelAlgorithm::PER_CHANNEL, bd, p);
}

__attribute__((visibility("default"))) int refcuda_defect_adaptive(uint8_t* data, int w, int h, int pattern, int bd,
                                                                   float threshold) {
    defect_correct::DefectCorrectParams p;
    p.threshold = threshold;
    return (int)defect_correct::process_defect_correct_cuda(data, w, h, static_cast<imop::BayerPattern>(pattern),
                                                            defect_correct::DefectCorrectAlgorithm::ADAPTIVE, bd, p);
}

__attribute__((visibility("default"))) int refcuda_demosaic(const uint8_t* in, uint8_t* rgb, int w, int h, int pattern,
                                                            int algorithm, int bd) {
    return (int)imop::demosaic_cuda(in, rgb, w, h, static_cast<imop::BayerPattern>(pattern),
                                    static_cast<imop::DemosaicAlgorithm>(algorithm), bd, false);
}

}  // extern "C"
