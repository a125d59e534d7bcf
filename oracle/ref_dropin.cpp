// ref_dropin.cpp - TEST INFRASTRUCTURE ONLY.
//
// extern "C" entry points into the reference's own module dispatchers, linked (oracle/Makefile,
// target dropin) with the reference's CPU sources and with this project's libimop_isp.so in place
// of the reference's GPU glue (src/gpu_dispatch.cpp, src/algorithms/cuda_dispatch.cpp,
// src/jpeg_codec/cuda_dispatch.cpp).  Each dispatcher then calls the library's has_cuda() and
// process_*_cuda(), exactly as it would in a reference build configured with this library: on a
// host with a GPU the library serves the call, without one the dispatcher runs its CPU code.
// Nothing here copies reference code - it only calls it.

#include <cstdint>
#include <cstring>
#include <vector>

#include "algorithms/common.hpp"
#include "black_level/algorithms.hpp"
#include "ccm/algorithms.hpp"
#include "defect_correct/algorithms.hpp"
#include "imop/algorithms.hpp"
#include "lens_shading/algorithms.hpp"
#include "tone/algorithms.hpp"
#include "white_balance/algorithms.hpp"

extern "C" long long imop_shim_calls_served(void);

namespace {
// AMAZE's FloatBufferPool::get resizes the outer vector while earlier references are alive
// (src/algorithms/common.hpp:16-23 with amaze.cpp:152-154); reserving the slots once per thread
// before the first CPU call keeps those references valid
void reserve_pool() {
    thread_local bool done = false;
    if (!done) {
        imop::detail::thread_local_pool().get(1, 11);
        done = true;
    }
}
}  // namespace

extern "C" {

long long dropin_served(void) { return imop_shim_calls_served(); }

// black_level::process_black_level on the reference's storage (u8 for bd <= 8, u16 otherwise), in place
int dropin_black_level(uint8_t* data, int w, int h, int pattern, int bd, int mode, const float off[4]) {
    black_level::BlackLevelParams p;
    p.r_offset = off[0]; p.gr_offset = off[1]; p.gb_offset = off[2]; p.b_offset = off[3];
    return (int)black_level::process_black_level(data, w, h, static_cast<imop::BayerPattern>(pattern),
                                                 mode ? black_level::BlackLevelAlgorithm::GLOBAL
                                                      : black_level::BlackLevelAlgorithm::PER_CHANNEL, bd, p);
}

int dropin_defect_adaptive(uint8_t* data, int w, int h, int pattern, int bd, float threshold) {
    defect_correct::DefectCorrectParams p;
    p.threshold = threshold;
    return (int)defect_correct::process_defect_correct(data, w, h, static_cast<imop::BayerPattern>(pattern),
                                                       defect_correct::DefectCorrectAlgorithm::ADAPTIVE, bd, p);
}

// imop::demosaic (src/algorithms/dispatch.cpp:89-113), raw storage in, RGB storage out
int dropin_demosaic(const uint8_t* raw, uint8_t* rgb, int w, int h, int pattern, int algo, int bd, int packed) {
    reserve_pool();
    return (int)imop::demosaic(raw, rgb, w, h, static_cast<imop::BayerPattern>(pattern),
                               static_cast<imop::DemosaicAlgorithm>(algo), bd, packed != 0);
}

int dropin_white_balance(const uint8_t* in, uint8_t* out, int w, int h, int bd, const float g[3]) {
    white_balance::WBCoefficients c;
    c.r_gain = g[0]; c.g_gain = g[1]; c.b_gain = g[2];
    return (int)white_balance::process_white_balance(in, out, w, h, 3, white_balance::WhiteBalanceAlgorithm::MANUAL,
                                                     bd, 6.0f, c);
}

int dropin_ccm(const uint8_t* in, uint8_t* out, int w, int h, int bd, const float m[9]) {
    ccm::CCMatrix3x3 mat;
    for (int i = 0; i < 9; i++) mat.m[i] = m[i];
    return (int)ccm::process_ccm(in, out, w, h, 3, ccm::CCMAlgorithm::LINEAR_3X3, bd, &mat);
}

// p = gamma, contrast, shadows, highlights, black_point, white_point, mid_point
int dropin_tone(const uint8_t* in, uint8_t* out, int w, int h, int bd, int algo, const float p[7]) {
    tone::ToneParams tp;
    tp.gamma = p[0]; tp.contrast = p[1]; tp.shadows = p[2]; tp.highlights = p[3];
    tp.black_point = p[4]; tp.white_point = p[5]; tp.mid_point = p[6];
    return (int)tone::process_tone(in, out, w, h, 3, static_cast<tone::ToneAlgorithm>(algo), bd, tp);
}

}  // extern "C"
