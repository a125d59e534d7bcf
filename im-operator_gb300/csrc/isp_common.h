// isp_common.h - definitions shared by host and device code of the ISP hot path.
#pragma once

#include <stddef.h>
#include <stdint.h>
#include <vector_types.h>

#ifdef __CUDACC__
#define IMOP_HD __host__ __device__ __forceinline__
#else
#define IMOP_HD inline
#endif

namespace imop {

// input storage formats
enum InFormat : int {
    FMT_U8 = 0,    // 1 byte per pixel (bit depth <= 8)
    FMT_U16 = 1,   // little-endian u16 per pixel, LSB-aligned
    FMT_P10 = 2,   // MIPI RAW10: 4 pixels in 5 bytes, global pixel order, no row padding
    FMT_P12 = 3,   // MIPI RAW12: 2 pixels in 3 bytes
    FMT_PBITS = 4  // other packed depths: one LSB-first bit stream, bit_depth bits per pixel
};

// input format of a parameter set: MIPI RAW10 / RAW12, other packed depths as a bit stream
// (pixel::get_packed_raw, include/imop/pixel_utils.hpp:58-118 of the reference), else u8 / u16
IMOP_HD int input_format_of(int packed, int bd) {
    if (packed) return bd == 10 ? FMT_P10 : (bd == 12 ? FMT_P12 : FMT_PBITS);
    return bd <= 8 ? FMT_U8 : FMT_U16;
}

// demosaic kernels (values of imop::DemosaicAlgorithm)
enum Demosaic : int { DM_HQLI = 1, DM_MG = 2, DM_AMAZE = 6 };

// how the RGB borders are filled (see border_source below)
enum BorderMode : int {
    BORDER_ROWS_THEN_COLS = 0,  // fill_intermediate_borders / fill_rgb_borders once
    BORDER_BOTH = 1             // AMAZE 8-bit: intermediate fill, then fill_rgb_borders again
};

// PatternOffsets::from_pattern (include/imop/types.hpp:88-101 of the reference)
struct PatternOffsets {
    int r_row, r_col, b_row, b_col;
};
IMOP_HD PatternOffsets pattern_offsets(int pattern) {
    switch (pattern) {
        case 1: return {1, 1, 0, 0};  // BGGR
        case 2: return {0, 1, 1, 0};  // GRBG
        case 3: return {1, 0, 0, 1};  // GBRG
        default: return {0, 0, 1, 1}; // RGGB
    }
}
// colour index 0=R 1=Gr 2=Gb 3=B (src/black_level/common.hpp:29-35 of the reference)
IMOP_HD int bayer_color(int row, int col, PatternOffsets po) {
    if ((row & 1) == po.r_row && (col & 1) == po.r_col) return 0;
    if ((row & 1) == po.b_row && (col & 1) == po.b_col) return 3;
    if ((row & 1) == po.r_row) return 1;
    return 2;
}
inline int bayer_color_host(int row, int col, int pattern) {
    return bayer_color(row, col, pattern_offsets(pattern));
}
IMOP_HD int max_val_of(int bd) { return bd >= 16 ? 65535 : (1 << bd) - 1; }

IMOP_HD size_t input_bytes_of(int fmt, int bd, int w, int h) {
    size_t n = (size_t)w * (size_t)h;
    switch (fmt) {
        case FMT_U8: return n;
        case FMT_U16: return 2 * n;
        case FMT_P10: return (n * 10 + 7) / 8;
        case FMT_P12: return (n * 12 + 7) / 8;
        default: return (n * (size_t)bd + 7) / 8;
    }
}

// Device-resident parameters of one frame (expanded from ImopIspParams by the host).
struct FrameParams {
    // geometry / format
    int w, h, bd, mv;
    int fmt, pattern, demosaic, border_mode;
    unsigned stages;
    int stage_order;
    int out_format;      // 0 RGB8, 1 native
    int out_bpc;         // bytes per output channel (1 or 2)
    size_t in_bytes;     // size of the input buffer (packed tail rule)
    // black level: per CFA colour (R, Gr, Gb, B), already max(0, .)
    float bl[4];
    int bl_int;          // all offsets integral and < 65536: exact as a saturating u16 subtract
    uint32_t bl2[2];     // packed (x even, x odd) offsets for even / odd rows
    int bl_i[2][2];      // integral offsets [row parity][column parity]
    uint32_t mv2;        // (mv, mv)
    // defect correction
    int dpc_mode;        // 0 adaptive, 1 map
    int dpc_thr;         // absolute threshold
    uint32_t thr2;       // (thr, thr)
    const int* map_row_ptr;   // h+1 offsets into map_ent (map mode)
    const int2* map_ent;      // (x, value slot) per unique map pixel, sorted by row then x
    const int* map_val;       // resolved value per slot (written by the resolve kernel)
    // lens shading
    int lsc_mode;        // 0 grid, 1 polynomial
    int gw, gh;
    const float* grid;   // [gh][gw][4]
    float poly[4][3];
    float lsc_cx, lsc_cy, lsc_max_r;
    // white balance per CFA colour (Bayer order) and per RGB channel (RGB order)
    float wb_cfa[4];
    float wb_rgb[3];
    // colour correction
    float ccm[9];
    // tone: 2^bd-entry u8 table
    const uint8_t* tone8;
    // the demosaic's u16 read shifts MSB-aligned samples (no earlier stage clamped them)
    int need_align;
    // data
    const uint8_t* in;
    uint8_t* out;
    // defect-chain seeds (adaptive mode): raster indices, appended by the fused kernel
    int* seed_count;
    int* seeds;
    int seed_cap;
    int* status;         // sticky error word (IMOP_ERR_*), 0 when fine
    int* tile_counter;   // next-tile counter of the fused launch (one per launch, zeroed before it)
    unsigned long long* seg_words;  // work-claim words of the streaming kernel (seg_cap of them)
    int seg_cap;
    // defect-chain fix-up scratch of this frame (heap, sorted override list)
    int* fix_heap;
    int* fix_ov_idx;
    int* fix_ov_val;
    int* fix_n_ov;
    int fix_cap;         // entries of fix_heap / fix_ov_*
    int tiles_x, tiles_y;  // tile grid of this frame
    // -0.0f, read at run time: the addend of the packed products (see dev::pmul)
    float neg_zero;
    // optional 3D LUT after the CCM (stage bit 5): size^3 x 3 floats, R-major
    const float* lut3d;
    int lut3d_size;
    // lens-shading grid gains all finite and within [0, 15] (the streaming kernel's packed halves)
    int lsc_bounded;
};

}  // namespace imop
