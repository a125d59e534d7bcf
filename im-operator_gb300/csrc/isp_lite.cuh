// isp_lite.cuh - the fused RAW->RGB8 pipeline for chains without defect correction and lens
// shading, demosaiced by HQLI: black level, white balance (Bayer or RGB order), HQLI, tone -> RGB8
// (the chain of the reference's plain per-module composition).
//
// HQLI reads one pixel around each output, so this kernel needs no shared tile and no CTA-wide
// barrier in its main loop.  Each warp works alone on a strip of up to 256 columns (8 per lane) of
// one frame, walking down a band of rows:
//   * lane 0 stages every raw row's byte window into the warp's ring of shared-memory slots with a
//     1-D bulk copy (cp.async.bulk, completing on the slot's mbarrier), kLiteRing rows ahead and
//     across the end of one band into the next band the warp claims, so the next rows are in
//     flight while the current one is computed;
//   * each lane unpacks, black-levels and (Bayer-order) white-balances its eight samples of a row
//     once; the columns to its left and right come from the neighbouring lanes by shuffles;
//   * three rows live in registers (a sliding window), so HQLI of the middle row is integer sums;
//   * RGB-order white balance and the tone LUT fold into one shared-memory table per output
//     channel (T_c[v] = tone8[round(v * wb_c)], built once per launch: the frames of a launch share
//     their tables), so each output byte is one lookup and no float-to-int conversion (an eighth of
//     the FP32 rate on this part) is in the loop;
//   * a row's 24 bytes per lane are assembled at the output's 16-byte phase in the warp's staging
//     row and leave as 16-byte vector stores.
// The reference's RGB border copies (fill_rgb_borders, src/algorithms/common.hpp:47-96) copy
// pixels; the RGB white balance and the tone are per-pixel maps, so copying output bytes gives the
// same result.  Columns 0, 1 / w-2, w-1 of a row take the bytes of column 2 / w-3 of that row;
// rows 0, 1 / h-2, h-1 are emitted with row 2 / h-3, their corner pixels (never written by the
// reference's HQLI, so zero) mapped through the tables.
#pragma once

#include "isp_device.cuh"
#include "isp_kernels.h"
#include "isp_ptx.cuh"
#include "isp_tile.cuh"

namespace imop {

constexpr int kLiteLanePx = 8;                   // pixels per lane
constexpr int kLiteStripMax = 32 * kLiteLanePx;  // columns of a strip
constexpr int kLiteBandH = 16;                   // rows of a band (the last absorbs a remainder below 4)
constexpr int kLiteRing = 4;                     // staged rows per warp
constexpr int kLiteWarps = 8;

struct LiteWarpSmem {
    // byte window of pixels [x0 - 8, x0 + 264) of a row in the widest format (u16), its 16-byte
    // alignment slack, and readable bytes past it for the unpack's word loads
    static constexpr int RAW_PITCH = round16(2 * (kLiteStripMax + 16) + 32 + 16);
    static constexpr int OUT_PITCH = round16(3 * kLiteStripMax + 16);
    alignas(16) uint8_t raw[kLiteRing][RAW_PITCH];
    alignas(16) uint8_t out[OUT_PITCH];
    int a0[kLiteRing];   // first staged byte of each slot's row (offset in the input frame)
    int len[kLiteRing];  // staged bytes (0: a row outside the frame)
    alignas(8) uint64_t bar[kLiteRing];
};

struct LiteSmem {
    alignas(16) uint8_t tab[3][4096];  // output byte per channel and sample value
    LiteWarpSmem w[kLiteWarps];
};

// width of a frame's strips: at most 256 columns, chosen so the last strip holds at least three
// columns (the right border copies column w-3 into w-2 and w-1 of the same strip)
__host__ __device__ inline int lite_strip_w(int w) {
    if (w <= kLiteStripMax) return kLiteStripMax;
    for (int s = kLiteStripMax; s > 64; s -= 8)
        if (w % s == 0 || w % s >= 3) return s;
    return 64;
}
__host__ __device__ inline int lite_strips(int w) {
    const int s = lite_strip_w(w);
    return (w + s - 1) / s;
}
__host__ __device__ inline int lite_bands(int h) { return tiles_along(h, kLiteBandH); }

// geometry of one band of one frame's strip (a warp's unit of work)
struct LiteUnit {
    int f;        // frame index in the launch
    int x0, npx;  // first column and columns of the strip
    int y0, bh;   // first row and rows of the band
    int nrows;    // staged rows: y0 - 1 .. y0 + bh
};

namespace lite {

// bytes [o, o + 4K) of a staged row as K words, for any byte offset o
template <int K>
__device__ __forceinline__ void load_words(const uint8_t* row, int o, uint32_t (&w)[K]) {
    const uint32_t* p = reinterpret_cast<const uint32_t*>(row + (o & ~3));
    const int sh = 8 * (o & 3);
    uint32_t a = p[0];
#pragma unroll
    for (int k = 0; k < K; k++) {
        const uint32_t b = p[k + 1];
        w[k] = __funnelshift_r(a, b, sh);
        a = b;
    }
}

// eight raw samples x .. x+7 of a staged row, pixel x at byte offset o (for the MIPI formats x
// lies on a pair / group boundary); bytes per eight samples: 8, 16, 12, 10
template <int FMT>
__device__ __forceinline__ void decode8(const uint8_t* row, int o, int (&v)[8]) {
    if (FMT == FMT_U8) {
        uint32_t w[2];
        load_words(row, o, w);
#pragma unroll
        for (int k = 0; k < 8; k++) v[k] = (w[k >> 2] >> (8 * (k & 3))) & 0xFF;
    } else if (FMT == FMT_U16) {
        uint32_t w[4];
        load_words(row, o, w);
#pragma unroll
        for (int k = 0; k < 4; k++) {
            v[2 * k] = w[k] & 0xFFFF;
            v[2 * k + 1] = w[k] >> 16;
        }
    } else if (FMT == FMT_P12) {
        uint32_t w[3];
        load_words(row, o, w);
        const uint32_t g[4] = {w[0], __funnelshift_r(w[0], w[1], 24), __funnelshift_r(w[1], w[2], 16), w[2] >> 8};
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const uint32_t p = unpack12_pair(g[k]);
            v[2 * k] = p & 0xFFFF;
            v[2 * k + 1] = p >> 16;
        }
    } else {
        uint32_t w[3];
        load_words(row, o, w);
        const uint32_t lo4[2] = {w[0], __funnelshift_r(w[1], w[2], 8)};
        const uint32_t b4[2] = {w[1] & 0xFF, w[2] >> 8};
#pragma unroll
        for (int g = 0; g < 2; g++)
#pragma unroll
            for (int s = 0; s < 4; s++)
                v[4 * g + s] = (int)((((lo4[g] >> (8 * s)) & 0xFF) << 2) | ((b4[g] >> (2 * s)) & 3));
    }
}

template <int FMT>
__host__ __device__ constexpr int bytes8() {
    return FMT == FMT_U8 ? 8 : FMT == FMT_U16 ? 16 : FMT == FMT_P12 ? 12 : 10;
}

// byte offset of pixel index i (on a pair / group boundary for the MIPI formats)
template <int FMT>
__device__ __forceinline__ int byte_of(int i) {
    return FMT == FMT_U8 ? i : FMT == FMT_U16 ? 2 * i : FMT == FMT_P12 ? 3 * (i >> 1) : 5 * (i >> 2);
}

// RGB of the 8 pixels of a lane's row (m) from the rows above (u) and below (d): detail::hqli_core
// (src/algorithms/interp_core.hpp:39-65) at interior sites; index 0 / 9 hold the columns left /
// right of the lane's pixels.  RB: which pixel of each pair is the red / blue site; RR: the row is
// a red row.  The samples never exceed the bit depth's maximum here (lite_eligible), so the
// reference's clamps of the averages to that maximum are identities.
template <int RB, bool RR>
__device__ __forceinline__ void hqli8(const int (&u)[10], const int (&m)[10], const int (&d)[10], int (&R)[8],
                                      int (&G)[8], int (&B)[8]) {
#pragma unroll
    for (int p = 0; p < 8; p++) {
        const int i = p + 1;
        if ((p & 1) == RB) {
            const int own = m[i];
            const int gq = (m[i - 1] + m[i + 1] + u[i] + d[i] + 2) >> 2;
            const int oq = (u[i - 1] + u[i + 1] + d[i - 1] + d[i + 1] + 2) >> 2;
            R[p] = RR ? own : oq;
            B[p] = RR ? oq : own;
            G[p] = gq;
        } else {
            const int hz = (m[i - 1] + m[i + 1] + 1) >> 1;
            const int vt = (u[i] + d[i] + 1) >> 1;
            G[p] = m[i];
            R[p] = RR ? hz : vt;
            B[p] = RR ? vt : hz;
        }
    }
}

}  // namespace lite

}  // namespace imop
