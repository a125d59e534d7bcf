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
constexpr int kLiteBandH = 16;                   // default rows of a band (the last absorbs a remainder below 4)
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

// A row of a lane as packed u16 pairs: P[j] = pixel 2j | pixel 2j+1 << 16 (j = 0..3), Lw = the
// column left of the lane << 16, R = the column right of it.  Samples are at most 4095 (bit depth
// <= 12), so sums of up to four of them never carry from one half-word into the other.
struct Row {
    uint32_t P[4];
    uint32_t Lw, R;
};

// byte k of word w replaced by byte 0 of t
__device__ __forceinline__ uint32_t put_byte(uint32_t w, uint32_t t, int k) {
    return __byte_perm(w, t, k == 0 ? 0x3214 : k == 1 ? 0x3240 : k == 2 ? 0x3410 : 0x4210);
}

// HQLI (detail::hqli_core, src/algorithms/interp_core.hpp:39-65) of the lane's 8 pixels of row m
// from rows u and d, two pixels per 32-bit operation, each output through its channel's table
// (tab[c][v]) into 24 bytes (ob, pixel-interleaved RGB).  RB: the pixel of each pair at the red /
// blue site (0 even, 1 odd); RR: the row holds red sites.  Per pair j (pixels 2j, 2j+1):
//   Hp = horizontal neighbour sums (m[p-1] + m[p+1]) of both pixels    = Me[j] + Me[j+1]
//   Vp = vertical sums (u[p] + d[p])                                  = U[j] + D[j]
//   Dg = diagonal sums (u + d at p-1 plus at p+1)                      = Ve[j] + Ve[j+1]
// where Me / Ve are the rows shifted by one pixel (pairs 2j-1, 2j).  A red / blue site takes
// (Hp + Vp + 2) >> 2 for green and (Dg + 2) >> 2 for the other colour; a green site
// (Hp + 1) >> 1 and (Vp + 1) >> 1 for the horizontal / vertical colour.  The samples never exceed
// the bit depth's maximum (lite_eligible), so the reference's clamps of these averages are
// identities.
template <int RB, bool RR>
__device__ __forceinline__ void hqli_row(const Row& u, const Row& m, const Row& d, const uint8_t (*tab)[4096],
                                         uint32_t (&ob)[6]) {
    uint32_t VN[4];
#pragma unroll
    for (int j = 0; j < 4; j++) VN[j] = u.P[j] + d.P[j];
    const uint32_t VL = u.Lw + d.Lw, VR = u.R + d.R;
    const uint32_t vs[6] = {VL, VN[0], VN[1], VN[2], VN[3], VR};
    const uint32_t ms[6] = {m.Lw, m.P[0], m.P[1], m.P[2], m.P[3], m.R};
    uint32_t Ve[5], Me[5];
#pragma unroll
    for (int j = 0; j < 5; j++) {
        Ve[j] = __funnelshift_r(vs[j], vs[j + 1], 16);
        Me[j] = __funnelshift_r(ms[j], ms[j + 1], 16);
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const uint32_t Hp = Me[j] + Me[j + 1], Dg = Ve[j] + Ve[j + 1], Vp = VN[j], Own = m.P[j];
        uint32_t gq, hz, vt, oq, own, g;
        if (RB == 0) {
            const uint32_t X = Hp + (Vp & 0xFFFFu) + 0x00010002u;
            gq = (X & 0xFFFFu) >> 2;
            hz = X >> 17;
            vt = (Vp + 0x10000u) >> 17;
            oq = ((Dg + 2u) & 0xFFFFu) >> 2;
            own = Own & 0xFFFFu;
            g = Own >> 16;
        } else {
            const uint32_t X = Hp + (Vp & 0xFFFF0000u) + 0x00020001u;
            hz = (X & 0xFFFFu) >> 1;
            gq = X >> 18;
            vt = ((Vp + 1u) & 0xFFFFu) >> 1;
            oq = (Dg + 0x20000u) >> 18;
            own = Own >> 16;
            g = Own & 0xFFFFu;
        }
        // the red / blue site and the green site of the pair
        const uint32_t rs_r = RR ? own : oq, rs_b = RR ? oq : own;
        const uint32_t gs_r = RR ? hz : vt, gs_b = RR ? vt : hz;
        const uint32_t r0 = RB == 0 ? rs_r : gs_r, g0 = RB == 0 ? gq : g, b0 = RB == 0 ? rs_b : gs_b;
        const uint32_t r1 = RB == 0 ? gs_r : rs_r, g1 = RB == 0 ? g : gq, b1 = RB == 0 ? gs_b : rs_b;
        const uint32_t t[6] = {tab[0][r0], tab[1][g0], tab[2][b0], tab[0][r1], tab[1][g1], tab[2][b1]};
#pragma unroll
        for (int c = 0; c < 6; c++) {
            const int n = 6 * j + c;
            ob[n >> 2] = (n & 3) == 0 ? t[c] : put_byte(ob[n >> 2], t[c], n & 3);
        }
    }
}

// The output tables replicated per rounding, for HQLI on the packed sums without the shifts:
// t1[c][v] is the output byte of channel c for sample value v, t2[c][k] = t1[c][k >> 1] and
// t4[c][k] = t1[c][k >> 2], so a half or quarter sum indexes t2 / t4 directly and the rounding
// constant (+1 / +2) is part of the load's address.
template <int N>  // entries of t1 per channel (the samples' range)
struct LiteTables {
    alignas(16) uint8_t t1[3][4096];
    alignas(16) uint8_t t2[3][2 * N];
    alignas(16) uint8_t t4[3][4 * N];
};

// hqli_row through the replicated tables: per pair j, S = Hp + Vp holds the red / blue site's four
// neighbours in the site's half, Dg its diagonals, Hp and Vp the green site's horizontal and
// vertical pairs in the other half (no half of a sum of four 12-bit samples carries into the
// other).  Same bytes as hqli_row, with fewer integer-pipe instructions.
template <int RB, bool RR, int N>
__device__ __forceinline__ void hqli_row_t(const Row& u, const Row& m, const Row& d, const LiteTables<N>& T,
                                           uint32_t (&ob)[6]) {
    uint32_t VN[4];
#pragma unroll
    for (int j = 0; j < 4; j++) VN[j] = u.P[j] + d.P[j];
    const uint32_t VL = u.Lw + d.Lw, VR = u.R + d.R;
    const uint32_t vs[6] = {VL, VN[0], VN[1], VN[2], VN[3], VR};
    const uint32_t ms[6] = {m.Lw, m.P[0], m.P[1], m.P[2], m.P[3], m.R};
    uint32_t Ve[5], Me[5];
#pragma unroll
    for (int j = 0; j < 5; j++) {
        Ve[j] = __funnelshift_r(vs[j], vs[j + 1], 16);
        Me[j] = __funnelshift_r(ms[j], ms[j + 1], 16);
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const uint32_t Hp = Me[j] + Me[j + 1], Dg = Ve[j] + Ve[j + 1], Vp = VN[j], Own = m.P[j];
        const uint32_t S = Hp + Vp;
        // the site's half (RB 0: low, 1: high) and the green site's half
        const uint32_t i_q = RB == 0 ? (S & 0xFFFFu) : (S >> 16);    // four neighbours: green at the site
        const uint32_t i_d = RB == 0 ? (Dg & 0xFFFFu) : (Dg >> 16);  // four diagonals: the other colour
        const uint32_t i_h = RB == 0 ? (Hp >> 16) : (Hp & 0xFFFFu);  // horizontal pair at the green site
        const uint32_t i_v = RB == 0 ? (Vp >> 16) : (Vp & 0xFFFFu);  // vertical pair at the green site
        const uint32_t own = RB == 0 ? (Own & 0xFFFFu) : (Own >> 16);
        const uint32_t g = RB == 0 ? (Own >> 16) : (Own & 0xFFFFu);
        // the red / blue site: its own colour, green, the other colour
        const uint32_t s_r = RR ? T.t1[0][own] : T.t4[0][i_d + 2];
        const uint32_t s_g = T.t4[1][i_q + 2];
        const uint32_t s_b = RR ? T.t4[2][i_d + 2] : T.t1[2][own];
        // the green site: the row's colour horizontally, the other vertically
        const uint32_t g_r = RR ? T.t2[0][i_h + 1] : T.t2[0][i_v + 1];
        const uint32_t g_g = T.t1[1][g];
        const uint32_t g_b = RR ? T.t2[2][i_v + 1] : T.t2[2][i_h + 1];
        const uint32_t t[6] = {RB == 0 ? s_r : g_r, RB == 0 ? s_g : g_g, RB == 0 ? s_b : g_b,
                               RB == 0 ? g_r : s_r, RB == 0 ? g_g : s_g, RB == 0 ? g_b : s_b};
#pragma unroll
        for (int c = 0; c < 6; c++) {
            const int n = 6 * j + c;
            ob[n >> 2] = (n & 3) == 0 ? t[c] : put_byte(ob[n >> 2], t[c], n & 3);
        }
    }
}

}  // namespace lite

}  // namespace imop
