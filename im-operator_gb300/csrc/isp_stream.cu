// isp_stream.cu - the warp-streamed fused kernel for the AMAZE chains: unpack, black level,
// adaptive defect correction, lens shading (grid), Bayer-order white balance, AMAZE, CCM and tone
// -> RGB8, for the interior of each frame (the border rows and columns, where the reference's
// stages take their edge rules, go to the tile kernel as rectangles of the same batch).
//
// Each warp works alone on a strip of 256 columns (8 per lane, as packed u16 pairs) of one frame
// and walks down a band of rows.  The stages are row recurrences with short vertical reach, so a
// warp keeps each intermediate row once, in small per-warp rings of shared memory, and reads every
// row it needs back from them instead of re-staging a 2-D apron per tile:
//   input row n    -> orig ring      (unpack + black level)
//   bay row n-2    -> jac, bay rings (3x3 same-colour min / max test, the median only where it
//                                     fails; lens shading; white balance)
//   green row n-4  -> cd ring        (AMAZE green at the red / blue site of each pair, and the
//                                     colour difference there)
//   output row n-5                   (colour differences, CCM, tone, 24-byte stores per lane)
// Neighbouring columns across lanes come by shuffles; lanes 0 and 31 only feed their neighbours,
// so a strip emits 240 columns.  Raw rows are read by plain coalesced word loads one row ahead:
// no lane stages for the others and nothing waits on a barrier.
//
// Integer stages run on both samples of a pair at once (samples are at most 4095, so sums and
// biased differences never carry across the halves).  Floating-point stages run as f32x2 pairs
// with the reference's roundings; the float -> integer conversions are one round-toward-zero
// add of 1.5 * 2^23 (the low bits of the sum are floor(x)) instead of a conversion instruction,
// and int -> float conversions place the sample under the exponent of 2^23 and subtract it.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "imop_isp.h"
#include "isp_device.cuh"
#include "isp_fused_kernel.cuh"
#include "isp_kernels.h"
#include "isp_rows.cuh"
#include "isp_segments.cuh"
#include "isp_tile.cuh"

namespace imop {
namespace {

constexpr int kStLanePx = 8;
constexpr int kStWin = 32 * kStLanePx;          // window columns of a strip
constexpr int kStOut = kStWin - 2 * kStLanePx;  // output columns of a strip (lanes 1..30)
constexpr int kStWarps = 12;  // one CTA per SM: every SM streams the same number of units
constexpr int kStThreads = 32 * kStWarps;
constexpr int kMaxDev = 64;

struct StreamWarpSmem {
    uint4 orig[5][32];        // black-levelled samples, packed pairs, [row mod 5][lane]
    uint4 jac[3][32];         // defect-corrected samples (Jacobi), [row mod 3][lane]
    uint4 bay[5][32];         // samples after lens shading and white balance, [row mod 5][lane]
    float4 cd[3][32];         // colour difference at the red / blue site of each pair, [row mod 3][lane]
    float cde[3][32];         // the neighbouring lane's colour difference each row needs
    float4 lsc[2][4][2][32];  // [row parity][pair][0: (A0, A1, B0, B1), 1: (C0, C1, D0, D1)][lane]
};
struct StreamSmem {
    alignas(16) uint8_t tone[4096];
    StreamWarpSmem w[kStWarps];
};

// Work claiming (isp_segments.cuh): a segment of a strip, its output columns and rows
struct SSeg {
    int f;
    int xw;        // first window column (output columns start 8 later)
    int ox0, ox1;  // output columns
    int s0, len;   // output rows of the segment
    int nb;        // bands
};

__device__ __forceinline__ void seg_of(const BatchLaunch& bl, int seg, SSeg& G) {
    const int r = item_rect(bl, seg);
    const TileRect& R = bl.rects[r];
    const int t = seg - bl.rect_start[r];
    const int ty = t / R.tiles_x, tx = t - ty * R.tiles_x;
    G.f = R.frame;
    G.ox0 = R.x0 + kStOut * tx;
    G.ox1 = min(G.ox0 + kStOut, R.x0 + R.w);
    G.xw = G.ox0 - kStLanePx;
    segs::split_rows(R.y0, R.h, R.tiles_y, ty, G.s0, G.len);
    G.nb = max(1, (G.len + bl.band_h - 1) / bl.band_h);
}
__device__ __forceinline__ void band_rows(const SSeg& G, int i, int& y0, int& bh) {
    segs::band_of(G.s0, G.len, G.nb, i, y0, bh);
}

// ---- packed helpers ------------------------------------------------------------------------
constexpr uint32_t kExp23 = 0x4B000000u;  // bits of 2^23
constexpr float kTwo23 = 8388608.0f;
constexpr float kMagic = 12582912.0f;     // 1.5 * 2^23: x + kMagic rounded toward zero holds floor(x)
constexpr uint32_t kMagicBits = 0x4B400000u;

__device__ __forceinline__ float2 fadd2_rz(float2 a, float2 b) {
    unsigned long long x = *reinterpret_cast<unsigned long long*>(&a), y = *reinterpret_cast<unsigned long long*>(&b), r;
    asm("add.rz.f32x2 %0, %1, %2;" : "=l"(r) : "l"(x), "l"(y));
    return *reinterpret_cast<float2*>(&r);
}
// 2^23 + the low (H = 0) or high (H = 1) half of w, as float bits
template <int H>
__device__ __forceinline__ float half_biased(uint32_t w) {
    return __uint_as_float(__byte_perm(w, kExp23, H ? 0x7432 : 0x7410));
}
// both halves of w as exact floats
__device__ __forceinline__ float2 halves_f2(uint32_t w) {
    return dev::fadd2(make_float2(half_biased<0>(w), half_biased<1>(w)), make_float2(-kTwo23, -kTwo23));
}
// low 16 bits of the float bits of each component, packed (lo = a)
__device__ __forceinline__ uint32_t low_halves(float2 s) {
    return __byte_perm(__float_as_uint(s.x), __float_as_uint(s.y), 0x5410);
}
// min(trunc(t), mv) of both components for 0 <= t < 65536 (the (int)(v * g + 0.5f) stages)
__device__ __forceinline__ uint32_t trunc_pack_u(float2 t, uint32_t mv2) {
    return __vimin3_u16x2(low_halves(fadd2_rz(t, make_float2(kMagic, kMagic))), mv2, mv2);
}
// clamp(floor(t), 0, mv) of both components for |t| < 32768: C's (int) cast followed by a clamp
// at 0 agrees with it (truncation and floor differ only below 0)
__device__ __forceinline__ uint32_t floor_pack_s(float2 t, uint32_t mv2) {
    return __viaddmin_s16x2_relu(low_halves(fadd2_rz(t, make_float2(kMagic, kMagic))), 0u, mv2);
}
// round_plane of both components: clamp((int)(v + 0.5f), 0, mv)
__device__ __forceinline__ uint32_t round_pack(float2 v, uint32_t mv2) {
    return floor_pack_s(dev::fadd2(v, make_float2(0.5f, 0.5f)), mv2);
}

// ---- defect correction: the median of the flagged samples, and defect-chain seeds --------------
// Jacobi value of every flagged sample of the lane (fl: bit i = pixel i), from the orig ring
// rows b-2, b, b+2 (slots o0, o2, o4); the window's outer two columns never take the median (their
// values feed no output)
__device__ __noinline__ uint4 jacobi_slow(const StreamWarpSmem& ws, int o0, int o2, int o4, uint4 J, unsigned fl,
                                         int lane, int thr) {
    const uint16_t* r0 = reinterpret_cast<const uint16_t*>(&ws.orig[o0][0]);
    const uint16_t* r2 = reinterpret_cast<const uint16_t*>(&ws.orig[o2][0]);
    const uint16_t* r4 = reinterpret_cast<const uint16_t*>(&ws.orig[o4][0]);
    uint32_t Jw[4] = {J.x, J.y, J.z, J.w};
#pragma unroll 1
    for (; fl; fl &= fl - 1) {
        const int i = __ffs(fl) - 1;
        const int x = kStLanePx * lane + i;
        if (x < 2 || x >= kStWin - 2) continue;
        const int nb[8] = {r0[x - 2], r0[x], r0[x + 2], r2[x - 2], r2[x + 2], r4[x - 2], r4[x], r4[x + 2]};
        const uint32_t v = (uint32_t)dev::dpc_apply(r2[x], nb, 0xFFu, thr);
#pragma unroll
        for (int j = 0; j < 4; j++)
            if ((i >> 1) == j) Jw[j] = (i & 1) ? ((Jw[j] & 0xFFFFu) | (v << 16)) : ((Jw[j] & 0xFFFF0000u) | v);
    }
    return make_uint4(Jw[0], Jw[1], Jw[2], Jw[3]);
}

// Seeds among the lane's own pixels of row b (the tile kernel's test): a pixel whose raster-earlier
// neighbours (x-2, b-2), (x, b-2), (x+2, b-2), (x-2, b) include a corrected one, and whose value
// re-evaluated against those corrections differs from its Jacobi value.  Rings: jac rows b-2 / b
// (j0, j2), orig rows b-2, b, b+2 (o0, o2, o4).
__device__ __noinline__ void seeds_slow(const StreamWarpSmem& ws, const FrameParams& fp, int o0, int o2, int o4,
                                       int j0, int j2, int lane, int xl, int y) {
    const uint16_t* r0 = reinterpret_cast<const uint16_t*>(&ws.orig[o0][0]);
    const uint16_t* r2 = reinterpret_cast<const uint16_t*>(&ws.orig[o2][0]);
    const uint16_t* r4 = reinterpret_cast<const uint16_t*>(&ws.orig[o4][0]);
    const uint16_t* q0 = reinterpret_cast<const uint16_t*>(&ws.jac[j0][0]);
    const uint16_t* q2 = reinterpret_cast<const uint16_t*>(&ws.jac[j2][0]);
#pragma unroll 1
    for (int i = 0; i < kStLanePx; i++) {
        const int x = kStLanePx * lane + i;
        const bool cand = q0[x - 2] != r0[x - 2] || q0[x] != r0[x] || q0[x + 2] != r0[x + 2] || q2[x - 2] != r2[x - 2];
        if (!cand) continue;
        const int nb[8] = {q0[x - 2], q0[x], q0[x + 2], q2[x - 2], r2[x + 2], r4[x - 2], r4[x], r4[x + 2]};
        if (dev::dpc_apply(r2[x], nb, 0xFFu, fp.dpc_thr) != (int)q2[x]) {
            const int slot = atomicAdd(fp.seed_count, 1);
            if (slot < fp.seed_cap) fp.seeds[slot] = y * fp.w + xl + i;
            else atomicExch(fp.status, 104 /* IMOP_ERR_CAPACITY */);
        }
    }
}

// ---- lens shading: the per-column terms of the bilinear gain for one cell row ---------------
// (src/lens_shading/flat_field.cpp:84-105: gain = ((g00*ofx*ofy + g10*fx*ofy) + g01*ofx*fy) +
// g11*fx*fy, products left to right); A = g00*ofx, B = g10*fx, C = g01*ofx, D = g11*fx for the
// lane's 8 columns and both row parities (the colour of a sample depends on the row parity)
__device__ __noinline__ void lsc_table(StreamWarpSmem& ws, const FrameParams& fp, int gy, int xw, int lane,
                                       PatternOffsets po) {
    const int W = fp.w, gw = fp.gw;
#pragma unroll 1
    for (int j = 0; j < 4; j++) {
        int gx[2];
        float fx[2], ofx[2];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int x = min(max(xw + kStLanePx * lane + 2 * j + h, 0), W - 1);
            const float gx_f = __fdiv_rn(dev::fmul((float)x, (float)(gw - 1)), (float)(W - 1));
            gx[h] = dev::clampi(dev::ftoi(gx_f), 0, gw - 2);
            fx[h] = dev::fsub(gx_f, (float)gx[h]);
            ofx[h] = dev::fsub(1.0f, fx[h]);
        }
#pragma unroll
        for (int par = 0; par < 2; par++) {
            float A[2], B[2], C[2], D[2];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int c = bayer_color(par, h, po);
                const float* g0 = fp.grid + (gy * gw + gx[h]) * 4 + c;
                const float* g1 = g0 + 4 * gw;
                A[h] = dev::fmul(__ldg(g0), ofx[h]);
                B[h] = dev::fmul(__ldg(g0 + 4), fx[h]);
                C[h] = dev::fmul(__ldg(g1), ofx[h]);
                D[h] = dev::fmul(__ldg(g1 + 4), fx[h]);
            }
            ws.lsc[par][j][0][lane] = make_float4(A[0], A[1], B[0], B[1]);
            ws.lsc[par][j][1][lane] = make_float4(C[0], C[1], D[0], D[1]);
        }
    }
}

// ---- AMAZE green at the red / blue site of each pair of row g, and the colour difference there --
// (src/algorithms/amaze.cpp:166-180; gradients and sums as (horizontal, vertical) halves of one
// word, biased by 0x4000 per half so no half goes negative).  m2, m1, c0, p1, p2: bay rows g-2 .. g+2;
// L / R: the pairs left and right of the lane in row g.  RBH: the half at the red / blue site.
template <int RBH>
__device__ __forceinline__ void green_row(const uint32_t (&m2)[4], const uint32_t (&m1)[4], const uint32_t (&c0)[4],
                                          const uint32_t (&p1)[4], const uint32_t (&p2)[4], uint32_t L, uint32_t R,
                                          float2 z2, float (&green)[4], float (&cd)[4]) {
    const uint32_t bias = 0x40004000u;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const uint32_t cm = j > 0 ? c0[j - 1] : L, cc = c0[j], cp = j < 3 ? c0[j + 1] : R;
        uint32_t A1, B1, A2, B2, C;
        if (RBH == 0) {
            A1 = __byte_perm(cm, m1[j], 0x5432);  // (x-1 of row g, x of row g-1)
            B1 = __byte_perm(cc, p1[j], 0x5432);  // (x+1, x of row g+1)
            A2 = __byte_perm(cm, m2[j], 0x5410);  // (x-2, x of row g-2)
            B2 = __byte_perm(cp, p2[j], 0x5410);  // (x+2, x of row g+2)
            C = __byte_perm(cc, 0u, 0x1010);
        } else {
            A1 = __byte_perm(cc, m1[j], 0x7610);
            B1 = __byte_perm(cp, p1[j], 0x7610);
            A2 = __byte_perm(cm, m2[j], 0x7632);
            B2 = __byte_perm(cp, p2[j], 0x7632);
            C = __byte_perm(cc, 0u, 0x3232);
        }
        const uint32_t S2n = bias - A2 - B2;             // 0x4000 - (m2 + p2)
        const uint32_t X = C + C + S2n;                  // 0x4000 + lap, lap = 2c - m2 - p2
        const uint32_t Xn = 0x80008000u - X;             // 0x4000 - lap
        const uint32_t Ml = __vimax3_u16x2(X, Xn, X);    // 0x4000 + |lap|
        const uint32_t E = A1 - B1 + bias, En = B1 - A1 + bias;
        const uint32_t Md = __vimax3_u16x2(E, En, E);    // 0x4000 + |m1 - p1|
        const uint32_t G1 = Ml + Md + 0x80008001u;       // 1 + gradient
        const uint32_t T = A1 + B1;
        const uint32_t Gs = T + T + X;                   // 0x4000 + 2 (m1 + p1) + lap
        const float2 f1 = halves_f2(G1);                 // (1 + gH, 1 + gV)
        const float2 y0 = make_float2(dev::rcp_estimate(f1.x), dev::rcp_estimate(f1.y));
        const float2 e = dev::fma2(make_float2(-f1.x, -f1.y), y0, make_float2(1.0f, 1.0f));
        const float2 wt = dev::fma2(e, y0, y0);          // 1 / (1 + g), correctly rounded
        const float2 w = dev::weight_quotients(wt.x, wt.y, z2);
        const float2 gs = dev::fadd2(make_float2(half_biased<0>(Gs), half_biased<1>(Gs)),
                                     make_float2(-(kTwo23 + 16384.0f), -(kTwo23 + 16384.0f)));
        const float2 p = dev::pmul(w, gs, z2);
        const float g = dev::fmul(dev::fadd(p.x, p.y), 0.25f);
        green[j] = g;
        const float cf = dev::fsub(half_biased<RBH>(cc), kTwo23);
        cd[j] = dev::fsub(cf, g);
    }
}

// ---- output row q: AMAZE colour differences (src/algorithms/common.hpp:142-199), CCM, tone ------
// cdm / cdc / cdp: colour differences of rows q-1, q, q+1 with the neighbouring lane's value each
// needs (em / ec / ep: pair -1 or 4); gq: green of row q; bq: bay row q.  RBH: the half at the red /
// blue site; rrow: the row holds red sites (a row of blue sites is the same with R and B swapped).
template <int RBH>
__device__ __forceinline__ void out_row(bool rrow, const float (&cdm)[4], float em, const float (&cdc)[4], float ec,
                                        const float (&cdp)[4], float ep, const float (&gq)[4], const uint32_t (&bq)[4],
                                        const float (&m)[9], bool ccm_on, int mv, uint32_t mv2, float2 z2,
                                        const uint8_t* tone, uint32_t (&ob)[6]) {
    // neighbour pairs: diagonals of rows q +- 1 at pairs j+pa, j+pa+1; horizontals of row q at j+pl, j+pl+1
    auto at = [&](const float (&r)[4], float e, int i) -> float { return i < 0 ? e : (i > 3 ? e : r[i]); };
    constexpr int pa = RBH ? 0 : -1, pl = RBH ? -1 : 0;
    const float2 h5 = make_float2(0.5f, 0.5f);
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const float c00 = at(cdm, em, j + pa), c01 = at(cdm, em, j + pa + 1);
        const float c10 = at(cdp, ep, j + pa), c11 = at(cdp, ep, j + pa + 1);
        const float sum = dev::fadd(dev::fadd(dev::fadd(c00, c01), c10), c11);
        const float other = __fmaf_rn(sum, 0.25f, gq[j]);  // x * 0.25 is exact: one rounding, like the add
        const float fgg = dev::fsub(half_biased<1 - RBH>(bq[j]), kTwo23);
        const float2 hv = dev::fadd2(make_float2(at(cdc, ec, j + pl), cdm[j]), make_float2(at(cdc, ec, j + pl + 1), cdp[j]));
        const float2 rb2 = dev::fma2(hv, h5, make_float2(fgg, fgg));
        const uint32_t W1 = round_pack(make_float2(other, gq[j]), mv2);  // (other colour, green) at the R/B site
        const uint32_t W2 = round_pack(rb2, mv2);                           // (horizontal, vertical) at the G site
        // sources of R, G, B of both pixels, (word, half), in a row of red sites: R/B site R = own,
        // G = green, B = other; G site R = horizontal, G = own, B = vertical
        const uint32_t wb = bq[j];
        uint32_t Rw, Gw, Bw;  // (pixel 0, pixel 1) per channel
        const uint32_t rs_r = wb, rs_b = W1;  // word holding R / B at the R/B site
        const int rs_rh = RBH, rs_bh = 0;     // its half
        const int gs_rh = 0, gs_bh = 1;       // halves of W2 holding R / B at the G site
        // pixel 0 is the R/B site when RBH == 0
        auto sel = [&](uint32_t w0, int h0, uint32_t w1, int h1) -> uint32_t {
            // (half h0 of w0) | (half h1 of w1) << 16
            return __byte_perm(w0, w1, (h0 ? 0x0032 : 0x0010) | (h1 ? 0x7600 : 0x5400));
        };
        if (RBH == 0) {
            Rw = sel(rs_r, rs_rh, W2, gs_rh);
            Gw = sel(W1, 1, wb, 1);
            Bw = sel(rs_b, rs_bh, W2, gs_bh);
        } else {
            Rw = sel(W2, gs_rh, rs_r, rs_rh);
            Gw = sel(wb, 0, W1, 1);
            Bw = sel(W2, gs_bh, rs_b, rs_bh);
        }
        if (!rrow) {
            const uint32_t t = Rw;
            Rw = Bw;
            Bw = t;
        }
        uint32_t i0[3], i1[3];  // tone indices of pixels 0 and 1, per channel
        if (ccm_on) {
            const float2 rr = halves_f2(Rw), gg = halves_f2(Gw), bb = halves_f2(Bw);
            auto M = [&](int k) { return make_float2(m[k], m[k]); };
            // ((m0*r + m1*g) + m2*b) + 0.5, each product rounded on its own (src/ccm/ccm.cpp order)
            const float2 ro = dev::fadd2(dev::fadd2(dev::fadd2(dev::pmul(M(0), rr, z2), dev::pmul(M(1), gg, z2)),
                                                    dev::pmul(M(2), bb, z2)), h5);
            const float2 go = dev::fadd2(dev::fadd2(dev::fadd2(dev::pmul(M(3), rr, z2), dev::pmul(M(4), gg, z2)),
                                                    dev::pmul(M(5), bb, z2)), h5);
            const float2 bo = dev::fadd2(dev::fadd2(dev::fadd2(dev::pmul(M(6), rr, z2), dev::pmul(M(7), gg, z2)),
                                                    dev::pmul(M(8), bb, z2)), h5);
            // clamp((int)t, 0, mv) straight from the bits of t + 1.5 * 2^23 (floor(t) above their
            // bias; C's truncation differs from floor only below 0, where both clamp to 0)
            const float2 o[3] = {ro, go, bo};
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const float2 f = fadd2_rz(o[c], make_float2(kMagic, kMagic));
                i0[c] = (uint32_t)__viaddmin_s32_relu((int)__float_as_uint(f.x), -(int)kMagicBits, mv);
                i1[c] = (uint32_t)__viaddmin_s32_relu((int)__float_as_uint(f.y), -(int)kMagicBits, mv);
            }
        } else {
            const uint32_t w[3] = {Rw, Gw, Bw};
#pragma unroll
            for (int c = 0; c < 3; c++) {
                i0[c] = w[c] & 0xFFFFu;
                i1[c] = w[c] >> 16;
            }
        }
        const uint32_t t0 = tone[i0[0]], t1 = tone[i0[1]], t2 = tone[i0[2]];
        const uint32_t t3 = tone[i1[0]], t4 = tone[i1[1]], t5 = tone[i1[2]];
        // bytes 6j .. 6j+5 of the lane's 24
        const uint32_t lo = t0 | (t1 << 8) | (t2 << 16) | (t3 << 24), hi = t4 | (t5 << 8);
        if ((j & 1) == 0) {
            ob[3 * (j >> 1)] = lo;
            ob[3 * (j >> 1) + 1] = hi;
        } else {
            ob[3 * (j >> 1) + 1] |= lo << 16;
            ob[3 * (j >> 1) + 2] = (lo >> 16) | (hi << 16);
        }
    }
}

__device__ __forceinline__ int mod5(int v) { return v >= 5 ? v - 5 : v; }
__device__ __forceinline__ int mod3(int v) { return v >= 3 ? v - 3 : v; }

// Streams band (y0, bh) of segment G; own: the segment's word when this warp owns it, so that it
// continues with the segment's next bands while it gets them.  CHAIN: every frame of the launch
// runs all five stages (black level, adaptive defect correction, grid shading, Bayer white
// balance, CCM), fixed at compile time; 0: each frame's own stage set.
template <int FMT, int CHAIN>
__device__ __forceinline__ void stream_unit(const BatchLaunch& bl, const StreamSmem& sm, StreamWarpSmem& ws,
                                            const SSeg& U, int y0, int bh, unsigned long long* own, int lane) {
    const unsigned full = 0xffffffffu;
    // the frame's parameters in registers for the unit (the parameter block is read through an
    // indexed constant bank)
    const FrameParams& fp = bl.frames[U.f];
    const int W = fp.w, H = fp.h, mv = fp.mv;
    const unsigned stages = fp.stages;
    const bool bl_on = CHAIN || (stages & 1u) != 0, dpc_on = CHAIN || (stages & 2u) != 0,
               lsc_on = CHAIN || (stages & 4u) != 0, wb_on = CHAIN || (stages & 8u) != 0,
               ccm_on = CHAIN || (stages & 16u) != 0;
    const PatternOffsets po = pattern_offsets(fp.pattern);
    const uint32_t mv2 = fp.mv2;
    const int thr = fp.dpc_thr;
    const uint32_t b16 = (uint32_t)(0x7FFF - thr) * 0x00010001u;
    const float2 z2 = make_float2(fp.neg_zero, fp.neg_zero);
    const float2 h5 = make_float2(0.5f, 0.5f);
    // per row parity (selected, never indexed: an indexed local array would live in memory)
    const int bl_e0 = fp.bl_i[0][0], bl_o0 = fp.bl_i[0][1], bl_e1 = fp.bl_i[1][0], bl_o1 = fp.bl_i[1][1];
    const uint32_t nbl0 = ((uint32_t)(-bl_e0) & 0xFFFFu) | ((uint32_t)(-bl_o0) << 16);
    const uint32_t nbl1 = ((uint32_t)(-bl_e1) & 0xFFFFu) | ((uint32_t)(-bl_o1) << 16);
    const float2 wb0 = make_float2(fp.wb_cfa[bayer_color(0, 0, po)], fp.wb_cfa[bayer_color(0, 1, po)]);
    const float2 wb1 = make_float2(fp.wb_cfa[bayer_color(1, 0, po)], fp.wb_cfa[bayer_color(1, 1, po)]);
    float ccm[9];
#pragma unroll
    for (int i = 0; i < 9; i++) ccm[i] = fp.ccm[i];
    const int xl = U.xw + kStLanePx * lane;  // the lane's first column
    const bool lane_in = xl < W;              // the width is a multiple of 8
    const bool lane_out = xl >= U.ox0 && xl < U.ox1;
    // pixels of the lane whose corrected value feeds an output of the strip (columns ox0 - 5 ..
    // ox1 + 4): only they take the median where the min / max test fails (beyond the frame's last
    // column the lanes hold zeros, which would fail the test on every row)
    unsigned need = 0;
#pragma unroll
    for (int i = 0; i < kStLanePx; i++)
        need |= (xl + i >= U.ox0 - 5 && xl + i < U.ox1 + 5) ? 1u << i : 0u;
    const int lane_byte = xl * rows::bytes_num<FMT>() / rows::bytes_den<FMT>();
    const size_t pitch = (size_t)W * rows::bytes_num<FMT>() / rows::bytes_den<FMT>();
    uint8_t* const out = fp.out;
    const uintptr_t out_base = reinterpret_cast<uintptr_t>(out);
    const int n0 = y0 - 5;
    int nrows = bh + 10, y_end = y0 + bh;  // grow as the segment's next bands are claimed

    const uint8_t* rowp = fp.in + (size_t)n0 * pitch;  // input row n (then n + 1 once loaded)
    uint8_t* outp = out + ((size_t)y0 * W + xl) * 3;  // the lane's bytes of output row q
    uint32_t rw[4];
    rows::load8<FMT>(rowp, lane_byte, lane_in, rw);
    int m5 = 0, m3 = 0;           // k mod 5, k mod 3
    unsigned modrows = 0;         // bit i: jac row b - i differs from orig row b - i in the warp
    int lsc_gy = -1;              // cell row of the lens-shading table
    int rt_base = -1 << 30;       // row table: lane l holds row rt_base + l
    int rt_gy = 0;
    float rt_fy = 0.0f;
    float gprev[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 1
    for (int k = 0; k < nrows; k++) {
        const int n = n0 + k;
        // ---- A: samples of row n -------------------------------------------------------------
        uint32_t P[4];
        rows::decode8<FMT>(rw, P);
        if (own && k + 1 == nrows) {
            // the segment's next band continues this stream
            int j = 0;
            if (lane == 0) j = segs::claim_front(own, bl.seg_words + bl.n_items);
            j = __shfl_sync(full, j, 0);
            if (j >= 0) {
                int yb, hb;
                band_rows(U, j, yb, hb);
                nrows += hb;
                y_end += hb;
            } else {
                own = nullptr;
            }
        }
        rowp += pitch;
        if (k + 1 < nrows) rows::load8<FMT>(rowp, lane_byte, lane_in, rw);
        if (bl_on) {
            const int par = n & 1;
            const int bl_e = par ? bl_e1 : bl_e0, bl_o = par ? bl_o1 : bl_o0;
            // u16 samples above 32767 do not fit the pairs' signed add: per sample
            if (FMT == FMT_U16 && ((P[0] | P[1] | P[2] | P[3]) & 0x80008000u) != 0) {
#pragma unroll
                for (int j = 0; j < 4; j++)
                    P[j] = (uint32_t)__viaddmin_s32_relu((int)(P[j] & 0xFFFFu), -bl_e, mv) |
                           ((uint32_t)__viaddmin_s32_relu((int)(P[j] >> 16), -bl_o, mv) << 16);
            } else {
#pragma unroll
                for (int j = 0; j < 4; j++) P[j] = __viaddmin_s16x2_relu(P[j], par ? nbl1 : nbl0, mv2);
            }
        }
        ws.orig[m5][lane] = make_uint4(P[0], P[1], P[2], P[3]);

        // B and C run from the first row: until their inputs are streamed (k < 4, k < 8) they work
        // on the rings' earlier contents, and nothing they leave there reaches an output or a seed
        {
            // ---- B: bay row b = n - 2 ------------------------------------------------------------
            const int b = n - 2;
            const int so0 = mod5(m5 + 1), so2 = mod5(m5 + 3);  // orig rows b-2, b
            const uint4 o2 = ws.orig[so2][lane];
            uint32_t J[4] = {o2.x, o2.y, o2.z, o2.w};
            const int sj = mod3(m3 + 1);  // kb mod 3
            if (dpc_on) {
                const uint4 o0 = ws.orig[so0][lane];
                const uint32_t R0[4] = {o0.x, o0.y, o0.z, o0.w};
                uint32_t vn[4], vx[4];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    vn[j] = __vimin3_u16x2(R0[j], J[j], P[j]);
                    vx[j] = __vimax3_u16x2(R0[j], J[j], P[j]);
                }
                const uint32_t vnL = __shfl_up_sync(full, vn[3], 1), vnR = __shfl_down_sync(full, vn[0], 1);
                const uint32_t vxL = __shfl_up_sync(full, vx[3], 1), vxR = __shfl_down_sync(full, vx[0], 1);
                unsigned fl = 0;
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    // |c - median| <= thr is certain when c - min and max - c are (min / max over the
                    // 3x3 same-colour box: including c changes neither test)
                    const uint32_t mn = __vimin3_u16x2(j ? vn[j - 1] : vnL, vn[j], j < 3 ? vn[j + 1] : vnR);
                    const uint32_t mx = __vimax3_u16x2(j ? vx[j - 1] : vxL, vx[j], j < 3 ? vx[j + 1] : vxR);
                    const uint32_t d = ((J[j] - mn + b16) | (mx - J[j] + b16)) & 0x80008000u;
                    fl |= ((d >> 15) & 1u) << (2 * j) | (d >> 31) << (2 * j + 1);
                }
                fl &= need;
                unsigned rowmod = 0;
                if (__any_sync(full, fl != 0)) {
                    __syncwarp();
                    const uint4 jn = jacobi_slow(ws, so0, so2, m5, make_uint4(J[0], J[1], J[2], J[3]), fl, lane, thr);
                    J[0] = jn.x;
                    J[1] = jn.y;
                    J[2] = jn.z;
                    J[3] = jn.w;
                    __syncwarp();  // every lane's reads of the rings come before the next row's writes
                    rowmod = __any_sync(full, ((J[0] ^ o2.x) | (J[1] ^ o2.y) | (J[2] ^ o2.z) | (J[3] ^ o2.w)) != 0);
                }
                modrows = (modrows << 1) | rowmod;
                ws.jac[sj][lane] = make_uint4(J[0], J[1], J[2], J[3]);
                if ((modrows & 5u) && b >= y0 && b < y_end) {
                    __syncwarp();
                    if (lane_out) seeds_slow(ws, fp, so0, so2, m5, mod3(sj + 1), sj, lane, xl, b);
                    __syncwarp();
                }
            }
            uint32_t Bq[4] = {J[0], J[1], J[2], J[3]};
            const int par = b & 1;
            if (lsc_on) {
                if (b - rt_base >= 32) {
                    // row terms of the next 32 rows, one per lane (src/lens_shading/flat_field.cpp:84-105)
                    rt_base = b;
                    const int y = min(b + lane, H - 1);
                    const float gy_f = __fdiv_rn(dev::fmul((float)y, (float)(fp.gh - 1)), (float)(H - 1));
                    rt_gy = dev::clampi(dev::ftoi(gy_f), 0, fp.gh - 2);
                    rt_fy = dev::fsub(gy_f, (float)rt_gy);
                }
                const int gy = __shfl_sync(full, rt_gy, b - rt_base);
                const float fy = __shfl_sync(full, rt_fy, b - rt_base);
                if (gy != lsc_gy) {
                    lsc_table(ws, fp, gy, U.xw, lane, po);
                    lsc_gy = gy;
                }
                const float ofy = dev::fsub(1.0f, fy);
                const float2 fy2 = make_float2(fy, fy), ofy2 = make_float2(ofy, ofy);
                const float2 wb = par ? wb1 : wb0;
                const uint32_t top = kMagicBits + (uint32_t)mv;
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const float4 ab = ws.lsc[par][j][0][lane], cv = ws.lsc[par][j][1][lane];
                    const float2 gain = dev::fadd2(
                        dev::fadd2(dev::fadd2(dev::pmul(make_float2(ab.x, ab.y), ofy2, z2), dev::pmul(make_float2(ab.z, ab.w), ofy2, z2)),
                                   dev::pmul(make_float2(cv.x, cv.y), fy2, z2)),
                        dev::pmul(make_float2(cv.z, cv.w), fy2, z2));
                    const float2 t = dev::fadd2(dev::pmul(halves_f2(Bq[j]), gain, z2), h5);
                    if (wb_on) {
                        // min(trunc(t), mv) as the float of the sum's bits, then white balance
                        const float2 s = fadd2_rz(t, make_float2(kMagic, kMagic));
                        const float2 u = dev::fadd2(make_float2(__uint_as_float(min(__float_as_uint(s.x), top)),
                                                                __uint_as_float(min(__float_as_uint(s.y), top))),
                                                    make_float2(-kMagic, -kMagic));
                        Bq[j] = trunc_pack_u(dev::fadd2(dev::pmul(u, wb, z2), h5), mv2);
                    } else {
                        Bq[j] = trunc_pack_u(t, mv2);
                    }
                }
            } else if (wb_on) {
                const float2 wb = par ? wb1 : wb0;
#pragma unroll
                for (int j = 0; j < 4; j++) Bq[j] = trunc_pack_u(dev::fadd2(dev::pmul(halves_f2(Bq[j]), wb, z2), h5), mv2);
            }
            const int sb = mod5(m5 + 3);  // kb mod 5
            ws.bay[sb][lane] = make_uint4(Bq[0], Bq[1], Bq[2], Bq[3]);

            {
                // ---- C: green row g = b - 2 (bay rows g-2 .. g+2 = slots kb-4 .. kb) ------------
                const int g = b - 2;
                const uint4 q0 = ws.bay[mod5(sb + 1)][lane], q1 = ws.bay[mod5(sb + 2)][lane];
                const uint4 q2 = ws.bay[mod5(sb + 3)][lane], q3 = ws.bay[mod5(sb + 4)][lane];
                const uint32_t m2[4] = {q0.x, q0.y, q0.z, q0.w}, m1[4] = {q1.x, q1.y, q1.z, q1.w};
                const uint32_t c0[4] = {q2.x, q2.y, q2.z, q2.w}, p1[4] = {q3.x, q3.y, q3.z, q3.w};
                const uint32_t L = __shfl_up_sync(full, c0[3], 1), R = __shfl_down_sync(full, c0[0], 1);
                const bool grow = (g & 1) == po.r_row;
                const int rbh_g = grow ? po.r_col : po.b_col;
                float gr[4], cd[4];
                if (rbh_g == 0) green_row<0>(m2, m1, c0, p1, Bq, L, R, z2, gr, cd);
                else green_row<1>(m2, m1, c0, p1, Bq, L, R, z2, gr, cd);
                // the one neighbour value each row is read with: pair -1 (left lane's pair 3) when its
                // red / blue site is the odd column, else pair 4 (right lane's pair 0)
                const float ce = __shfl_sync(full, rbh_g ? cd[3] : cd[0], rbh_g ? lane - 1 : lane + 1);
                const int sc = mod3(m3 + 2);  // kg = k - 4 mod 3
                ws.cd[sc][lane] = make_float4(cd[0], cd[1], cd[2], cd[3]);
                ws.cde[sc][lane] = ce;

                if (k >= 10) {
                    // ---- D: output row q = g - 1 -------------------------------------------------
                    const int q = g - 1;
                    const int sm1 = mod3(sc + 1), sq = mod3(sc + 2);  // cd rows q-1, q
                    const float4 a = ws.cd[sm1][lane], c = ws.cd[sq][lane];
                    const float cdm[4] = {a.x, a.y, a.z, a.w}, cdc[4] = {c.x, c.y, c.z, c.w};
                    const float em = ws.cde[sm1][lane], ec = ws.cde[sq][lane];
                    const uint32_t(&bq)[4] = m1;  // bay row q = g - 1
                    const bool rrow = (q & 1) == po.r_row;
                    const int rbh = rrow ? po.r_col : po.b_col;
                    uint32_t ob[6];
                    if (rbh == 0) out_row<0>(rrow, cdm, em, cdc, ec, cd, ce, gprev, bq, ccm, ccm_on, mv, mv2, z2, sm.tone, ob);
                    else out_row<1>(rrow, cdm, em, cdc, ec, cd, ce, gprev, bq, ccm, ccm_on, mv, mv2, z2, sm.tone, ob);
                    if (lane_out) {
                        uint8_t* dst = outp;
                        if ((out_base & 7) == 0) {
                            uint2* d2 = reinterpret_cast<uint2*>(dst);
                            d2[0] = make_uint2(ob[0], ob[1]);
                            d2[1] = make_uint2(ob[2], ob[3]);
                            d2[2] = make_uint2(ob[4], ob[5]);
                        } else if ((out_base & 3) == 0) {
                            uint32_t* d4 = reinterpret_cast<uint32_t*>(dst);
#pragma unroll
                            for (int i = 0; i < 6; i++) d4[i] = ob[i];
                        } else {
#pragma unroll
                            for (int i = 0; i < 24; i++) dst[i] = (uint8_t)(ob[i >> 2] >> (8 * (i & 3)));
                        }
                    }
                    outp += (size_t)3 * W;
                }
#pragma unroll
                for (int j = 0; j < 4; j++) gprev[j] = gr[j];
            }
        }
        m5 = m5 == 4 ? 0 : m5 + 1;
        m3 = m3 == 2 ? 0 : m3 + 1;
    }
}

template <int FMT, int CHAIN>
__global__ void __launch_bounds__(kStThreads, 1) stream_kernel(const __grid_constant__ BatchLaunch bl) {
    extern __shared__ __align__(16) uint8_t dsm[];
    auto& sm = *reinterpret_cast<StreamSmem*>(dsm);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    {
        // every frame of the launch shares its tone table; the rings start zeroed
        const FrameParams& f0 = bl.frames[0];
        for (int i = threadIdx.x; i <= f0.mv; i += kStThreads) sm.tone[i] = __ldg(f0.tone8 + i);
        uint4* r = reinterpret_cast<uint4*>(&sm.w[warp]);
        for (int i = lane; i < (int)(sizeof(StreamWarpSmem) / 16); i += 32) r[i] = make_uint4(0u, 0u, 0u, 0u);
    }
    __syncthreads();
    segs::wait_init();
    // the border tile launches may start now (the init kernel, which zeroed their counters, is
    // complete); their CTAs take the SMs this kernel's CTAs leave
    segs::release_dependents();
    const int nseg = bl.n_items;
    const int gw = (int)blockIdx.x * kStWarps + warp;
    // the warp's own segment, band after band from the front, then bands from the back of others
    segs::Walk walk(gw, nseg, (int)gridDim.x * kStWarps, bl.owners);
    int seg, band, nbands;
    bool own;
    while (walk.next(bl.seg_words, nseg, gw, lane, seg, band, nbands, own)) {
        SSeg S;
        seg_of(bl, seg, S);
        // bands band .. band + nbands - 1: contiguous rows
        int y0, bh, yl, hl;
        band_rows(S, band, y0, bh);
        band_rows(S, band + nbands - 1, yl, hl);
        bh = yl + hl - y0;
        stream_unit<FMT, CHAIN>(bl, sm, sm.w[warp], S, y0, bh, own ? bl.seg_words + seg : nullptr, lane);
    }
}

// the launch's claim words: each segment's band count with zero claims, then the taken count (and
// the border launches' tile counters)
__global__ void stream_seg_init_kernel(const __grid_constant__ BatchLaunch bl) {
    segs::release_dependents();
    const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i < bl.n_items) {
        SSeg G;
        seg_of(bl, i, G);
        bl.seg_words[i] = segs::initial_word(G.nb);
    } else if (i == bl.n_items) {
        bl.seg_words[i] = 0ull;
        // the tile counters of the batch's border-row and border-column launches
        if (bl.tile_counter) *bl.tile_counter = 0;
        bl.seg_words[kStreamSegCap - 1] = 0ull;
    }
}

int g_stream_grid[kMaxDev];

template <int FMT>
cudaError_t launch_fmt(const BatchLaunch& bl, bool chain, int grid, size_t smem, cudaStream_t st) {
    return chain ? launch_dependent(stream_kernel<FMT, 1>, grid, kStThreads, smem, st, bl)
                 : launch_dependent(stream_kernel<FMT, 0>, grid, kStThreads, smem, st, bl);
}

}  // namespace

// interior of a frame: output columns [8, xe), rows [7, h-7)
static int stream_xe(int w) { return 8 + 8 * ((w - 15) / 8); }

bool stream_eligible(const FrameParams& fp) {
    if (fp.demosaic != DM_AMAZE || fp.bd > 12 || fp.out_format != 0 || fp.out_bpc != 1 || (fp.stages & 32u)) return false;
    if (fp.fmt != FMT_U8 && fp.fmt != FMT_U16 && fp.fmt != FMT_P10 && fp.fmt != FMT_P12) return false;
    if (fp.w % 8 != 0 || fp.w < 64 || fp.h < 32 || (reinterpret_cast<uintptr_t>(fp.in) & 15) != 0) return false;
    if (!fp.seg_words || fp.seg_cap < kStreamSegCap) return false;  // the work-claim words of a launch
    const unsigned s = fp.stages;
    const bool bl_on = (s & 1u) != 0, lsc = (s & 4u) != 0, wb = (s & 8u) != 0;
    if (bl_on) {
        if (!fp.bl_int) return false;
        for (int c = 0; c < 4; c++)
            if (fp.bl[c] > (float)fp.mv) return false;
    }
    if ((s & 2u) && (fp.dpc_mode != 0 || fp.dpc_thr < 0 || fp.dpc_thr > 0x7FFF)) return false;
    // gains of at most 15 keep (int)(v * g + 0.5f) below 65536 (one unsigned half)
    if (lsc && (fp.lsc_mode != 0 || !fp.lsc_bounded)) return false;
    if (wb) {
        if (fp.stage_order != 0) return false;
        for (int c = 0; c < 4; c++)
            if (!(fp.wb_cfa[c] >= 0.0f && fp.wb_cfa[c] <= 15.0f)) return false;
    }
    if (s & 16u) {
        // CCM outputs within a signed half before their clamp
        for (int r = 0; r < 3; r++) {
            const double a = std::fabs((double)fp.ccm[3 * r]) + std::fabs((double)fp.ccm[3 * r + 1]) +
                             std::fabs((double)fp.ccm[3 * r + 2]);
            if (!(a * fp.mv + 1.0 < 32000.0)) return false;
        }
    }
    // samples of at most 4095 for the packed arithmetic, and at most the bit depth's maximum when
    // they reach the demosaic (a stage clamps them, a packed format, or full 8-bit bytes)
    if (!bl_on && fp.fmt == FMT_U16) return false;
    return bl_on || lsc || wb || fp.fmt == FMT_P10 || fp.fmt == FMT_P12 || fp.bd == 8;
}

long long stream_table_key(const FrameParams& fp) {
    return (long long)((uint64_t)reinterpret_cast<uintptr_t>(fp.tone8) * 0x9E3779B97F4A7C15ull >> 8);
}

void stream_rects(const FrameParams& fp, TileRect& interior, TileRect (&border)[4]) {
    const int W = fp.w, H = fp.h, xe = stream_xe(W);
    interior = {0, 8, 7, xe - 8, H - 14, (xe - 8 + kStOut - 1) / kStOut, 1};
    border[0] = {0, 0, 0, W, 7, 0, 0};
    border[1] = {0, 0, H - 7, W, 7, 0, 0};
    border[2] = {0, 0, 7, 8, H - 14, 0, 0};
    border[3] = {0, xe, 7, W - xe, H - 14, 0, 0};
}

bool choose_segments(BatchLaunch& bl, int warps, int seg_percent, int band_rows) {
    long long strip_rows = 0, strips = 0;
    for (int r = 0; r < bl.n_rects; r++) {
        strip_rows += (long long)bl.rects[r].tiles_x * bl.rects[r].h;
        strips += bl.rects[r].tiles_x;
    }
    if (strips > kSegMax) return false;  // one segment per strip is the fewest
    double per = std::max(1.0, (double)strip_rows / std::max(1, warps) * seg_percent / 100.0);
    // the segment count the spread aims at (one per warp at 100 %), within the cap
    const long long target = std::min<long long>(kSegMax, std::max<long long>(strips, std::llround(warps * 100.0 / seg_percent)));
    // each rectangle's count rounded down, then one more for the rectangles of the height with the
    // largest remainder — all rectangles of that height at once, so their segments stay equal — while
    // the total stays within the target (at 100 % every segment has its warp and no warp starts with
    // two); above the cap, longer segments until the count fits (it shrinks with every pass and
    // reaches one per strip)
    for (;;) {
        long long items = 0;
        double rem[kMaxRects];
        for (int r = 0; r < bl.n_rects; r++) {
            TileRect& R = bl.rects[r];
            const double t = R.h / per;
            R.tiles_y = std::max(1, std::min(R.h, (int)std::floor(t)));
            rem[r] = R.tiles_y < R.h ? t - R.tiles_y : -1.0;
            items += (long long)R.tiles_x * R.tiles_y;
        }
        for (;;) {
            int best = -1;
            long long add_best = 0;
            for (int r = 0; r < bl.n_rects; r++) {
                if (rem[r] <= 0.0 || (best >= 0 && rem[r] <= rem[best])) continue;
                long long add = 0;  // one more segment per strip of every rectangle of this height
                for (int q = 0; q < bl.n_rects; q++)
                    if (bl.rects[q].h == bl.rects[r].h && rem[q] > 0.0) add += bl.rects[q].tiles_x;
                if (items + add <= target) {
                    best = r;
                    add_best = add;
                }
            }
            if (best < 0) break;
            const int h = bl.rects[best].h;
            for (int q = 0; q < bl.n_rects; q++)
                if (bl.rects[q].h == h && rem[q] > 0.0) {
                    bl.rects[q].tiles_y++;
                    rem[q] = -1.0;
                }
            items += add_best;
        }
        if (items <= kSegMax) break;
        per *= (double)items / kSegMax * 1.01;
    }
    int items = 0;
    for (int r = 0; r < bl.n_rects; r++) {
        bl.rect_start[r] = items;
        items += bl.rects[r].tiles_x * bl.rects[r].tiles_y;
    }
    bl.rect_start[bl.n_rects] = bl.n_items = items;
    // at most segs::kMaxBands bands per segment (the claim word's band count field)
    int longest = 0;
    for (int r = 0; r < bl.n_rects; r++)
        longest = std::max(longest, (bl.rects[r].h + bl.rects[r].tiles_y - 1) / bl.rects[r].tiles_y);
    bl.band_h = std::max(band_rows, (longest + segs::kMaxBands - 1) / segs::kMaxBands);
    return true;
}

cudaError_t launch_stream(const BatchLaunch& bl_in, cudaStream_t st) {
    const size_t smem = sizeof(StreamSmem);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDev) return cudaErrorInvalidDevice;
    int limit;
    {
        std::lock_guard<std::mutex> lock(device_setup_mutex());
        if (!g_stream_grid[dev]) {
            void (*ks[8])(BatchLaunch) = {stream_kernel<FMT_U8, 0>,  stream_kernel<FMT_U16, 0>, stream_kernel<FMT_P10, 0>,
                                          stream_kernel<FMT_P12, 0>, stream_kernel<FMT_U8, 1>,  stream_kernel<FMT_U16, 1>,
                                          stream_kernel<FMT_P10, 1>, stream_kernel<FMT_P12, 1>};
            for (int k = 0; k < 8 && e == cudaSuccess; k++)
                e = cudaFuncSetAttribute(ks[k], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            int n = 0, m = 0;
            if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ks[3], kStThreads, smem);
            if (e == cudaSuccess) e = cudaDeviceGetAttribute(&m, cudaDevAttrMultiProcessorCount, dev);
            if (e != cudaSuccess) return e;
            g_stream_grid[dev] = m * (n > 0 ? n : 1);
        }
        limit = g_stream_grid[dev];
    }
    BatchLaunch bl = bl_in;
    bl.owners = 0;
    int wmax = 0;
    for (int f = 0; f < bl.n_frames; f++) wmax = std::max(wmax, bl.frames[f].w);
    const TuneParams tp = tuning_for(IMOP_KERNEL_STREAM, bl.fmt, wmax);
    if (!choose_segments(bl, limit * kStWarps, tp.seg_percent, tp.band_rows)) return cudaErrorInvalidValue;
    if (bl.n_items <= 0) return cudaSuccess;
    if (bl.n_items > kSegMax || !bl.seg_words) return cudaErrorInvalidValue;
    stream_seg_init_kernel<<<(bl.n_items + 256) / 256, 256, 0, st>>>(bl);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // one CTA per 12 segments (a warp that starts without a segment of its own would take bands
    // from the others from the start, each with 10 warm-up rows: slower than the idle SMs)
    const int want = (bl.n_items + kStWarps - 1) / kStWarps;
    const int grid = want < limit ? want : limit;
    count_launch(2);
    // the instantiation with every stage fixed on when each frame runs all five
    bool chain = true;
    for (int f = 0; f < bl.n_frames; f++) chain = chain && (bl.frames[f].stages & 31u) == 31u;
    switch (bl.fmt) {
        case FMT_U8: return launch_fmt<FMT_U8>(bl, chain, grid, smem, st);
        case FMT_U16: return launch_fmt<FMT_U16>(bl, chain, grid, smem, st);
        case FMT_P10: return launch_fmt<FMT_P10>(bl, chain, grid, smem, st);
        case FMT_P12: return launch_fmt<FMT_P12>(bl, chain, grid, smem, st);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace imop
