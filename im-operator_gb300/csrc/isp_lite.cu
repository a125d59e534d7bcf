// isp_lite.cu - the light-chain kernel (isp_lite.cuh) in two variants.  The staged one: persistent
// CTAs whose warps each claim bands of frame strips from a device counter and stream them row by
// row from a ring of bulk-copied rows (any frame).  The direct-read one: frames 16-byte aligned
// with a width that is a multiple of 8; lanes load their samples with plain coalesced loads two
// rows ahead, and each warp streams a whole segment of its strip (isp_segments.cuh).

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "imop_isp.h"
#include "isp_fused_kernel.cuh"
#include "isp_kernels.h"
#include "isp_lite.cuh"
#include "isp_rows.cuh"
#include "isp_segments.cuh"

namespace imop {
namespace {

constexpr int kMaxDev = 64;

// unit `item` of the launch: its rectangle (frame) by binary search, then the band and strip
__device__ __forceinline__ void unit_of(const BatchLaunch& bl, int item, LiteUnit& U) {
    const int r = item_rect(bl, item);
    const TileRect& R = bl.rects[r];
    const int t = item - bl.rect_start[r];
    const int ty = t / R.tiles_x, tx = t - ty * R.tiles_x;
    const int sw = lite_strip_w(R.w);
    U.f = R.frame;
    U.x0 = R.x0 + tx * sw;
    U.npx = min(sw, R.w - tx * sw);
    int y0, bh;
    tile_span(R.h, bl.band_h, R.tiles_y, ty, y0, bh);
    U.y0 = R.y0 + y0;
    U.bh = bh;
    U.nrows = bh + 2;
}

// lane 0: stage row k (y = y0 - 1 + k) of unit U into slot s: the bytes of pixels
// [x0 - 8, x0 + npx + 8) of the frame, widened to 16-byte boundaries inside the buffer; a row
// outside the frame (or a frame pointer the copy engine cannot take) completes its barrier phase
// with no bytes
template <int FMT>
__device__ __forceinline__ void stage_row(LiteWarpSmem& ws, const FrameParams& fp, const LiteUnit& U, int k, int s) {
    const int y = U.y0 - 1 + k;
    const int W = fp.w;
    int a0 = 0, len = 0;
    if (y >= 0 && y < fp.h) {
        const int xs = max(0, U.x0 - 8), xe = min(W, U.x0 + U.npx + 8);
        int b0, b1;
        pixel_bytes(FMT, fp.bd, y * W + xs, y * W + xe, b0, b1);
        b1 = min(b1, (int)fp.in_bytes);
        a0 = b0 & ~15;
        const int a1 = min((b1 + 15) & ~15, (int)(fp.in_bytes & ~(size_t)15));
        len = max(a1 - a0, 0);
    }
    ws.a0[s] = a0;
    ws.len[s] = len;
    if (len > 0 && (reinterpret_cast<uintptr_t>(fp.in) & 15) == 0) {
        ptx::mbar_arrive_expect_tx(&ws.bar[s], (uint32_t)len);
        ptx::bulk_g2s(ws.raw[s], fp.in + a0, (uint32_t)len, &ws.bar[s]);
    } else {
        ptx::mbar_arrive_expect_tx(&ws.bar[s], 0);
    }
}

// the 8 raw samples x .. x+7 (x even) of staged row y as packed pairs (a0 / len: the slot's
// window): word loads from the slot where the samples lie whole inside it on a pair / group
// boundary, else one by one with the packed-tail rule of pixel::get_packed_raw (frame edge,
// unaligned rows)
template <int FMT>
__device__ __forceinline__ void decode_pairs(const FrameParams& fp, const uint8_t* row, int a0, int len, int y, int x,
                                             uint32_t (&P)[4]) {
    const int W = fp.w;
    const int i0 = y * W + x;
    const int o = lite::byte_of<FMT>(i0) - a0;
    const bool pair_ok = FMT == FMT_U8 || FMT == FMT_U16 || (FMT == FMT_P12 && (i0 & 1) == 0) ||
                         (FMT == FMT_P10 && (i0 & 3) == 0);
    if (x + 8 <= W && pair_ok && o >= 0 && o + lite::bytes8<FMT>() <= len) {
        if (FMT == FMT_U8) {
            uint32_t w[2];
            lite::load_words(row, o, w);
            P[0] = __byte_perm(w[0], 0u, 0x4140);
            P[1] = __byte_perm(w[0], 0u, 0x4342);
            P[2] = __byte_perm(w[1], 0u, 0x4140);
            P[3] = __byte_perm(w[1], 0u, 0x4342);
        } else if (FMT == FMT_U16) {
            lite::load_words(row, o, P);
        } else if (FMT == FMT_P12) {
            uint32_t w[3];
            lite::load_words(row, o, w);
            P[0] = unpack12_pair(w[0]);
            P[1] = unpack12_pair(__funnelshift_r(w[0], w[1], 24));
            P[2] = unpack12_pair(__funnelshift_r(w[1], w[2], 16));
            P[3] = unpack12_pair(w[2] >> 8);
        } else {
            int v[8];
            lite::decode8<FMT>(row, o, v);
#pragma unroll
            for (int j = 0; j < 4; j++) P[j] = (uint32_t)v[2 * j] | ((uint32_t)v[2 * j + 1] << 16);
        }
    } else {
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const uint32_t lo = (x + 2 * j < W) ? (uint32_t)staged_raw(fp, a0, len, row, i0 + 2 * j) : 0u;
            const uint32_t hi = (x + 2 * j + 1 < W) ? (uint32_t)staged_raw(fp, a0, len, row, i0 + 2 * j + 1) : 0u;
            P[j] = lo | (hi << 16);
        }
    }
}

// black level and Bayer-order white balance of a row, its parameters in registers for a unit (the
// parameter block is read through an indexed constant bank)
struct LiteLevels {
    uint32_t nbl0, nbl1, mv2;  // the negated black levels of even / odd rows as pairs; the maximum twice
    int nbb0, nbb1, mv;        // the negated black level of the lane's outer sample, even / odd rows
    bool bl_on, per_sample;    // per_sample: Bayer-order white balance or the MSB-aligned read
};
__device__ __forceinline__ LiteLevels lite_levels_of(const FrameParams& fp, int lane) {
    LiteLevels L;
    const int e0 = fp.bl_i[0][0], o0 = fp.bl_i[0][1], e1 = fp.bl_i[1][0], o1 = fp.bl_i[1][1];
    L.nbl0 = ((uint32_t)(-e0) & 0xFFFFu) | ((uint32_t)(-o0) << 16);
    L.nbl1 = ((uint32_t)(-e1) & 0xFFFFu) | ((uint32_t)(-o1) << 16);
    // lane 0's outer sample (column x0 - 1) is in an odd column, lane 31's (x0 + 256) in an even one
    L.nbb0 = lane == 0 ? -o0 : -e0;
    L.nbb1 = lane == 0 ? -o1 : -e1;
    L.mv = fp.mv;
    L.mv2 = (uint32_t)fp.mv | ((uint32_t)fp.mv << 16);
    L.bl_on = (fp.stages & 1u) != 0;
    L.per_sample = ((fp.stages & 8u) && fp.stage_order == 0) || fp.need_align != 0;
    return L;
}

// one sample at a time: black level, Bayer-order white balance, the MSB-aligned read
__device__ __forceinline__ void lite_levels_each(const FrameParams& fp, PatternOffsets po, int y, int lane,
                                                 uint32_t (&P)[4], int& nb) {
    const int mv = fp.mv, p = y & 1;
    const int bl_e = fp.bl_i[p][0], bl_o = fp.bl_i[p][1];
    const bool bl_on = (fp.stages & 1u) != 0, wb_bayer = (fp.stages & 8u) && fp.stage_order == 0;
    const bool need_align = fp.need_align != 0;
    const float wb_e = fp.wb_cfa[bayer_color(y, 0, po)], wb_o = fp.wb_cfa[bayer_color(y, 1, po)];
    auto one = [&](int v, bool odd) {
        if (bl_on) v = __viaddmin_s32_relu(v, odd ? -bl_o : -bl_e, mv);
        if (wb_bayer) v = dev::gain_round(v, odd ? wb_o : wb_e, mv);
        if (need_align && v > mv) v >>= (16 - fp.bd);
        return v;
    };
#pragma unroll
    for (int j = 0; j < 4; j++)
        P[j] = (uint32_t)one((int)(P[j] & 0xFFFFu), false) | ((uint32_t)one((int)(P[j] >> 16), true) << 16);
    nb = one(nb, lane == 0);
}

// the lane's pairs P and the strip's outer neighbour nb (lane 0: column x0 - 1, lane 31: column
// x0 + 256) of row y
template <int FMT>
__device__ __forceinline__ void lite_levels(const FrameParams& fp, const LiteLevels& L, PatternOffsets po, int y,
                                            int lane, uint32_t (&P)[4], int& nb) {
    // u16 samples above 32767 (beyond any bit depth here) do not fit the pairs' signed 16-bit add:
    // those lanes take the per-sample path
    const bool per_sample =
        L.per_sample || (FMT == FMT_U16 && L.bl_on && ((P[0] | P[1] | P[2] | P[3]) & 0x80008000u) != 0);
    if (!per_sample) {
        // black level (integral offsets <= the maximum: lite_eligible) on both samples of a pair at
        // once: (int)((float)v - off) clamped to [0, mv]
        if (L.bl_on) {
            const bool odd = (y & 1) != 0;
            const uint32_t nbl = odd ? L.nbl1 : L.nbl0;
#pragma unroll
            for (int j = 0; j < 4; j++) P[j] = __viaddmin_s16x2_relu(P[j], nbl, L.mv2);
            nb = __viaddmin_s32_relu(nb, odd ? L.nbb1 : L.nbb0, L.mv);
        }
    } else {
        lite_levels_each(fp, po, y, lane, P, nb);
    }
}

// the output row from the staging row of the warp: the row's bytes at their 16-byte phase, the
// border columns fixed, vector stores of the whole 16-byte chunks; rows 0, 1 / h-2, h-1 with row
// 2 / h-3
__device__ __forceinline__ void lite_emit_staged(const uint8_t (*tab)[4096], uint8_t* wout, uint8_t* out, int W, int H,
                                              int x0, int npx, int lane, int yo, uint4 oa, uint2 ob2) {
    const uint32_t ob[6] = {oa.x, oa.y, oa.z, oa.w, ob2.x, ob2.y};
    const uintptr_t out_base = reinterpret_cast<uintptr_t>(out);
    const int xl = x0 + kLiteLanePx * lane;
    const bool edge_l = x0 == 0, edge_r = x0 + npx == W;
    const int g0 = (yo * W + x0) * 3;
    // otherwise: stage at the output row's 16-byte phase, fix the border columns, store
    const int shift = (int)((out_base + (uintptr_t)g0) & 15);
    const int nbytes = 3 * npx;
    uint8_t* st = wout + shift + 24 * lane;
    if (xl < x0 + npx) {
        if ((shift & 7) == 0) {
            uint2* q2 = reinterpret_cast<uint2*>(st);
            q2[0] = make_uint2(ob[0], ob[1]);
            q2[1] = make_uint2(ob[2], ob[3]);
            q2[2] = make_uint2(ob[4], ob[5]);
        } else if ((shift & 3) == 0) {
            uint32_t* q4 = reinterpret_cast<uint32_t*>(st);
#pragma unroll
            for (int q = 0; q < 6; q++) q4[q] = ob[q];
        } else {
#pragma unroll
            for (int q = 0; q < 24; q++) st[q] = (uint8_t)(ob[q >> 2] >> (8 * (q & 3)));
        }
    }
    __syncwarp();
    uint8_t* so = wout + shift;
    if (edge_l || edge_r) {
        if (lane < 6) {
            // columns 0, 1 <- 2 and w-2, w-1 <- w-3 (lanes 0-2 / 3-5, one byte each)
            const int b = lane % 3;
            if (lane < 3 && edge_l) so[b] = so[3 + b] = so[6 + b];
            if (lane >= 3 && edge_r) {
                const int c3 = W - 3 - x0;
                so[3 * (c3 + 1) + b] = so[3 * (c3 + 2) + b] = so[3 * c3 + b];
            }
        }
        __syncwarp();
    }
    // the row, and rows 0, 1 with row 2 / rows h-2, h-1 with row h-3 (their corner pixels
    // zero: the tables' bytes of 0)
    const int copies = (yo == 2 || yo == H - 3) ? 3 : 1;
    for (int rep = 0; rep < copies; rep++) {
        const int yt = rep == 0 ? yo : (yo == 2 ? rep - 1 : H - 3 + rep);
        if (rep == 1) {
            if (lane < 6) {
                const int b = lane % 3;
                const uint8_t z = tab[b][0];
                if (lane < 3 && edge_l) so[b] = so[3 + b] = z;
                if (lane >= 3 && edge_r) {
                    const int c3 = W - 3 - x0;
                    so[3 * (c3 + 1) + b] = so[3 * (c3 + 2) + b] = z;
                }
            }
            __syncwarp();
        }
        const int gt = (yt * W + x0) * 3;
        if ((int)((out_base + (uintptr_t)gt) & 15) == shift) {
            // staging bytes [A, E) <-> output bytes from gt: whole 16-byte chunks as vector
            // stores, the head and tail bytes one per lane
            uint8_t* base = out + gt - shift;  // 16-byte aligned
            const int A = shift, E = shift + nbytes;
            const int F = (A + 15) & ~15, L = E & ~15;
            if (F < L) {
                for (int c = F / 16 + lane; c < L / 16; c += 32)
                    ptx::st_global_v4(base + 16 * c, *reinterpret_cast<const uint4*>(wout + 16 * c));
                if (A + lane < F) base[A + lane] = wout[A + lane];
                if (L + lane < E) base[L + lane] = wout[L + lane];
            } else if (A + lane < E) {
                base[A + lane] = wout[A + lane];
            }
        } else {
            uint8_t* d8 = out + gt;
            for (int b = lane; b < nbytes; b += 32) d8[b] = so[b];
        }
    }
    __syncwarp();
}

// output row y - 1 from rows u, m, d (y - 2 .. y) of the strip at x0 (npx columns): HQLI through
// the output tables, the reference's border copies, 24-byte stores per lane or staged rows
__device__ __forceinline__ void lite_emit(const uint8_t (*tab)[4096], uint8_t* wout, int W, int H, uint8_t* out,
                                          PatternOffsets po, int x0, int npx, int lane, int y, const lite::Row& Ur,
                                          const lite::Row& Mr, const lite::Row& Dr) {
    const uintptr_t out_base = reinterpret_cast<uintptr_t>(out);
    const int xl = x0 + kLiteLanePx * lane;
    const bool edge_l = x0 == 0, edge_r = x0 + npx == W;
    const bool lane_in = xl + kLiteLanePx <= x0 + npx;
    // ---- output row yo = y - 1 -------------------------------------------------------------
    const int yo = y - 1;
    if (yo < 2 || yo >= H - 2) return;  // emitted with row 2 / h-3
    uint32_t ob[6];
    const bool rrow = (yo & 1) == po.r_row;
    const int rb = rrow ? po.r_col : po.b_col;
    if (rb == 0) {
        if (rrow) lite::hqli_row<0, true>(Ur, Mr, Dr, tab, ob);
        else lite::hqli_row<0, false>(Ur, Mr, Dr, tab, ob);
    } else {
        if (rrow) lite::hqli_row<1, true>(Ur, Mr, Dr, tab, ob);
        else lite::hqli_row<1, false>(Ur, Mr, Dr, tab, ob);
    }
    const int g0 = (yo * W + x0) * 3;
    // an interior strip whose row starts 8-byte aligned: each lane stores its 24 bytes
    if (!edge_l && !edge_r && yo != 2 && yo != H - 3 && ((out_base + (uintptr_t)g0) & 7) == 0) {
        if (lane_in) {
            uint2* q = reinterpret_cast<uint2*>(out + g0 + 24 * lane);
            q[0] = make_uint2(ob[0], ob[1]);
            q[1] = make_uint2(ob[2], ob[3]);
            q[2] = make_uint2(ob[4], ob[5]);
        }
        return;
    }
    lite_emit_staged(tab, wout, out, W, H, x0, npx, lane, yo, make_uint4(ob[0], ob[1], ob[2], ob[3]),
                     make_uint2(ob[4], ob[5]));
}

template <int FMT>
__global__ void __launch_bounds__(kThreads, 3) lite_batch_kernel(const __grid_constant__ BatchLaunch bl) {
    extern __shared__ __align__(16) uint8_t dsm[];
    auto& sm = *reinterpret_cast<LiteSmem*>(dsm);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    LiteWarpSmem& ws = sm.w[warp];
    const int n_items = bl.n_items;

    // tables of the launch (every frame shares them): T_c[v] = tone8[round(v * wb_rgb[c])] when white
    // balance runs on RGB, else tone8[v]
    {
        const FrameParams& f0 = bl.frames[0];
        const int mv = f0.mv;
        const bool wb_rgb = (f0.stages & 8u) && f0.stage_order == 1;
        for (int i = threadIdx.x; i < 3 * (mv + 1); i += kThreads) {
            const int c = i / (mv + 1), v = i - c * (mv + 1);
            const int q = wb_rgb ? dev::gain_round(v, f0.wb_rgb[c], mv) : v;
            sm.tab[c][v] = __ldg(f0.tone8 + q);
        }
    }
    if (lane == 0) {
        for (int s = 0; s < kLiteRing; s++) ptx::mbar_init(&ws.bar[s], 1);
        ptx::fence_mbar_init();
    }
    __syncthreads();

    // The warp's stream of staged rows: the rows of unit `cur`, then those of unit `nxt`, claimed
    // when staging reaches the end of `cur` (a few rows before `cur` is done, so the claims stay
    // balanced across warps).  `issued` / `used` count rows over the whole stream: slot = count %
    // ring, barrier phase = (count / ring) & 1.
    int cur_item = 0;
    if (lane == 0) cur_item = atomicAdd(bl.tile_counter, 1);
    cur_item = __shfl_sync(0xffffffffu, cur_item, 0);
    if (cur_item >= n_items) return;
    int nxt_item = -1;  // -1: not claimed yet
    LiteUnit cur, nxt;
    unit_of(bl, cur_item, cur);
    nxt = cur;
    unsigned issued = 0, used = 0;
    int iss_unit = 0, iss_k = 0;  // staging position: unit (0 cur, 1 nxt) and row in it
    // stage the stream's next row (all lanes call it, lane 0 issues); false at the end of the work
    auto issue_next = [&]() -> bool {
        if (iss_unit == 0 && iss_k == cur.nrows) {
            iss_unit = 1;
            iss_k = 0;
        }
        if (iss_unit == 1) {
            if (nxt_item < 0) {
                int it = 0;
                if (lane == 0) it = atomicAdd(bl.tile_counter, 1);
                nxt_item = __shfl_sync(0xffffffffu, it, 0);
                if (nxt_item < n_items) unit_of(bl, nxt_item, nxt);
            }
            if (nxt_item >= n_items || iss_k == nxt.nrows) return false;
        }
        const LiteUnit& U = iss_unit == 0 ? cur : nxt;
        if (lane == 0) stage_row<FMT>(ws, bl.frames[U.f], U, iss_k, (int)(issued % kLiteRing));
        issued++;
        iss_k++;
        return true;
    };
    for (int i = 0; i < kLiteRing; i++)
        if (!issue_next()) break;

    lite::Row Ur, Mr, Dr;  // rows y-2, y-1, y of the lane (packed pairs)
    while (true) {
        const FrameParams& fp = bl.frames[cur.f];
        const int W = fp.w;
        const PatternOffsets po = pattern_offsets(fp.pattern);
        const LiteLevels L = lite_levels_of(fp, lane);
        const bool aligned_in = (reinterpret_cast<uintptr_t>(fp.in) & 15) == 0;
        const int xl = cur.x0 + kLiteLanePx * lane;  // the lane's first column
        for (int k = 0; k < cur.nrows; k++) {
            const int s = (int)(used % kLiteRing);
            const uint32_t parity = (used / kLiteRing) & 1u;
            const bool ok = wait_bar(&ws.bar[s], parity);
            if (!__all_sync(0xffffffffu, ok)) {
                // leave no copy in flight into this CTA's shared memory: wait (bounded) for the other
                // staged rows, then report
                for (unsigned c = used + 1; c < issued; c++) wait_bar(&ws.bar[c % kLiteRing], (c / kLiteRing) & 1u);
                if (lane == 0) atomicExch(fp.status, 103 /* IMOP_ERR_TIMEOUT */);
                return;
            }
            const uint8_t* row = ws.raw[s];
            const int a0 = ws.a0[s], len = ws.len[s];
            const int y = cur.y0 - 1 + k;
            if (!aligned_in && len > 0) {
                // the frame pointer is not 16-byte aligned: the lanes copy the window themselves
                uint8_t* dst = ws.raw[s];
                for (int b = lane; b < len; b += 32) dst[b] = __ldg(fp.in + a0 + b);
                __syncwarp();
            }
            // ---- this lane's 8 samples of row y (packed pairs) and the strip's outer neighbour
            // (lane 0: column x0 - 1, lane 31: column x0 + 256), black-levelled and white-balanced --
            uint32_t P[4] = {0u, 0u, 0u, 0u};
            int nb = 0;
            if (len > 0) {
                if (xl < W) decode_pairs<FMT>(fp, row, a0, len, y, xl, P);
                if (lane == 0 || lane == 31) {
                    const int xn = lane == 0 ? cur.x0 - 8 : cur.x0 + kLiteStripMax;
                    if (xn >= 0 && xn < W) {
                        uint32_t t[4];
                        decode_pairs<FMT>(fp, row, a0, len, y, xn, t);
                        nb = lane == 0 ? (int)(t[3] >> 16) : (int)(t[0] & 0xFFFFu);
                    }
                }
                lite_levels<FMT>(fp, L, po, y, lane, P, nb);
                if (lane == 0 && cur.x0 == 0) nb = 0;
            }
            uint32_t Lw = __shfl_up_sync(0xffffffffu, P[3], 1) & 0xFFFF0000u;
            uint32_t Rn = __shfl_down_sync(0xffffffffu, P[0], 1) & 0xFFFFu;
            if (lane == 0) Lw = (uint32_t)nb << 16;
            if (lane == 31) Rn = (uint32_t)nb;
            // the slot is consumed: every lane's reads of it come before the copy that refills it
            ptx::fence_proxy_async_smem();
            __syncwarp();
            used++;
            issue_next();
            // slide the window
            Ur = Mr;
            Mr = Dr;
#pragma unroll
            for (int j = 0; j < 4; j++) Dr.P[j] = P[j];
            Dr.Lw = Lw;
            Dr.R = Rn;
            if (k < 2) continue;

            lite_emit(sm.tab, ws.out, W, fp.h, fp.out, po, cur.x0, cur.npx, lane, y, Ur, Mr, Dr);
        }
        // the next unit: `nxt` (claimed while `cur`'s last rows were staged) becomes current
        if (nxt_item < 0) {
            int it = 0;
            if (lane == 0) it = atomicAdd(bl.tile_counter, 1);
            nxt_item = __shfl_sync(0xffffffffu, it, 0);
            if (nxt_item < n_items) unit_of(bl, nxt_item, nxt);
            iss_unit = 1;
            iss_k = 0;
        }
        if (nxt_item >= n_items) return;
        cur_item = nxt_item;
        cur = nxt;
        nxt_item = -1;
        iss_unit = 0;  // staging continues inside the new `cur` at row iss_k
        while (issued - used < (unsigned)kLiteRing)
            if (!issue_next()) break;
    }
}

// ---- the direct-read variant ---------------------------------------------------------------
// Frames whose rows start on a word (direct_ok) skip the shared staging of whole rows: each lane copies the words of its own 8 samples of a row (lanes 0 and 31 also the sample
// beside the strip) into its slot of a ring of kDirRing rows with per-thread asynchronous copies,
// kDirRing - 1 rows ahead of their use, and reads them back itself: no lane waits for another,
// no barrier, and the rows in flight hold no registers.  A warp streams a whole segment of its
// strip band after band, so only bands taken from the back of another warp's segment (the
// end-of-launch balancing) re-read the two rows above them.  One CTA per SM builds the output
// tables once.
constexpr int kDirWarps = 24;
constexpr int kDirThreads = 32 * kDirWarps;
constexpr int kDirRing = 4;

// u8 frames (samples of at most 8 bits) use the replicated output tables (lite::hqli_row_t): fewer
// integer-pipe instructions per pixel, which binds this kernel; for the others (4096-entry tables)
// the larger tables measured slower
template <int FMT>
struct LiteDirectSmem {
    lite::LiteTables<FMT == FMT_U8 ? 256 : 1> tab;
    alignas(16) uint8_t out[kDirWarps][LiteWarpSmem::OUT_PITCH];
    uint4 ring[kDirWarps][kDirRing][32];   // the lanes' words of each row in flight
    uint2 ring_e[kDirWarps][kDirRing][32];  // the words of the sample beside the strip (lanes 0, 31)
};
static_assert(kDirWarps * LiteWarpSmem::OUT_PITCH >= 4096, "the staging rows hold the tone table at start");
template <int FMT>
constexpr size_t direct_smem() { return sizeof(LiteDirectSmem<FMT>); }

// a segment of a strip (isp_segments.cuh): columns [x0, x0 + npx), output rows [s0, s0 + len)
struct LSeg {
    int f, x0, npx, s0, len, nb;
};

__device__ __forceinline__ void lseg_of(const BatchLaunch& bl, int seg, LSeg& G) {
    const int r = item_rect(bl, seg);
    const TileRect& R = bl.rects[r];
    const int t = seg - bl.rect_start[r];
    const int ty = t / R.tiles_x, tx = t - ty * R.tiles_x;
    const int sw = lite_strip_w(R.w);
    G.f = R.frame;
    G.x0 = R.x0 + tx * sw;
    G.npx = min(sw, R.w - tx * sw);
    segs::split_rows(R.y0, R.h, R.tiles_y, ty, G.s0, G.len);
    G.nb = max(1, (G.len + bl.band_h - 1) / bl.band_h);
}

// where a lane's samples of strip U's rows are: its 8 samples and (lanes 0 and 31) the sample
// beside the strip
// WORDS: u8 / u16 rows that start on a word but not on the lanes' 8- / 16-byte loads (a width
// that is not a multiple of 8, or an input that is not 16-byte aligned)
template <int FMT, bool WORDS>
struct DirectRows {
    int pitch, lane_byte, edge_byte;
    bool lane_in, edge_in, edge_lane;
    __device__ __forceinline__ DirectRows(const FrameParams& fp, const LSeg& U, int lane) {
        const int W = fp.w;
        edge_lane = lane == 0 || lane == 31;
        const int xl = U.x0 + kLiteLanePx * lane;
        lane_in = xl < W;  // the width is a multiple of 8
        // lane 0: the sample left of the strip (column x0 - 1); lane 31: the one right of it
        const int xe = lane == 0 ? U.x0 - 1 : U.x0 + kLiteStripMax;
        edge_in = (lane == 0 || lane == 31) && xe >= 0 && xe < W;
        lane_byte = xl * rows::bytes_num<FMT>() / rows::bytes_den<FMT>();
        edge_byte = !edge_in ? 0 : lane == 0 ? rows::edge_byte<FMT, true>(xe) : rows::edge_byte<FMT, false>(xe);
        pitch = W * rows::bytes_num<FMT>() / rows::bytes_den<FMT>();
    }
    // row n of frame fp into the lane's ring slots (zeros outside the frame)
    __device__ __forceinline__ void issue(const FrameParams& fp, int n, uint32_t main, uint32_t edge) const {
        const bool row_in = (unsigned)n < (unsigned)fp.h;
        const uint8_t* rp = fp.in + (row_in ? (long long)n * pitch : 0ll);
        if (WORDS)
            rows::ring_load8_words<FMT>(main, rp, lane_byte, pitch - lane_byte, row_in && lane_in, fp.in);
        else
            rows::ring_load8<FMT>(main, rp, lane_byte, row_in && lane_in, fp.in);
        // only lanes 0 and 31 use the sample beside the strip
        if (edge_lane) rows::ring_load_edge<FMT>(edge, rp, edge_byte, row_in && edge_in, fp.in);
    }
    // row n back from the slots (after its copies completed): the lane's words and the edge words
    __device__ __forceinline__ void read(const FrameParams& fp, int n, const uint4& main, const uint2& edge,
                                         uint32_t (&w)[4], rows::Edge<FMT>& e) const {
        if (FMT == FMT_U8) {
            const uint2 m = *reinterpret_cast<const uint2*>(&main);  // 8 bytes hold the 8 samples
            w[0] = m.x;
            w[1] = m.y;
            w[2] = w[3] = 0u;
        } else {
            const uint4 m = main;
            w[0] = m.x;
            w[1] = m.y;
            w[2] = m.z;
            w[3] = m.w;
        }
        e.g[0] = edge.x;
        if (FMT == FMT_P10) {
            // the byte offsets of the samples in the first copied words
            const bool row_in = (unsigned)n < (unsigned)fp.h;
            const uint8_t* rp = fp.in + (row_in ? (long long)n * pitch : 0ll);
            w[3] = rows::ring_offset(rp, lane_byte);
            e.g[1] = edge.y;
            e.g[2] = rows::ring_offset(rp, edge_byte);
        }
    }
};

// output rows [y0, y0 + bh) of segment U and, while `own` is set, the segment's next bands from
// the front: input rows y0 - 1 .. (the row below the last output row)
template <int FMT, bool WORDS>
__device__ __forceinline__ void direct_unit(const BatchLaunch& bl, const lite::LiteTables<FMT == FMT_U8 ? 256 : 1>& tab,
                                            uint8_t* wout,
                                            uint4 (*ring)[32], uint2 (*ring_e)[32], const LSeg& U, int y0, int bh,
                                            unsigned long long* own, int lane) {
    const unsigned full = 0xffffffffu;
    const FrameParams& fp = bl.frames[U.f];
    const int W = fp.w, H = fp.h;
    uint8_t* const out = fp.out;
    const PatternOffsets po = pattern_offsets(fp.pattern);
    const LiteLevels L = lite_levels_of(fp, lane);
    const int xl = U.x0 + kLiteLanePx * lane;
    const DirectRows<FMT, WORDS> src(fp, U, lane);
    const int n0 = y0 - 1;
    int nrows = bh + 2;
    // output: on an interior strip every lane stores its 24 bytes straight, in words as wide as the
    // row's 8-byte phase allows (the same for every lane of a row; one phase for all rows of a
    // frame whose width is a multiple of 8); the lane's bytes of output row n - 1 lie at out + ooff
    const bool lane_st = xl + kLiteLanePx <= U.x0 + U.npx;
    const bool interior = U.x0 != 0 && U.x0 + U.npx != W;
    const bool fast = interior && ((reinterpret_cast<uintptr_t>(out) + 3u * U.x0) & 7) == 0;  // !WORDS
    long long ooff = ((long long)(n0 - 1) * W + xl) * 3;
    // the HQLI variant (red / blue site column, red row) of even and odd output rows
    const bool rr_e = po.r_row == 0;
    const int v_e = 2 * (rr_e ? po.r_col : po.b_col) + (rr_e ? 1 : 0);
    const int v_o = 2 * (rr_e ? po.b_col : po.r_col) + (rr_e ? 0 : 1);
    // rows n0 .. n0 + kDirRing - 2 on their way (one commit group per row, empty past the unit's
    // rows, so that the group of row k is always kDirRing - 1 groups before the newest)
    const uint32_t main0 = ptx::smem_u32(&ring[0][lane]), edge0 = ptx::smem_u32(&ring_e[0][lane]);
    constexpr uint32_t kMainStep = sizeof(ring[0]), kEdgeStep = sizeof(ring_e[0]);
#pragma unroll
    for (int r = 0; r < kDirRing - 1; r++) {
        if (r < nrows) src.issue(fp, n0 + r, main0 + r * kMainStep, edge0 + r * kEdgeStep);
        ptx::cp_async_commit();
    }
    lite::Row Ur, Mr, Dr;  // rows n - 2, n - 1, n of the lane
    // the owner's claim of the segment's next band is in flight a band ahead of its use (lane 0
    // holds the counter's old value), so the warp never waits for the atomic
    unsigned long long pend = 0;
    if (own && lane == 0) pend = atomicAdd(own, segs::kFrontOne);
#pragma unroll 1
    for (int k = 0; k < nrows; k++) {
        const int n = n0 + k;
        if (own && k + kDirRing - 1 == nrows) {
            // the segment's next band continues this stream
            int j = 0;
            if (lane == 0) j = segs::settle_front(pend, bl.seg_words + bl.n_items);
            j = __shfl_sync(full, j, 0);
            if (j >= 0) {
                int yb, hb;
                segs::band_of(U.s0, U.len, U.nb, j, yb, hb);
                nrows += hb;
                if (lane == 0) pend = atomicAdd(own, segs::kFrontOne);
            } else {
                own = nullptr;
            }
        }
        // row n + kDirRing - 1 into the slot row n - 1 left, then row n's copies complete
        const int ahead = (k + kDirRing - 1) & (kDirRing - 1);
        if (k + kDirRing - 1 < nrows) src.issue(fp, n + kDirRing - 1, main0 + ahead * kMainStep, edge0 + ahead * kEdgeStep);
        ptx::cp_async_commit();
        ptx::cp_async_wait<kDirRing - 1>();
        const int slot = k & (kDirRing - 1);
        uint32_t w[4];
        rows::Edge<FMT> e;
        src.read(fp, n, ring[slot][lane], ring_e[slot][lane], w, e);
        uint32_t P[4];
        rows::decode8<FMT>(w, P);
        int nb = lane == 0 ? rows::decode_edge<FMT, true>(e) : rows::decode_edge<FMT, false>(e);
        lite_levels<FMT>(fp, L, po, n, lane, P, nb);
        uint32_t Lw = __shfl_up_sync(full, P[3], 1) & 0xFFFF0000u;
        uint32_t Rn = __shfl_down_sync(full, P[0], 1) & 0xFFFFu;
        if (lane == 0) Lw = (uint32_t)nb << 16;
        if (lane == 31) Rn = (uint32_t)nb;
        Ur = Mr;
        Mr = Dr;
#pragma unroll
        for (int j = 0; j < 4; j++) Dr.P[j] = P[j];
        Dr.Lw = Lw;
        Dr.R = Rn;
        const int yo = n - 1;  // rows 0, 1 / h-2, h-1 are emitted with row 2 / h-3
        if (k >= 2 && yo >= 2 && yo <= H - 3) {
            uint32_t ob[6];
            const int v = (yo & 1) ? v_o : v_e;
            if (FMT == FMT_U8) {
                if (v == 0) lite::hqli_row_t<0, false>(Ur, Mr, Dr, tab, ob);
                else if (v == 1) lite::hqli_row_t<0, true>(Ur, Mr, Dr, tab, ob);
                else if (v == 2) lite::hqli_row_t<1, false>(Ur, Mr, Dr, tab, ob);
                else lite::hqli_row_t<1, true>(Ur, Mr, Dr, tab, ob);
            } else {
                if (v == 0) lite::hqli_row<0, false>(Ur, Mr, Dr, tab.t1, ob);
                else if (v == 1) lite::hqli_row<0, true>(Ur, Mr, Dr, tab.t1, ob);
                else if (v == 2) lite::hqli_row<1, false>(Ur, Mr, Dr, tab.t1, ob);
                else lite::hqli_row<1, true>(Ur, Mr, Dr, tab.t1, ob);
            }
            // one phase for all rows unless WORDS
            const int phase = WORDS ? (int)((reinterpret_cast<uintptr_t>(out) + (uintptr_t)ooff) & 7) : 0;
            if ((WORDS ? interior && (phase & 1) == 0 : fast) && yo != 2 && yo != H - 3) {
                if (lane_st) {
                    uint8_t* q = out + ooff;
                    if (!WORDS || phase == 0) {
                        uint2* q2 = reinterpret_cast<uint2*>(q);
                        q2[0] = make_uint2(ob[0], ob[1]);
                        q2[1] = make_uint2(ob[2], ob[3]);
                        q2[2] = make_uint2(ob[4], ob[5]);
                    } else if (phase == 4) {
                        uint32_t* q4 = reinterpret_cast<uint32_t*>(q);
#pragma unroll
                        for (int w = 0; w < 6; w++) q4[w] = ob[w];
                    } else {
                        // two bytes, five words from the next word boundary on, two bytes
                        reinterpret_cast<uint16_t*>(q)[0] = (uint16_t)(ob[0] & 0xFFFFu);
                        uint32_t* q4 = reinterpret_cast<uint32_t*>(q + 2);
#pragma unroll
                        for (int w = 0; w < 5; w++) q4[w] = __funnelshift_r(ob[w], ob[w + 1], 16);
                        reinterpret_cast<uint16_t*>(q + 22)[0] = (uint16_t)(ob[5] >> 16);
                    }
                }
            } else {
                lite_emit_staged(tab.t1, wout, out, W, H, U.x0, U.npx, lane, yo, make_uint4(ob[0], ob[1], ob[2], ob[3]),
                                 make_uint2(ob[4], ob[5]));
            }
        }
        ooff += 3 * W;
    }
}

template <int FMT, bool WORDS>
__global__ void __launch_bounds__(kDirThreads, 1) lite_direct_kernel(const __grid_constant__ BatchLaunch bl) {
    extern __shared__ __align__(16) uint8_t dsm[];
    auto& sm = *reinterpret_cast<LiteDirectSmem<FMT>*>(dsm);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nseg = bl.n_items;
    const int gw = (int)blockIdx.x * kDirWarps + warp;
    {
        // tables of the launch, as in the staged variant; the tone table first comes into the
        // warps' staging rows by 16-byte loads (its buffer holds at least 4096 bytes)
        const FrameParams& f0 = bl.frames[0];
        const int mv = f0.mv, nv = mv + 1;
        const bool wb_rgb = (f0.stages & 8u) && f0.stage_order == 1;
        uint8_t* tone_s = &sm.out[0][0];
        for (int i = threadIdx.x; i < (nv + 15) / 16; i += kDirThreads)
            reinterpret_cast<uint4*>(tone_s)[i] = __ldg(reinterpret_cast<const uint4*>(f0.tone8) + i);
        __syncthreads();
#pragma unroll 1
        for (int c = 0; c < 3; c++) {
            const float g = f0.wb_rgb[c];
            for (int v = threadIdx.x; v < nv; v += kDirThreads) sm.tab.t1[c][v] = tone_s[wb_rgb ? dev::gain_round(v, g, mv) : v];
        }
        __syncthreads();
        // the replicated tables (u8), four entries per word: t2 words hold t1[2w], t1[2w], t1[2w+1],
        // t1[2w+1]; t4 words four copies of t1[w] (nv is a power of two, 2 to 256)
#pragma unroll 1
        for (int c = 0; c < (FMT == FMT_U8 ? 3 : 0); c++) {
            uint32_t* t2 = reinterpret_cast<uint32_t*>(sm.tab.t2[c]);
            uint32_t* t4 = reinterpret_cast<uint32_t*>(sm.tab.t4[c]);
            for (int w = threadIdx.x; w < nv / 2; w += kDirThreads)
                t2[w] = (uint32_t)sm.tab.t1[c][2 * w] * 0x0101u | (uint32_t)sm.tab.t1[c][2 * w + 1] * 0x01010000u;
            for (int w = threadIdx.x; w < nv; w += kDirThreads) t4[w] = (uint32_t)sm.tab.t1[c][w] * 0x01010101u;
        }
    }
    __syncthreads();
    segs::wait_init();
    uint8_t* wout = sm.out[warp];
    // the warp's own segment (its band 0 claimed for it by the init kernel), band after band from
    // the front, then bands from the back of others
    segs::Walk walk(gw, nseg, (int)gridDim.x * kDirWarps, bl.owners);
    int seg, band, nbands;
    bool own;
    while (walk.next(bl.seg_words, nseg, gw, lane, seg, band, nbands, own)) {
        LSeg S;
        lseg_of(bl, seg, S);
        // a segment of one band is taken with the claim made for its warp
        if (seg < bl.owners && band == 0 && S.nb == 1 && lane == 0) atomicAdd(bl.seg_words + nseg, 1ull);
        // bands band .. band + nbands - 1: contiguous rows
        int y0, bh, yl, hl;
        segs::band_of(S.s0, S.len, S.nb, band, y0, bh);
        segs::band_of(S.s0, S.len, S.nb, band + nbands - 1, yl, hl);
        bh = yl + hl - y0;
        direct_unit<FMT, WORDS>(bl, sm.tab, wout, sm.ring[warp], sm.ring_e[warp], S, y0, bh,
                                own ? bl.seg_words + seg : nullptr,
                         lane);
    }
}

// the launch's claim words: each segment's band count with zero claims, then the taken count
__global__ void lite_seg_init_kernel(const __grid_constant__ BatchLaunch bl) {
    segs::release_dependents();
    const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i < bl.n_items) {
        LSeg G;
        lseg_of(bl, i, G);
        bl.seg_words[i] = segs::initial_word(G.nb) + (i < bl.owners ? segs::kFrontOne : 0ull);
    } else if (i == bl.n_items) {
        bl.seg_words[i] = 0ull;
    }
}

int g_direct_grid[kMaxDev];

template <int FMT, bool WORDS>
cudaError_t launch_direct_fmt(const BatchLaunch& bl, int grid, cudaStream_t st) {
    return launch_dependent(lite_direct_kernel<FMT, WORDS>, grid, kDirThreads, direct_smem<FMT>(), st, bl);
}

int g_lite_grid[kMaxDev];

template <int FMT>
cudaError_t launch_fmt(const BatchLaunch& bl, int grid, size_t smem, cudaStream_t st) {
    lite_batch_kernel<FMT><<<grid, kThreads, smem, st>>>(bl);
    return cudaGetLastError();
}

}  // namespace

bool lite_eligible(const FrameParams& fp) {
    const bool fmt_ok = fp.fmt == FMT_U8 || fp.fmt == FMT_U16 || (fp.fmt == FMT_P12 && (fp.w & 1) == 0) ||
                        (fp.fmt == FMT_P10 && (fp.w & 3) == 0);
    // integral black levels (one add-min-relu per sample), and samples no larger than the bit depth's
    // maximum when they reach the demosaic (a stage clamps them, the MSB-aligned u16 read, a packed
    // format, or full 8-bit bytes), so HQLI needs no clamps
    bool bl_ok = !(fp.stages & 1u) || fp.bl_int;
    for (int c = 0; c < 4; c++) bl_ok = bl_ok && (!(fp.stages & 1u) || fp.bl[c] <= (float)fp.mv);
    const bool bounded =
        (fp.stages & 1u) || ((fp.stages & 8u) && fp.stage_order == 0) || fp.fmt != FMT_U8 || fp.bd == 8;
    return fmt_ok && bl_ok && bounded && fp.bd <= 12 && fp.demosaic == DM_HQLI &&
           !(fp.stages & (2u | 4u | 16u | 32u)) && fp.out_format == 0 && fp.out_bpc == 1 && fp.w >= 6 && fp.h >= 6;
}

// frames of one launch share their output tables: same tone table, white-balance order and RGB gains
long long lite_table_key(const FrameParams& fp) {
    const bool wb_rgb = (fp.stages & 8u) && fp.stage_order == 1;
    uint64_t h = (uint64_t)reinterpret_cast<uintptr_t>(fp.tone8) * 0x9E3779B97F4A7C15ull;
    h ^= wb_rgb ? 1u : 0u;
    if (wb_rgb)
        for (int c = 0; c < 3; c++) {
            uint32_t b;
            std::memcpy(&b, &fp.wb_rgb[c], 4);
            h = (h ^ b) * 0xBF58476D1CE4E5B9ull;
        }
    return (long long)(h >> 8);
}

int lite_units_x(int w) { return lite_strips(w); }
int lite_units_y(int h, int band_rows) { return tiles_along(h, band_rows); }

// frames the direct-read variant takes: rows that start on a word (the input word-aligned, and a
// width that is a multiple of 8 for the MIPI formats, even for u16, a multiple of 4 for u8), claim
// words
static bool direct_ok(const FrameParams& fp) {
    const int wmul = fp.fmt == FMT_U16 ? 2 : fp.fmt == FMT_U8 ? 4 : 8;
    return fp.w % wmul == 0 && (reinterpret_cast<uintptr_t>(fp.in) & 3) == 0 && fp.seg_words &&
           fp.seg_cap >= kStreamSegCap;
}
// u8 / u16 frames whose lanes' 8- / 16-byte loads do not all start on their size: word copies
static bool needs_words(const FrameParams& fp) {
    return (fp.fmt == FMT_U8 || fp.fmt == FMT_U16) && (fp.w % 8 != 0 || (reinterpret_cast<uintptr_t>(fp.in) & 15) != 0);
}

static cudaError_t launch_direct(const BatchLaunch& bl_in, cudaStream_t st) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDev) return cudaErrorInvalidDevice;
    int limit;
    {
        std::lock_guard<std::mutex> lock(device_setup_mutex());
        if (!g_direct_grid[dev]) {
            void (*ks[6])(BatchLaunch) = {lite_direct_kernel<FMT_U8, false>,  lite_direct_kernel<FMT_U16, false>,
                                          lite_direct_kernel<FMT_P10, false>, lite_direct_kernel<FMT_P12, false>,
                                          lite_direct_kernel<FMT_U8, true>,   lite_direct_kernel<FMT_U16, true>};
            const size_t sm[6] = {direct_smem<FMT_U8>(),  direct_smem<FMT_U16>(), direct_smem<FMT_P10>(),
                                  direct_smem<FMT_P12>(), direct_smem<FMT_U8>(),  direct_smem<FMT_U16>()};
            for (int k = 0; k < 6 && e == cudaSuccess; k++)
                e = cudaFuncSetAttribute(ks[k], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm[k]);
            // every variant holds one CTA per SM (24 warps at 80 registers); the largest sets the grid
            int n = 0, m = 0;
            if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ks[0], kDirThreads, sm[0]);
            if (e == cudaSuccess) e = cudaDeviceGetAttribute(&m, cudaDevAttrMultiProcessorCount, dev);
            if (e != cudaSuccess) return e;
            g_direct_grid[dev] = m * (n > 0 ? n : 1);
        }
        limit = g_direct_grid[dev];
    }
    BatchLaunch bl = bl_in;
    int wmax = 0;
    for (int f = 0; f < bl.n_frames; f++) wmax = std::max(wmax, bl.frames[f].w);
    const TuneParams tp = tuning_for(IMOP_KERNEL_LITE, bl.fmt, wmax);
    if (!choose_segments(bl, limit * kDirWarps, tp.seg_percent, tp.band_rows)) return cudaErrorNotSupported;
    if (bl.n_items <= 0) return cudaSuccess;
    if (bl.n_items > kSegMax) return cudaErrorInvalidValue;
    bl.seg_words = bl.frames[0].seg_words;
    // every SM once the launch has work for half of them (warps without a segment of their own
    // take bands from the others from the start); fewer CTAs for a small launch
    const int want = (bl.n_items + kDirWarps - 1) / kDirWarps;
    const int grid = want >= limit / 2 ? limit : want;
    bl.owners = grid * kDirWarps;  // every warp starts on its own segment's band 0
    lite_seg_init_kernel<<<(bl.n_items + 256) / 256, 256, 0, st>>>(bl);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    count_launch(IMOP_KERNEL_LITE);
    count_launch(IMOP_KERNEL_LITE_DIRECT);
    bool words = false;  // word copies, stores by the rows' phases
    for (int f = 0; f < bl.n_frames; f++) words = words || needs_words(bl.frames[f]);
    switch (bl.fmt) {
        case FMT_U8: return words ? launch_direct_fmt<FMT_U8, true>(bl, grid, st)
                                  : launch_direct_fmt<FMT_U8, false>(bl, grid, st);
        case FMT_U16: return words ? launch_direct_fmt<FMT_U16, true>(bl, grid, st)
                                   : launch_direct_fmt<FMT_U16, false>(bl, grid, st);
        case FMT_P10: return launch_direct_fmt<FMT_P10, false>(bl, grid, st);
        case FMT_P12: return launch_direct_fmt<FMT_P12, false>(bl, grid, st);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_lite(const BatchLaunch& bl, cudaStream_t st) {
    bool direct = bl.n_frames > 0;
    for (int f = 0; f < bl.n_frames; f++)
        direct = direct && direct_ok(bl.frames[f]) && bl.frames[f].seg_words == bl.frames[0].seg_words;
    if (direct) {
        const cudaError_t e = launch_direct(bl, st);
        if (e != cudaErrorNotSupported) return e;  // else more strips than claim words: the staged variant
    }
    const size_t smem = sizeof(LiteSmem);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDev) return cudaErrorInvalidDevice;
    int limit;
    {
        std::lock_guard<std::mutex> lock(device_setup_mutex());
        if (!g_lite_grid[dev]) {
            void (*ks[4])(BatchLaunch) = {lite_batch_kernel<FMT_U8>, lite_batch_kernel<FMT_U16>,
                                          lite_batch_kernel<FMT_P10>, lite_batch_kernel<FMT_P12>};
            for (int k = 0; k < 4 && e == cudaSuccess; k++)
                e = cudaFuncSetAttribute(ks[k], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            int n = 0, m = 0;
            if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ks[1], kThreads, smem);
            if (e == cudaSuccess) e = cudaDeviceGetAttribute(&m, cudaDevAttrMultiProcessorCount, dev);
            if (e != cudaSuccess) return e;
            g_lite_grid[dev] = m * (n > 0 ? n : 1);
        }
        limit = g_lite_grid[dev];
    }
    if (bl.n_items <= 0) return cudaSuccess;
    if ((e = cudaMemsetAsync(bl.tile_counter, 0, sizeof(int), st)) != cudaSuccess) return e;
    // enough CTAs that every warp has a unit, at most the resident limit
    const int want = (bl.n_items + kLiteWarps - 1) / kLiteWarps;
    const int grid = want < limit ? want : limit;
    count_launch(1);
    switch (bl.fmt) {
        case FMT_U8: return launch_fmt<FMT_U8>(bl, grid, smem, st);
        case FMT_U16: return launch_fmt<FMT_U16>(bl, grid, smem, st);
        case FMT_P10: return launch_fmt<FMT_P10>(bl, grid, smem, st);
        case FMT_P12: return launch_fmt<FMT_P12>(bl, grid, smem, st);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace imop
