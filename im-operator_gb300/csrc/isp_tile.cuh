// isp_tile.cuh - one output tile of the fused RAW->RGB pipeline (sm_103a).
//
// A CTA of 256 threads owns a tw x th tile of output pixels and works on horizontal pixel pairs
// (x even, x+1).  In every Bayer row a pair holds exactly one green and one red/blue site, so the
// demosaic code is the same for every thread (no CFA-colour divergence).
//
//   stage   region (radius around the tile)   storage
//   raw     rows +-5, columns +-6            bytes, one 1-D TMA bulk copy per row (mbarrier);
//                                            two buffers, so the next tile is staged while this
//                                            one is computed
//   orig    rows +-5, columns +-6            int per pixel: unpacked, black-levelled
//   bay     rows +-3, columns +-4            int per pixel: defect-corrected (Jacobi), LSC, WB
//   green   rows +-1, columns +-2            f32 per pair: green at the pair's red/blue site
//                                            (in the tile's raw buffer, free after unpacking)
//   out     the tile                         bytes, shifted to the output's 16-byte phase
//                                            (in the orig plane, free after the seed check)
//
// Output (x,y) needs demosaic inputs within 1 (HQLI) or, through green, 3 pixels (AMAZE, MG);
// defect correction reads 2 more.  Border pixels copy from pixels at most 2 away (border_source),
// which lie in the same tile because every tile is at least 4 pixels wide and high.
//
// Tiles whose whole apron lies inside the frame with margin take a specialisation (FULL) with
// compile-time extents and no bounds checks; frame-edge tiles, ragged last tiles and the defect
// fix-up windows take the general path.
#pragma once

#include "isp_device.cuh"
#include "isp_ptx.cuh"

namespace imop {

constexpr int kThreads = 256;

// tile grid along one axis: n tiles of `t` pixels, the last absorbing a remainder below 4
__host__ __device__ inline int tiles_along(int extent, int t) {
    int n = (extent + t - 1) / t;
    int rem = extent - (n - 1) * t;
    if (n > 1 && rem < 4) n--;
    return n;
}
__host__ __device__ inline void tile_span(int extent, int t, int n, int i, int& start, int& len) {
    start = i * t;
    len = (i == n - 1) ? extent - start : t;
}

// sorted override list lookup (defect-chain fix-up): value or -1
__device__ __forceinline__ int find_override(const int* ov_idx, const int* ov_val, int n, int key) {
    int lo = 0, hi = n - 1;
    while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        int v = ov_idx[mid];
        if (v == key) return ov_val[mid];
        if (v < key) lo = mid + 1;
        else hi = mid - 1;
    }
    return -1;
}

// map-mode lookup: resolved value of map pixel (x,y) or -1
__device__ __forceinline__ int map_lookup(const FrameParams& fp, int x, int y) {
    int lo = __ldg(fp.map_row_ptr + y), hi = __ldg(fp.map_row_ptr + y + 1) - 1;
    while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        int2 e = fp.map_ent[mid];
        if (e.x == x) return fp.map_val[e.y];
        if (e.x < x) lo = mid + 1;
        else hi = mid - 1;
    }
    return -1;
}

struct Overrides {
    const int* idx;
    const int* val;
    int n;
};

__host__ __device__ constexpr int cmax(int a, int b) { return a > b ? a : b; }
__host__ __device__ constexpr int round16(int a) { return (a + 15) / 16 * 16; }

template <int TW, int TH, int OUTB>
struct TileGeom {
    static_assert(TW % 2 == 0, "tile width must be even");
    static constexpr int TWM = TW + 3, THM = TH + 3;  // a merged last tile
    static constexpr int TWP = (TWM + 1) / 2;         // pairs of own pixels
    static constexpr int OPW = TWP + 6, ORH = THM + 10, OW = 2 * OPW;
    static constexpr int BPW = TWP + 4, BRH = THM + 6, BW = 2 * BPW;
    static constexpr int GPW = TWP + 2, GRH = THM + 2;
    static constexpr int RAW_PITCH = round16(4 * OPW + 32);
    static constexpr int OUT_PITCH = round16(TWM * OUTB + 16);
    static constexpr int RAW_BYTES = cmax(ORH * RAW_PITCH, GRH * GPW * 4);
    static constexpr int B_BYTES = cmax(ORH * OW * 4, THM * OUT_PITCH);
    // region extents of a full (nominal) tile, in pairs / rows
    static constexpr int F_OPW = (TW + 13) / 2, F_OH = TH + 10;
    static constexpr int F_BPW = (TW + 9) / 2, F_BH = TH + 6;
    static constexpr int F_GPW = (TW + 5) / 2, F_GH = TH + 2;
    static constexpr int F_TPW = (TW + 1) / 2;
    // full tiles give every warp one of two blocks of 32 pair columns
    static_assert(F_BPW <= 64 && F_GPW <= 64 && F_TPW <= 64, "full-tile loops cover two blocks of 32 pair columns");
};

template <int TW, int TH, int OUTB>
struct TileSmem {
    using G = TileGeom<TW, TH, OUTB>;
    alignas(16) uint8_t raw[2][G::RAW_BYTES];  // raw staging; green of the computed tile reuses it
    alignas(16) uint8_t regB[G::B_BYTES];      // orig samples (int per pixel), then output staging
    alignas(16) int bay[G::BRH * G::BW];       // samples after defect correction, lens shading, WB
    alignas(16) uint8_t tone8[4096];           // tone table (bit depth <= 12)
    alignas(16) FrameParams fp[2];             // parameters of the frame of each staged tile
    uint8_t mod[G::BRH * G::BPW];              // bit h: pixel h of the pair was corrected
    int row_a0[2][G::ORH];                     // staged byte window [a0, a0 + len) of each raw row
    int row_len[2][G::ORH];
    int row_base[2][G::ORH];                   // staged offset of the region's first pair, or -1
    int col_gx[2 * G::BPW];
    float col_fx[2 * G::BPW];
    int row_gy[G::BRH];
    float row_fy[G::BRH];
    int tile[2][4];                            // x0, y0, tw, th of each staged tile
    int next_item[2];                          // item staged into each buffer (>= n_items: none)
    const uint8_t* tone_src;                   // the tone table held in tone8
    alignas(8) uint64_t bar[2];
};

// ---- small helpers -----------------------------------------------------------------------------
// byte range [b0, b1) of pixels [i0, i1) (pixel indices) in the input stream
__device__ __forceinline__ void pixel_bytes(int fmt, int bd, int i0, int i1, int& b0, int& b1) {
    switch (fmt) {
        case FMT_U8: b0 = i0; b1 = i1; break;
        case FMT_U16: b0 = 2 * i0; b1 = 2 * i1; break;
        case FMT_P12: b0 = 3 * (i0 >> 1); b1 = 3 * ((i1 - 1) >> 1) + 3; break;
        case FMT_P10: b0 = 5 * (i0 >> 2); b1 = 5 * ((i1 - 1) >> 2) + 5; break;
        default: b0 = (int)(((long long)i0 * bd) >> 3); b1 = (int)(((long long)i1 * bd + 7) >> 3); break;
    }
}

// sample at bit `shift` of the staged bytes from `rel` on (8 bytes readable there), bit stream
// formats
__device__ __forceinline__ int bits_at(const uint8_t* row, int rel, int shift, int mv) {
    const int o4 = rel & ~3;
    const uint32_t w0 = *reinterpret_cast<const uint32_t*>(row + o4);
    const uint32_t w1 = *reinterpret_cast<const uint32_t*>(row + o4 + 4);
    return (int)((__funnelshift_r(w0, w1, 8 * (rel & 3)) >> shift) & (uint32_t)mv);
}

// one raw byte of the staged row (or of global memory past the staged window)
__device__ __forceinline__ int staged_byte(const FrameParams& fp, int a0, int len, const uint8_t* row, int off) {
    int rel = off - a0;
    if (rel >= 0 && rel < len) return row[rel];
    return __ldg(fp.in + off);
}

// unpacked sample of pixel index i of a staged row; the packed-tail rule of
// pixel::get_packed_raw (a group ending at or past the buffer end reads 0) is kept
__device__ __forceinline__ int staged_raw(const FrameParams& fp, int a0, int len, const uint8_t* row, int i) {
    switch (fp.fmt) {
        case FMT_U8: return staged_byte(fp, a0, len, row, i);
        case FMT_U16: return staged_byte(fp, a0, len, row, 2 * i) | (staged_byte(fp, a0, len, row, 2 * i + 1) << 8);
        case FMT_P12: {
            int off = (i >> 1) * 3;
            if (off + 2 >= (int)fp.in_bytes) return 0;
            int b1 = staged_byte(fp, a0, len, row, off + 1);
            if ((i & 1) == 0) return ((staged_byte(fp, a0, len, row, off) << 4) | (b1 & 0xF)) & fp.mv;
            return ((staged_byte(fp, a0, len, row, off + 2) << 4) | (b1 >> 4)) & fp.mv;
        }
        case FMT_P10: {
            int off = (i >> 2) * 5;
            int sub = i & 3;
            if (off + 4 >= (int)fp.in_bytes) return 0;
            int b = staged_byte(fp, a0, len, row, off + sub), b4 = staged_byte(fp, a0, len, row, off + 4);
            return ((b << 2) | ((b4 >> (2 * sub)) & 3)) & fp.mv;
        }
        default: {
            const long long bit = (long long)i * fp.bd;
            const int off = (int)(bit >> 3), shift = (int)(bit & 7);
            if (off >= (int)fp.in_bytes) return 0;
            const int n = min((fp.bd + shift + 7) >> 3, (int)fp.in_bytes - off);
            uint32_t v = 0;
            for (int k = 0; k < n; k++) v |= (uint32_t)staged_byte(fp, a0, len, row, off + k) << (8 * k);
            return (int)((v >> shift) & (uint32_t)fp.mv);
        }
    }
}

// MIPI RAW12 pair from its three bytes (b0 | b1 << 8 | b2 << 16): p0 = b0<<4 | b1&15, p1 = b2<<4 | b1>>4
__device__ __forceinline__ uint32_t unpack12_pair(uint32_t v) {
    uint32_t hi8 = __byte_perm(v, 0u, 0x4240u);           // b0 | b2 << 16
    uint32_t b1 = __byte_perm(v, 0u, 0x4141u);            // b1 | b1 << 16
    return (hi8 << 4) | (b1 & 0x0000000Fu) | ((b1 >> 4) & 0x000F0000u);
}

// scalar defect kernel on the orig plane (edges and the rare non-fast pixels)
template <class OrigAt>
__device__ __forceinline__ int dpc_scalar(const FrameParams& fp, OrigAt orig, int x, int y) {
    unsigned m = dev::dpc_valid_mask(x, y, fp.w, fp.h);
    int nb[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (m & 1u) nb[0] = orig(x - 2, y - 2);
    if (m & 2u) nb[1] = orig(x, y - 2);
    if (m & 4u) nb[2] = orig(x + 2, y - 2);
    if (m & 8u) nb[3] = orig(x - 2, y);
    if (m & 16u) nb[4] = orig(x + 2, y);
    if (m & 32u) nb[5] = orig(x - 2, y + 2);
    if (m & 64u) nb[6] = orig(x, y + 2);
    if (m & 128u) nb[7] = orig(x + 2, y + 2);
    return dev::dpc_apply(orig(x, y), nb, m, fp.dpc_thr);
}

// bounded wait on a staging barrier (about a second at most); false when it gave up
__device__ __forceinline__ bool wait_bar(uint64_t* bar, uint32_t parity) {
    for (uint32_t it = 0; it < (1u << 22); it++)
        if (ptx::mbar_try_wait(bar, parity)) return true;
    return false;
}

template <int TW, int TH, int OUTB>
__device__ void tile_init(TileSmem<TW, TH, OUTB>& sm) {
    if (threadIdx.x == 0) {
        ptx::mbar_init(&sm.bar[0], 1);
        ptx::mbar_init(&sm.bar[1], 1);
        ptx::fence_mbar_init();
        sm.tone_src = nullptr;
    }
    __syncthreads();
}

// A tile with the nominal extents whose raw apron, defect apron and demosaic support lie inside
// the frame with margin (and whose packed rows start on a pair boundary): no bounds checks.
template <int TW, int TH>
__device__ __forceinline__ bool tile_is_full(const FrameParams& fp, int x0, int y0, int tw, int th) {
    const bool even_rows = fp.fmt == FMT_U8 || fp.fmt == FMT_U16 || fp.fmt == FMT_PBITS || (fp.w & 1) == 0;
    return tw == TW && th == TH && x0 >= 8 && y0 >= 8 && x0 + TW + 8 <= fp.w && y0 + TH + 8 <= fp.h && even_rows;
}

// green value of a pixel inside the green region: the stored red/blue-site green, or the
// green-site sample (AMAZE only inside the interior; MG everywhere)
struct GreenAt {
    const float* green;
    const int* bay;
    int xg0, yg0, xb, yb, gpitch, bpitch, W, H, r_row, r_col, b_col, mg;
    __device__ __forceinline__ float operator()(int x, int y) const {
        int rbh = ((y & 1) == r_row) ? r_col : b_col;
        if ((x & 1) == rbh) return green[(y - yg0) * gpitch + ((x - xg0) >> 1)];
        bool interior = x >= 2 && x < W - 2 && y >= 2 && y < H - 2;
        if (!(interior || mg)) return -1.0f;
        return (float)bay[(y - yb) * bpitch + (x - xb)];
    }
};

__device__ __forceinline__ int u16q(float t, int mv) { return (int)min(__float2uint_rz(t), (unsigned)mv); }

// bytes [a, b) of one 16-byte window (dst and src agree modulo 16): naturally aligned 1/2/4/8-byte
// pieces, rising to the window's alignment and then falling to its end
__device__ __forceinline__ void store_piece(uint8_t* dst, const uint8_t* src, int a, int b) {
    int q = a;
    if ((q & 1) && q + 1 <= b) { dst[q] = src[q]; q += 1; }
    if ((q & 2) && q + 2 <= b) { *reinterpret_cast<uint16_t*>(dst + q) = *reinterpret_cast<const uint16_t*>(src + q); q += 2; }
    if ((q & 4) && q + 4 <= b) { *reinterpret_cast<uint32_t*>(dst + q) = *reinterpret_cast<const uint32_t*>(src + q); q += 4; }
    if ((q & 8) && q + 8 <= b) { *reinterpret_cast<uint2*>(dst + q) = *reinterpret_cast<const uint2*>(src + q); q += 8; }
    for (; q + 8 <= b; q += 8) *reinterpret_cast<uint2*>(dst + q) = *reinterpret_cast<const uint2*>(src + q);
    if (q + 4 <= b) { *reinterpret_cast<uint32_t*>(dst + q) = *reinterpret_cast<const uint32_t*>(src + q); q += 4; }
    if (q + 2 <= b) { *reinterpret_cast<uint16_t*>(dst + q) = *reinterpret_cast<const uint16_t*>(src + q); q += 2; }
    if (q < b) dst[q] = src[q];
}

// ---- staging (warp 0): row windows of buffer b, bulk copies completing on bar[b] ----------------
// sm.fp[b] holds the tile's frame parameters.  With an input pointer that is not 16-byte aligned
// nothing is copied here: compute_tile copies the same windows with plain loads.
template <int TW, int TH, int OUTB>
__device__ void stage_tile(TileSmem<TW, TH, OUTB>& sm, int b, int x0, int y0, int tw, int th) {
    using G = TileGeom<TW, TH, OUTB>;
    const FrameParams& fp = sm.fp[b];
    const int lane = threadIdx.x & 31;
    const int W = fp.w, H = fp.h;
    const int xo = x0 - 6, yo = y0 - 5;
    const int opw = (tw + 13) / 2, oh = th + 10;
    const int in16 = (int)(fp.in_bytes & ~(size_t)15);
    const bool bulk_ok = ((reinterpret_cast<uintptr_t>(fp.in) & 15) == 0);
    uint32_t bytes = 0;
    for (int r = lane; r < oh; r += 32) {
        int y = yo + r;
        int a0 = 0, len = 0, base = -1;
        if (y >= 0 && y < H) {
            int xs = max(0, xo), xe = min(W, xo + 2 * opw);
            int b0, b1;
            pixel_bytes(fp.fmt, fp.bd, y * W + xs, y * W + xe, b0, b1);
            b1 = min(b1, (int)fp.in_bytes);
            a0 = b0 & ~15;
            int a1 = min((b1 + 15) & ~15, in16);
            len = max(a1 - a0, 0);
            int i = y * W + xo;  // pixel index of the region's first pair (may lie left of the frame)
            switch (fp.fmt) {
                case FMT_U8: base = i - a0; break;
                case FMT_U16: base = 2 * i - a0; break;
                case FMT_P12: base = ((i & 1) == 0) ? 3 * (i >> 1) - a0 : -1; break;
                case FMT_P10: base = ((i & 1) == 0) ? 5 * (i >> 2) - a0 : -1; break;
                default: base = -1; break;  // bit streams: per-sample offsets (full tiles only)
            }
        }
        sm.row_a0[b][r] = a0;
        sm.row_len[b][r] = len;
        sm.row_base[b][r] = base;
        bytes += (uint32_t)len;
    }
    if (lane == 0) {
        sm.tile[b][0] = x0;
        sm.tile[b][1] = y0;
        sm.tile[b][2] = tw;
        sm.tile[b][3] = th;
    }
    if (!bulk_ok) return;
    for (int o = 16; o > 0; o >>= 1) bytes += __shfl_xor_sync(0xffffffffu, bytes, o);
    if (lane == 0) ptx::mbar_arrive_expect_tx(&sm.bar[b], bytes);
    __syncwarp();
    for (int r = lane; r < oh; r += 32) {
        int n = sm.row_len[b][r];
        if (n > 0) ptx::bulk_g2s(sm.raw[b] + r * G::RAW_PITCH, fp.in + sm.row_a0[b][r], (uint32_t)n, &sm.bar[b]);
    }
}

// ---- compute one staged tile (all threads) ------------------------------------------------------
// `parity` is buffer b's barrier phase, flipped when its bytes are consumed.  Returns false, the
// same on every thread, when the staged bytes never arrived (the status word is set).
// EXTRA = false leaves out the bit-stream unpack and the 3D LUT, DM != 0 fixes the demosaic
// algorithm, SPEC != 0 fixes the input format (SPEC & 7 = format + 1) and, with SPEC & 8, the
// common stage configuration (adaptive or no defect correction, no polynomial shading, RGB8
// output; white balance in either order); SPEC & 16 also leaves out defect correction and lens
// shading (frames that use neither): a launch whose frames allow it runs a copy of the kernel
// without the other paths' code (unused paths cost the kernel through its instruction footprint:
// ~2 % for the 3D LUT alone, ~5 % for all of them on a C2 batch)
template <int TW, int TH, int OUTB, bool FULL, bool EXTRA = true, int DM = 0, int SPEC = 0>
__device__ bool compute_tile(TileSmem<TW, TH, OUTB>& sm, int b, Overrides ov, bool detect_seeds, uint32_t& parity) {
    using G = TileGeom<TW, TH, OUTB>;
    const FrameParams& fp = sm.fp[b];
    const int x0 = sm.tile[b][0], y0 = sm.tile[b][1];
    const int tw = FULL ? TW : sm.tile[b][2], th = FULL ? TH : sm.tile[b][3];
    const int W = fp.w, H = fp.h, mv = fp.mv;
    const PatternOffsets po = pattern_offsets(fp.pattern);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned stages = fp.stages;
    const bool dpc_on = !(SPEC & 16) && (stages & 2u) != 0;
    const bool adaptive = dpc_on && ((SPEC & 8) || fp.dpc_mode == 0);
    const int demosaic = DM ? DM : fp.demosaic;
    const int xo = x0 - 6, yo = y0 - 5;  // orig region origin (xo even)
    const int opw = FULL ? G::F_OPW : (tw + 13) / 2, oh = FULL ? G::F_OH : th + 10;
    const int xb = x0 - 4, yb = y0 - 3;  // bay region origin
    const int bpw = FULL ? G::F_BPW : (tw + 9) / 2, bh = FULL ? G::F_BH : th + 6;
    const int xg0 = x0 - 2, yg0 = y0 - 1;  // green region origin
    const int gpw = FULL ? G::F_GPW : (tw + 5) / 2, gh = FULL ? G::F_GH : th + 2;
    const int tpw = FULL ? G::F_TPW : (tw + 1) / 2;  // own pairs
    const bool tone_smem = fp.out_format == 0 && fp.bd <= 12;
    const float2 z2 = make_float2(fp.neg_zero, fp.neg_zero);  // addend of the packed products
    uint8_t* raw = sm.raw[b];

    // tone table (when the frame's table changed) and lens-shading tables, then the staged bytes
    if (tone_smem && sm.tone_src != fp.tone8) {
        int n = mv + 1;
        for (int k = tid * 4; k < n; k += kThreads * 4)
            *reinterpret_cast<uint32_t*>(sm.tone8 + k) = __ldg(reinterpret_cast<const uint32_t*>(fp.tone8 + k));
    }
    if (!(SPEC & 16) && (stages & 4u) && fp.lsc_mode == 0) {
        for (int c = tid; c < 2 * bpw; c += kThreads) {
            int x = min(max(xb + c, 0), W - 1);
            float gx_f = __fdiv_rn(dev::fmul((float)x, (float)(fp.gw - 1)), (float)(W - 1));
            int gx_i = dev::clampi(dev::ftoi(gx_f), 0, fp.gw - 2);
            sm.col_gx[c] = gx_i;
            sm.col_fx[c] = dev::fsub(gx_f, (float)gx_i);
        }
        for (int r = tid; r < bh; r += kThreads) {
            int y = min(max(yb + r, 0), H - 1);
            float gy_f = __fdiv_rn(dev::fmul((float)y, (float)(fp.gh - 1)), (float)(H - 1));
            int gy_i = dev::clampi(dev::ftoi(gy_f), 0, fp.gh - 2);
            sm.row_gy[r] = gy_i;
            sm.row_fy[r] = dev::fsub(gy_f, (float)gy_i);
        }
    }
    bool arrived = true;
    if ((reinterpret_cast<uintptr_t>(fp.in) & 15) == 0) {
        arrived = wait_bar(&sm.bar[b], parity);
        parity ^= 1u;
    } else {
        // unaligned input pointer: threads copy the staged windows byte by byte
        __syncthreads();
        for (int r = 0; r < oh; r++) {
            int n = sm.row_len[b][r];
            for (int k = tid; k < n; k += kThreads) raw[r * G::RAW_PITCH + k] = __ldg(fp.in + sm.row_a0[b][r] + k);
        }
    }
    if (__syncthreads_or(!arrived)) {
        if (tid == 0) atomicExch(fp.status, 103 /* IMOP_ERR_TIMEOUT */);
        return false;
    }
    if (tid == 0 && tone_smem) sm.tone_src = fp.tone8;

    // ---- 2. unpack + black level -> orig samples (one int per pixel) ------------------------
    int* orig = reinterpret_cast<int*>(sm.regB);
    const bool bl_on = (stages & 1u) != 0;
    const bool bl_int = fp.bl_int != 0;
    const int fmt = (SPEC & 7) ? (SPEC & 7) - 1 : fp.fmt;
    constexpr int OPW_LOOP = FULL ? G::F_OPW : G::OPW;
    constexpr int OH_LOOP = FULL ? G::F_OH : G::ORH;
    for (int s = tid; s < OH_LOOP * OPW_LOOP; s += kThreads) {
        int r = s / OPW_LOOP, pc = s - r * OPW_LOOP;
        if (!FULL && (r >= oh || pc >= opw)) continue;
        int y = yo + r, x = xo + 2 * pc;
        int v0 = 0, v1 = 0;
        if (FULL || (y >= 0 && y < H)) {
            const uint8_t* row = raw + r * G::RAW_PITCH;
            const int base = sm.row_base[b][r], len = sm.row_len[b][r];
            const bool in0 = FULL || (x >= 0 && x < W), in1 = FULL || (x + 1 >= 0 && x + 1 < W);
            bool done = false;
            if (FULL || (in0 && in1 && base >= 0)) {
                if (fmt == FMT_P12) {
                    int off = base + 3 * pc;
                    if (FULL || (off >= 0 && off + 3 <= len)) {
                        int o4 = off & ~3;
                        uint32_t w0 = *reinterpret_cast<const uint32_t*>(row + o4);
                        uint32_t w1 = *reinterpret_cast<const uint32_t*>(row + o4 + 4);
                        uint32_t w = unpack12_pair(__funnelshift_r(w0, w1, 8 * (off & 3)));
                        v0 = (int)(w & 0xFFFFu);
                        v1 = (int)(w >> 16);
                        done = true;
                    }
                } else if (fmt == FMT_U16) {
                    int off = base + 4 * pc;
                    if (FULL || (off >= 0 && off + 4 <= len)) {
                        uint32_t w = ((off & 3) == 0) ? *reinterpret_cast<const uint32_t*>(row + off)
                                                      : (uint32_t)*reinterpret_cast<const uint16_t*>(row + off) |
                                                            ((uint32_t)*reinterpret_cast<const uint16_t*>(row + off + 2) << 16);
                        v0 = (int)(w & 0xFFFFu);
                        v1 = (int)(w >> 16);
                        done = true;
                    }
                } else if (fmt == FMT_U8) {
                    int off = base + 2 * pc;
                    if (FULL || (off >= 0 && off + 2 <= len)) {
                        v0 = row[off];
                        v1 = row[off + 1];
                        done = true;
                    }
                } else if (EXTRA && fmt == FMT_PBITS) {
                    // bit stream: each sample from its own bit offset (full tiles stage every
                    // byte the pair needs, and the row buffer has 8 readable bytes past it)
                    const long long bit0 = ((long long)y * W + x) * fp.bd;
                    const int a0r = sm.row_a0[b][r];
                    v0 = bits_at(row, (int)((bit0 >> 3) - a0r), (int)(bit0 & 7), mv);
                    const long long bit1 = bit0 + fp.bd;
                    v1 = bits_at(row, (int)((bit1 >> 3) - a0r), (int)(bit1 & 7), mv);
                    done = true;
                } else {
                    // MIPI RAW10: the pair is sample 0-1 or 2-3 of its 5-byte group
                    const int i = y * W + x;
                    const int goff = base + 5 * ((i >> 2) - ((y * W + xo) >> 2));
                    const int sub = i & 2;
                    if (FULL || (goff >= 0 && goff + 5 <= len)) {
                        const int b4 = row[goff + 4];
                        v0 = (row[goff + sub] << 2) | ((b4 >> (2 * sub)) & 3);
                        v1 = (row[goff + sub + 1] << 2) | ((b4 >> (2 * sub + 2)) & 3);
                        done = true;
                    }
                }
            }
            if (!FULL && !done) {
                const int i = y * W + x, a0 = sm.row_a0[b][r];
                if (in0) v0 = staged_raw(fp, a0, len, row, i);
                if (in1) v1 = staged_raw(fp, a0, len, row, i + 1);
            }
            if (bl_on) {
                if (bl_int) {
                    // (int)((float)v - off) == v - off for an integral offset; clamp(v - off, 0, mv)
                    // as one add-min-relu
                    const int p = y & 1;
                    v0 = __viaddmin_s32_relu(v0, -fp.bl_i[p][0], mv);
                    v1 = __viaddmin_s32_relu(v1, -fp.bl_i[p][1], mv);
                } else {
                    v0 = dev::black_level(fp, v0, bayer_color(y, x, po));
                    v1 = dev::black_level(fp, v1, bayer_color(y, x + 1, po));
                }
            }
            if (!FULL) {
                if (!in0) v0 = 0;
                if (!in1) v1 = 0;
            }
        }
        *reinterpret_cast<int2*>(orig + r * G::OW + 2 * pc) = make_int2(v0, v1);
    }
    __syncthreads();

    auto ORIGV = [&](int x, int y) -> int { return orig[(y - yo) * G::OW + (x - xo)]; };

    // ---- 3. defect correction (Jacobi), lens shading, Bayer WB -> bay samples ---------------
    // warp-rows: a warp takes 32 pair columns of one row; with two column blocks every warp
    // keeps one row parity and one column pair, so its colour constants stay in registers
    int local_mod = 0;
    const bool lsc_grid = !(SPEC & 16) && (stages & 4u) && fp.lsc_mode == 0;
    const bool lsc_poly = !(SPEC & 8) && (stages & 4u) && fp.lsc_mode == 1;
    const bool wb_bayer = (stages & 8u) && fp.stage_order == 0;
    const bool need_align = fp.need_align != 0;
    const int thr = fp.dpc_thr;
    const float2 h5 = make_float2(0.5f, 0.5f);
    if constexpr (FULL) {
        // a warp keeps one block of 32 pair columns and the rows r0, r0 + 4, ... (one row
        // parity), so its colours, gains and lens-shading columns are loop constants
        const int pc = (warp & 1) * 32 + lane;
        const int r0 = warp >> 1;
        const int p = (yb + r0) & 1;
        const int c0 = bayer_color(p, 0, po), c1 = bayer_color(p, 1, po);
        const float2 WB = make_float2(fp.wb_cfa[c0], fp.wb_cfa[c1]);
        const int x = xb + 2 * pc;
        if (pc < G::F_BPW) {
            float f0 = 0.f, f1 = 0.f;
            int gxa = 0, gxb = 0;
            if (lsc_grid) {
                f0 = sm.col_fx[2 * pc];
                f1 = sm.col_fx[2 * pc + 1];
                gxa = sm.col_gx[2 * pc];
                gxb = sm.col_gx[2 * pc + 1];
            }
            const float2 f01 = make_float2(f0, f1);
            const float2 of01 = make_float2(dev::fsub(1.0f, f0), dev::fsub(1.0f, f1));
            int cache_gy = -1;
            float2 A = make_float2(0.f, 0.f), B = A, C = A, D = A;
            const int* ob = orig + 2 * G::OW + (x - xo);
            for (int r = r0; r < G::F_BH; r += 4) {
                const int y = yb + r;
                const int* o = ob + r * G::OW;
                const int2 c = *reinterpret_cast<const int2*>(o);
                int j0 = c.x, j1 = c.y;
                if (adaptive) {
                    int2 n0 = *reinterpret_cast<const int2*>(o - 2 * G::OW - 2);
                    int2 n1 = *reinterpret_cast<const int2*>(o - 2 * G::OW);
                    int2 n2 = *reinterpret_cast<const int2*>(o - 2 * G::OW + 2);
                    int2 n3 = *reinterpret_cast<const int2*>(o - 2);
                    int2 n4 = *reinterpret_cast<const int2*>(o + 2);
                    int2 n5 = *reinterpret_cast<const int2*>(o + 2 * G::OW - 2);
                    int2 n6 = *reinterpret_cast<const int2*>(o + 2 * G::OW);
                    int2 n7 = *reinterpret_cast<const int2*>(o + 2 * G::OW + 2);
                    const int mn0 = dev::min8(n0.x, n1.x, n2.x, n3.x, n4.x, n5.x, n6.x, n7.x);
                    const int mx0 = dev::max8(n0.x, n1.x, n2.x, n3.x, n4.x, n5.x, n6.x, n7.x);
                    const int mn1 = dev::min8(n0.y, n1.y, n2.y, n3.y, n4.y, n5.y, n6.y, n7.y);
                    const int mx1 = dev::max8(n0.y, n1.y, n2.y, n3.y, n4.y, n5.y, n6.y, n7.y);
                    // |c - median| <= thr is certain when c - min <= thr and max - c <= thr
                    if (max(c.x - mn0, mx0 - c.x) > thr) {
                        int nb[8] = {n0.x, n1.x, n2.x, n3.x, n4.x, n5.x, n6.x, n7.x};
                        j0 = dev::dpc_apply(c.x, nb, 0xFFu, thr);
                    }
                    if (max(c.y - mn1, mx1 - c.y) > thr) {
                        int nb[8] = {n0.y, n1.y, n2.y, n3.y, n4.y, n5.y, n6.y, n7.y};
                        j1 = dev::dpc_apply(c.y, nb, 0xFFu, thr);
                    }
                } else if (!(SPEC & 8) && dpc_on && fp.dpc_mode == 1 && __ldg(fp.map_row_ptr + y + 1) > __ldg(fp.map_row_ptr + y)) {
                    int sv = map_lookup(fp, x, y);
                    if (sv >= 0) j0 = sv;
                    sv = map_lookup(fp, x + 1, y);
                    if (sv >= 0) j1 = sv;
                }
                const int m = (j0 != c.x) | ((j1 != c.y) << 1);
                local_mod |= m;
                sm.mod[r * G::BPW + pc] = (uint8_t)m;
                int u0 = j0, u1 = j1;
                if (lsc_grid) {
                    const int gy_i = sm.row_gy[r];
                    if (gy_i != cache_gy) {
                        // g00*(1-fx), g10*fx, g01*(1-fx), g11*fx of both samples for this cell row
                        cache_gy = gy_i;
                        const float* g0 = fp.grid + (gy_i * fp.gw + gxa) * 4 + c0;
                        const float* g1 = fp.grid + (gy_i * fp.gw + gxb) * 4 + c1;
                        A = dev::pmul(make_float2(__ldg(g0), __ldg(g1)), of01, z2);
                        B = dev::pmul(make_float2(__ldg(g0 + 4), __ldg(g1 + 4)), f01, z2);
                        C = dev::pmul(make_float2(__ldg(g0 + 4 * fp.gw), __ldg(g1 + 4 * fp.gw)), of01, z2);
                        D = dev::pmul(make_float2(__ldg(g0 + 4 * fp.gw + 4), __ldg(g1 + 4 * fp.gw + 4)), f01, z2);
                    }
                    const float fy = sm.row_fy[r], ofy = dev::fsub(1.0f, fy);
                    const float2 fy2 = make_float2(fy, fy), ofy2 = make_float2(ofy, ofy);
                    float2 gain = dev::fadd2(dev::fadd2(dev::fadd2(dev::pmul(A, ofy2, z2), dev::pmul(B, ofy2, z2)),
                                                        dev::pmul(C, fy2, z2)),
                                             dev::pmul(D, fy2, z2));
                    float2 t = dev::fadd2(dev::pmul(make_float2((float)u0, (float)u1), gain, z2), h5);
                    u0 = u16q(t.x, mv);
                    u1 = u16q(t.y, mv);
                } else if (lsc_poly) {
                    u0 = dev::lsc_poly(fp, u0, x, y, c0);
                    u1 = dev::lsc_poly(fp, u1, x + 1, y, c1);
                }
                if (wb_bayer) {
                    float2 t = dev::fadd2(dev::pmul(make_float2((float)u0, (float)u1), WB, z2), h5);
                    u0 = u16q(t.x, mv);
                    u1 = u16q(t.y, mv);
                }
                if (need_align) {
                    if (u0 > mv) u0 >>= (16 - fp.bd);
                    if (u1 > mv) u1 >>= (16 - fp.bd);
                }
                *reinterpret_cast<int2*>(sm.bay + r * G::BW + 2 * pc) = make_int2(u0, u1);
            }
        }
    } else {
        // wide regions: a warp takes 32 pair columns of one row; narrow ones (border columns): the
        // (row, pair) items spread over all threads, so the lanes are not mostly idle
        const int nbk = (bpw + 31) >> 5;
        const bool flat = bpw <= 16;
        int cache_key = -1;
        float2 A = make_float2(0.f, 0.f), B = A, C = A, D = A, WB = make_float2(1.f, 1.f);
        for (int item = flat ? tid : warp; item < (flat ? bh * bpw : nbk * bh); item += flat ? kThreads : 8) {
            int r, pc;
            if (flat) {
                r = item / bpw;
                pc = item - r * bpw;
            } else {
                int blk;
                if (nbk == 2) { blk = item & 1; r = item >> 1; } else { blk = item % nbk; r = item / nbk; }
                pc = blk * 32 + lane;
                if (pc >= bpw) continue;
            }
            int y = yb + r, x = xb + 2 * pc;
            const int* o = orig + (r + 2) * G::OW + (x - xo);
            int2 c = *reinterpret_cast<const int2*>(o);
            int j0 = c.x, j1 = c.y;
            const bool yin = FULL || (y >= 0 && y < H);
            if (yin && adaptive) {
                const bool fast = FULL || (x >= 4 && x + 1 < W - 4 && y >= 4 && y < H - 4);
                if (fast) {
                    int2 n0 = *reinterpret_cast<const int2*>(o - 2 * G::OW - 2);
                    int2 n1 = *reinterpret_cast<const int2*>(o - 2 * G::OW);
                    int2 n2 = *reinterpret_cast<const int2*>(o - 2 * G::OW + 2);
                    int2 n3 = *reinterpret_cast<const int2*>(o - 2);
                    int2 n4 = *reinterpret_cast<const int2*>(o + 2);
                    int2 n5 = *reinterpret_cast<const int2*>(o + 2 * G::OW - 2);
                    int2 n6 = *reinterpret_cast<const int2*>(o + 2 * G::OW);
                    int2 n7 = *reinterpret_cast<const int2*>(o + 2 * G::OW + 2);
                    const int mn0 = dev::min8(n0.x, n1.x, n2.x, n3.x, n4.x, n5.x, n6.x, n7.x);
                    const int mx0 = dev::max8(n0.x, n1.x, n2.x, n3.x, n4.x, n5.x, n6.x, n7.x);
                    const int mn1 = dev::min8(n0.y, n1.y, n2.y, n3.y, n4.y, n5.y, n6.y, n7.y);
                    const int mx1 = dev::max8(n0.y, n1.y, n2.y, n3.y, n4.y, n5.y, n6.y, n7.y);
                    // |c - median| <= thr is certain when c - min <= thr and max - c <= thr
                    if (max(c.x - mn0, mx0 - c.x) > thr) {
                        int nb[8] = {n0.x, n1.x, n2.x, n3.x, n4.x, n5.x, n6.x, n7.x};
                        j0 = dev::dpc_apply(c.x, nb, 0xFFu, thr);
                    }
                    if (max(c.y - mn1, mx1 - c.y) > thr) {
                        int nb[8] = {n0.y, n1.y, n2.y, n3.y, n4.y, n5.y, n6.y, n7.y};
                        j1 = dev::dpc_apply(c.y, nb, 0xFFu, thr);
                    }
                } else {
                    if (x >= 2 && x < W - 2 && y >= 2 && y < H - 2) j0 = dpc_scalar(fp, ORIGV, x, y);
                    if (x + 1 >= 2 && x + 1 < W - 2 && y >= 2 && y < H - 2) j1 = dpc_scalar(fp, ORIGV, x + 1, y);
                }
                if (!FULL && ov.n > 0 && y >= 2 && y < H - 2) {
                    if (x >= 2 && x < W - 2) { int sv = find_override(ov.idx, ov.val, ov.n, y * W + x); if (sv >= 0) j0 = sv; }
                    if (x + 1 >= 2 && x + 1 < W - 2) { int sv = find_override(ov.idx, ov.val, ov.n, y * W + x + 1); if (sv >= 0) j1 = sv; }
                }
            } else if (!(SPEC & 8) && yin && dpc_on && fp.dpc_mode == 1 && y >= 2 && y < H - 2 &&
                       __ldg(fp.map_row_ptr + y + 1) > __ldg(fp.map_row_ptr + y)) {
                if (x >= 2 && x < W - 2) { int sv = map_lookup(fp, x, y); if (sv >= 0) j0 = sv; }
                if (x + 1 >= 2 && x + 1 < W - 2) { int sv = map_lookup(fp, x + 1, y); if (sv >= 0) j1 = sv; }
            }
            int m = (j0 != c.x) | ((j1 != c.y) << 1);
            local_mod |= m;
            sm.mod[r * G::BPW + pc] = (uint8_t)m;
            // lens shading + white balance: scalar products (packed FP32 multiply-add pairs would be
            // fused into one rounding), packed sums
            int u0 = 0, u1 = 0;
            if (yin) {
                const int p = y & 1;
                const int c0 = bayer_color(p, 0, po), c1 = bayer_color(p, 1, po);
                u0 = j0;
                u1 = j1;
                if (lsc_grid) {
                    int gy_i = sm.row_gy[r];
                    int key = (gy_i * 2 + p) * 1024 + pc;
                    if (key != cache_key) {
                        // g00*(1-fx), g10*fx, g01*(1-fx), g11*fx of both samples for this cell row
                        cache_key = key;
                        const float2 f01 = make_float2(sm.col_fx[2 * pc], sm.col_fx[2 * pc + 1]);
                        const float2 of01 = make_float2(dev::fsub(1.0f, f01.x), dev::fsub(1.0f, f01.y));
                        const float* g0 = fp.grid + (gy_i * fp.gw + sm.col_gx[2 * pc]) * 4 + c0;
                        const float* g1 = fp.grid + (gy_i * fp.gw + sm.col_gx[2 * pc + 1]) * 4 + c1;
                        A = dev::pmul(make_float2(__ldg(g0), __ldg(g1)), of01, z2);
                        B = dev::pmul(make_float2(__ldg(g0 + 4), __ldg(g1 + 4)), f01, z2);
                        C = dev::pmul(make_float2(__ldg(g0 + 4 * fp.gw), __ldg(g1 + 4 * fp.gw)), of01, z2);
                        D = dev::pmul(make_float2(__ldg(g0 + 4 * fp.gw + 4), __ldg(g1 + 4 * fp.gw + 4)), f01, z2);
                        WB = make_float2(fp.wb_cfa[c0], fp.wb_cfa[c1]);
                    }
                    const float fy = sm.row_fy[r], ofy = dev::fsub(1.0f, fy);
                    const float2 fy2 = make_float2(fy, fy), ofy2 = make_float2(ofy, ofy);
                    float2 gain = dev::fadd2(dev::fadd2(dev::fadd2(dev::pmul(A, ofy2, z2), dev::pmul(B, ofy2, z2)),
                                                        dev::pmul(C, fy2, z2)),
                                             dev::pmul(D, fy2, z2));
                    float2 t = dev::fadd2(dev::pmul(make_float2((float)u0, (float)u1), gain, z2), h5);
                    u0 = u16q(t.x, mv);
                    u1 = u16q(t.y, mv);
                } else {
                    if (lsc_poly) {
                        u0 = dev::lsc_poly(fp, u0, x, y, c0);
                        u1 = dev::lsc_poly(fp, u1, x + 1, y, c1);
                    }
                    WB = make_float2(fp.wb_cfa[c0], fp.wb_cfa[c1]);
                }
                if (wb_bayer) {
                    float2 t = dev::fadd2(dev::pmul(make_float2((float)u0, (float)u1), WB, z2), h5);
                    u0 = u16q(t.x, mv);
                    u1 = u16q(t.y, mv);
                }
                if (need_align) {
                    if (u0 > mv) u0 >>= (16 - fp.bd);
                    if (u1 > mv) u1 >>= (16 - fp.bd);
                }
                if (!FULL) {
                    if (x < 0 || x >= W) u0 = 0;
                    if (x + 1 < 0 || x + 1 >= W) u1 = 0;
                }
            }
            *reinterpret_cast<int2*>(sm.bay + r * G::BW + 2 * pc) = make_int2(u0, u1);
        }
    }
    const int any_mod = __syncthreads_or(local_mod);

    auto BAYV = [&](int x, int y) -> int { return sm.bay[(y - yb) * G::BW + (x - xb)]; };
    float* green = reinterpret_cast<float*>(raw);  // one float per pair row: the R/B site

    // ---- 4a. defect-chain seeds among own pixels (only tiles with a corrected pixel) ---------
    if (detect_seeds && adaptive && any_mod) {
        for (int s = tid; s < G::THM * G::TWP; s += kThreads) {
            int r = s / G::TWP, pc = s - r * G::TWP;
            if (r >= th || pc >= tpw) continue;
            int y = y0 + r;
            // quick reject: no corrected pixel among the earlier neighbours of either sample
            const uint8_t* mr = sm.mod + (r + 1) * G::BPW + (pc + 2);  // row y-2, pair of x
            const uint8_t* m0 = sm.mod + (r + 3) * G::BPW + (pc + 2);  // row y
            if ((mr[-1] | mr[0] | mr[1] | m0[-1]) == 0) continue;
            for (int h = 0; h < 2; h++) {
                int x = x0 + 2 * pc + h;
                if (x >= x0 + tw || x < 2 || x >= W - 2 || y < 2 || y >= H - 2) continue;
                unsigned valid = dev::dpc_valid_mask(x, y, W, H);
                auto MOD = [&](int xx, int yy) { return (sm.mod[(yy - yb) * G::BPW + ((xx - xb) >> 1)] >> ((xx - xb) & 1)) & 1; };
                bool any = ((valid & 1u) && MOD(x - 2, y - 2)) || ((valid & 2u) && MOD(x, y - 2)) ||
                           ((valid & 4u) && MOD(x + 2, y - 2)) || ((valid & 8u) && MOD(x - 2, y));
                if (!any) continue;
                int nb[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                const int ex[4] = {x - 2, x, x + 2, x - 2}, ey[4] = {y - 2, y - 2, y - 2, y};
                for (int k = 0; k < 4; k++)
                    if ((valid >> k) & 1u) nb[k] = MOD(ex[k], ey[k]) ? dpc_scalar(fp, ORIGV, ex[k], ey[k]) : ORIGV(ex[k], ey[k]);
                if (valid & 16u) nb[4] = ORIGV(x + 2, y);
                if (valid & 32u) nb[5] = ORIGV(x - 2, y + 2);
                if (valid & 64u) nb[6] = ORIGV(x, y + 2);
                if (valid & 128u) nb[7] = ORIGV(x + 2, y + 2);
                int s1 = dev::dpc_apply(ORIGV(x, y), nb, valid, fp.dpc_thr);
                int jp = MOD(x, y) ? dpc_scalar(fp, ORIGV, x, y) : ORIGV(x, y);
                if (s1 != jp) {
                    int slot = atomicAdd(fp.seed_count, 1);
                    if (slot < fp.seed_cap) fp.seeds[slot] = y * W + x;
                    else atomicExch(fp.status, 104 /* IMOP_ERR_CAPACITY */);
                }
            }
        }
    }

    // ---- 4b. green at the red/blue site of each pair (AMAZE, MG) ---------------------------
    if (FULL && demosaic != DM_HQLI) {
        // one column block and one row parity per warp, as in the defect phase
        const bool fast_div = fp.bd <= 12;
        const int pc = (warp & 1) * 32 + lane;
        const int r0 = warp >> 1;
        const int rbh = (((yg0 + r0) & 1) == po.r_row) ? po.r_col : po.b_col;
        if (pc < G::F_GPW) {
            const int* bp0 = sm.bay + 2 * G::BW + (xg0 + 2 * pc + rbh - xb);
            for (int r = r0; r < G::F_GH; r += 4) {
                const int* bp = bp0 + r * G::BW;
                const int cc = bp[0], hm1 = bp[-1], hp1 = bp[1], hm2 = bp[-2], hp2 = bp[2];
                const int vm1 = bp[-G::BW], vp1 = bp[G::BW], vm2 = bp[-2 * G::BW], vp2 = bp[2 * G::BW];
                float g;
                if (demosaic == DM_AMAZE) {
                    g = dev::amaze_green_fast(cc, hm1, hp1, hm2, hp2, vm1, vp1, vm2, vp2, fast_div, z2);
                } else if (fp.bd <= 8) {
                    // src/algorithms/mg.cpp:58-69 (integer Malvar-He-Cutler green)
                    g = (float)dev::clampi((4 * cc + 2 * (vm1 + vp1 + hp1 + hm1) - (vm2 + vp2 + hp2 + hm2) + 4) >> 3, 0, mv);
                } else {
                    // src/algorithms/mg.cpp:187-196, exact in FP32 for integer samples
                    float t = dev::fsub(dev::fadd(dev::fmul(4.0f, (float)cc), dev::fmul(2.0f, (float)(vm1 + vp1 + hp1 + hm1))),
                                        (float)(vm2 + vp2 + hp2 + hm2));
                    g = __fdiv_rn(t, 8.0f);
                }
                green[r * G::GPW + pc] = g;
            }
        }
    } else if (demosaic != DM_HQLI) {
        const int nbk = (gpw + 31) >> 5;
        const bool flat = gpw <= 16;
        const bool fast_div = fp.bd <= 12;
        for (int item = flat ? tid : warp; item < (flat ? gh * gpw : nbk * gh); item += flat ? kThreads : 8) {
            int r, pc;
            if (flat) {
                r = item / gpw;
                pc = item - r * gpw;
            } else {
                int blk;
                if (nbk == 2) { blk = item & 1; r = item >> 1; } else { blk = item % nbk; r = item / nbk; }
                pc = blk * 32 + lane;
                if (pc >= gpw) continue;
            }
            int y = yg0 + r;
            int rbh = ((y & 1) == po.r_row) ? po.r_col : po.b_col;
            int x = xg0 + 2 * pc + rbh;
            float g = -1.0f;
            if (FULL || (x >= 2 && x < W - 2 && y >= 2 && y < H - 2)) {
                const int* bp = sm.bay + (r + 2) * G::BW + (x - xb);
                int cc = bp[0], hm1 = bp[-1], hp1 = bp[1], hm2 = bp[-2], hp2 = bp[2];
                int vm1 = bp[-G::BW], vp1 = bp[G::BW], vm2 = bp[-2 * G::BW], vp2 = bp[2 * G::BW];
                if (demosaic == DM_AMAZE) {
                    g = dev::amaze_green_fast(cc, hm1, hp1, hm2, hp2, vm1, vp1, vm2, vp2, fast_div, z2);
                } else if (fp.bd <= 8) {
                    // src/algorithms/mg.cpp:58-69 (integer Malvar-He-Cutler green)
                    g = (float)dev::clampi((4 * cc + 2 * (vm1 + vp1 + hp1 + hm1) - (vm2 + vp2 + hp2 + hm2) + 4) >> 3, 0, mv);
                } else {
                    // src/algorithms/mg.cpp:187-196, exact in FP32 for integer samples
                    float t = dev::fsub(dev::fadd(dev::fmul(4.0f, (float)cc), dev::fmul(2.0f, (float)(vm1 + vp1 + hp1 + hm1))),
                                        (float)(vm2 + vp2 + hp2 + hm2));
                    g = __fdiv_rn(t, 8.0f);
                }
            }
            green[r * G::GPW + pc] = g;
        }
    }
    __syncthreads();

    const GreenAt GRNV{green, sm.bay, xg0, yg0, xb, yb, G::GPW, G::BW, W, H, po.r_row, po.r_col, po.b_col,
                       demosaic == DM_MG};

    // demosaic of one pixel at (sx, sy) (general path: border tiles, MG and fix-up windows)
    auto demosaic_at = [&](int sx, int sy, int& R, int& Gv, int& B) {
        bool at_r = ((sy & 1) == po.r_row) && ((sx & 1) == po.r_col);
        bool at_b = ((sy & 1) == po.b_row) && ((sx & 1) == po.b_col);
        R = Gv = B = 0;
        if (demosaic == DM_HQLI) {
            // detail::hqli_core (src/algorithms/interp_core.hpp:39-65)
            if (sx >= 2 && sx < W - 2 && sy >= 2 && sy < H - 2) {
                int n4 = BAYV(sx - 1, sy) + BAYV(sx + 1, sy) + BAYV(sx, sy - 1) + BAYV(sx, sy + 1);
                int d4 = BAYV(sx - 1, sy - 1) + BAYV(sx + 1, sy - 1) + BAYV(sx - 1, sy + 1) + BAYV(sx + 1, sy + 1);
                if (at_r) { R = BAYV(sx, sy); Gv = (n4 + 2) / 4; B = (d4 + 2) / 4; }
                else if (at_b) { R = (d4 + 2) / 4; Gv = (n4 + 2) / 4; B = BAYV(sx, sy); }
                else {
                    Gv = BAYV(sx, sy);
                    int hz = (BAYV(sx - 1, sy) + BAYV(sx + 1, sy) + 1) / 2;
                    int vt = (BAYV(sx, sy - 1) + BAYV(sx, sy + 1) + 1) / 2;
                    if ((sy & 1) == po.r_row) { R = hz; B = vt; } else { B = hz; R = vt; }
                }
                R = min(R, mv); Gv = min(Gv, mv); B = min(B, mv);
            }
        } else if (demosaic == DM_MG && fp.bd <= 8) {
            // integer colour differences (src/algorithms/mg.cpp:74-146)
            int g = (int)GRNV(sx, sy);
            int Ri = 0, Bi = 0;
            if (sx >= 1 && sx < W - 1 && sy >= 1 && sy < H - 1) {
                auto cdi = [&](int x, int y) { return BAYV(x, y) - (int)GRNV(x, y); };
                if (at_r || at_b) {
                    int sum = cdi(sx - 1, sy - 1) + cdi(sx + 1, sy - 1) + cdi(sx - 1, sy + 1) + cdi(sx + 1, sy + 1);
                    int other = g + (sum + 2) / 4;
                    if (at_r) { Ri = BAYV(sx, sy); Bi = other; } else { Bi = BAYV(sx, sy); Ri = other; }
                } else {
                    int hz = cdi(sx - 1, sy) + cdi(sx + 1, sy), vt = cdi(sx, sy - 1) + cdi(sx, sy + 1);
                    int rc = ((sy & 1) == po.r_row) ? hz : vt, bc = ((sy & 1) == po.r_row) ? vt : hz;
                    Ri = g + (rc + 1) / 2;
                    Bi = g + (bc + 1) / 2;
                }
            }
            R = dev::clampi(Ri, 0, mv); Gv = dev::clampi(g, 0, mv); B = dev::clampi(Bi, 0, mv);
        } else {
            // float colour differences (src/algorithms/common.hpp:142-199, amaze.cpp:62-114)
            float g = GRNV(sx, sy), Rf = 0.0f, Bf = 0.0f;
            if (sx >= 1 && sx < W - 1 && sy >= 1 && sy < H - 1) {
                auto cd = [&](int x, int y) { return dev::fsub((float)BAYV(x, y), GRNV(x, y)); };
                if (at_r || at_b) {
                    float sum = dev::fadd(dev::fadd(dev::fadd(cd(sx - 1, sy - 1), cd(sx + 1, sy - 1)), cd(sx - 1, sy + 1)),
                                          cd(sx + 1, sy + 1));
                    float other = dev::fadd(g, dev::fmul(sum, 0.25f));
                    if (at_r) { Rf = (float)BAYV(sx, sy); Bf = other; } else { Bf = (float)BAYV(sx, sy); Rf = other; }
                } else {
                    float hz = dev::fadd(cd(sx - 1, sy), cd(sx + 1, sy));
                    float vt = dev::fadd(cd(sx, sy - 1), cd(sx, sy + 1));
                    bool rrow = (sy & 1) == po.r_row;
                    Rf = dev::fadd(g, dev::fmul(rrow ? hz : vt, 0.5f));
                    Bf = dev::fadd(g, dev::fmul(rrow ? vt : hz, 0.5f));
                }
            }
            R = dev::round_plane(Rf, mv); Gv = dev::round_plane(g, mv); B = dev::round_plane(Bf, mv);
        }
    };

    // ---- 5. demosaic + RGB WB/CCM + tone for own pairs -> output staging ---------------------
    uint8_t* outs = sm.regB;
    const int bpc = fp.out_bpc;
    const uintptr_t out_base = reinterpret_cast<uintptr_t>(fp.out);
    const int out_format = (SPEC & 8) ? 0 : fp.out_format;
    const bool border_tile = !FULL && (x0 < 2 || x0 + tw > W - 2 || y0 < 2 || y0 + th > H - 2);
    const bool ccm_on = (stages & 16u) != 0;
    const bool lut3d_on = (stages & 32u) != 0;
    const bool wb_rgb = (stages & 8u) && fp.stage_order == 1;
    const float wr = fp.wb_rgb[0], wg = fp.wb_rgb[1], wbl = fp.wb_rgb[2];
    // RGB WB, CCM and tone of pair (x, x+1) in tile row r, staged for the stores
    auto finish = [&](int r, int y, int pc, int x, int R0, int G0, int B0, int R1, int G1, int B1) {
        // RGB-domain white balance (reference call order), CCM: scalar products, packed sums
        if (wb_rgb) {
            float2 t;
            t = dev::fadd2(dev::pmul(make_float2((float)R0, (float)R1), make_float2(wr, wr), z2), h5);
            R0 = u16q(t.x, mv); R1 = u16q(t.y, mv);
            t = dev::fadd2(dev::pmul(make_float2((float)G0, (float)G1), make_float2(wg, wg), z2), h5);
            G0 = u16q(t.x, mv); G1 = u16q(t.y, mv);
            t = dev::fadd2(dev::pmul(make_float2((float)B0, (float)B1), make_float2(wbl, wbl), z2), h5);
            B0 = u16q(t.x, mv); B1 = u16q(t.y, mv);
        }
        if (ccm_on) {
            const float* m = fp.ccm;
            const float2 rr = make_float2((float)R0, (float)R1), gg = make_float2((float)G0, (float)G1),
                         bb = make_float2((float)B0, (float)B1);
            auto M = [&](int k) { return make_float2(m[k], m[k]); };
            // ((m0*r + m1*g) + m2*b) + 0.5 for both samples, each product rounded on its own
            float2 ro = dev::fadd2(dev::fadd2(dev::fadd2(dev::pmul(M(0), rr, z2), dev::pmul(M(1), gg, z2)),
                                              dev::pmul(M(2), bb, z2)), h5);
            float2 go = dev::fadd2(dev::fadd2(dev::fadd2(dev::pmul(M(3), rr, z2), dev::pmul(M(4), gg, z2)),
                                              dev::pmul(M(5), bb, z2)), h5);
            float2 bo = dev::fadd2(dev::fadd2(dev::fadd2(dev::pmul(M(6), rr, z2), dev::pmul(M(7), gg, z2)),
                                              dev::pmul(M(8), bb, z2)), h5);
            // (int)(v + 0.5) clamped to [0, mv]: truncation saturating at 0, then min
            R0 = u16q(ro.x, mv); R1 = u16q(ro.y, mv);
            G0 = u16q(go.x, mv); G1 = u16q(go.y, mv);
            B0 = u16q(bo.x, mv); B1 = u16q(bo.y, mv);
        }
        if (EXTRA && lut3d_on) {
            dev::lut3d_apply(fp.lut3d, fp.lut3d_size, mv, R0, G0, B0);
            dev::lut3d_apply(fp.lut3d, fp.lut3d_size, mv, R1, G1, B1);
        }
        int g0 = (y * W + x0) * 3 * bpc;
        int shift = (int)((out_base + (uintptr_t)g0) & 15);
        uint8_t* q = outs + r * G::OUT_PITCH + shift + 2 * pc * 3 * bpc;
        const bool has1 = FULL || x + 1 < x0 + tw;
        if (out_format == 0) {
            const uint8_t* tt = tone_smem ? sm.tone8 : fp.tone8;
            int t0 = tt[R0], t1 = tt[G0], t2 = tt[B0];
            if (((shift & 1) == 0) && has1) {
                int t3 = tt[R1], t4 = tt[G1], t5 = tt[B1];
                uint16_t* q16 = reinterpret_cast<uint16_t*>(q);
                q16[0] = (uint16_t)(t0 | (t1 << 8));
                q16[1] = (uint16_t)(t2 | (t3 << 8));
                q16[2] = (uint16_t)(t4 | (t5 << 8));
            } else {
                q[0] = (uint8_t)t0; q[1] = (uint8_t)t1; q[2] = (uint8_t)t2;
                if (has1) { q[3] = tt[R1]; q[4] = tt[G1]; q[5] = tt[B1]; }
            }
        } else if (bpc == 1) {
            q[0] = (uint8_t)R0; q[1] = (uint8_t)G0; q[2] = (uint8_t)B0;
            if (has1) { q[3] = (uint8_t)R1; q[4] = (uint8_t)G1; q[5] = (uint8_t)B1; }
        } else {
            int v[6] = {R0, G0, B0, R1, G1, B1};
            for (int k = 0; k < (has1 ? 6 : 3); k++) { q[2 * k] = (uint8_t)v[k]; q[2 * k + 1] = (uint8_t)(v[k] >> 8); }
        }
    };
    if (FULL && demosaic != DM_MG) {
        // one column block and one row parity per warp: the red/blue column, the row colours and
        // every neighbour offset are loop constants
        const int pc = (warp & 1) * 32 + lane;
        const int r0 = warp >> 1;
        const bool rrow = ((y0 + r0) & 1) == po.r_row;
        const int rbh = rrow ? po.r_col : po.b_col;  // sample of the pair at the red/blue site
        if (pc < G::F_TPW) {
            const int x = x0 + 2 * pc;
            const int* br0 = sm.bay + 3 * G::BW + (x + rbh - xb);
            const int* bg0 = sm.bay + 3 * G::BW + (x + 1 - rbh - xb);
            const float* gr0 = green + G::GPW + (pc + 1);
            // pair offsets of columns xr-1 / xr+1 (diagonals) and xg-1 / xg+1 (horizontal)
            const int pa = rbh ? 0 : -1, pl = rbh ? -1 : 0;
            for (int r = r0; r < TH; r += 4) {
                int R0, G0, B0, R1, G1, B1;
                const int* br = br0 + r * G::BW;  // red/blue site
                const int* bg = bg0 + r * G::BW;  // green site
                int own, gq, oq, gg, hz, vt;  // R/B site: own, green, other; G site: green, horizontal, vertical
                if (demosaic == DM_HQLI) {
                    // detail::hqli_core (src/algorithms/interp_core.hpp:39-65)
                    int n4 = br[-1] + br[1] + br[-G::BW] + br[G::BW];
                    int d4 = br[-G::BW - 1] + br[-G::BW + 1] + br[G::BW - 1] + br[G::BW + 1];
                    own = min(br[0], mv);
                    gq = min((n4 + 2) / 4, mv);
                    oq = min((d4 + 2) / 4, mv);
                    gg = min(bg[0], mv);
                    hz = min((bg[-1] + bg[1] + 1) / 2, mv);
                    vt = min((bg[-G::BW] + bg[G::BW] + 1) / 2, mv);
                } else {
                    // AMAZE colour differences (src/algorithms/common.hpp:142-199, amaze.cpp:62-114).
                    // Red/blue site xr: the other colour from the four diagonals, the red/blue sites of
                    // rows y-1, y+1 at columns xr-1, xr+1.  Green site xg: horizontal neighbours are
                    // this row's red/blue sites, vertical ones those of rows y-1, y+1.
                    const float* gr = gr0 + r * G::GPW;  // this pair row's R/B green
                    float g_rb = gr[0];
                    float c00 = dev::fsub((float)br[-G::BW - 1], gr[-G::GPW + pa]);
                    float c01 = dev::fsub((float)br[-G::BW + 1], gr[-G::GPW + pa + 1]);
                    float c10 = dev::fsub((float)br[G::BW - 1], gr[G::GPW + pa]);
                    float c11 = dev::fsub((float)br[G::BW + 1], gr[G::GPW + pa + 1]);
                    float sum = dev::fadd(dev::fadd(dev::fadd(c00, c01), c10), c11);
                    float fgq = (float)bg[0];
                    float2 hv = dev::fadd2(make_float2(dev::fsub((float)bg[-1], gr[pl]), dev::fsub((float)bg[-G::BW], gr[-G::GPW])),
                                           make_float2(dev::fsub((float)bg[1], gr[pl + 1]), dev::fsub((float)bg[G::BW], gr[G::GPW])));
                    // x*0.25 and x*0.5 are exact, so one fused multiply-add rounds like the add
                    float other = __fmaf_rn(sum, 0.25f, g_rb);
                    float2 rb2 = dev::fma2(hv, make_float2(0.5f, 0.5f), make_float2(fgq, fgq));
                    // the float plane's rounding of an integer sample is a clamp
                    own = dev::clampi(br[0], 0, mv);
                    oq = dev::round_plane(other, mv);
                    gq = dev::round_plane(g_rb, mv);
                    gg = dev::clampi(bg[0], 0, mv);
                    hz = dev::round_plane(rb2.x, mv);
                    vt = dev::round_plane(rb2.y, mv);
                }
                // red/blue site: R,B = own/other by row; green site: R,B = horizontal/vertical by row
                int rr_rb = rrow ? own : oq, bb_rb = rrow ? oq : own;
                int rr_g = rrow ? hz : vt, bb_g = rrow ? vt : hz;
                if (rbh == 0) { R0 = rr_rb; G0 = gq; B0 = bb_rb; R1 = rr_g; G1 = gg; B1 = bb_g; }
                else { R1 = rr_rb; G1 = gq; B1 = bb_rb; R0 = rr_g; G0 = gg; B0 = bb_g; }
                finish(r, y0 + r, pc, x, R0, G0, B0, R1, G1, B1);
            }
        }
    } else {
        const int nbk = FULL ? (G::F_TPW + 31) / 32 : (tpw + 31) >> 5;
        const bool flat = !FULL && tpw <= 16;
        for (int item = flat ? tid : warp; item < (flat ? th * tpw : nbk * th); item += flat ? kThreads : 8) {
            int r, pc;
            if (flat) {
                r = item / tpw;
                pc = item - r * tpw;
            } else {
                int blk;
                if (nbk == 2) { blk = item & 1; r = item >> 1; } else { blk = item % nbk; r = item / nbk; }
                pc = blk * 32 + lane;
                if (pc >= tpw) continue;
            }
            int y = y0 + r, x = x0 + 2 * pc;
            int R0, G0, B0, R1, G1, B1;
            if (!border_tile && demosaic != DM_MG) {
                const bool rrow = (y & 1) == po.r_row;
                const int rbh = rrow ? po.r_col : po.b_col;  // sample of the pair at the red/blue site
                const int xr = x + rbh, xg = x + 1 - rbh;
                const int* br = sm.bay + (r + 3) * G::BW + (xr - xb);  // red/blue site
                const int* bg = sm.bay + (r + 3) * G::BW + (xg - xb);  // green site
                int own, gq, oq, gg, hz, vt;  // R/B site: own, green, other; G site: green, horizontal, vertical
                if (demosaic == DM_HQLI) {
                    // detail::hqli_core (src/algorithms/interp_core.hpp:39-65)
                    int n4 = br[-1] + br[1] + br[-G::BW] + br[G::BW];
                    int d4 = br[-G::BW - 1] + br[-G::BW + 1] + br[G::BW - 1] + br[G::BW + 1];
                    own = min(br[0], mv);
                    gq = min((n4 + 2) / 4, mv);
                    oq = min((d4 + 2) / 4, mv);
                    gg = min(bg[0], mv);
                    hz = min((bg[-1] + bg[1] + 1) / 2, mv);
                    vt = min((bg[-G::BW] + bg[G::BW] + 1) / 2, mv);
                } else {
                    // AMAZE colour differences (src/algorithms/common.hpp:142-199, amaze.cpp:62-114).
                    // Red/blue site xr: the other colour from the four diagonals, the red/blue sites of
                    // rows y-1, y+1 at columns xr-1, xr+1.  Green site xg: horizontal neighbours are
                    // this row's red/blue sites, vertical ones those of rows y-1, y+1.
                    const float* gr = green + (r + 1) * G::GPW + (pc + 1);  // this pair row's R/B green
                    // pair offsets of columns xr-1 / xr+1 (diagonals) and xg-1 / xg+1 (horizontal)
                    const int pa = rbh ? 0 : -1, pl = rbh ? -1 : 0;
                    float g_rb = gr[0];
                    float c00 = dev::fsub((float)br[-G::BW - 1], gr[-G::GPW + pa]);
                    float c01 = dev::fsub((float)br[-G::BW + 1], gr[-G::GPW + pa + 1]);
                    float c10 = dev::fsub((float)br[G::BW - 1], gr[G::GPW + pa]);
                    float c11 = dev::fsub((float)br[G::BW + 1], gr[G::GPW + pa + 1]);
                    float sum = dev::fadd(dev::fadd(dev::fadd(c00, c01), c10), c11);
                    float fgq = (float)bg[0];
                    float2 hv = dev::fadd2(make_float2(dev::fsub((float)bg[-1], gr[pl]), dev::fsub((float)bg[-G::BW], gr[-G::GPW])),
                                           make_float2(dev::fsub((float)bg[1], gr[pl + 1]), dev::fsub((float)bg[G::BW], gr[G::GPW])));
                    // x*0.25 and x*0.5 are exact, so one fused multiply-add rounds like the add
                    float other = __fmaf_rn(sum, 0.25f, g_rb);
                    float2 rb2 = dev::fma2(hv, make_float2(0.5f, 0.5f), make_float2(fgq, fgq));
                    // the float plane's rounding of an integer sample is a clamp
                    own = dev::clampi(br[0], 0, mv);
                    oq = dev::round_plane(other, mv);
                    gq = dev::round_plane(g_rb, mv);
                    gg = dev::clampi(bg[0], 0, mv);
                    hz = dev::round_plane(rb2.x, mv);
                    vt = dev::round_plane(rb2.y, mv);
                }
                // red/blue site: R,B = own/other by row; green site: R,B = horizontal/vertical by row
                int rr_rb = rrow ? own : oq, bb_rb = rrow ? oq : own;
                int rr_g = rrow ? hz : vt, bb_g = rrow ? vt : hz;
                if (rbh == 0) { R0 = rr_rb; G0 = gq; B0 = bb_rb; R1 = rr_g; G1 = gg; B1 = bb_g; }
                else { R1 = rr_rb; G1 = gq; B1 = bb_rb; R0 = rr_g; G0 = gg; B0 = bb_g; }
            } else {
                int sx, sy;
                dev::border_source(x, y, W, H, fp.border_mode, sx, sy);
                demosaic_at(sx, sy, R0, G0, B0);
                dev::border_source(x + 1, y, W, H, fp.border_mode, sx, sy);
                demosaic_at(sx, sy, R1, G1, B1);
            }
            finish(r, y, pc, x, R0, G0, B0, R1, G1, B1);
        }
    }
    __syncthreads();

    // ---- 6. store: 16-byte vector stores on the output's own 16-byte grid --------------------
    const int len = tw * 3 * bpc;
    constexpr int CH = G::OUT_PITCH / 16;
    for (int s = tid; s < G::THM * CH; s += kThreads) {
        int r = s / CH, k = s - r * CH;
        if (r >= th) continue;
        int g0 = ((y0 + r) * W + x0) * 3 * bpc;
        int shift = (int)((out_base + (uintptr_t)g0) & 15);
        int lo = 16 * k, hi = lo + 16;  // staging bytes [lo, hi) <-> output bytes g0 - shift + [lo, hi)
        if (hi <= shift || lo >= shift + len) continue;
        const uint8_t* src = outs + r * G::OUT_PITCH;
        uint8_t* dst = fp.out + g0 - shift;
        if (lo >= shift && hi <= shift + len) {
            ptx::st_global_v4(dst + lo, *reinterpret_cast<const uint4*>(src + lo));
        } else {
            store_piece(dst, src, max(lo, shift), min(hi, shift + len));
        }
    }
    // this tile's generic reads and writes of its raw buffer come before the bulk copy that
    // stages a later tile into it
    ptx::fence_proxy_async_smem();
    __syncthreads();
    return true;
}

// One tile of frame sm.fp[0] through buffer 0, staged and computed in turn (fix-up windows).
template <int TW, int TH, int OUTB>
__device__ bool process_tile_sync(TileSmem<TW, TH, OUTB>& sm, int x0, int y0, int tw, int th, Overrides ov,
                                  uint32_t& parity) {
    if (threadIdx.x < 32) stage_tile(sm, 0, x0, y0, tw, th);
    __syncthreads();
    return compute_tile<TW, TH, OUTB, false>(sm, 0, ov, false, parity);
}

}  // namespace imop
