// isp_adjoint.cu - the differentiable calibration chain on sm_103a: forward render and adjoint.
//
// Chain (per pixel, FP32, no rounding between stages; the reference's stage formulas):
//   b = clamp(raw - bl[c], 0, mv)      l = clamp(b * gain(x, y, c), 0, mv)     u = clamp(l * wb[c], 0, mv)
//   demosaic(u) -> clamp(., 0, mv) -> o = clamp(M . rgb, 0, mv) -> t = knots lerp at o / mv
// Demosaic is HQLI or AMAZE (gradient-weighted green at red/blue sites, colour differences with
// the -1 green sentinel outside [2,w-2)x[2,h-2), border copies from rows / columns 2 and -3).
//
// The adjoint recomputes the forward per tile (32 x 32 output pixels; the last tile of a row or
// column absorbs a remainder below 4 so that every border copy source lies inside its tile) into
// shared planes: u with a 3-pixel apron, green with a 1-pixel apron.  It back-propagates dL/dt
// of the tile's own pixels into gradient planes of the same extent (shared atomics), then the
// green plane into u, then u into the per-pixel parameters.  A u or green sample in the apron
// holds only the contributions of this tile's outputs; its parameter terms are linear in those
// contributions, so each tile adds its share and no tile needs another tile's gradients.
//
// Parameter gradients: BL, WB, CCM and the loss in registers, tone knots in shared accumulators,
// the lens-shading grid in the CTA's partial vector; each CTA of the persistent grid writes one
// partial vector and a second kernel adds the partials in a fixed order.

#include <cuda_runtime.h>

#include "isp_adjoint.h"
#include "isp_kernels.h"
#include "isp_device.cuh"
#include "isp_tile.cuh"

namespace imop {
namespace {

constexpr int kAdjThreads = 256;
constexpr int kTX = 32, kTY = 32;  // 64 x 16 measured 1 % slower, 64 x 32 (2 CTAs / SM) 9 %
constexpr int kUW = kTX + 3 + 6, kUH = kTY + 3 + 6;  // u region: tile (merged) +- 3
constexpr int kGW = kTX + 3 + 2, kGH = kTY + 3 + 2;  // green region: tile +- 1
constexpr int kVW = kTX + 3 + 4, kVH = kTY + 3 + 4;  // demosaic-output gradients: tile +- 2
constexpr int kMaxParams = 16 + 4 * kAdjMaxGridNodes + 33;

// tile-local lens-shading nodes: a tile's u region spans at most kLNX x kLNY grid nodes in the
// local table (wider spans add straight into the CTA's partial vector)
constexpr int kLNX = 4, kLNY = 3, kLocalNodes = 4 * kLNX * kLNY;

// Under 56 KB, so that four CTAs share an SM: the lens-shading grid's sums live in the CTA's
// partial vector in global memory (a tile adds its local nodes there once), raw samples are kept
// as u16, and the green plane's adjoint reuses the green plane, which nothing reads once the pixel
// pass is done.
struct AdjSmem {
    float th[kMaxParams];
    float acc_knots[33];
    // Accumulators with one column per lane index, entry [k][lane]: the lanes of a warp never meet
    // on an address (and hit 32 different banks); only warps with the same lane index can, so the
    // shared atomics here rarely retry.
    float knot_lane[33 * 32];
    float node_lane[kLocalNodes * 32];
    float u[kUH * kUW];
    float gu[kUH * kUW];
    union {
        float G[kGH * kGW];   // forward and pixel pass
        float gG[kGH * kGW];  // demosaic adjoint
    };
    // dL/d(demosaic output) per channel, summed at each output's source pixel (border copies add
    // into their source); zero outside the tile's own pixels
    float gV[3][kVH * kVW];
    int col_gx[kUW];
    float col_fx[kUW];
    int row_gy[kUH];
    float row_fy[kUH];
    float red[kAdjThreads / 32][18];
    int next_item[2];  // the tile claimed during tile k, in slot k & 1
    uint16_t raw[kUH * kUW];
};

__device__ __forceinline__ float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }

// (row, column) of element s = r * w + c of a w-wide region, for a loop whose s starts at s0 and
// steps by kAdjThreads: one division at the start, then a carry per step
struct Walk2D {
    int r, c, dr, dc, w;
    __device__ __forceinline__ Walk2D(int s0, int w_) : w(w_) {
        r = s0 / w;
        c = s0 - r * w;
        dr = kAdjThreads / w;
        dc = kAdjThreads - dr * w;
    }
    __device__ __forceinline__ void step() {
        r += dr;
        c += dc;
        if (c >= w) {
            c -= w;
            r++;
        }
    }
};


__device__ __forceinline__ float inside(float v, float lo, float hi) { return (v > lo && v < hi) ? 1.0f : 0.0f; }
__device__ __forceinline__ float sgnf(float v) { return v > 0.0f ? 1.0f : (v < 0.0f ? -1.0f : 0.0f); }

struct TileCtx {
    const AdjFrame* f;
    PatternOffsets po;
    int x0, y0, tw, th;
    int xu, yu;  // u region origin (x0 - 3, y0 - 3)
    int xg, yg;  // green region origin (x0 - 1, y0 - 1)
    __device__ int cfa(int x, int y) const { return bayer_color(y, x, po); }
    __device__ bool at_r(int x, int y) const { return ((y & 1) == po.r_row) && ((x & 1) == po.r_col); }
    __device__ bool at_b(int x, int y) const { return ((y & 1) == po.b_row) && ((x & 1) == po.b_col); }
    __device__ bool rb(int x, int y) const { return at_r(x, y) || at_b(x, y); }
    __device__ int ui(int x, int y) const { return (y - yu) * kUW + (x - xu); }
    __device__ int gi(int x, int y) const { return (y - yg) * kGW + (x - xg); }
    __device__ int vi(int x, int y) const { return (y - yg + 1) * kVW + (x - xg + 1); }
};

__device__ __forceinline__ float wb_of(const float* th, int c) { return th[4 + (c == 0 ? 0 : (c == 3 ? 2 : 1))]; }

// AMAZE green at a red/blue site from the u plane; parts receive the terms the adjoint needs
__device__ float amaze_df(const AdjSmem& sm, const TileCtx& t, int x, int y, float* parts) {
    const float* u = sm.u;
    int i = t.ui(x, y);
    float c = u[i], hm1 = u[i - 1], hp1 = u[i + 1], hm2 = u[i - 2], hp2 = u[i + 2];
    float vm1 = u[i - kUW], vp1 = u[i + kUW], vm2 = u[i - 2 * kUW], vp2 = u[i + 2 * kUW];
    float lapH = 2.0f * c - hm2 - hp2, lapV = 2.0f * c - vm2 - vp2;
    float gH = fabsf(hm1 - hp1) + fabsf(lapH), gV = fabsf(vm1 - vp1) + fabsf(lapV);
    // the chain is FP32 to a tolerance, not bit-exact: approximate reciprocals (2 ulp) suffice
    float a = __fdividef(1.0f, 1.0f + gH), b = __fdividef(1.0f, 1.0f + gV);
    float rs = __fdividef(1.0f, a + b);
    float wh = a * rs, wv = b * rs;
    float gh = (hm1 + hp1) * 0.5f + lapH * 0.25f, gv = (vm1 + vp1) * 0.5f + lapV * 0.25f;
    if (parts) {
        parts[0] = a; parts[1] = b; parts[2] = wh; parts[3] = wv; parts[4] = gh; parts[5] = gv;
        parts[6] = sgnf(hm1 - hp1); parts[7] = sgnf(lapH); parts[8] = sgnf(vm1 - vp1); parts[9] = sgnf(lapV);
    }
    return wh * gh + wv * gv;
}

template <int DM>
__device__ void demosaic_df(const AdjSmem& sm, const TileCtx& t, int x, int y, float v[3]) {
    const AdjFrame& f = *t.f;
    const float* u = sm.u;
    v[0] = v[1] = v[2] = 0.0f;
    const bool ar = t.at_r(x, y), ab = t.at_b(x, y), rrow = (y & 1) == t.po.r_row;
    const int i = t.ui(x, y);
    if (DM == DM_HQLI) {
        if (x < 2 || x >= f.w - 2 || y < 2 || y >= f.h - 2) return;
        float n4 = u[i - 1] + u[i + 1] + u[i - kUW] + u[i + kUW];
        float d4 = u[i - kUW - 1] + u[i - kUW + 1] + u[i + kUW - 1] + u[i + kUW + 1];
        if (ar) { v[0] = u[i]; v[1] = n4 * 0.25f; v[2] = d4 * 0.25f; }
        else if (ab) { v[0] = d4 * 0.25f; v[1] = n4 * 0.25f; v[2] = u[i]; }
        else {
            float hz = (u[i - 1] + u[i + 1]) * 0.5f, vt = (u[i - kUW] + u[i + kUW]) * 0.5f;
            v[1] = u[i];
            v[0] = rrow ? hz : vt;
            v[2] = rrow ? vt : hz;
        }
        return;
    }
    const float* G = sm.G;
    const int j = t.gi(x, y);
    float g = G[j];
    v[1] = g;
    if (x < 1 || x >= f.w - 1 || y < 1 || y >= f.h - 1) return;
    // colour differences d = u - G at four neighbours, chosen by the site so that the lanes of a
    // warp (alternating sites along a row) run one path: at a red / blue site the diagonals, the
    // other channel g + (d1 + d2 + d3 + d4) / 4; at a G site the horizontal pair d1 + d2 and the
    // vertical pair d3 + d4, the row's colour from the first, the other colour from the second
    const bool rbs = ar || ab;
    const int u1 = rbs ? -kUW - 1 : -1, u2 = rbs ? -kUW + 1 : 1, u3 = rbs ? kUW - 1 : -kUW, u4 = rbs ? kUW + 1 : kUW;
    const int g1 = rbs ? -kGW - 1 : -1, g2 = rbs ? -kGW + 1 : 1, g3 = rbs ? kGW - 1 : -kGW, g4 = rbs ? kGW + 1 : kGW;
    const float d12 = (u[i + u1] - G[j + g1]) + (u[i + u2] - G[j + g2]);
    const float d3 = u[i + u3] - G[j + g3], d4 = u[i + u4] - G[j + g4];
    const float other = g + ((d12 + d3) + d4) * 0.25f;
    const float d34 = d3 + d4;
    const float own = u[i];
    v[0] = ar ? own : (ab ? other : g + (rrow ? d12 : d34) * 0.5f);
    v[2] = ab ? own : (ar ? other : g + (rrow ? d34 : d12) * 0.5f);
}

// one pixel (x, y) of the green region, at region row r, column c; rbs: a red / blue site
template <int DM>
__device__ __forceinline__ void gather_site(AdjSmem& sm, const TileCtx& t, int x, int y, int r, int c, bool rbs) {
    const AdjFrame& f = *t.f;
    const float* V0 = sm.gV[0];
    const float* V1 = sm.gV[1];
    const float* V2 = sm.gV[2];
    const bool hqli = DM == DM_HQLI;
    const int lo = hqli ? 2 : 1;  // sources with colour interpolation: [lo, w - lo) x [lo, h - lo)
    const int v = t.vi(x, y), i = t.ui(x, y), j = r * kGW + c;
    auto in_lo = [&](int xx, int yy) { return xx >= lo && xx < f.w - lo && yy >= lo && yy < f.h - lo; };
    float gu = 0.0f, gG = 0.0f;
    if (rbs) {
        const bool ar = t.at_r(x, y);
        // own source: the own channel reads u(q); AMAZE's green and other channel read G(q)
        if (in_lo(x, y)) {
            gu += ar ? V0[v] : V2[v];
            if (!hqli) gG += V1[v] + (ar ? V2[v] : V0[v]);
        } else if (!hqli) {
            gG += V1[v];
        }
        // diagonals: R/B sites of the other colour, whose other channel is this colour
        const float* Vd = ar ? V0 : V2;  // at a blue diagonal the other channel is red, and back
        float nb = 0.0f;
        if (in_lo(x - 1, y - 1)) nb += 0.25f * Vd[v - kVW - 1];
        if (in_lo(x + 1, y - 1)) nb += 0.25f * Vd[v - kVW + 1];
        if (in_lo(x - 1, y + 1)) nb += 0.25f * Vd[v + kVW - 1];
        if (in_lo(x + 1, y + 1)) nb += 0.25f * Vd[v + kVW + 1];
        // horizontal / vertical neighbours: G sites; a G site in a red row interpolates red
        // horizontally and blue vertically
        const bool rrow = (y & 1) == t.po.r_row;  // the neighbours x +- 1 share this row
        // (the horizontal pair feeds the row's colour, the vertical pair the other row's other
        // colour: both are this site's colour)
        const float* Vn = rrow ? V0 : V2;
        if (in_lo(x - 1, y)) nb += 0.5f * Vn[v - 1];
        if (in_lo(x + 1, y)) nb += 0.5f * Vn[v + 1];
        if (in_lo(x, y - 1)) nb += 0.5f * Vn[v - kVW];
        if (in_lo(x, y + 1)) nb += 0.5f * Vn[v + kVW];
        gu += nb;
        if (!hqli) gG -= nb;
    } else {
        // G site: its own green channel
        if (hqli) {
            if (in_lo(x, y)) gu += V1[v];
            // the green of each horizontal / vertical R/B neighbour reads 1/4 of u(q)
            float nb = 0.0f;
            if (in_lo(x - 1, y)) nb += V1[v - 1];
            if (in_lo(x + 1, y)) nb += V1[v + 1];
            if (in_lo(x, y - 1)) nb += V1[v - kVW];
            if (in_lo(x, y + 1)) nb += V1[v + kVW];
            gu += 0.25f * nb;
        } else {
            gG += in_lo(x, y) ? V0[v] + V1[v] + V2[v] : V1[v];
        }
    }
    sm.gu[i] = gu;
    if (!hqli) sm.gG[j] = gG;
}

// Adjoint of the demosaic as a gather: every pixel q of the green region (own pixels +- 1) adds up
// what the demosaic outputs that read u(q) or G(q) send back, from the gV planes (zero outside the
// own pixels).  These are the transposes of demosaic_df's expressions:
//   HQLI, source p in [2,w-2)^2: R/B site: own channel <- u(p); green <- 1/4 of the four
//     horizontal / vertical neighbours; other channel <- 1/4 of the four diagonals.  G site:
//     green <- u(p); the row's colour <- 1/2 (u(p-1) + u(p+1)), the other <- 1/2 (u(p-W) + u(p+W)).
//   AMAZE, source p in [1,w-1)^2 (else only green <- G(p)): green <- G(p); R/B site: own <- u(p),
//     other <- G(p) + 1/4 sum over diagonals d of (u(d) - G(d)); G site: R, B <- G(p) + 1/2 sum of
//     (u - G) over the horizontal or the vertical pair.
// By Bayer pairs (frame columns 2k, 2k + 1): every lane takes its pair's red / blue site, then its
// green site, so the lanes of a warp run the same path.
template <int DM>
__device__ void demosaic_gather(AdjSmem& sm, const TileCtx& t) {
    const int gw = t.tw + 2, gh = t.th + 2;
    const int xp0 = t.xg & ~1, np = (((t.xg + gw - 1) & ~1) - xp0) / 2 + 1;
    Walk2D wg(threadIdx.x, np);
    for (int s = threadIdx.x; s < np * gh; s += kAdjThreads, wg.step()) {
        const int r = wg.r, y = t.yg + r, xp = xp0 + 2 * wg.c;
        const int rbh = t.rb(xp, y) ? 0 : 1;  // the red / blue site of the pair
        int x = xp + rbh, c = x - t.xg;
        if (c >= 0 && c < gw) gather_site<DM>(sm, t, x, y, r, c, true);
        x = xp + 1 - rbh;
        c = x - t.xg;
        if (c >= 0 && c < gw) gather_site<DM>(sm, t, x, y, r, c, false);
    }
}

__device__ __forceinline__ void tile_of(const AdjLaunch& L, int item, int& fi, TileCtx& t) {
    const AdjFrame& f = L.f;
    const int per = f.tiles_x * f.tiles_y;
    fi = item / per;
    int k = item - fi * per;
    int ty = k / f.tiles_x, tx = k - ty * f.tiles_x;
    t.f = &L.f;
    t.po = pattern_offsets(f.pattern);
    tile_span(f.w, kTX, f.tiles_x, tx, t.x0, t.tw);
    tile_span(f.h, kTY, f.tiles_y, ty, t.y0, t.th);
    t.xu = t.x0 - 3;
    t.yu = t.y0 - 3;
    t.xg = t.x0 - 1;
    t.yg = t.y0 - 1;
}

// one raw sample of frame f (pixel formats of the product path)
__device__ __forceinline__ int adj_raw(const AdjFrame& f, const uint8_t* in, int x, int y) {
    // u16 frames (2-byte aligned: every frame of a launch is 2 w h bytes): one 16-bit load
    if (f.fmt == FMT_U16) return (int)__ldg(reinterpret_cast<const uint16_t*>(in) + (size_t)y * f.w + x);
    FrameParams fp;
    fp.w = f.w;
    fp.bd = f.bd;
    fp.mv = f.mv;
    fp.fmt = f.fmt;
    fp.in = in;
    fp.in_bytes = f.in_bytes;
    return dev::load_raw(fp, x, y);
}

// forward planes of one tile: raw, u (apron 3), green (apron 1); gradient planes cleared
template <bool BACKWARD, int DM>
__device__ void tile_forward(AdjSmem& sm, const TileCtx& t, const uint8_t* in) {
    const AdjFrame& f = *t.f;
    const int tid = threadIdx.x;
    const float mvf = (float)f.mv;
    const int uw = t.tw + 6, uh = t.th + 6;
    for (int c = tid; c < uw; c += kAdjThreads) {
        int x = min(max(t.xu + c, 0), f.w - 1);
        // gx = x (gw-1) / (w-1), the apply loop's grid position
        float gxf = (float)x * (float)(f.gw - 1) / (float)(f.w - 1);
        int gi = min(max((int)gxf, 0), f.gw - 2);
        sm.col_gx[c] = gi;
        sm.col_fx[c] = gxf - (float)gi;
    }
    for (int r = tid; r < uh; r += kAdjThreads) {
        int y = min(max(t.yu + r, 0), f.h - 1);
        float gyf = (float)y * (float)(f.gh - 1) / (float)(f.h - 1);
        int gi = min(max((int)gyf, 0), f.gh - 2);
        sm.row_gy[r] = gi;
        sm.row_fy[r] = gyf - (float)gi;
    }
    __syncthreads();
    const float* grid = sm.th + 16;
    Walk2D wk(tid, uw);
    for (int s = tid; s < uw * uh; s += kAdjThreads, wk.step()) {
        const int r = wk.r, c = wk.c;
        int x = t.xu + c, y = t.yu + r;
        int i = r * kUW + c;
        int ri = 0;
        float uv = 0.0f;
        if (x >= 0 && x < f.w && y >= 0 && y < f.h) {
            int cc = t.cfa(x, y);
            ri = adj_raw(f, in, x, y);
            const float rv = (float)ri;
            float b = clampf(rv - sm.th[cc], 0.0f, mvf);
            int gx = sm.col_gx[c], gy = sm.row_gy[r];
            float fx = sm.col_fx[c], fy = sm.row_fy[r];
            const float* g0 = grid + (gy * f.gw + gx) * 4 + cc;
            float gain = g0[0] * (1.0f - fx) * (1.0f - fy) + g0[4] * fx * (1.0f - fy) +
                         g0[4 * f.gw] * (1.0f - fx) * fy + g0[4 * f.gw + 4] * fx * fy;
            float l = clampf(b * gain, 0.0f, mvf);
            uv = clampf(l * wb_of(sm.th, cc), 0.0f, mvf);
        }
        sm.raw[i] = (uint16_t)ri;  // samples of at most 16 bits
        sm.u[i] = uv;
        if (BACKWARD) sm.gu[i] = 0.0f;
    }
    if (BACKWARD) {
        for (int s = tid; s < 3 * kVH * kVW; s += kAdjThreads) (&sm.gV[0][0])[s] = 0.0f;
    }
    __syncthreads();
    if (DM == DM_AMAZE) {
        // by Bayer pairs (frame columns 2k, 2k + 1): every lane takes the pair's red / blue site
        // (AMAZE's weighted green) and its green site (a copy), so no lane idles beside another.
        // (The demosaic adjoint writes every gG of the green region, so gG needs no clearing.)
        const int gw = t.tw + 2, gh = t.th + 2;
        const int xp0 = t.xg & ~1, np = (((t.xg + gw - 1) & ~1) - xp0) / 2 + 1;
        Walk2D wg(tid, np);
        for (int s = tid; s < np * gh; s += kAdjThreads, wg.step()) {
            const int r = wg.r, y = t.yg + r, xp = xp0 + 2 * wg.c;
            const int rbh = t.rb(xp, y) ? 0 : 1;  // the red / blue site of the pair
            const bool rows_in = y >= 2 && y < f.h - 2;
            int x = xp + rbh, c = x - t.xg;
            if (c >= 0 && c < gw)
                sm.G[r * kGW + c] = rows_in && x >= 2 && x < f.w - 2 ? amaze_df(sm, t, x, y, nullptr) : -1.0f;
            x = xp + 1 - rbh;
            c = x - t.xg;
            if (c >= 0 && c < gw) sm.G[r * kGW + c] = rows_in && x >= 2 && x < f.w - 2 ? sm.u[t.ui(x, y)] : -1.0f;
        }
        __syncthreads();
    }
}

__device__ __forceinline__ void tone_df(const float* knots, float o, float o_to_knot, float& t, int& idx, float& frac) {
    float fi = o * o_to_knot;
    int k = (int)fi;
    float fr = fi - (float)k;
    if (k > 31) { k = 31; fr = 1.0f; }
    if (k < 0) { k = 0; fr = 0.0f; }
    idx = k;
    frac = fr;
    t = knots[k] * (1.0f - fr) + knots[k + 1] * fr;
}

struct RegAcc {
    float bl[4], wb[3], ccm[9], loss;
};

// forward (+ adjoint) of the tile's own pixels
template <bool BACKWARD, int DM>
__device__ void tile_pixels(AdjSmem& sm, const TileCtx& t, int fi, const AdjLaunch& L, RegAcc& acc) {
    const AdjFrame& f = *t.f;
    const float mvf = (float)f.mv;
    const float* M = sm.th + 7;
    const float* knots = sm.th + 16 + 4 * f.gw * f.gh;
    const size_t frame_px = (size_t)f.w * f.h;
    const float o_to_knot = 32.0f / mvf;
    const int n_own = t.tw * t.th;
    float* knot_lane = sm.knot_lane + (threadIdx.x & 31);
    const bool border_tile = t.x0 < 2 || t.x0 + t.tw > f.w - 2 || t.y0 < 2 || t.y0 + t.th > f.h - 2;
    // whole warps iterate together (the knot sums are warp-wide); lanes past the end repeat the
    // last pixel with zero weight
    Walk2D wp(threadIdx.x, t.tw);
    for (int s0 = threadIdx.x & ~31; s0 < n_own; s0 += kAdjThreads, wp.step()) {
        const bool valid = s0 + (int)(threadIdx.x & 31) < n_own;
        int r = wp.r, c = wp.c;
        if (!valid) {
            r = t.th - 1;  // the last pixel, with zero weight
            c = t.tw - 1;
        }
        int x = t.x0 + c, y = t.y0 + r;
        int sx = x, sy = y;  // the source is the pixel itself away from the frame's border
        if (border_tile) dev::border_source(x, y, f.w, f.h, f.border_mode, sx, sy);
        float v[3], rgb[3], pre[3], o[3], tt[3], fr[3];
        int idx[3];
        demosaic_df<DM>(sm, t, sx, sy, v);
#pragma unroll
        for (int k = 0; k < 3; k++) rgb[k] = clampf(v[k], 0.0f, mvf);
#pragma unroll
        for (int q = 0; q < 3; q++) {
            pre[q] = M[3 * q] * rgb[0] + M[3 * q + 1] * rgb[1] + M[3 * q + 2] * rgb[2];
            o[q] = clampf(pre[q], 0.0f, mvf);
        }
#pragma unroll
        for (int k = 0; k < 3; k++) tone_df(knots, o[k], o_to_knot, tt[k], idx[k], fr[k]);
        const size_t pi = ((size_t)fi * frame_px + (size_t)y * f.w + x) * 3;
        if constexpr (!BACKWARD) {
            if (valid) {
#pragma unroll
                for (int k = 0; k < 3; k++) L.rgb_out[pi + k] = tt[k];
            }
        } else {
        float gt[3], go[3], grgb[3] = {0.0f, 0.0f, 0.0f}, gv[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            float rv = L.ref[pi + k];
            if (L.mode == 0) {
                float e = tt[k] - rv;
                gt[k] = valid ? 2.0f * e : 0.0f;
                if (valid) acc.loss += e * e;
            } else {
                gt[k] = valid ? rv : 0.0f;
                if (valid) acc.loss += tt[k] * rv;
            }
            if (valid) {
                atomicAdd(&knot_lane[idx[k] * 32], gt[k] * (1.0f - fr[k]));
                atomicAdd(&knot_lane[(idx[k] + 1) * 32], gt[k] * fr[k]);
            }
            go[k] = gt[k] * (knots[idx[k] + 1] - knots[idx[k]]) * o_to_knot;
        }
#pragma unroll
        for (int q = 0; q < 3; q++) {
            float gp = go[q] * inside(pre[q], 0.0f, mvf);
#pragma unroll
            for (int j = 0; j < 3; j++) {
                acc.ccm[3 * q + j] += gp * rgb[j];
                grgb[j] += M[3 * q + j] * gp;
            }
        }
#pragma unroll
        for (int k = 0; k < 3; k++) gv[k] = grgb[k] * inside(v[k], 0.0f, mvf);
        if (valid) {
            // border copies add into their source, which its own output also writes: atomics in
            // tiles with border outputs, plain stores elsewhere
            const int vi = t.vi(sx, sy);
            if (border_tile) {
#pragma unroll
                for (int k = 0; k < 3; k++) atomicAdd(&sm.gV[k][vi], gv[k]);
            } else {
#pragma unroll
                for (int k = 0; k < 3; k++) sm.gV[k][vi] = gv[k];
            }
        }
        }
    }
}

// adjoint of the green plane into u, then of u into the per-pixel parameters; acc_grid: the
// CTA's lens-shading sums (global memory, written by this CTA alone)
template <int DM>
__device__ void tile_back_planes(AdjSmem& sm, const TileCtx& t, RegAcc& acc, float* acc_grid) {
    const AdjFrame& f = *t.f;
    const int tid = threadIdx.x;
    const float mvf = (float)f.mv;
    __syncthreads();
    if (DM == DM_AMAZE) {
        // by Bayer pairs, as the forward green loop: each lane the pair's green site (one add)
        // and its red / blue site (AMAZE's adjoint)
        const int gw = t.tw + 2, gh = t.th + 2;
        const int xp0 = t.xg & ~1, np = (((t.xg + gw - 1) & ~1) - xp0) / 2 + 1;
        Walk2D wg(tid, np);
        for (int s = tid; s < np * gh; s += kAdjThreads, wg.step()) {
          const int r = wg.r, y = t.yg + r, xp = xp0 + 2 * wg.c;
          const int rbh = t.rb(xp, y) ? 0 : 1;  // the red / blue site of the pair
          // the green site first
          {
              const int x = xp + 1 - rbh, c = x - t.xg;
              if (c >= 0 && c < gw && x >= 2 && x < f.w - 2 && y >= 2 && y < f.h - 2) {
                  const float g = sm.gG[r * kGW + c];
                  if (g != 0.0f) atomicAdd(&sm.gu[t.ui(x, y)], g);
              }
          }
          {
            const int x = xp + rbh, c = x - t.xg;
            if (c < 0 || c >= gw) continue;
            float g = sm.gG[r * kGW + c];
            if (g == 0.0f || x < 2 || x >= f.w - 2 || y < 2 || y >= f.h - 2) continue;
            int i = t.ui(x, y);
            float P[10];
            amaze_df(sm, t, x, y, P);
            float a = P[0], b = P[1], wh = P[2], wv = P[3], gh_ = P[4], gv_ = P[5];
            float rs = __fdividef(1.0f, a + b);
            float rs2 = rs * rs;
            float dgH = -a * a * b * (gh_ - gv_) * rs2;
            float dgV = -b * b * a * (gv_ - gh_) * rs2;
            float tH = g * (wh * 0.25f + dgH * P[7]);
            float tV = g * (wv * 0.25f + dgV * P[9]);
            atomicAdd(&sm.gu[i - 1], g * (wh * 0.5f + dgH * P[6]));
            atomicAdd(&sm.gu[i + 1], g * (wh * 0.5f - dgH * P[6]));
            atomicAdd(&sm.gu[i - 2], -tH);
            atomicAdd(&sm.gu[i + 2], -tH);
            atomicAdd(&sm.gu[i - kUW], g * (wv * 0.5f + dgV * P[8]));
            atomicAdd(&sm.gu[i + kUW], g * (wv * 0.5f - dgV * P[8]));
            atomicAdd(&sm.gu[i - 2 * kUW], -tV);
            atomicAdd(&sm.gu[i + 2 * kUW], -tV);
            atomicAdd(&sm.gu[i], 2.0f * (tH + tV));
          }
        }
        __syncthreads();
    }
    const int uw = t.tw + 6, uh = t.th + 6, nu = uw * uh;
    const float* grid = sm.th + 16;
    // the tile's lens-shading cells: local node (lx, ly) is grid node (gx_lo + lx, gy_lo + ly)
    const int gx_lo = sm.col_gx[0], gy_lo = sm.row_gy[0];
    const bool local = sm.col_gx[uw - 1] + 1 - gx_lo < kLNX && sm.row_gy[uh - 1] + 1 - gy_lo < kLNY;
    const int gnode[4] = {0, 4, 4 * f.gw, 4 * f.gw + 4};
    const int lnode[4] = {0, 4 * 32, 4 * kLNX * 32, (4 * kLNX + 4) * 32};
    float* node_lane = sm.node_lane + (tid & 31);
    Walk2D wu(tid, uw);
    for (int s = tid; s < nu; s += kAdjThreads, wu.step()) {
        const int r = wu.r, c = wu.c;
        int i = r * kUW + c;
        float g = sm.gu[i];
        int x = t.xu + c, y = t.yu + r;
        float gw4[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (g != 0.0f && x >= 0 && x < f.w && y >= 0 && y < f.h) {
            int cc = t.cfa(x, y);
            float rv = (float)sm.raw[i];
            float b = clampf(rv - sm.th[cc], 0.0f, mvf);
            int gx = sm.col_gx[c], gy = sm.row_gy[r];
            float fx = sm.col_fx[c], fy = sm.row_fy[r];
            int n0 = (gy * f.gw + gx) * 4 + cc;
            const float* g0 = grid + n0;
            float w00 = (1.0f - fx) * (1.0f - fy), w10 = fx * (1.0f - fy), w01 = (1.0f - fx) * fy, w11 = fx * fy;
            float gain = g0[0] * w00 + g0[4] * w10 + g0[4 * f.gw] * w01 + g0[4 * f.gw + 4] * w11;
            float l = clampf(b * gain, 0.0f, mvf);
            float wb = wb_of(sm.th, cc);
            if (l * wb > 0.0f && l * wb < mvf) {
                float gwb = g * l;
                if (cc == 0) acc.wb[0] += gwb; else if (cc == 3) acc.wb[2] += gwb; else acc.wb[1] += gwb;
                float gl = g * wb;
                if (b * gain > 0.0f && b * gain < mvf) {
                    float ggain = gl * b;
                    gw4[0] = ggain * w00;
                    gw4[1] = ggain * w10;
                    gw4[2] = ggain * w01;
                    gw4[3] = ggain * w11;
                    if (local) {
                        float* q = node_lane + (((gy - gy_lo) * kLNX + (gx - gx_lo)) * 4 + cc) * 32;
#pragma unroll
                        for (int k = 0; k < 4; k++) atomicAdd(q + lnode[k], gw4[k]);
                    } else {
#pragma unroll
                        for (int k = 0; k < 4; k++) atomicAdd(acc_grid + n0 + gnode[k], gw4[k]);
                    }
                    float v = rv - sm.th[cc];
                    if (v > 0.0f && v < mvf) {
                        float gb = -gl * gain;
                        if (cc == 0) acc.bl[0] += gb; else if (cc == 1) acc.bl[1] += gb; else if (cc == 2) acc.bl[2] += gb; else acc.bl[3] += gb;
                    }
                }
            }
        }
    }
    __syncthreads();
    if (local) {
        // local nodes into the CTA's sums: warp w takes nodes w, w + 8, ...; its lanes add the
        // node's 32 lane columns by a fixed butterfly and lane 0 adds the sum to the partial
        // vector (a reduction in global memory: the barriers between tiles order a node's
        // additions).  The table is cleared for the next tile.
        const int lane = tid & 31, warp = tid >> 5;
        for (int e = warp; e < kLocalNodes; e += kAdjThreads / 32) {
            float v = sm.node_lane[e * 32 + lane];
            sm.node_lane[e * 32 + lane] = 0.0f;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            const int lx = (e >> 2) % kLNX, ly = (e >> 2) / kLNX;
            if (lane == 0 && v != 0.0f && gx_lo + lx < f.gw && gy_lo + ly < f.gh)
                atomicAdd(acc_grid + ((gy_lo + ly) * f.gw + gx_lo + lx) * 4 + (e & 3), v);
        }
        __syncthreads();
    }
}

// DM: the launch's demosaic algorithm (every frame of a launch shares the descriptor)
template <bool BACKWARD, int DM>
__global__ void __launch_bounds__(kAdjThreads, 4) adjoint_kernel(const __grid_constant__ AdjLaunch L) {
    extern __shared__ __align__(16) uint8_t dsm[];
    AdjSmem& sm = *reinterpret_cast<AdjSmem*>(dsm);
    const int tid = threadIdx.x;
    const int ng = 4 * L.f.gw * L.f.gh;
    // this CTA's partial vector: BL, WB, CCM, the lens-shading grid (summed in place), the knots
    float* part = BACKWARD ? L.partials + (size_t)blockIdx.x * (L.n_params + 1) : nullptr;
    for (int k = tid; k < L.n_params; k += kAdjThreads) sm.th[k] = L.theta[k];
    if (BACKWARD) {
        for (int k = tid; k < ng; k += kAdjThreads) part[16 + k] = 0.0f;
        for (int k = tid; k < 33; k += kAdjThreads) sm.acc_knots[k] = 0.0f;
        for (int k = tid; k < 33 * 32; k += kAdjThreads) sm.knot_lane[k] = 0.0f;
        for (int k = tid; k < kLocalNodes * 32; k += kAdjThreads) sm.node_lane[k] = 0.0f;
    }
    __syncthreads();
    RegAcc acc;
#pragma unroll
    for (int k = 0; k < 4; k++) acc.bl[k] = 0.0f;
#pragma unroll
    for (int k = 0; k < 3; k++) acc.wb[k] = 0.0f;
#pragma unroll
    for (int k = 0; k < 9; k++) acc.ccm[k] = 0.0f;
    acc.loss = 0.0f;
    // Tiles: the first wave by CTA index, then (backward) claimed from the launch's counter one
    // tile ahead, so that CTAs given costlier tiles (frame borders, wider last columns) take fewer
    // of them; the render launch keeps the fixed stride.  Thread 0 writes slot k & 1 at the start
    // of tile k and every thread reads it after the tile's barriers; the slot is written again at
    // tile k + 2, after tile k + 1's barriers.
    unsigned* const counter = BACKWARD ? L.tile_counter : nullptr;
    int item = blockIdx.x;
    for (int k = 0; item < L.n_items; k++) {
        if (counter && tid == 0) sm.next_item[k & 1] = (int)gridDim.x + (int)atomicAdd(counter, 1u);
        int fi;
        TileCtx t;
        tile_of(L, item, fi, t);
        const uint8_t* in = L.raw + (size_t)fi * L.f.in_bytes;
        tile_forward<BACKWARD, DM>(sm, t, in);
        tile_pixels<BACKWARD, DM>(sm, t, fi, L, acc);
        if (BACKWARD) {
            __syncthreads();
            demosaic_gather<DM>(sm, t);
            tile_back_planes<DM>(sm, t, acc, part + 16);
        }
        else __syncthreads();
        item = counter ? sm.next_item[k & 1] : item + (int)gridDim.x;
    }
    if constexpr (BACKWARD) {
        // the partial reduction may start once every CTA is here (it waits for this grid's end)
        asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
        // the last CTA to finish (counter[1]) clears both words for the next launch: every other
        // CTA made its last claim before counting itself
        if (tid == 0) {
            __threadfence();
            if (atomicAdd(counter + 1, 1u) == gridDim.x - 1) {
                counter[0] = 0u;
                counter[1] = 0u;
            }
        }
    }
    if constexpr (BACKWARD) {
        // block reduction of the register accumulators, warps in order
        float vals[17];
#pragma unroll
        for (int k = 0; k < 4; k++) vals[k] = acc.bl[k];
#pragma unroll
        for (int k = 0; k < 3; k++) vals[4 + k] = acc.wb[k];
#pragma unroll
        for (int k = 0; k < 9; k++) vals[7 + k] = acc.ccm[k];
        vals[16] = acc.loss;
        const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
        for (int k = 0; k < 17; k++) {
            float v = vals[k];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) sm.red[warp][k] = v;
        }
        __syncthreads();
        if (tid < 17) {
            float v = 0.0f;
            for (int w = 0; w < kAdjThreads / 32; w++) v += sm.red[w][tid];
            if (tid < 16) part[tid] = v;
            else part[L.n_params] = v;
        }
        for (int k = tid; k < 33; k += kAdjThreads) {
            float v = sm.acc_knots[k];
            for (int l = 0; l < 32; l++) v += sm.knot_lane[k * 32 + l];
            part[16 + ng + k] = v;
        }
    }
}

// grad[k] = sum over CTAs of partial[cta][k]; loss likewise (index n_params).  32 parameters per
// block of 32 x kRedRows threads: row j adds CTAs j, j + kRedRows, ... in order (coalesced over
// the parameters), then the rows are added in order, so the sum is the same in every run.
constexpr int kRedRows = 16;
__global__ void __launch_bounds__(32 * kRedRows) reduce_partials_kernel(const float* partials, int n_parts,
                                                                       int n_params, float* grad, float* loss) {
    __shared__ float rows[kRedRows][33];
    asm volatile("griddepcontrol.wait;" ::: "memory");  // launched as the adjoint's dependent
    const int k = blockIdx.x * 32 + threadIdx.x;
    float s = 0.0f;
    if (k <= n_params)
        for (int c = threadIdx.y; c < n_parts; c += kRedRows) s += partials[(size_t)c * (n_params + 1) + k];
    rows[threadIdx.y][threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.y == 0 && k <= n_params) {
        float t = 0.0f;
        for (int j = 0; j < kRedRows; j++) t += rows[j][threadIdx.x];
        if (k < n_params) grad[k] = t;
        else if (loss) *loss = t;
    }
}

}  // namespace

int adj_tile_grid(int w, int h, int& tx, int& ty) {
    tx = tiles_along(w, kTX);
    ty = tiles_along(h, kTY);
    return tx * ty;
}

size_t adj_smem_bytes() { return sizeof(AdjSmem); }

cudaError_t adj_grid_limit(int& limit) {
    static int cached[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(device_setup_mutex());
    if (!cached[dev]) {
        const int smem = (int)sizeof(AdjSmem);
        if ((e = cudaFuncSetAttribute(adjoint_kernel<true, DM_AMAZE>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) ||
            (e = cudaFuncSetAttribute(adjoint_kernel<false, DM_AMAZE>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) ||
            (e = cudaFuncSetAttribute(adjoint_kernel<true, DM_HQLI>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) ||
            (e = cudaFuncSetAttribute(adjoint_kernel<false, DM_HQLI>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)))
            return e;
        int n = 0, sms = 0;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, adjoint_kernel<true, DM_AMAZE>, kAdjThreads, smem)) ||
            (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)))
            return e;
        cached[dev] = sms * (n > 0 ? n : 1);
    }
    limit = cached[dev];
    return cudaSuccess;
}

cudaError_t launch_adjoint(const AdjLaunch& L, bool backward, int grid, float* d_grad, float* d_loss, cudaStream_t st) {
    const size_t smem = sizeof(AdjSmem);
    const bool hqli = L.f.demosaic == DM_HQLI;
    if (backward) {
        if (hqli)
            adjoint_kernel<true, DM_HQLI><<<grid, kAdjThreads, smem, st>>>(L);
        else
            adjoint_kernel<true, DM_AMAZE><<<grid, kAdjThreads, smem, st>>>(L);
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((L.n_params + 1 + 31) / 32);
        cfg.blockDim = dim3(32, kRedRows);
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        const float* parts = L.partials;
        const cudaError_t e = cudaLaunchKernelEx(&cfg, reduce_partials_kernel, parts, grid, L.n_params, d_grad, d_loss);
        if (e != cudaSuccess) return e;
    } else if (hqli) {
        adjoint_kernel<false, DM_HQLI><<<grid, kAdjThreads, smem, st>>>(L);
    } else {
        adjoint_kernel<false, DM_AMAZE><<<grid, kAdjThreads, smem, st>>>(L);
    }
    return cudaGetLastError();
}

}  // namespace imop
