// isp_tile.cuh - one output tile of the fused RAW->RGB pipeline.
//
// A CTA owns a tw x th tile of output pixels.  It stages the tile plus a 5-pixel apron of the
// unpacked, black-levelled mosaic in shared memory, corrects defects and applies lens shading
// and white balance on a 3-pixel apron, interpolates green on a 1-pixel apron, then produces
// demosaic -> CCM -> tone for its own pixels and writes them out.  Each pixel reads its RAW bytes
// from global memory once per CTA that needs it (aprons are L2 hits) and each RGB byte is
// written once.
//
// Apron radii: output (x,y) needs demosaic inputs within 1 (HQLI) or, through green, 3 pixels
// (AMAZE / MG); the defect kernel reads 2 more.  Border pixels copy from pixels at most 2 away
// (border_source), which lie inside the same tile because tiles are at least 4 pixels wide.
#pragma once

#include "isp_device.cuh"

namespace imop {

constexpr int kThreads = 256;
constexpr int kHaloRaw = 5;
constexpr int kHaloBay = 3;
constexpr int kHaloG = 1;

// The nominal tile is TW x TH; the last tile of a row/column absorbs a remainder below 4.
template <int TW, int TH>
struct TileGeom {
    static constexpr int TWM = TW + 3, THM = TH + 3;
    static constexpr int OR_W = TWM + 2 * kHaloRaw, OR_H = THM + 2 * kHaloRaw;
    static constexpr int DP_W = TWM + 2 * kHaloBay, DP_H = THM + 2 * kHaloBay;
    static constexpr int GG_W = TWM + 2 * kHaloG, GG_H = THM + 2 * kHaloG;
    static constexpr int OUT_PITCH = TWM * 6;
};

template <int TW, int TH>
struct TileSmem {
    using G = TileGeom<TW, TH>;
    uint16_t orig[G::OR_H * G::OR_W];
    uint16_t dpc[G::DP_H * G::DP_W];
    uint16_t bay[G::DP_H * G::DP_W];
    float green[G::GG_H * G::GG_W];
    uint8_t out[G::THM * G::OUT_PITCH];
};

// tile grid of one frame along one axis: n tiles of `t` pixels, the last one absorbing a
// remainder smaller than 4
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

template <int TW, int TH>
__device__ void process_tile(const FrameParams& fp, int x0, int y0, int tw, int th, TileSmem<TW, TH>& sm,
                             Overrides ov, bool detect_seeds) {
    using G = TileGeom<TW, TH>;
    const int W = fp.w, H = fp.h, mv = fp.mv;
    const PatternOffsets po = pattern_offsets(fp.pattern);
    const int tid = threadIdx.x;
    const bool dpc_on = (fp.stages & 2u) != 0;
    const bool adaptive = dpc_on && fp.dpc_mode == 0;

    // ---- 1. unpack + black level over the tile and a 5-pixel apron ----------------------
    const int ow = tw + 2 * kHaloRaw, oh = th + 2 * kHaloRaw;
    for (int i = tid; i < ow * oh; i += kThreads) {
        int r = i / ow, c = i - r * ow;
        int gx = x0 - kHaloRaw + c, gy = y0 - kHaloRaw + r;
        int v = 0;
        if (gx >= 0 && gx < W && gy >= 0 && gy < H) v = dev::orig_value(fp, gx, gy, po);
        sm.orig[r * G::OR_W + c] = (uint16_t)v;
    }
    __syncthreads();

    auto ORIG = [&](int gx, int gy) -> int {
        return sm.orig[(gy - y0 + kHaloRaw) * G::OR_W + (gx - x0 + kHaloRaw)];
    };
    auto DPC = [&](int gx, int gy) -> int { return sm.dpc[(gy - y0 + kHaloBay) * G::DP_W + (gx - x0 + kHaloBay)]; };
    auto BAY = [&](int gx, int gy) -> int { return sm.bay[(gy - y0 + kHaloBay) * G::DP_W + (gx - x0 + kHaloBay)]; };

    // ---- 2. defect correction (Jacobi), lens shading, Bayer white balance, 3-pixel apron ---
    const int dw = tw + 2 * kHaloBay, dh = th + 2 * kHaloBay;
    for (int i = tid; i < dw * dh; i += kThreads) {
        int r = i / dw, c = i - r * dw;
        int gx = x0 - kHaloBay + c, gy = y0 - kHaloBay + r;
        int o = ORIG(gx, gy);
        int j = o, b = 0;
        if (gx >= 0 && gx < W && gy >= 0 && gy < H) {
            if (adaptive && gx >= 2 && gx < W - 2 && gy >= 2 && gy < H - 2) {
                int nb[8] = {ORIG(gx - 2, gy - 2), ORIG(gx, gy - 2), ORIG(gx + 2, gy - 2), ORIG(gx - 2, gy),
                             ORIG(gx + 2, gy), ORIG(gx - 2, gy + 2), ORIG(gx, gy + 2), ORIG(gx + 2, gy + 2)};
                j = dev::dpc_apply(o, nb, dev::dpc_valid_mask(gx, gy, W, H), fp.dpc_thr);
                if (ov.n > 0) {
                    int s = find_override(ov.idx, ov.val, ov.n, gy * W + gx);
                    if (s >= 0) j = s;
                }
            } else if (dpc_on && fp.dpc_mode == 1 && gx >= 2 && gx < W - 2 && gy >= 2 && gy < H - 2) {
                int s = map_lookup(fp, gx, gy);
                if (s >= 0) j = s;
            }
            b = dev::bayer_tail(fp, j, gx, gy, bayer_color(gy, gx, po));
        }
        sm.dpc[r * G::DP_W + c] = (uint16_t)j;
        sm.bay[r * G::DP_W + c] = (uint16_t)b;
    }
    __syncthreads();

    // ---- 3. defect-chain seeds: own pixels whose raster-earlier neighbour was corrected and
    //         whose value changes when those corrections are seen (sequential semantics) ----
    if (detect_seeds && adaptive) {
        for (int i = tid; i < tw * th; i += kThreads) {
            int r = i / tw, c = i - r * tw;
            int gx = x0 + c, gy = y0 + r;
            if (gx < 2 || gx >= W - 2 || gy < 2 || gy >= H - 2) continue;
            unsigned valid = dev::dpc_valid_mask(gx, gy, W, H);
            const int ex[4] = {gx - 2, gx, gx + 2, gx - 2}, ey[4] = {gy - 2, gy - 2, gy - 2, gy};
            bool any = false;
#pragma unroll
            for (int k = 0; k < 4; k++)
                if ((valid >> k) & 1u) any |= DPC(ex[k], ey[k]) != ORIG(ex[k], ey[k]);
            if (!any) continue;
            int nb[8] = {DPC(gx - 2, gy - 2), DPC(gx, gy - 2), DPC(gx + 2, gy - 2), DPC(gx - 2, gy),
                         ORIG(gx + 2, gy), ORIG(gx - 2, gy + 2), ORIG(gx, gy + 2), ORIG(gx + 2, gy + 2)};
            int s1 = dev::dpc_apply(ORIG(gx, gy), nb, valid, fp.dpc_thr);
            if (s1 != DPC(gx, gy)) {
                int slot = atomicAdd(fp.seed_count, 1);
                if (slot < fp.seed_cap) fp.seeds[slot] = gy * W + gx;
                else atomicExch(fp.status, 104 /* IMOP_ERR_CAPACITY */);
            }
        }
    }

    // ---- 4. green plane on a 1-pixel apron (AMAZE, MG) ------------------------------------
    const int gwid = tw + 2 * kHaloG, ghgt = th + 2 * kHaloG;
    if (fp.demosaic != DM_HQLI) {
        for (int i = tid; i < gwid * ghgt; i += kThreads) {
            int r = i / gwid, c = i - r * gwid;
            int gx = x0 - kHaloG + c, gy = y0 - kHaloG + r;
            float g = -1.0f;
            if (gx >= 0 && gx < W && gy >= 0 && gy < H) {
                bool at_r = ((gy & 1) == po.r_row) && ((gx & 1) == po.r_col);
                bool at_b = ((gy & 1) == po.b_row) && ((gx & 1) == po.b_col);
                bool interior = gx >= 2 && gx < W - 2 && gy >= 2 && gy < H - 2;
                if (!at_r && !at_b) {
                    // AMAZE sets green only inside the interior; MG at every green site
                    if (interior || fp.demosaic == DM_MG) g = (float)BAY(gx, gy);
                } else if (interior) {
                    int cc = BAY(gx, gy);
                    if (fp.demosaic == DM_AMAZE) {
                        g = dev::amaze_green(cc, BAY(gx - 1, gy), BAY(gx + 1, gy), BAY(gx - 2, gy), BAY(gx + 2, gy),
                                             BAY(gx, gy - 1), BAY(gx, gy + 1), BAY(gx, gy - 2), BAY(gx, gy + 2));
                    } else {
                        int n1 = BAY(gx, gy - 1) + BAY(gx, gy + 1) + BAY(gx + 1, gy) + BAY(gx - 1, gy);
                        int n2 = BAY(gx, gy - 2) + BAY(gx, gy + 2) + BAY(gx + 2, gy) + BAY(gx - 2, gy);
                        if (fp.bd <= 8) {
                            // src/algorithms/mg.cpp:58-69 (integer Malvar-He-Cutler)
                            g = (float)dev::clampi((4 * cc + 2 * n1 - n2 + 4) >> 3, 0, mv);
                        } else {
                            // src/algorithms/mg.cpp:187-196: (4c + 2*(n+s+e+w) - (n2+s2+e2+w2)) / 8
                            float t = dev::fsub(dev::fadd(dev::fmul(4.0f, (float)cc), dev::fmul(2.0f, (float)n1)),
                                                (float)n2);
                            g = __fdiv_rn(t, 8.0f);
                        }
                    }
                }
            }
            sm.green[r * G::GG_W + c] = g;
        }
    }
    __syncthreads();
    auto GRN = [&](int gx, int gy) -> float { return sm.green[(gy - y0 + kHaloG) * G::GG_W + (gx - x0 + kHaloG)]; };

    // ---- 5. demosaic + RGB tail + tone for own pixels --------------------------------------
    const int bpc = fp.out_bpc;
    for (int i = tid; i < tw * th; i += kThreads) {
        int r = i / tw, c = i - r * tw;
        int gx = x0 + c, gy = y0 + r;
        int sx, sy;
        dev::border_source(gx, gy, W, H, fp.border_mode, sx, sy);
        bool at_r = ((sy & 1) == po.r_row) && ((sx & 1) == po.r_col);
        bool at_b = ((sy & 1) == po.b_row) && ((sx & 1) == po.b_col);
        int R = 0, Gv = 0, B = 0;
        if (fp.demosaic == DM_HQLI) {
            // detail::hqli_core (src/algorithms/interp_core.hpp:39-65); outside the interior the
            // reference leaves the zeroed output untouched
            if (sx >= 2 && sx < W - 2 && sy >= 2 && sy < H - 2) {
                int n4 = BAY(sx - 1, sy) + BAY(sx + 1, sy) + BAY(sx, sy - 1) + BAY(sx, sy + 1);
                int d4 = BAY(sx - 1, sy - 1) + BAY(sx + 1, sy - 1) + BAY(sx - 1, sy + 1) + BAY(sx + 1, sy + 1);
                if (at_r) {
                    R = BAY(sx, sy); Gv = (n4 + 2) / 4; B = (d4 + 2) / 4;
                } else if (at_b) {
                    R = (d4 + 2) / 4; Gv = (n4 + 2) / 4; B = BAY(sx, sy);
                } else {
                    Gv = BAY(sx, sy);
                    int hz = (BAY(sx - 1, sy) + BAY(sx + 1, sy) + 1) / 2;
                    int vt = (BAY(sx, sy - 1) + BAY(sx, sy + 1) + 1) / 2;
                    if ((sy & 1) == po.r_row) { R = hz; B = vt; } else { B = hz; R = vt; }
                }
                R = min(R, mv); Gv = min(Gv, mv); B = min(B, mv);
            }
        } else if (fp.demosaic == DM_MG && fp.bd <= 8) {
            // integer colour differences (src/algorithms/mg.cpp:74-146)
            int g = (int)GRN(sx, sy);
            int Ri = 0, Bi = 0, Gi = g;
            if (sx >= 1 && sx < W - 1 && sy >= 1 && sy < H - 1) {
                auto cdi = [&](int x, int y) { return BAY(x, y) - (int)GRN(x, y); };
                if (at_r || at_b) {
                    int s = cdi(sx - 1, sy - 1) + cdi(sx + 1, sy - 1) + cdi(sx - 1, sy + 1) + cdi(sx + 1, sy + 1);
                    int other = g + (s + 2) / 4;
                    if (at_r) { Ri = BAY(sx, sy); Bi = other; } else { Bi = BAY(sx, sy); Ri = other; }
                } else {
                    int hz = cdi(sx - 1, sy) + cdi(sx + 1, sy), vt = cdi(sx, sy - 1) + cdi(sx, sy + 1);
                    int rc = ((sy & 1) == po.r_row) ? hz : vt, bc = ((sy & 1) == po.r_row) ? vt : hz;
                    Ri = g + (rc + 1) / 2;
                    Bi = g + (bc + 1) / 2;
                }
            }
            R = dev::clampi(Ri, 0, mv); Gv = dev::clampi(Gi, 0, mv); B = dev::clampi(Bi, 0, mv);
        } else {
            // float colour differences (src/algorithms/common.hpp:142-199, amaze.cpp:62-114)
            float g = GRN(sx, sy), Rf = 0.0f, Bf = 0.0f;
            if (sx >= 1 && sx < W - 1 && sy >= 1 && sy < H - 1) {
                auto cd = [&](int x, int y) { return dev::fsub((float)BAY(x, y), GRN(x, y)); };
                if (at_r || at_b) {
                    float s = dev::fadd(dev::fadd(dev::fadd(cd(sx - 1, sy - 1), cd(sx + 1, sy - 1)), cd(sx - 1, sy + 1)),
                                        cd(sx + 1, sy + 1));
                    float other = dev::fadd(g, dev::fmul(s, 0.25f));
                    if (at_r) { Rf = (float)BAY(sx, sy); Bf = other; } else { Bf = (float)BAY(sx, sy); Rf = other; }
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
        dev::rgb_tail(fp, R, Gv, B);
        uint8_t* o = sm.out + r * G::OUT_PITCH + c * 3 * bpc;
        if (fp.out_format == 0) {
            o[0] = __ldg(fp.tone8 + R); o[1] = __ldg(fp.tone8 + Gv); o[2] = __ldg(fp.tone8 + B);
        } else if (bpc == 1) {
            o[0] = (uint8_t)R; o[1] = (uint8_t)Gv; o[2] = (uint8_t)B;
        } else {
            o[0] = (uint8_t)R; o[1] = (uint8_t)(R >> 8); o[2] = (uint8_t)Gv;
            o[3] = (uint8_t)(Gv >> 8); o[4] = (uint8_t)B; o[5] = (uint8_t)(B >> 8);
        }
    }
    __syncthreads();

    // ---- 6. write the tile rows (3*bpc*tw contiguous bytes per row) ------------------------
    const int rowbytes = tw * 3 * bpc;
    for (int i = tid; i < rowbytes * th; i += kThreads) {
        int r = i / rowbytes, b = i - r * rowbytes;
        size_t goff = ((size_t)(y0 + r) * W + x0) * 3 * bpc + b;
        fp.out[goff] = sm.out[r * G::OUT_PITCH + b];
    }
    __syncthreads();
}

}  // namespace imop
