/*
 * isp_oracle.c - CPU oracle of the RAW->RGB hot path.  TEST INFRASTRUCTURE ONLY: used by
 * tests/, __graft_entry__.smoke() and bench.py's CPU baseline as the checker, never by the
 * product library.
 *
 * Each function restates one reference stage and cites the im-operator file:line it follows.
 * Floating-point expressions keep the reference's evaluation order; the file is compiled with
 * -ffp-contract=off so that a*b+c is never fused (the reference's own results depend on that
 * flag, see oracle/Makefile).  Loops that the reference runs under OpenMP (its DLOOP macro,
 * src/algorithms/common.hpp:37-42) carry the same pragma here; the Bayer stages, which the
 * reference runs single-threaded, stay single-threaded, so the timed CPU baseline has the
 * reference's parallel structure.
 */
#include "isp_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#define OR_DLOOP _Pragma("omp parallel for schedule(static)")
#else
#define OR_DLOOP
#endif

/* safe_max_val for 1..16 bits (include/imop/pixel_utils.hpp:15-19,
 * src/black_level/common.hpp:11-15: the module variants agree on 1..16). */
int or_max_val(int bd) {
    if (bd <= 0) return 255;
    if (bd >= 16) return 65535;
    return (1 << bd) - 1;
}

/* PatternOffsets::from_pattern (include/imop/types.hpp:88-101) */
static void pattern_offsets(int pattern, int* r_row, int* r_col, int* b_row, int* b_col) {
    switch (pattern) {
        case IMOP_BGGR: *r_row = 1; *r_col = 1; *b_row = 0; *b_col = 0; break;
        case IMOP_GRBG: *r_row = 0; *r_col = 1; *b_row = 1; *b_col = 0; break;
        case IMOP_GBRG: *r_row = 1; *r_col = 0; *b_row = 0; *b_col = 1; break;
        default: *r_row = 0; *r_col = 0; *b_row = 1; *b_col = 1; break;
    }
}

typedef struct { int r_row, r_col, b_row, b_col; } PO;
static PO po_of(int pattern) {
    PO po;
    pattern_offsets(pattern, &po.r_row, &po.r_col, &po.b_row, &po.b_col);
    return po;
}
static inline int is_r(PO po, int row, int col) { return ((row & 1) == po.r_row) && ((col & 1) == po.r_col); }
static inline int is_b(PO po, int row, int col) { return ((row & 1) == po.b_row) && ((col & 1) == po.b_col); }

/* bayer_color: 0=R, 1=Gr, 2=Gb, 3=B (src/black_level/common.hpp:29-35) */
int or_bayer_color(int row, int col, int pattern) {
    PO po = po_of(pattern);
    if ((row & 1) == po.r_row && (col & 1) == po.r_col) return 0;
    if ((row & 1) == po.b_row && (col & 1) == po.b_col) return 3;
    if ((row & 1) == po.r_row) return 1;
    return 2;
}

/* ------------------------------------------------------------------------------------ */
/* a1: pixel::get_packed_raw (include/imop/pixel_utils.hpp:58-118) with the byte size the
 * reference derives from the height (:64-65).  MIPI RAW12: pair k at byte 3k (:69-80);
 * MIPI RAW10: group k at byte 5k (:82-98); other depths: LSB-first bit stream (:100-117).
 * Pixels whose group would end at or past the buffer end read as 0 (:71, :85). */
int or_get_packed_raw(const uint8_t* data, int x, int y, int w, int h, int bd) {
    if (bd < 1 || bd > 16) return 0;
    if (x < 0 || y < 0 || x >= w || (h > 0 && y >= h)) return 0;
    size_t idx = (size_t)y * (size_t)w + (size_t)x;
    size_t size = ((size_t)w * (size_t)h * (size_t)bd + 7) / 8;
    int mv = or_max_val(bd);
    if (bd == 12) {
        size_t off = idx / 2 * 3;
        if (off + 2 >= size) return 0;
        uint8_t b0 = data[off], b1 = data[off + 1], b2 = data[off + 2];
        if ((idx & 1) == 0) return ((b0 << 4) | (b1 & 0xF)) & mv;
        return ((b2 << 4) | (b1 >> 4)) & mv;
    }
    if (bd == 10) {
        size_t off = idx / 4 * 5;
        int sub = (int)(idx & 3);
        if (off + 4 >= size) return 0;
        uint8_t b = data[off + (size_t)sub], b4 = data[off + 4];
        return ((b << 2) | ((b4 >> (2 * sub)) & 0x3)) & mv;
    }
    size_t bit = idx * (size_t)bd;
    size_t off = bit / 8;
    int shift = (int)(bit % 8);
    int nbytes = (bd + shift + 7) / 8;
    if (off >= size) return 0;
    if ((size_t)nbytes > size - off) nbytes = (int)(size - off);
    uint32_t v = 0;
    for (int i = 0; i < nbytes; i++) v |= (uint32_t)data[off + (size_t)i] << (8 * i);
    return (int)((v >> shift) & (uint32_t)mv);
}

/* a2: unpacked storage is read as stored (u8 for bd <= 8, little-endian u16 otherwise),
 * which is what the first Bayer stage reads (src/black_level/common.hpp:17-21). */
void or_unpack(const uint8_t* in, int w, int h, int bd, int packed, uint16_t* out) {
    size_t n = (size_t)w * (size_t)h;
    if (bd <= 8) {
        for (size_t i = 0; i < n; i++) out[i] = in[i];
    } else if (packed) {
        for (int y = 0; y < h; y++)
            for (int x = 0; x < w; x++)
                out[(size_t)y * w + x] = (uint16_t)or_get_packed_raw(in, x, y, w, h, bd);
    } else {
        for (size_t i = 0; i < n; i++) out[i] = (uint16_t)(in[2 * i] | (in[2 * i + 1] << 8));
    }
}

/* a3: black_level::process_per_channel (src/black_level/per_channel.cpp:6-33) and
 * process_global (src/black_level/global.cpp:6-24). */
void or_black_level(uint16_t* d, int w, int h, int pattern, int bd, int mode, const float off[4]) {
    int mv = or_max_val(bd);
    float o[4];
    for (int c = 0; c < 4; c++) {
        float v = (mode == IMOP_BL_GLOBAL) ? off[0] : off[c];
        o[c] = v > 0.0f ? v : 0.0f; /* std::max(0.0f, offset) */
    }
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            size_t i = (size_t)y * w + x;
            int c = or_bayer_color(y, x, pattern);
            int nv = (int)((float)d[i] - o[c]);
            if (nv < 0) nv = 0;
            if (nv > mv) nv = mv;
            d[i] = (uint16_t)nv;
        }
    }
}

/* sort a handful of ints (std::sort result) */
static void isort(int* a, int n) {
    for (int i = 1; i < n; i++) {
        int v = a[i], j = i - 1;
        while (j >= 0 && a[j] > v) { a[j + 1] = a[j]; j--; }
        a[j + 1] = v;
    }
}

/* Same-colour neighbours at step 2 inside [2,w-2)x[2,h-2), median = sorted[n/2]
 * (src/defect_correct/adaptive.cpp:31-49).  Returns -1 when there is none. */
static int dpc_median(const uint16_t* d, int w, int h, int x, int y, int pattern) {
    int nb[8], n = 0;
    int color = or_bayer_color(y, x, pattern);
    for (int dy = -2; dy <= 2; dy += 2) {
        for (int dx = -2; dx <= 2; dx += 2) {
            if (dx == 0 && dy == 0) continue;
            int nx = x + dx, ny = y + dy;
            if (nx >= 2 && nx < w - 2 && ny >= 2 && ny < h - 2) {
                if (or_bayer_color(ny, nx, pattern) == color) nb[n++] = d[(size_t)ny * w + nx];
            }
        }
    }
    if (n == 0) return -1;
    isort(nb, n);
    return nb[n / 2];
}

/* a4: defect_correct::process_adaptive (src/defect_correct/adaptive.cpp:8-61): raster order,
 * in place, so later pixels see the corrected values of earlier ones. */
void or_dpc_adaptive(uint16_t* d, int w, int h, int pattern, int bd, float threshold) {
    if (w < 5 || h < 5) return;
    int mv = or_max_val(bd);
    float t = threshold < 1.0f ? threshold : 1.0f;
    t = t > 0.05f ? t : 0.05f;
    int thr = (int)(t * (float)mv);
    for (int y = 2; y < h - 2; y++) {
        for (int x = 2; x < w - 2; x++) {
            int center = d[(size_t)y * w + x];
            int med = dpc_median(d, w, h, x, y, pattern);
            if (med < 0) continue;
            int diff = center - med;
            if (diff < 0) diff = -diff;
            if (diff > thr) d[(size_t)y * w + x] = (uint16_t)med;
        }
    }
}

/* a4': defect_correct::process_map_based (src/defect_correct/map_based.cpp:8-46): map order,
 * unconditional replacement, in place. */
void or_dpc_map(uint16_t* d, int w, int h, int pattern, int bd, const ImopDefectPoint* map, int n) {
    (void)bd;
    if (!map || n <= 0) return;
    for (int i = 0; i < n; i++) {
        int x = map[i].x, y = map[i].y;
        if (x < 2 || x >= w - 2 || y < 2 || y >= h - 2) continue;
        int med = dpc_median(d, w, h, x, y, pattern);
        if (med >= 0) d[(size_t)y * w + x] = (uint16_t)med;
    }
}

/* a5: the apply loop of lens_shading::process_flat_field (src/lens_shading/flat_field.cpp:78-107)
 * with an explicit gw x gh x 4 grid in place of the fixed 32x24 one. */
void or_lsc_grid(uint16_t* d, int w, int h, int pattern, int bd, const float* g, int gw, int gh) {
    int mv = or_max_val(bd);
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            int c = or_bayer_color(y, x, pattern);
            float gx_f = (float)x * (float)(gw - 1) / (float)(w - 1);
            float gy_f = (float)y * (float)(gh - 1) / (float)(h - 1);
            int gx_i = (int)gx_f;
            int gy_i = (int)gy_f;
            if (gx_i < 0) gx_i = 0;
            if (gx_i > gw - 2) gx_i = gw - 2;
            if (gy_i < 0) gy_i = 0;
            if (gy_i > gh - 2) gy_i = gh - 2;
            float fx = gx_f - (float)gx_i;
            float fy = gy_f - (float)gy_i;
            float g00 = g[(gy_i * gw + gx_i) * 4 + c];
            float g10 = g[(gy_i * gw + gx_i + 1) * 4 + c];
            float g01 = g[((gy_i + 1) * gw + gx_i) * 4 + c];
            float g11 = g[((gy_i + 1) * gw + gx_i + 1) * 4 + c];
            float gain = g00 * (1.0f - fx) * (1.0f - fy) + g10 * fx * (1.0f - fy) +
                         g01 * (1.0f - fx) * fy + g11 * fx * fy;
            size_t i = (size_t)y * w + x;
            int nv = (int)((float)d[i] * gain + 0.5f);
            if (nv < 0) nv = 0;
            if (nv > mv) nv = mv;
            d[i] = (uint16_t)nv;
        }
    }
}

/* a5': lens_shading::process_polynomial (src/lens_shading/polynomial.cpp:13-52) */
void or_lsc_poly(uint16_t* d, int w, int h, int pattern, int bd, const float coef[4][3], float cxn,
                 float cyn) {
    int mv = or_max_val(bd);
    float cx = cxn * (float)w;
    float cy = cyn * (float)h;
    float max_r = sqrtf(cx * cx + cy * cy);
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            float dx = (float)x - cx;
            float dy = (float)y - cy;
            float r = sqrtf(dx * dx + dy * dy) / max_r;
            int c = or_bayer_color(y, x, pattern);
            float r2 = r * r;
            float r4 = r2 * r2;
            float r6 = r4 * r2;
            float gain = 1.0f + coef[c][0] * r2 + coef[c][1] * r4 + coef[c][2] * r6;
            size_t i = (size_t)y * w + x;
            int nv = (int)((float)d[i] * gain + 0.5f);
            if (nv < 0) nv = 0;
            if (nv > mv) nv = mv;
            d[i] = (uint16_t)nv;
        }
    }
}

static int read_store(const void* p, size_t i, int bd) {
    if (bd <= 8) return ((const uint8_t*)p)[i];
    const uint8_t* b = (const uint8_t*)p + 2 * i;
    return b[0] | (b[1] << 8);
}

/* Grid construction of lens_shading::process_flat_field (src/lens_shading/flat_field.cpp:30-76):
 * per-channel centre targets, then a 32x24 grid of target/mean. */
int or_lsc_flat_field_grid(const void* ff, int ffw, int ffh, int pattern, int bd, float* gm) {
    if (!ff) return IMOP_ERR_NULL_INPUT;
    if (ffw <= 0 || ffh <= 0) return IMOP_ERR_INVALID_DIMENSIONS;
    int mv = or_max_val(bd);
    float targets[4] = {0, 0, 0, 0};
    int counts[4] = {0, 0, 0, 0};
    int cx0 = ffw * 3 / 10, cx1 = ffw * 7 / 10;
    int cy0 = ffh * 3 / 10, cy1 = ffh * 7 / 10;
    for (int y = cy0; y < cy1; y += 2)
        for (int x = cx0; x < cx1; x += 2) {
            int c = or_bayer_color(y, x, pattern);
            targets[c] += (float)read_store(ff, (size_t)y * ffw + x, bd);
            counts[c]++;
        }
    for (int c = 0; c < 4; c++)
        targets[c] = (counts[c] > 0) ? targets[c] / (float)counts[c] : (float)mv;
    const int gw = 32, gh = 24;
    for (int i = 0; i < gw * gh * 4; i++) gm[i] = 1.0f;
    for (int gy = 0; gy < gh; gy++) {
        for (int gx = 0; gx < gw; gx++) {
            int fx0 = gx * ffw / gw, fx1 = (gx + 1) * ffw / gw;
            int fy0 = gy * ffh / gh, fy1 = (gy + 1) * ffh / gh;
            float sum[4] = {0, 0, 0, 0};
            int cnt[4] = {0, 0, 0, 0};
            for (int y = fy0; y < fy1; y += 2)
                for (int x = fx0; x < fx1; x += 2) {
                    int c = or_bayer_color(y, x, pattern);
                    sum[c] += (float)read_store(ff, (size_t)y * ffw + x, bd);
                    cnt[c]++;
                }
            for (int c = 0; c < 4; c++) {
                float mean = (cnt[c] > 0) ? sum[c] / (float)cnt[c] : targets[c];
                float den = mean > 1e-6f ? mean : 1e-6f; /* std::max(1e-6f, mean) */
                gm[(gy * gw + gx) * 4 + c] = targets[c] / den;
            }
        }
    }
    return 0;
}

/* a6': Bayer-domain white balance: the per-sample rule of white_balance::process_manual_wb
 * (src/white_balance/manual.cpp:29-31) applied at each CFA site with the gain of its colour. */
void or_wb_bayer(uint16_t* d, int w, int h, int pattern, int bd, const float gain[3]) {
    int mv = or_max_val(bd);
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            int c = or_bayer_color(y, x, pattern);
            float g = (c == 0) ? gain[0] : (c == 3) ? gain[2] : gain[1];
            size_t i = (size_t)y * w + x;
            int nv = (int)((float)d[i] * g + 0.5f);
            if (nv < 0) nv = 0;
            if (nv > mv) nv = mv;
            d[i] = (uint16_t)nv;
        }
    }
}

/* detail::fill_rgb_borders (src/algorithms/common.hpp:47-96) on a u16 x 3 plane. */
static void fill_rgb_borders(uint16_t* rgb, int w, int h, int border) {
    if (border <= 0 || w <= border * 2 || h <= border * 2) return;
    size_t stride = (size_t)w * 3;
    int ref_top = border, ref_bottom = h - 1 - border;
    for (int y = 0; y < border; y++)
        memcpy(rgb + (size_t)y * stride, rgb + (size_t)ref_top * stride, stride * sizeof(uint16_t));
    for (int y = h - border; y < h; y++)
        memcpy(rgb + (size_t)y * stride, rgb + (size_t)ref_bottom * stride, stride * sizeof(uint16_t));
    for (int y = border; y < h - border; y++) {
        uint16_t* row = rgb + (size_t)y * stride;
        uint16_t* l = row + (size_t)border * 3;
        uint16_t* r = row + (size_t)(w - 1 - border) * 3;
        for (int x = 0; x < border; x++) { row[x * 3] = l[0]; row[x * 3 + 1] = l[1]; row[x * 3 + 2] = l[2]; }
        for (int x = w - border; x < w; x++) { row[x * 3] = r[0]; row[x * 3 + 1] = r[1]; row[x * 3 + 2] = r[2]; }
    }
}

/* detail::fill_intermediate_borders (src/algorithms/common.hpp:98-135) on float planes. */
static void fill_intermediate_borders(float* R, float* G, float* B, int w, int h, int border) {
    if (border <= 0 || w <= border * 2 || h <= border * 2) return;
    for (int y = 0; y < border; y++) {
        size_t di = (size_t)y * w, ri = (size_t)border * w;
        for (int x = 0; x < w; x++) { R[di + x] = R[ri + x]; G[di + x] = G[ri + x]; B[di + x] = B[ri + x]; }
    }
    for (int y = h - border; y < h; y++) {
        size_t di = (size_t)y * w, ri = (size_t)(h - 1 - border) * w;
        for (int x = 0; x < w; x++) { R[di + x] = R[ri + x]; G[di + x] = G[ri + x]; B[di + x] = B[ri + x]; }
    }
    OR_DLOOP
    for (int y = border; y < h - border; y++) {
        size_t ry = (size_t)y * w, rl = ry + border, rr = ry + (w - 1 - border);
        for (int x = 0; x < border; x++) { R[ry + x] = R[rl]; G[ry + x] = G[rl]; B[ry + x] = B[rl]; }
        for (int x = w - border; x < w; x++) { R[ry + x] = R[rr]; G[ry + x] = G[rr]; B[ry + x] = B[rr]; }
    }
}

/* a7: imop::process_hqli -> detail::hqli_core (src/algorithms/interp_core.hpp:28-68), the
 * AVX2 8-bit path (src/algorithms/avx2.cpp:257-352) has the same integer arithmetic, then
 * fill_rgb_borders(2) (src/algorithms/hqli.cpp:41).  The output plane starts zeroed: the four
 * 2x2 corner blocks are copied by fill_rgb_borders from row-2 / row-(h-3) pixels the interior
 * loop never writes, so they keep the caller's buffer contents; a zeroed buffer is what the
 * reference's GPU path uses (cudaMemset in src/algorithms/cuda_dispatch.cpp:100). */
void or_demosaic_hqli(const uint16_t* bay, uint16_t* rgb, int w, int h, int pattern, int bd) {
    PO po = po_of(pattern);
    int mv = or_max_val(bd);
    memset(rgb, 0, (size_t)w * h * 3 * sizeof(uint16_t));
#define PIX(X, Y) ((int)bay[(size_t)(Y) * w + (X)])
    OR_DLOOP
    for (int y = 2; y < h - 2; y++) {
        int is_gr_row = ((y & 1) == po.r_row);
        for (int x = 2; x < w - 2; x++) {
            int r, g, b;
            if (is_r(po, y, x)) {
                r = PIX(x, y);
                g = (PIX(x - 1, y) + PIX(x + 1, y) + PIX(x, y - 1) + PIX(x, y + 1) + 2) / 4;
                b = (PIX(x - 1, y - 1) + PIX(x + 1, y - 1) + PIX(x - 1, y + 1) + PIX(x + 1, y + 1) + 2) / 4;
            } else if (is_b(po, y, x)) {
                r = (PIX(x - 1, y - 1) + PIX(x + 1, y - 1) + PIX(x - 1, y + 1) + PIX(x + 1, y + 1) + 2) / 4;
                g = (PIX(x - 1, y) + PIX(x + 1, y) + PIX(x, y - 1) + PIX(x, y + 1) + 2) / 4;
                b = PIX(x, y);
            } else {
                g = PIX(x, y);
                if (is_gr_row) {
                    r = (PIX(x - 1, y) + PIX(x + 1, y) + 1) / 2;
                    b = (PIX(x, y - 1) + PIX(x, y + 1) + 1) / 2;
                } else {
                    b = (PIX(x - 1, y) + PIX(x + 1, y) + 1) / 2;
                    r = (PIX(x, y - 1) + PIX(x, y + 1) + 1) / 2;
                }
            }
            if (r > mv) r = mv;
            if (g > mv) g = mv;
            if (b > mv) b = mv;
            uint16_t* o = rgb + ((size_t)y * w + x) * 3;
            o[0] = (uint16_t)r; o[1] = (uint16_t)g; o[2] = (uint16_t)b;
        }
    }
#undef PIX
    fill_rgb_borders(rgb, w, h, 2);
}

/* Colour-difference R/B (src/algorithms/common.hpp:142-199, inlined in
 * src/algorithms/amaze.cpp:62-114) followed by fill_intermediate_borders(2) and the float ->
 * int writer (src/algorithms/common.hpp:201-214). Shared by AMAZE and the float MG path. */
static void colour_difference_and_write(const uint16_t* bay, float* R, float* G, float* B,
                                        uint16_t* rgb, int w, int h, PO po, int bd) {
#define RAW(X, Y) ((float)bay[(size_t)(Y) * w + (X)])
#define GV(X, Y) (G[(size_t)(Y) * w + (X)])
    OR_DLOOP
    for (int y = 1; y < h - 1; y++) {
        for (int x = 1; x < w - 1; x++) {
            size_t idx = (size_t)y * w + x;
            float g = G[idx];
            if (is_r(po, y, x)) {
                R[idx] = RAW(x, y);
                float cd = 0.0f; int cnt = 0;
                static const int dg[4][2] = {{-1, -1}, {1, -1}, {-1, 1}, {1, 1}};
                for (int k = 0; k < 4; k++) {
                    int nx = x + dg[k][0], ny = y + dg[k][1];
                    if (nx >= 0 && nx < w && ny >= 0 && ny < h && is_b(po, ny, nx)) {
                        cd += RAW(nx, ny) - GV(nx, ny);
                        cnt++;
                    }
                }
                B[idx] = g + (cnt > 0 ? cd / (float)cnt : 0.0f);
            } else if (is_b(po, y, x)) {
                B[idx] = RAW(x, y);
                float cd = 0.0f; int cnt = 0;
                static const int dg[4][2] = {{-1, -1}, {1, -1}, {-1, 1}, {1, 1}};
                for (int k = 0; k < 4; k++) {
                    int nx = x + dg[k][0], ny = y + dg[k][1];
                    if (nx >= 0 && nx < w && ny >= 0 && ny < h && is_r(po, ny, nx)) {
                        cd += RAW(nx, ny) - GV(nx, ny);
                        cnt++;
                    }
                }
                R[idx] = g + (cnt > 0 ? cd / (float)cnt : 0.0f);
            } else {
                float rc = 0.0f, bc = 0.0f; int rn = 0, bn = 0;
                if (is_r(po, y - 1, x)) { rc += RAW(x, y - 1) - GV(x, y - 1); rn++; }
                if (is_r(po, y + 1, x)) { rc += RAW(x, y + 1) - GV(x, y + 1); rn++; }
                if (is_r(po, y, x - 1)) { rc += RAW(x - 1, y) - GV(x - 1, y); rn++; }
                if (is_r(po, y, x + 1)) { rc += RAW(x + 1, y) - GV(x + 1, y); rn++; }
                if (is_b(po, y - 1, x)) { bc += RAW(x, y - 1) - GV(x, y - 1); bn++; }
                if (is_b(po, y + 1, x)) { bc += RAW(x, y + 1) - GV(x, y + 1); bn++; }
                if (is_b(po, y, x - 1)) { bc += RAW(x - 1, y) - GV(x - 1, y); bn++; }
                if (is_b(po, y, x + 1)) { bc += RAW(x + 1, y) - GV(x + 1, y); bn++; }
                R[idx] = g + (rn > 0 ? rc / (float)rn : 0.0f);
                B[idx] = g + (bn > 0 ? bc / (float)bn : 0.0f);
            }
        }
    }
#undef RAW
#undef GV
    fill_intermediate_borders(R, G, B, w, h, 2);
    int mv = or_max_val(bd);
    OR_DLOOP
    for (int y = 0; y < h; y++) {
        for (int x = 0; x < w; x++) {
            size_t idx = (size_t)y * w + x;
            int ro = (int)(R[idx] + 0.5f), go = (int)(G[idx] + 0.5f), bo = (int)(B[idx] + 0.5f);
            ro = ro < 0 ? 0 : (ro > mv ? mv : ro);
            go = go < 0 ? 0 : (go > mv ? mv : go);
            bo = bo < 0 ? 0 : (bo > mv ? mv : bo);
            uint16_t* o = rgb + idx * 3;
            o[0] = (uint16_t)ro; o[1] = (uint16_t)go; o[2] = (uint16_t)bo;
        }
    }
    /* the 8-bit path re-fills the RGB borders (src/algorithms/amaze.cpp:142) */
    if (bd <= 8) fill_rgb_borders(rgb, w, h, 2);
}

/* a8: imop::process_amaze (src/algorithms/amaze.cpp:130-201; 8-bit core :7-128).
 * G starts at -1 everywhere (:155), the gradient-weighted green fills [2,h-2)x[2,w-2)
 * (:159-183), and the colour-difference pass reads the -1 sentinel near the border. */
void or_demosaic_amaze(const uint16_t* bay, uint16_t* rgb, int w, int h, int pattern, int bd) {
    PO po = po_of(pattern);
    size_t n = (size_t)w * h;
    float* G = (float*)malloc(n * sizeof(float));
    float* R = (float*)malloc(n * sizeof(float));
    float* B = (float*)malloc(n * sizeof(float));
    for (size_t i = 0; i < n; i++) { G[i] = -1.0f; R[i] = 0.0f; B[i] = 0.0f; }
#define RAW(X, Y) ((float)bay[(size_t)(Y) * w + (X)])
    OR_DLOOP
    for (int y = 2; y < h - 2; y++) {
        for (int x = 2; x < w - 2; x++) {
            size_t idx = (size_t)y * w + x;
            if (!is_r(po, y, x) && !is_b(po, y, x)) {
                G[idx] = RAW(x, y);
            } else {
                float c = RAW(x, y);
                float hm1 = RAW(x - 1, y), hp1 = RAW(x + 1, y), hm2 = RAW(x - 2, y), hp2 = RAW(x + 2, y);
                float vm1 = RAW(x, y - 1), vp1 = RAW(x, y + 1), vm2 = RAW(x, y - 2), vp2 = RAW(x, y + 2);
                float gradH = fabsf(hm1 - hp1) + fabsf(2.0f * c - hm2 - hp2);
                float gradV = fabsf(vm1 - vp1) + fabsf(2.0f * c - vm2 - vp2);
                float wh = 1.0f / (1.0f + gradH);
                float wv = 1.0f / (1.0f + gradV);
                float sum_w = wh + wv;
                wh /= sum_w;
                wv /= sum_w;
                float gh = (hm1 + hp1) * 0.5f;
                float gv = (vm1 + vp1) * 0.5f;
                float lapH = 2.0f * c - hm2 - hp2;
                float lapV = 2.0f * c - vm2 - vp2;
                gh += lapH * 0.25f;
                gv += lapV * 0.25f;
                G[idx] = wh * gh + wv * gv;
            }
        }
    }
#undef RAW
    colour_difference_and_write(bay, R, G, B, rgb, w, h, po, bd);
    free(G); free(R); free(B);
}

/* a8': imop::process_mg.  For bd <= 8 and unpacked data the reference runs the integer path
 * (src/algorithms/mg.cpp:23-161; the AVX2 variant src/algorithms/avx2.cpp:422-687 is used when
 * available); otherwise the float path (src/algorithms/mg.cpp:163-216). */
void or_demosaic_mg(const uint16_t* bay, uint16_t* rgb, int w, int h, int pattern, int bd) {
    PO po = po_of(pattern);
    size_t n = (size_t)w * h;
    int mv = or_max_val(bd);
    if (bd <= 8) {
        int* G = (int*)malloc(n * sizeof(int));
        int* R = (int*)calloc(n, sizeof(int));
        int* B = (int*)calloc(n, sizeof(int));
        for (size_t i = 0; i < n; i++) G[i] = -1;
        for (int y = 0; y < h; y++)
            for (int x = 0; x < w; x++)
                if (!is_r(po, y, x) && !is_b(po, y, x)) G[(size_t)y * w + x] = bay[(size_t)y * w + x];
#define P(X, Y) ((int)bay[(size_t)(Y) * w + (X)])
        OR_DLOOP
        for (int y = 2; y < h - 2; y++)
            for (int x = 2; x < w - 2; x++)
                if (is_r(po, y, x) || is_b(po, y, x)) {
                    int c = P(x, y);
                    int gv = (4 * c + 2 * (P(x, y - 1) + P(x, y + 1) + P(x + 1, y) + P(x - 1, y)) -
                              (P(x, y - 2) + P(x, y + 2) + P(x + 2, y) + P(x - 2, y)) + 4) >> 3;
                    if (gv < 0) gv = 0; else if (gv > mv) gv = mv;
                    G[(size_t)y * w + x] = gv;
                }
        OR_DLOOP
        for (int y = 1; y < h - 1; y++) {
            for (int x = 1; x < w - 1; x++) {
                size_t idx = (size_t)y * w + x;
                int g = G[idx];
                if (is_r(po, y, x) || is_b(po, y, x)) {
                    int at_r = is_r(po, y, x);
                    int s = 0, cnt = 0;
                    static const int dg[4][2] = {{-1, -1}, {1, -1}, {-1, 1}, {1, 1}};
                    for (int k = 0; k < 4; k++) {
                        int nx = x + dg[k][0], ny = y + dg[k][1];
                        if (at_r ? is_b(po, ny, nx) : is_r(po, ny, nx)) {
                            s += P(nx, ny) - G[(size_t)ny * w + nx];
                            cnt++;
                        }
                    }
                    int other = g + (cnt > 0 ? ((s + cnt / 2) / cnt) : 0);
                    if (at_r) { R[idx] = P(x, y); B[idx] = other; }
                    else { B[idx] = P(x, y); R[idx] = other; }
                } else {
                    int rc = 0, bc = 0, rn = 0, bn = 0;
                    static const int d4[4][2] = {{0, -1}, {0, 1}, {-1, 0}, {1, 0}};
                    for (int k = 0; k < 4; k++) {
                        int nx = x + d4[k][0], ny = y + d4[k][1];
                        if (is_r(po, ny, nx)) { rc += P(nx, ny) - G[(size_t)ny * w + nx]; rn++; }
                    }
                    for (int k = 0; k < 4; k++) {
                        int nx = x + d4[k][0], ny = y + d4[k][1];
                        if (is_b(po, ny, nx)) { bc += P(nx, ny) - G[(size_t)ny * w + nx]; bn++; }
                    }
                    R[idx] = g + (rn > 0 ? (rc + rn / 2) / rn : 0);
                    B[idx] = g + (bn > 0 ? (bc + bn / 2) / bn : 0);
                }
            }
        }
#undef P
        /* fill_intermediate_borders_int (src/algorithms/common.hpp:116-119) */
        {
            int border = 2;
            for (int y = 0; y < border; y++)
                for (int x = 0; x < w; x++) {
                    size_t di = (size_t)y * w + x, ri = (size_t)border * w + x;
                    R[di] = R[ri]; G[di] = G[ri]; B[di] = B[ri];
                }
            for (int y = h - border; y < h; y++)
                for (int x = 0; x < w; x++) {
                    size_t di = (size_t)y * w + x, ri = (size_t)(h - 1 - border) * w + x;
                    R[di] = R[ri]; G[di] = G[ri]; B[di] = B[ri];
                }
            for (int y = border; y < h - border; y++) {
                size_t ry = (size_t)y * w, rl = ry + border, rr = ry + (w - 1 - border);
                for (int x = 0; x < border; x++) { R[ry + x] = R[rl]; G[ry + x] = G[rl]; B[ry + x] = B[rl]; }
                for (int x = w - border; x < w; x++) { R[ry + x] = R[rr]; G[ry + x] = G[rr]; B[ry + x] = B[rr]; }
            }
        }
        for (size_t i = 0; i < n; i++) {
            int ro = R[i], go = G[i], bo = B[i];
            ro = ro < 0 ? 0 : (ro > mv ? mv : ro);
            go = go < 0 ? 0 : (go > mv ? mv : go);
            bo = bo < 0 ? 0 : (bo > mv ? mv : bo);
            rgb[i * 3] = (uint16_t)ro; rgb[i * 3 + 1] = (uint16_t)go; rgb[i * 3 + 2] = (uint16_t)bo;
        }
        free(G); free(R); free(B);
        return;
    }
    float* G = (float*)malloc(n * sizeof(float));
    float* R = (float*)malloc(n * sizeof(float));
    float* B = (float*)malloc(n * sizeof(float));
    for (size_t i = 0; i < n; i++) { G[i] = -1.0f; R[i] = 0.0f; B[i] = 0.0f; }
#define RAW(X, Y) ((float)bay[(size_t)(Y) * w + (X)])
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++)
            if (!is_r(po, y, x) && !is_b(po, y, x)) G[(size_t)y * w + x] = RAW(x, y);
    OR_DLOOP
    for (int y = 2; y < h - 2; y++)
        for (int x = 2; x < w - 2; x++)
            if (is_r(po, y, x) || is_b(po, y, x)) {
                float nn = RAW(x, y - 1), s = RAW(x, y + 1), e = RAW(x + 1, y), ww = RAW(x - 1, y);
                float n2 = RAW(x, y - 2), s2 = RAW(x, y + 2), e2 = RAW(x + 2, y), w2 = RAW(x - 2, y);
                float c = RAW(x, y);
                G[(size_t)y * w + x] = (4.0f * c + 2.0f * (nn + s + e + ww) - (n2 + s2 + e2 + w2)) / 8.0f;
            }
#undef RAW
    /* the float path never re-fills RGB borders, for any bit depth */
    colour_difference_and_write(bay, R, G, B, rgb, w, h, po, 16);
    /* colour_difference_and_write clamps to 65535 with bd=16; redo the clamp at bd */
    for (size_t i = 0; i < n * 3; i++)
        if (rgb[i] > mv) rgb[i] = (uint16_t)mv;
    free(G); free(R); free(B);
}

/* a6: white_balance::process_manual_wb (src/white_balance/manual.cpp:6-40) */
void or_wb_rgb(uint16_t* rgb, int w, int h, int bd, const float gain[3]) {
    int mv = or_max_val(bd);
    size_t n = (size_t)w * h;
    for (size_t i = 0; i < n; i++) {
        for (int c = 0; c < 3; c++) {
            int v = (int)((float)rgb[i * 3 + c] * gain[c] + 0.5f);
            rgb[i * 3 + c] = (uint16_t)(v < 0 ? 0 : (v > mv ? mv : v));
        }
    }
}

/* a11: lut::apply_lut (src/lut/core.cpp:11-39) with lut::detail::trilinear_lookup
 * (src/lut/common.hpp:44-106): v / max into the cube, interpolation along B, then G, then R,
 * (int)(v * max + 0.5f) clamped to [0, max]. */
void or_lut3d(uint16_t* rgb, int w, int h, int bd, const float* lut, int size) {
    const int mv = or_max_val(bd);
    const float mvf = (float)mv, s1 = (float)(size - 1);
    const size_t n = (size_t)w * (size_t)h;
    for (size_t i = 0; i < n; i++) {
        float sc[3];
        int lo[3], hi[3];
        float d[3];
        for (int c = 0; c < 3; c++) {
            sc[c] = ((float)rgb[3 * i + c] / mvf) * s1;
            int k = (int)sc[c];
            if (k > size - 2) k = size - 2;
            if (k < 0) k = 0;
            lo[c] = k;
            hi[c] = k + 1 < size - 1 ? k + 1 : size - 1;
            d[c] = sc[c] - (float)k;
        }
        float corner[2][2][3]; /* [r][g][channel], interpolated along B */
        for (int a = 0; a < 2; a++)
            for (int b = 0; b < 2; b++) {
                const int ri = a ? hi[0] : lo[0], gi = b ? hi[1] : lo[1];
                const float* p0 = lut + (((size_t)ri * size + (size_t)gi) * size + (size_t)lo[2]) * 3;
                const float* p1 = lut + (((size_t)ri * size + (size_t)gi) * size + (size_t)hi[2]) * 3;
                for (int c = 0; c < 3; c++) corner[a][b][c] = p0[c] + d[2] * (p1[c] - p0[c]);
            }
        for (int c = 0; c < 3; c++) {
            const float v0 = corner[0][0][c] + d[1] * (corner[0][1][c] - corner[0][0][c]);
            const float v1 = corner[1][0][c] + d[1] * (corner[1][1][c] - corner[1][0][c]);
            const float o = v0 + d[0] * (v1 - v0);
            int q = (int)(o * mvf + 0.5f);
            rgb[3 * i + c] = (uint16_t)(q < 0 ? 0 : (q > mv ? mv : q));
        }
    }
}

/* a9: ccm::process_linear_3x3 (src/ccm/linear_3x3.cpp:9-46) */
void or_ccm(uint16_t* rgb, int w, int h, int bd, const float m[9]) {
    int mv = or_max_val(bd);
    size_t n = (size_t)w * h;
    for (size_t i = 0; i < n; i++) {
        float r = (float)rgb[i * 3], g = (float)rgb[i * 3 + 1], b = (float)rgb[i * 3 + 2];
        float ro = m[0] * r + m[1] * g + m[2] * b;
        float go = m[3] * r + m[4] * g + m[5] * b;
        float bo = m[6] * r + m[7] * g + m[8] * b;
        int a = (int)(ro + 0.5f), c = (int)(go + 0.5f), d = (int)(bo + 0.5f);
        rgb[i * 3] = (uint16_t)(a < 0 ? 0 : (a > mv ? mv : a));
        rgb[i * 3 + 1] = (uint16_t)(c < 0 ? 0 : (c > mv ? mv : c));
        rgb[i * 3 + 2] = (uint16_t)(d < 0 ? 0 : (d > mv ? mv : d));
    }
}

/* a10: the tone stage ending in 8 bits.  LINEAR: v/max (tone/gamma.cpp:26 normalisation);
 * LUT: a caller table; KNOTS: the lerp rule of tone::process_curves_3point
 * (src/tone/curves_3point.cpp:128-134) over 33 knots (32 segments). */
float or_tone_value(int mode, const float* lut, const float* knots, int v, int bd) {
    float mv = (float)or_max_val(bd);
    if (mode == IMOP_TONE_LUT) return lut[v];
    if (mode == IMOP_TONE_KNOTS) {
        float norm = (float)v / mv;
        float fi = norm * 32.0f;
        int idx = (int)fi;
        float frac = fi - (float)idx;
        if (idx > 31) { idx = 31; frac = 1.0f; }
        return knots[idx] * (1.0f - frac) + knots[idx + 1] * frac;
    }
    return (float)v / mv;
}

/* (int)(t*255+0.5) clamped: the quantiser of src/tone/curves_3point.cpp:137-138 with max 255 */
uint8_t or_tone_to_u8(float t) {
    int q = (int)(t * 255.0f + 0.5f);
    return (uint8_t)(q < 0 ? 0 : (q > 255 ? 255 : q));
}

void or_tone_rgb8(const uint16_t* rgb, uint8_t* out, int w, int h, int bd, int mode,
                  const float* lut, const float* knots) {
    size_t n = (size_t)w * h * 3;
    for (size_t i = 0; i < n; i++) out[i] = or_tone_to_u8(or_tone_value(mode, lut, knots, rgb[i], bd));
}

/* ------------------------------------------------------------------------------------ */
static int validate(const ImopIspParams* p) {
    if (!p) return IMOP_ERR_NULL_INPUT;
    if (p->width <= 0 || p->height <= 0) return IMOP_ERR_INVALID_DIMENSIONS;
    if (p->bit_depth < 1 || p->bit_depth > 16) return IMOP_ERR_INVALID_BIT_DEPTH;
    if (p->pattern < 0 || p->pattern > 3) return IMOP_ERR_INVALID_PATTERN;
    if (p->width < 6 || p->height < 6) return IMOP_ERR_IMAGE_TOO_SMALL;
    if (p->demosaic != IMOP_DEMOSAIC_HQLI && p->demosaic != IMOP_DEMOSAIC_AMAZE &&
        p->demosaic != IMOP_DEMOSAIC_MG)
        return IMOP_ERR_UNSUPPORTED;
    return 0;
}

static void rgb_copy_fill(uint16_t* dst, const uint16_t* src, size_t n) {
    if (dst) memcpy(dst, src, n * sizeof(uint16_t));
}

int or_pipeline(const ImopIspParams* p, const void* in, void* out, OracleDumps* dumps) {
    int st = validate(p);
    if (st) return st;
    int w = p->width, h = p->height, bd = p->bit_depth;
    size_t n = (size_t)w * h;
    uint16_t* bay = (uint16_t*)malloc(n * sizeof(uint16_t));
    uint16_t* rgb = (uint16_t*)malloc(n * 3 * sizeof(uint16_t));
    OracleDumps none;
    memset(&none, 0, sizeof(none));
    if (!dumps) dumps = &none;

    or_unpack((const uint8_t*)in, w, h, bd, p->packed, bay);
    rgb_copy_fill(dumps->unpacked, bay, n);
    if (p->stages & IMOP_STAGE_BLACK_LEVEL) or_black_level(bay, w, h, p->pattern, bd, p->bl_mode, p->bl_offset);
    rgb_copy_fill(dumps->black_level, bay, n);
    if (p->stages & IMOP_STAGE_DEFECT) {
        if (p->dpc_mode == IMOP_DPC_MAP_BASED) or_dpc_map(bay, w, h, p->pattern, bd, p->dpc_map, p->dpc_map_count);
        else or_dpc_adaptive(bay, w, h, p->pattern, bd, p->dpc_threshold);
    }
    rgb_copy_fill(dumps->defect, bay, n);
    if (p->stages & IMOP_STAGE_LENS_SHADING) {
        if (p->lsc_mode == IMOP_LSC_POLYNOMIAL) {
            or_lsc_poly(bay, w, h, p->pattern, bd, p->lsc_poly, p->lsc_center[0], p->lsc_center[1]);
        } else if (p->lsc_mode == IMOP_LSC_FLAT_FIELD) {
            float grid[32 * 24 * 4];
            int e = or_lsc_flat_field_grid(p->lsc_flat_field, p->lsc_flat_w, p->lsc_flat_h, p->pattern, bd, grid);
            if (e) { free(bay); free(rgb); return e; }
            or_lsc_grid(bay, w, h, p->pattern, bd, grid, 32, 24);
        } else {
            or_lsc_grid(bay, w, h, p->pattern, bd, p->lsc_grid, p->lsc_grid_w, p->lsc_grid_h);
        }
    }
    rgb_copy_fill(dumps->lens_shading, bay, n);
    int wb = (p->stages & IMOP_STAGE_WHITE_BALANCE) != 0;
    if (wb && p->stage_order == IMOP_ORDER_BAYER_WB) {
        or_wb_bayer(bay, w, h, p->pattern, bd, p->wb_gain);
        rgb_copy_fill(dumps->white_balance, bay, n);
    }
    /* the demosaic reads u16 samples through align_raw_value (include/imop/pixel_utils.hpp:129-137):
     * a sample above max is taken as MSB-aligned; a no-op once any Bayer stage has clamped */
    if (bd > 8 && bd < 16) {
        int mv = or_max_val(bd);
        for (size_t i = 0; i < n; i++)
            if (bay[i] > mv) bay[i] = (uint16_t)(bay[i] >> (16 - bd));
    }
    if (p->demosaic == IMOP_DEMOSAIC_AMAZE) or_demosaic_amaze(bay, rgb, w, h, p->pattern, bd);
    else if (p->demosaic == IMOP_DEMOSAIC_MG) or_demosaic_mg(bay, rgb, w, h, p->pattern, bd);
    else or_demosaic_hqli(bay, rgb, w, h, p->pattern, bd);
    rgb_copy_fill(dumps->demosaic, rgb, n * 3);
    if (wb && p->stage_order == IMOP_ORDER_RGB_WB) {
        or_wb_rgb(rgb, w, h, bd, p->wb_gain);
        rgb_copy_fill(dumps->white_balance, rgb, n * 3);
    }
    if (p->stages & IMOP_STAGE_CCM) or_ccm(rgb, w, h, bd, p->ccm);
    rgb_copy_fill(dumps->ccm, rgb, n * 3);
    if (p->stages & IMOP_STAGE_LUT3D) or_lut3d(rgb, w, h, bd, p->lut3d, p->lut3d_size);
    if (p->out_format == IMOP_OUT_NATIVE) {
        if (bd <= 8) {
            uint8_t* o = (uint8_t*)out;
            for (size_t i = 0; i < n * 3; i++) o[i] = (uint8_t)rgb[i];
        } else {
            memcpy(out, rgb, n * 3 * sizeof(uint16_t));
        }
    } else {
        or_tone_rgb8(rgb, (uint8_t*)out, w, h, bd, p->tone_mode, p->tone_lut, p->tone_knots);
    }
    free(bay);
    free(rgb);
    return 0;
}
