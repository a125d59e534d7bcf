/*
 * isp_oracle_grad.c - FP64 differentiable forward and analytic (reverse-mode) gradient of the
 * calibration chain.  TEST INFRASTRUCTURE ONLY: the checker of the adjoint kernel, itself checked
 * by central finite differences in tests/.
 *
 * The chain restates the hot path's stages with the integer rounding dropped (the reference has
 * no gradients; its stage formulas are followed):
 *   b = clamp(raw - bl[c], 0, mv)                          black_level/per_channel.cpp:22-31
 *   l = clamp(b * gain(x, y, c), 0, mv)                    lens_shading/flat_field.cpp:84-105
 *   u = clamp(l * wb[c], 0, mv)                            white_balance/manual.cpp:29-31
 *   RGB = demosaic(u)  (HQLI interp_core.hpp:39-65; AMAZE amaze.cpp:159-183 and the colour
 *         differences of common.hpp:142-199 with the -1 green sentinel; border copies of
 *         common.hpp:47-135), then clamp(., 0, mv)
 *   o = clamp(M * RGB, 0, mv)                              ccm/linear_3x3.cpp:28-41
 *   t = knots lerp at o / mv, 32 segments                  tone/curves_3point.cpp:92-97
 * Clamps pass gradient strictly inside their range; |v| has derivative sign(v), sign(0) = 0.
 */
#include "isp_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct { int r_row, r_col, b_row, b_col; } APO;
static APO apo(int pattern) {
    APO p;
    switch (pattern) {
        case IMOP_BGGR: p.r_row = 1; p.r_col = 1; p.b_row = 0; p.b_col = 0; break;
        case IMOP_GRBG: p.r_row = 0; p.r_col = 1; p.b_row = 1; p.b_col = 0; break;
        case IMOP_GBRG: p.r_row = 1; p.r_col = 0; p.b_row = 0; p.b_col = 1; break;
        default: p.r_row = 0; p.r_col = 0; p.b_row = 1; p.b_col = 1; break;
    }
    return p;
}
static int a_is_r(APO p, int y, int x) { return ((y & 1) == p.r_row) && ((x & 1) == p.r_col); }
static int a_is_b(APO p, int y, int x) { return ((y & 1) == p.b_row) && ((x & 1) == p.b_col); }
static double clampd(double v, double lo, double hi) { return v < lo ? lo : (v > hi ? hi : v); }
static double inside(double v, double lo, double hi) { return (v > lo && v < hi) ? 1.0 : 0.0; }
static double sgn(double v) { return v > 0 ? 1.0 : (v < 0 ? -1.0 : 0.0); }

int or_adj_param_count(const ImopAdjointDesc* d) { return 16 + 4 * d->grid_w * d->grid_h + 33; }

/* border fill source: rows first (full width), then columns for interior rows; the 8-bit AMAZE
 * path fills the RGB borders again, which also clamps the columns of the copied rows */
static void border_src(int x, int y, int w, int h, int both, int* sx, int* sy) {
    *sy = y < 2 ? 2 : (y > h - 3 ? h - 3 : y);
    int row_interior = (y >= 2 && y < h - 2);
    *sx = (row_interior || both) ? (x < 2 ? 2 : (x > w - 3 ? w - 3 : x)) : x;
}

typedef struct {
    int w, h, mv, gw, gh, demosaic, both;
    APO po;
    const double* th;
    double *b, *gain, *l, *u, *G;         /* planes of one frame */
    double *gu, *gG;                      /* their gradients */
    int* c;                               /* CFA colour */
    double gwx[2], gwy[2];
} Frame;

#define TH_BL 0
#define TH_WB 4
#define TH_CCM 7
#define TH_GRID 16

static double wbc(const Frame* F, int c) { return F->th[TH_WB + (c == 0 ? 0 : (c == 3 ? 2 : 1))]; }

/* bilinear weights and base node of (x, y): the apply loop of flat_field.cpp:84-105 */
static void grid_pos(const Frame* F, int x, int y, int* gx, int* gy, double* fx, double* fy) {
    double gxf = (double)x * (F->gw - 1) / (double)(F->w - 1);
    double gyf = (double)y * (F->gh - 1) / (double)(F->h - 1);
    int ix = (int)gxf, iy = (int)gyf;
    if (ix < 0) ix = 0;
    if (ix > F->gw - 2) ix = F->gw - 2;
    if (iy < 0) iy = 0;
    if (iy > F->gh - 2) iy = F->gh - 2;
    *gx = ix; *gy = iy;
    *fx = gxf - ix; *fy = gyf - iy;
}

static double amaze_g(const Frame* F, int x, int y, double* out_parts) {
    const int w = F->w;
    const double* u = F->u;
#define U(X, Y) u[(size_t)(Y) * w + (X)]
    double c = U(x, y);
    double hm1 = U(x - 1, y), hp1 = U(x + 1, y), hm2 = U(x - 2, y), hp2 = U(x + 2, y);
    double vm1 = U(x, y - 1), vp1 = U(x, y + 1), vm2 = U(x, y - 2), vp2 = U(x, y + 2);
#undef U
    double lapH = 2 * c - hm2 - hp2, lapV = 2 * c - vm2 - vp2;
    double gH = fabs(hm1 - hp1) + fabs(lapH), gV = fabs(vm1 - vp1) + fabs(lapV);
    double a = 1.0 / (1.0 + gH), b = 1.0 / (1.0 + gV);
    double wh = a / (a + b), wv = b / (a + b);
    double gh = (hm1 + hp1) * 0.5 + lapH * 0.25, gv = (vm1 + vp1) * 0.5 + lapV * 0.25;
    if (out_parts) {
        out_parts[0] = a; out_parts[1] = b; out_parts[2] = wh; out_parts[3] = wv;
        out_parts[4] = gh; out_parts[5] = gv; out_parts[6] = sgn(hm1 - hp1); out_parts[7] = sgn(lapH);
        out_parts[8] = sgn(vm1 - vp1); out_parts[9] = sgn(lapV);
    }
    return wh * gh + wv * gv;
}

static void frame_forward_planes(Frame* F, const uint16_t* raw) {
    const int w = F->w, h = F->h, mv = F->mv;
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            size_t i = (size_t)y * w + x;
            int c = a_is_r(F->po, y, x) ? 0 : (a_is_b(F->po, y, x) ? 3 : (((y & 1) == F->po.r_row) ? 1 : 2));
            F->c[i] = c;
            double b = clampd((double)raw[i] - F->th[TH_BL + c], 0, mv);
            int gx, gy;
            double fx, fy;
            grid_pos(F, x, y, &gx, &gy, &fx, &fy);
            const double* g = F->th + TH_GRID;
            double g00 = g[(gy * F->gw + gx) * 4 + c], g10 = g[(gy * F->gw + gx + 1) * 4 + c];
            double g01 = g[((gy + 1) * F->gw + gx) * 4 + c], g11 = g[((gy + 1) * F->gw + gx + 1) * 4 + c];
            double gain = g00 * (1 - fx) * (1 - fy) + g10 * fx * (1 - fy) + g01 * (1 - fx) * fy + g11 * fx * fy;
            double l = clampd(b * gain, 0, mv);
            F->b[i] = b;
            F->gain[i] = gain;
            F->l[i] = l;
            F->u[i] = clampd(l * wbc(F, c), 0, mv);
        }
    for (size_t i = 0; i < (size_t)w * h; i++) F->G[i] = -1.0;
    if (F->demosaic == IMOP_DEMOSAIC_AMAZE)
        for (int y = 2; y < h - 2; y++)
            for (int x = 2; x < w - 2; x++) {
                size_t i = (size_t)y * w + x;
                F->G[i] = (a_is_r(F->po, y, x) || a_is_b(F->po, y, x)) ? amaze_g(F, x, y, NULL) : F->u[i];
            }
}

/* demosaic value (before the plane clamp) of pixel (x, y) */
static void demosaic_at(const Frame* F, int x, int y, double v[3]) {
    const int w = F->w, h = F->h;
    const double* u = F->u;
    const double* G = F->G;
#define U(X, Y) u[(size_t)(Y) * w + (X)]
#define GG(X, Y) G[(size_t)(Y) * w + (X)]
    v[0] = v[1] = v[2] = 0.0;
    int at_r = a_is_r(F->po, y, x), at_b = a_is_b(F->po, y, x), rrow = (y & 1) == F->po.r_row;
    if (F->demosaic == IMOP_DEMOSAIC_HQLI) {
        if (x < 2 || x >= w - 2 || y < 2 || y >= h - 2) return;
        double n4 = U(x - 1, y) + U(x + 1, y) + U(x, y - 1) + U(x, y + 1);
        double d4 = U(x - 1, y - 1) + U(x + 1, y - 1) + U(x - 1, y + 1) + U(x + 1, y + 1);
        if (at_r) { v[0] = U(x, y); v[1] = n4 / 4; v[2] = d4 / 4; }
        else if (at_b) { v[0] = d4 / 4; v[1] = n4 / 4; v[2] = U(x, y); }
        else {
            double hz = (U(x - 1, y) + U(x + 1, y)) / 2, vt = (U(x, y - 1) + U(x, y + 1)) / 2;
            v[1] = U(x, y);
            v[0] = rrow ? hz : vt;
            v[2] = rrow ? vt : hz;
        }
        return;
    }
    double g = GG(x, y);
    v[1] = g;
    if (x < 1 || x >= w - 1 || y < 1 || y >= h - 1) return;
    if (at_r || at_b) {
        double s = (U(x - 1, y - 1) - GG(x - 1, y - 1)) + (U(x + 1, y - 1) - GG(x + 1, y - 1)) +
                   (U(x - 1, y + 1) - GG(x - 1, y + 1)) + (U(x + 1, y + 1) - GG(x + 1, y + 1));
        double other = g + s / 4;
        if (at_r) { v[0] = U(x, y); v[2] = other; } else { v[2] = U(x, y); v[0] = other; }
    } else {
        double hz = (U(x - 1, y) - GG(x - 1, y)) + (U(x + 1, y) - GG(x + 1, y));
        double vt = (U(x, y - 1) - GG(x, y - 1)) + (U(x, y + 1) - GG(x, y + 1));
        v[0] = g + (rrow ? hz : vt) / 2;
        v[2] = g + (rrow ? vt : hz) / 2;
    }
#undef U
#undef GG
}

/* adjoint of demosaic_at: gradient gv[3] of the values into gu / gG */
static void demosaic_back(Frame* F, int x, int y, const double gv[3]) {
    const int w = F->w, h = F->h;
    double* gu = F->gu;
    double* gG = F->gG;
#define GU(X, Y) gu[(size_t)(Y) * w + (X)]
#define GGG(X, Y) gG[(size_t)(Y) * w + (X)]
    int at_r = a_is_r(F->po, y, x), at_b = a_is_b(F->po, y, x), rrow = (y & 1) == F->po.r_row;
    if (F->demosaic == IMOP_DEMOSAIC_HQLI) {
        if (x < 2 || x >= w - 2 || y < 2 || y >= h - 2) return;
        if (at_r || at_b) {
            double gown = at_r ? gv[0] : gv[2], goth = at_r ? gv[2] : gv[0];
            GU(x, y) += gown;
            GU(x - 1, y) += gv[1] / 4; GU(x + 1, y) += gv[1] / 4; GU(x, y - 1) += gv[1] / 4; GU(x, y + 1) += gv[1] / 4;
            GU(x - 1, y - 1) += goth / 4; GU(x + 1, y - 1) += goth / 4; GU(x - 1, y + 1) += goth / 4; GU(x + 1, y + 1) += goth / 4;
        } else {
            double ghz = rrow ? gv[0] : gv[2], gvt = rrow ? gv[2] : gv[0];
            GU(x, y) += gv[1];
            GU(x - 1, y) += ghz / 2; GU(x + 1, y) += ghz / 2;
            GU(x, y - 1) += gvt / 2; GU(x, y + 1) += gvt / 2;
        }
        return;
    }
    GGG(x, y) += gv[1];
    if (x < 1 || x >= w - 1 || y < 1 || y >= h - 1) return;
    if (at_r || at_b) {
        double goth = at_r ? gv[2] : gv[0];
        GU(x, y) += at_r ? gv[0] : gv[2];
        GGG(x, y) += goth;
        double q = goth / 4;
        GU(x - 1, y - 1) += q; GGG(x - 1, y - 1) -= q;
        GU(x + 1, y - 1) += q; GGG(x + 1, y - 1) -= q;
        GU(x - 1, y + 1) += q; GGG(x - 1, y + 1) -= q;
        GU(x + 1, y + 1) += q; GGG(x + 1, y + 1) -= q;
    } else {
        double ghz = (rrow ? gv[0] : gv[2]) / 2, gvt = (rrow ? gv[2] : gv[0]) / 2;
        GGG(x, y) += gv[0] + gv[2];
        GU(x - 1, y) += ghz; GGG(x - 1, y) -= ghz;
        GU(x + 1, y) += ghz; GGG(x + 1, y) -= ghz;
        GU(x, y - 1) += gvt; GGG(x, y - 1) -= gvt;
        GU(x, y + 1) += gvt; GGG(x, y + 1) -= gvt;
    }
#undef GU
#undef GGG
}

/* adjoint of the green plane: gG into gu */
static void green_back(Frame* F) {
    const int w = F->w, h = F->h;
    if (F->demosaic != IMOP_DEMOSAIC_AMAZE) return;
    for (int y = 2; y < h - 2; y++)
        for (int x = 2; x < w - 2; x++) {
            size_t i = (size_t)y * w + x;
            double g = F->gG[i];
            if (g == 0.0) continue;
            if (!(a_is_r(F->po, y, x) || a_is_b(F->po, y, x))) {
                F->gu[i] += g;
                continue;
            }
            double P[10];
            amaze_g(F, x, y, P);
            double a = P[0], b = P[1], wh = P[2], wv = P[3], gh = P[4], gv = P[5];
            double s = (a + b) * (a + b);
            double dgH = -a * a * b * (gh - gv) / s;  /* dG/dgradH */
            double dgV = -b * b * a * (gv - gh) / s;  /* dG/dgradV */
            double* gu = F->gu;
#define GU(X, Y) gu[(size_t)(Y) * w + (X)]
            /* horizontal: gh = 0.5 (h-1 + h+1) + 0.25 lapH; gradH = |h-1 - h+1| + |lapH| */
            double tH = g * (wh * 0.25 + dgH * P[7]);  /* d/dlapH */
            GU(x - 1, y) += g * (wh * 0.5 + dgH * P[6]);
            GU(x + 1, y) += g * (wh * 0.5 - dgH * P[6]);
            GU(x, y) += 2 * tH;
            GU(x - 2, y) -= tH;
            GU(x + 2, y) -= tH;
            double tV = g * (wv * 0.25 + dgV * P[9]);
            GU(x, y - 1) += g * (wv * 0.5 + dgV * P[8]);
            GU(x, y + 1) += g * (wv * 0.5 - dgV * P[8]);
            GU(x, y) += 2 * tV;
            GU(x, y - 2) -= tV;
            GU(x, y + 2) -= tV;
#undef GU
        }
}

static void tone_eval(const double* knots, double o, int mv, double* t, int* idx, double* frac) {
    double xn = o / (double)mv;
    double fi = xn * 32.0;
    int k = (int)fi;
    double f = fi - k;
    if (k > 31) { k = 31; f = 1.0; }
    if (k < 0) { k = 0; f = 0.0; }
    *idx = k;
    *frac = f;
    *t = knots[k] * (1 - f) + knots[k + 1] * f;
}

static int frame_alloc(Frame* F, int w, int h, int with_grad) {
    size_t n = (size_t)w * h;
    F->b = malloc(n * sizeof(double)); F->gain = malloc(n * sizeof(double));
    F->l = malloc(n * sizeof(double)); F->u = malloc(n * sizeof(double)); F->G = malloc(n * sizeof(double));
    F->c = malloc(n * sizeof(int));
    F->gu = with_grad ? calloc(n, sizeof(double)) : NULL;
    F->gG = with_grad ? calloc(n, sizeof(double)) : NULL;
    return F->b && F->gain && F->l && F->u && F->G && F->c && (!with_grad || (F->gu && F->gG));
}
static void frame_free(Frame* F) {
    free(F->b); free(F->gain); free(F->l); free(F->u); free(F->G); free(F->c); free(F->gu); free(F->gG);
}

/* One frame: forward (t into rgb_out when given); with `ref`, the loss against it (target or
 * upstream gradient, by `mode`); with `grad`, dL/dtheta of this frame added into grad. */
static int frame_run(const ImopAdjointDesc* d, const double* theta, const uint8_t* raw, double* rgb_out,
                     const float* ref, int mode, double* loss, double* grad) {
    const int w = d->width, h = d->height, mv = or_max_val(d->bit_depth);
    const size_t n = (size_t)w * h;
    uint16_t* r16 = malloc(n * sizeof(uint16_t));
    Frame F;
    memset(&F, 0, sizeof(F));
    if (!r16 || !frame_alloc(&F, w, h, grad != NULL)) {
        free(r16);
        frame_free(&F);
        return IMOP_ERR_INTERNAL;
    }
    F.w = w; F.h = h; F.mv = mv; F.gw = d->grid_w; F.gh = d->grid_h; F.demosaic = d->demosaic;
    F.both = (d->demosaic == IMOP_DEMOSAIC_AMAZE && d->bit_depth <= 8);
    F.po = apo(d->pattern);
    F.th = theta;
    const double* M = theta + TH_CCM;
    const double* knots = theta + TH_GRID + 4 * d->grid_w * d->grid_h;
    double* dk = grad ? grad + TH_GRID + 4 * d->grid_w * d->grid_h : NULL;
    double L = 0.0;
    or_unpack(raw, w, h, d->bit_depth, d->packed, r16);
    frame_forward_planes(&F, r16);
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            int sx, sy;
            border_src(x, y, w, h, F.both, &sx, &sy);
            double v[3], rgb[3], pre[3], o[3], t[3];
            demosaic_at(&F, sx, sy, v);
            for (int k = 0; k < 3; k++) rgb[k] = clampd(v[k], 0, mv);
            for (int r = 0; r < 3; r++) {
                pre[r] = M[3 * r] * rgb[0] + M[3 * r + 1] * rgb[1] + M[3 * r + 2] * rgb[2];
                o[r] = clampd(pre[r], 0, mv);
            }
            int idx[3];
            double fr[3];
            for (int k = 0; k < 3; k++) tone_eval(knots, o[k], mv, &t[k], &idx[k], &fr[k]);
            size_t pi = ((size_t)y * w + x) * 3;
            if (rgb_out)
                for (int k = 0; k < 3; k++) rgb_out[pi + k] = t[k];
            if (!ref) continue;
            double gt[3];
            for (int k = 0; k < 3; k++) {
                if (mode == IMOP_ADJ_TARGET) {
                    double e = t[k] - (double)ref[pi + k];
                    L += e * e;
                    gt[k] = 2 * e;
                } else {
                    gt[k] = (double)ref[pi + k];
                    L += t[k] * gt[k];
                }
            }
            if (!grad) continue;
            double go[3], grgb[3] = {0, 0, 0}, gv[3];
            for (int k = 0; k < 3; k++) {
                dk[idx[k]] += gt[k] * (1 - fr[k]);
                dk[idx[k] + 1] += gt[k] * fr[k];
                go[k] = gt[k] * (knots[idx[k] + 1] - knots[idx[k]]) * 32.0 / (double)mv;
            }
            for (int r = 0; r < 3; r++) {
                double gp = go[r] * inside(pre[r], 0, mv);
                for (int j = 0; j < 3; j++) {
                    grad[TH_CCM + 3 * r + j] += gp * rgb[j];
                    grgb[j] += M[3 * r + j] * gp;
                }
            }
            for (int k = 0; k < 3; k++) gv[k] = grgb[k] * inside(v[k], 0, mv);
            demosaic_back(&F, sx, sy, gv);
        }
    if (grad) {
        green_back(&F);
        for (int y = 0; y < h; y++)
            for (int x = 0; x < w; x++) {
                size_t i = (size_t)y * w + x;
                double g = F.gu[i];
                if (g == 0.0) continue;
                int c = F.c[i];
                double wb = wbc(&F, c);
                if (!inside(F.l[i] * wb, 0, mv)) continue;
                grad[TH_WB + (c == 0 ? 0 : (c == 3 ? 2 : 1))] += g * F.l[i];
                double gl = g * wb;
                if (!inside(F.b[i] * F.gain[i], 0, mv)) continue;
                double ggain = gl * F.b[i];
                int gx, gy;
                double fx, fy;
                grid_pos(&F, x, y, &gx, &gy, &fx, &fy);
                double* gg = grad + TH_GRID;
                gg[(gy * F.gw + gx) * 4 + c] += ggain * (1 - fx) * (1 - fy);
                gg[(gy * F.gw + gx + 1) * 4 + c] += ggain * fx * (1 - fy);
                gg[((gy + 1) * F.gw + gx) * 4 + c] += ggain * (1 - fx) * fy;
                gg[((gy + 1) * F.gw + gx + 1) * 4 + c] += ggain * fx * fy;
                double gb = gl * F.gain[i];
                if (inside((double)r16[i] - theta[TH_BL + c], 0, mv)) grad[TH_BL + c] -= gb;
            }
    }
    if (loss) *loss = L;
    free(r16);
    frame_free(&F);
    return 0;
}

/* All frames, one OpenMP task per frame; per-frame losses and gradients are summed in frame order. */
static int adj_run(const ImopAdjointDesc* d, const double* theta, const uint8_t* raw, double* rgb_out,
                   const float* ref, int mode, double* loss, double* grad) {
    const size_t n = (size_t)d->width * d->height;
    const size_t in_bytes = d->packed ? (n * (size_t)d->bit_depth + 7) / 8 : (d->bit_depth <= 8 ? n : 2 * n);
    const int P = or_adj_param_count(d), nf = d->n_frames;
    double* fl = calloc((size_t)nf, sizeof(double));
    double* fg = grad ? calloc((size_t)nf * P, sizeof(double)) : NULL;
    int* rc = calloc((size_t)nf, sizeof(int));
    if (!fl || !rc || (grad && !fg)) {
        free(fl); free(fg); free(rc);
        return IMOP_ERR_INTERNAL;
    }
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int f = 0; f < nf; f++)
        rc[f] = frame_run(d, theta, raw + (size_t)f * in_bytes, rgb_out ? rgb_out + (size_t)f * n * 3 : NULL,
                          ref ? ref + (size_t)f * n * 3 : NULL, mode, &fl[f], fg ? fg + (size_t)f * P : NULL);
    int status = 0;
    double L = 0.0;
    for (int f = 0; f < nf; f++) {
        if (rc[f]) status = rc[f];
        L += fl[f];
    }
    if (grad) {
        memset(grad, 0, (size_t)P * sizeof(double));
        for (int f = 0; f < nf; f++)
            for (int k = 0; k < P; k++) grad[k] += fg[(size_t)f * P + k];
    }
    if (loss) *loss = L;
    free(fl); free(fg); free(rc);
    return status;
}

int or_adj_forward(const ImopAdjointDesc* d, const double* theta, const uint8_t* raw, double* rgb_out) {
    return adj_run(d, theta, raw, rgb_out, NULL, 0, NULL, NULL);
}

int or_adj_loss_grad(const ImopAdjointDesc* d, const double* theta, const uint8_t* raw, const float* ref, int mode,
                     double* loss, double* grad) {
    return adj_run(d, theta, raw, NULL, ref, mode, loss, grad);
}

/* loss only (the finite-difference probe) */
int or_adj_loss(const ImopAdjointDesc* d, const double* theta, const uint8_t* raw, const float* ref, int mode,
                double* loss) {
    return adj_run(d, theta, raw, NULL, ref, mode, loss, NULL);
}
