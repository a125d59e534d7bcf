/*
 * isp_oracle.h - CPU oracle of the RAW->RGB hot path.  TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's CPU algorithm for every stage of the path,
 * used by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference arm as
 * the checker and as the timed CPU baseline.  The product library never links or calls it.
 *
 * Parity pin: the restatement is checked stage by stage against the reference's own CPU
 * functions compiled from source (oracle/Makefile -> oracle/_ref/) and against the golden
 * vectors under tests/golden/ that those functions produced (tests/golden/make_golden.py).
 *
 * Internal storage: Bayer planes are u16 per pixel for every bit depth and RGB planes are
 * u16 x 3 per pixel; the reference keeps u8 for bit depth <= 8, which holds the same values
 * because every stage clamps to 2^bd - 1.
 */
#ifndef IMOP_ISP_ORACLE_H
#define IMOP_ISP_ORACLE_H

#include <stddef.h>
#include <stdint.h>
#include "../include/imop_isp.h"

#ifdef __cplusplus
extern "C" {
#endif

int or_max_val(int bd);
int or_bayer_color(int row, int col, int pattern);

/* a1/a2: unpack one frame to u16 (packed MIPI RAW10/RAW12 or u8/u16 storage). */
void or_unpack(const uint8_t* in, int w, int h, int bd, int packed, uint16_t* out);
int or_get_packed_raw(const uint8_t* data, int x, int y, int w, int h, int bd);

/* a3 */
void or_black_level(uint16_t* d, int w, int h, int pattern, int bd, int mode, const float off[4]);
/* a4 / a4' (sequential, in place) */
void or_dpc_adaptive(uint16_t* d, int w, int h, int pattern, int bd, float threshold);
void or_dpc_map(uint16_t* d, int w, int h, int pattern, int bd, const ImopDefectPoint* map, int n);
/* a5 / a5' */
void or_lsc_grid(uint16_t* d, int w, int h, int pattern, int bd, const float* grid, int gw, int gh);
void or_lsc_poly(uint16_t* d, int w, int h, int pattern, int bd, const float coef[4][3], float cx,
                 float cy);
/* flat-field -> 32x24x4 grid (flat_field.cpp:30-76); returns 0 on success */
int or_lsc_flat_field_grid(const void* ff, int ffw, int ffh, int pattern, int bd, float* grid_out);
/* a6' Bayer-domain white balance */
void or_wb_bayer(uint16_t* d, int w, int h, int pattern, int bd, const float gain[3]);
/* a7 / a8 / a8': Bayer (u16) -> RGB (u16 x 3) at bit depth bd */
void or_demosaic_hqli(const uint16_t* bay, uint16_t* rgb, int w, int h, int pattern, int bd);
void or_demosaic_amaze(const uint16_t* bay, uint16_t* rgb, int w, int h, int pattern, int bd);
void or_demosaic_mg(const uint16_t* bay, uint16_t* rgb, int w, int h, int pattern, int bd);
/* a6 RGB-domain white balance, a9 CCM (in place on RGB u16 x 3) */
void or_wb_rgb(uint16_t* rgb, int w, int h, int bd, const float gain[3]);
void or_ccm(uint16_t* rgb, int w, int h, int bd, const float m[9]);
void or_lut3d(uint16_t* rgb, int w, int h, int bd, const float* lut, int size);
/* a10: tone value in [0,1] for an integer sample, then the 8-bit quantiser */
float or_tone_value(int mode, const float* lut, const float* knots, int v, int bd);
uint8_t or_tone_to_u8(float t);
void or_tone_rgb8(const uint16_t* rgb, uint8_t* out, int w, int h, int bd, int mode,
                  const float* lut, const float* knots);

/* Full chain.  Each non-NULL dump pointer receives that stage's frame. Returns 0 or an
 * IMOP_ERR_* code (same validation as the product's imop_isp_set_params). */
typedef struct OracleDumps {
    uint16_t* unpacked;
    uint16_t* black_level;
    uint16_t* defect;
    uint16_t* lens_shading;
    uint16_t* white_balance; /* Bayer (w*h) or RGB (w*h*3) depending on stage_order */
    uint16_t* demosaic;
    uint16_t* ccm;
} OracleDumps;
int or_pipeline(const ImopIspParams* p, const void* in, void* out, OracleDumps* dumps);

/* seeded synthetic frames (isp_oracle_scene.c): the workloads' scene, defect positions and MIPI
 * packing, equal to the product's generator byte for byte */
int or_scene_render(int w, int h, int bd, int pattern, uint64_t seed, float lo, float hi, float gain,
                    float read_sigma, void* out);
int or_scene_defects(int w, int h, uint64_t seed, int count, int* xy);
void or_scene_apply_defects(uint16_t* frame, int w, int bd, const int* xy, int count);
void or_pack_mipi(const uint16_t* in, size_t n, int bd, uint8_t* out);

/* Differentiable FP64 forward of the calibration pipeline (no integer rounding):
 * raw u16 -> BL -> LSC grid -> WB -> HQLI-style bilinear (same stencil) -> CCM -> knots curve.
 * theta layout = imop_isp_param_count().  rgb out: h*w*3 doubles. */
void or_render_f64(const uint16_t* raw, int w, int h, int bd, int pattern, int gw, int gh,
                   const double* theta, double* rgb);
/* Analytic FP64 gradient of 0.5*sum((render - target)^2) w.r.t. theta, accumulated into grad. */
double or_adjoint_f64(const uint16_t* raw, const float* target, int w, int h, int bd, int pattern,
                      int gw, int gh, const double* theta, double* grad);

/* FP64 differentiable calibration chain (isp_oracle_grad.c): parameter layout as
 * ImopAdjointDesc in include/imop_isp.h; raw frames back to back; rgb / ref are n_frames*h*w*3. */
int or_adj_param_count(const ImopAdjointDesc* d);
int or_adj_forward(const ImopAdjointDesc* d, const double* theta, const uint8_t* raw, double* rgb_out);
int or_adj_loss_grad(const ImopAdjointDesc* d, const double* theta, const uint8_t* raw, const float* ref, int mode,
                     double* loss, double* grad);
int or_adj_loss(const ImopAdjointDesc* d, const double* theta, const uint8_t* raw, const float* ref, int mode,
                double* loss);

/* Baseline JPEG encoder (isp_oracle_jpeg.c): the reference's process_encode_baseline byte for byte.
 * RGB8 interleaved input; returns 0 or the reference's JpegError value; *out_size in = capacity
 * (0: w*h*9 + 65536), out = bytes written. */
int or_jpeg_encode(const uint8_t* in, int w, int h, int bd, int quality, int subsample, uint8_t* out,
                   size_t* out_size);
void or_jpeg_scale_qtable(int q[64], const int base[64], int quality);

#ifdef __cplusplus
}
#endif
#endif
