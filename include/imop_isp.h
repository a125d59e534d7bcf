/*
 * imop_isp.h - C ABI of the GB300-native RAW->RGB ISP hot path.
 *
 * One fused sm_103a kernel runs
 *   unpack -> black_level -> defect_correct -> lens_shading -> white_balance
 *   -> Bayer demosaic (HQLI / AMAZE / MG) -> ccm -> tone LUT -> RGB8
 * over one frame or over a batch of frames of uneven sizes and formats.
 *
 * Every entry point takes plain pointers and sizes; no C++ or torch types cross
 * this boundary.  Status codes 0..6 are numerically equal to the reference's
 * imop::DemosaicError (include/imop/types.hpp:31-39 of im-operator) and to the
 * per-module error enums (e.g. include/black_level/types.hpp:13-21), so a
 * caller that maps "non-zero" to "fall back" keeps the reference's contract.
 *
 * Reference interfaces replaced (paths are relative to the im-operator tree):
 *   imop_isp_run_host      : the host-side composition of
 *                            black_level::process_black_level   (src/black_level/dispatch.cpp:44-63)
 *                            defect_correct::process_defect_correct (src/defect_correct/dispatch.cpp:44-63)
 *                            lens_shading::process_lens_shading  (src/lens_shading/dispatch.cpp:41-60)
 *                            imop::demosaic                      (src/algorithms/dispatch.cpp:89-113)
 *                            white_balance::process_white_balance (src/white_balance/dispatch.cpp:196-219)
 *                            ccm::process_ccm                    (src/ccm/dispatch.cpp:167-191)
 *                            tone::process_tone                  (src/tone/dispatch.cpp:66-86)
 *                            with their GPU glue in src/gpu_dispatch.cpp:292-571
 *   imop_isp_batch_*       : imop::demosaic_cuda_batch           (src/algorithms/cuda_dispatch.cpp:150-209)
 *   imop_op_*              : the per-operator *_cuda entry points of src/gpu_dispatch.cpp
 *                            and imop::demosaic_cuda (src/algorithms/cuda_dispatch.cpp:68-141)
 */
#ifndef IMOP_ISP_H
#define IMOP_ISP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define IMOP_ISP_ABI_VERSION 4

/* ---- status codes (0..6 == imop::DemosaicError) ---------------------------------- */
enum {
    IMOP_OK = 0,
    IMOP_ERR_NULL_INPUT = 1,
    IMOP_ERR_INVALID_DIMENSIONS = 2,
    IMOP_ERR_INVALID_BIT_DEPTH = 3,
    IMOP_ERR_INVALID_PATTERN = 4,
    IMOP_ERR_IMAGE_TOO_SMALL = 5,
    IMOP_ERR_INTERNAL = 6,
    /* codes beyond the reference enum; a DemosaicError-typed caller sees them as InternalError */
    IMOP_ERR_INVALID_ARGUMENT = 100, /* a parameter outside its documented range          */
    IMOP_ERR_UNSUPPORTED = 101,      /* format / algorithm combination not on this path     */
    IMOP_ERR_CUDA = 102,             /* a CUDA runtime call failed                          */
    IMOP_ERR_TIMEOUT = 103,          /* a bounded device-side wait expired                  */
    IMOP_ERR_CAPACITY = 104,         /* a device-side list (defect chain, queue) overflowed */
    IMOP_ERR_NO_DEVICE = 105,        /* no CUDA device visible                              */
    IMOP_ERR_INSUFFICIENT_PATCHES = 106, /* fewer than 3 patches for a CCM solve             */
    IMOP_ERR_SINGULAR = 107          /* singular normal equations in a CCM solve            */
};

/* imop::BayerPattern (include/imop/types.hpp:12-17) */
enum { IMOP_RGGB = 0, IMOP_BGGR = 1, IMOP_GRBG = 2, IMOP_GBRG = 3 };

/* imop::DemosaicAlgorithm values (include/imop/types.hpp:19-29) served by this path */
enum { IMOP_DEMOSAIC_HQLI = 1, IMOP_DEMOSAIC_MG = 2, IMOP_DEMOSAIC_AMAZE = 6 };

/* stage bits */
enum {
    IMOP_STAGE_BLACK_LEVEL = 1u << 0,
    IMOP_STAGE_DEFECT = 1u << 1,
    IMOP_STAGE_LENS_SHADING = 1u << 2,
    IMOP_STAGE_WHITE_BALANCE = 1u << 3,
    IMOP_STAGE_CCM = 1u << 4,
    IMOP_STAGE_ALL = 0x1Fu,
    /* optional 3D LUT after the CCM (lut::apply_lut, trilinear; not part of IMOP_STAGE_ALL) */
    IMOP_STAGE_LUT3D = 1u << 5
};

/* where white balance runs */
enum {
    IMOP_ORDER_BAYER_WB = 0, /* WB on the Bayer mosaic before demosaic (fused spec order)  */
    IMOP_ORDER_RGB_WB = 1    /* WB on RGB after demosaic (the order the reference's calls compose) */
};

/* black_level::BlackLevelAlgorithm (include/black_level/types.hpp:8-11) */
enum { IMOP_BL_PER_CHANNEL = 0, IMOP_BL_GLOBAL = 1 };
/* defect_correct::DefectCorrectAlgorithm (include/defect_correct/types.hpp:8-11) */
enum { IMOP_DPC_ADAPTIVE = 0, IMOP_DPC_MAP_BASED = 1 };
/* lens shading modes */
enum {
    IMOP_LSC_GRID = 0,       /* explicit gw x gh x 4 FP32 gain grid, bilinear (flat_field.cpp:78-107)  */
    IMOP_LSC_POLYNOMIAL = 1, /* lens_shading::process_polynomial (polynomial.cpp:13-52)                 */
    IMOP_LSC_FLAT_FIELD = 2  /* 32x24 grid derived from a flat-field frame (flat_field.cpp:30-76)       */
};
/* tone modes: every mode ends in an 8-bit value (int)(f(v)*255+0.5) clamped to [0,255] */
enum {
    IMOP_TONE_LINEAR = 0, /* f(v) = v / max                                         */
    IMOP_TONE_LUT = 1,    /* f(v) = lut[v], 2^bit_depth FP32 entries in [0,1]        */
    IMOP_TONE_KNOTS = 2   /* 33-knot piecewise-linear curve (curves_3point.cpp:114-135 rule) */
};
/* output format */
enum {
    IMOP_OUT_RGB8 = 0,  /* interleaved RGB, 3 bytes per pixel, after the tone stage            */
    IMOP_OUT_NATIVE = 1 /* interleaved RGB at the input bit depth (u8, or u16 when bd > 8); no tone */
};

/* defect_correct::DefectPoint (include/defect_correct/types.hpp:41-43): same layout */
typedef struct ImopDefectPoint {
    int x, y;
} ImopDefectPoint;

typedef struct ImopIspParams {
    int width, height;
    int bit_depth;   /* 1..16 */
    int packed;      /* 0: u8 (bd<=8) or u16 LSB-aligned; 1: MIPI RAW10 (4 px / 5 B), MIPI RAW12
                        (2 px / 3 B), other depths one LSB-first bit stream (RAW14, RAW16 ...) */
    int pattern;     /* IMOP_RGGB ... */
    int demosaic;    /* IMOP_DEMOSAIC_* */
    unsigned stages; /* IMOP_STAGE_* bits */
    int stage_order; /* IMOP_ORDER_* */

    int bl_mode;          /* IMOP_BL_* */
    float bl_offset[4];   /* R, Gr, Gb, B (GLOBAL uses [0]) */

    int dpc_mode;         /* IMOP_DPC_* */
    float dpc_threshold;  /* adaptive: relative threshold, clamped to [0.05, 1] */
    const ImopDefectPoint* dpc_map; /* map-based: copied by imop_isp_set_params */
    int dpc_map_count;

    int lsc_mode;         /* IMOP_LSC_* */
    const float* lsc_grid;        /* [grid_h][grid_w][4] (R, Gr, Gb, B); copied */
    int lsc_grid_w, lsc_grid_h;   /* >= 2 each */
    float lsc_poly[4][3];         /* per channel a2, a4, a6 */
    float lsc_center[2];          /* optical centre, normalised */
    const void* lsc_flat_field;   /* flat-field frame, same storage as an unpacked input; copied */
    int lsc_flat_w, lsc_flat_h;

    float wb_gain[3];     /* R, G, B */
    float ccm[9];         /* row-major 3x3, out = M * in */

    int tone_mode;        /* IMOP_TONE_* */
    const float* tone_lut; int tone_lut_len; /* copied; tone_lut_len == 2^bit_depth */
    float tone_knots[33];

    int out_format;       /* IMOP_OUT_* */

    /* IMOP_STAGE_LUT3D: lut3d_size^3 x 3 floats, R-major, RGB interleaved (lut::LUT3D); copied */
    const float* lut3d;
    int lut3d_size;       /* samples per axis, 2..65 */
} ImopIspParams;

/* Fill *p with the identity pipeline for a w x h frame: all stages off, HQLI, linear tone, RGB8. */
void imop_isp_params_default(ImopIspParams* p, int width, int height, int bit_depth, int packed);

/* Byte sizes of one input frame and one output frame for the given parameters. */
size_t imop_isp_input_bytes(const ImopIspParams* p);
size_t imop_isp_output_bytes(const ImopIspParams* p);

/* ---- context ----------------------------------------------------------------------- */
typedef struct imop_isp_ctx* imop_isp_t;

int imop_isp_create(imop_isp_t* out_ctx);
int imop_isp_destroy(imop_isp_t ctx);
/* Validates and uploads parameters (grid, LUT, defect map are copied to the device).
 * Same validation order and codes as the reference dispatchers. */
int imop_isp_set_params(imop_isp_t ctx, const ImopIspParams* p);

/* Drop-in semantics: host buffers, H2D + fused kernel + D2H, synchronous (the reference's
 * gpu_dispatch.cpp call shape).  in_bytes / out_bytes must be at least the frame sizes. */
int imop_isp_run_host(imop_isp_t ctx, const void* in, size_t in_bytes, void* out, size_t out_bytes);

/* Device pointers, asynchronous on `stream` (a cudaStream_t; NULL = legacy default stream). */
int imop_isp_run_device(imop_isp_t ctx, const void* d_in, void* d_out, void* stream);

/* Plain per-operator form: the same pipeline as one kernel per stage over full frames kept
 * in device memory (the comparator for the fused kernel).  Asynchronous on `stream`. */
int imop_isp_run_device_plain(imop_isp_t ctx, const void* d_in, void* d_out, void* stream);

/* Per-stage dumps through the plain per-operator kernels.  Each non-NULL host pointer receives
 * one full frame: Bayer stages as u16 per pixel (w*h*2 bytes), RGB stages as u16 x 3 per pixel
 * (w*h*6 bytes), the final output in the context's output format. Synchronous. */
typedef struct ImopStageDumps {
    uint16_t* unpacked;     /* raw values after unpack                  */
    uint16_t* black_level;  /* after black level                        */
    uint16_t* defect;       /* after defect correction                  */
    uint16_t* lens_shading; /* after lens shading                       */
    uint16_t* white_balance;/* after Bayer WB (ORDER_BAYER_WB) or RGB WB (ORDER_RGB_WB, 3 ch) */
    uint16_t* demosaic;     /* RGB at bit depth after demosaic          */
    uint16_t* ccm;          /* RGB at bit depth after CCM               */
    uint8_t* output;        /* final output                             */
} ImopStageDumps;
int imop_isp_dump_stages(imop_isp_t ctx, const void* in, size_t in_bytes, ImopStageDumps* dumps);

/* Tile shape of the fused kernel (0 = autotuned / default). */
int imop_isp_set_tile(imop_isp_t ctx, int tile_w, int tile_h);

/* Device-side defect-chain statistics of the last run (seeds re-resolved in raster order). */
int imop_isp_last_stats(imop_isp_t ctx, int* dpc_seeds, int* dpc_overrides);

/* Wait for the work this context enqueued on `stream`, then return and clear the sticky device
 * status (IMOP_ERR_CAPACITY when a defect-chain list overflowed, IMOP_ERR_TIMEOUT when a staging
 * wait gave up).  The asynchronous entry points do not read it themselves. */
int imop_isp_sync_status(imop_isp_t ctx, void* stream);

/* ---- batches -------------------------------------------------------------------------- */
/* Replaces imop::demosaic_cuda_batch (src/algorithms/cuda_dispatch.cpp:150-209), which takes
 * one size, one format and host pointers; a batch here mixes frame sizes, formats and
 * parameter sets. */
typedef struct ImopFrameDesc {
    const ImopIspParams* params; /* this frame's parameters; NULL = the context's (set_params) */
    const void* in;              /* input frame  (device memory for batch_submit, host for run_host_batch) */
    void* out;                   /* output frame (same) */
} ImopFrameDesc;

enum {
    IMOP_BATCH_GRAPH = 1, /* record the batch's launches into a CUDA graph once and replay it while
                             the descriptors (pointers and parameter contents) stay the same */
    IMOP_BATCH_PLAIN = 2  /* one plain per-operator pipeline per frame (the comparator) */
};

/* All frames through the persistent fused kernels: one launch per run of up to 32 frames with
 * the same output channel width, tiles of every frame pulled by the same CTAs, and one defect
 * fix-up launch.  Parameter tables are uploaded once per distinct content and cached in the
 * context.  Asynchronous on `stream`; device frames must stay valid until it completes. */
int imop_isp_batch_submit(imop_isp_t ctx, const ImopFrameDesc* frames, int n, unsigned flags, void* stream);

/* Host frames (the drop-in call shape of demosaic_cuda_batch): copies in, fused kernel and
 * copies out are pipelined over four device slots and separate streams for the copies in, the
 * tile kernels, the defect fix-up and the copies out, so the transfers of one frame overlap the
 * kernels of its neighbours.  Page-locked host buffers overlap fully; pageable
 * ones are copied synchronously by the CUDA runtime.  Synchronous; returns the device status. */
int imop_isp_run_host_batch(imop_isp_t ctx, const ImopFrameDesc* frames, int n);

/* ---- per-operator drop-ins ------------------------------------------------------------ */
/* One stage of the pipeline on host buffers, synchronous, with the semantics of the reference's
 * per-module CPU functions (the *_cuda glue of src/gpu_dispatch.cpp:292-571 replaced):
 *   imop_op_bayer_stage: stage IMOP_STAGE_BLACK_LEVEL, IMOP_STAGE_DEFECT or IMOP_STAGE_LENS_SHADING,
 *     in place on one unpacked Bayer frame (u8 for bit depth <= 8, u16 otherwise), as
 *     black_level::process_black_level_cuda, defect_correct::process_defect_correct_cuda and
 *     lens_shading::process_lens_shading_cuda do;
 *   imop_op_rgb_stage: stage IMOP_STAGE_WHITE_BALANCE, IMOP_STAGE_CCM or IMOP_STAGE_LUT3D, interleaved RGB
 *     (u8 x 3 for bit depth <= 8, u16 x 3 otherwise) from `in` to `out` (may alias), as
 *     white_balance::process_white_balance_cuda and ccm::process_ccm_cuda do.
 * The stage's parameters come from *p (width, height, bit_depth, pattern and the stage's own
 * fields; the stage bits and the other stages' fields are ignored). */
int imop_op_bayer_stage(imop_isp_t ctx, const ImopIspParams* p, unsigned stage, void* data);
int imop_op_rgb_stage(imop_isp_t ctx, const ImopIspParams* p, unsigned stage, const void* in, void* out);

/* ---- the reference's RGB tone curves (tone::process_tone) ------------------------------ */
/* tone::ToneAlgorithm values (include/tone/types.hpp:8-14 of im-operator) */
enum {
    IMOP_TONE_CURVE_GAMMA = 0,
    IMOP_TONE_CURVE_S_CURVE = 1,
    IMOP_TONE_CURVE_LEVELS = 2,
    IMOP_TONE_CURVE_3POINT = 3,
    IMOP_TONE_CURVE_SHADOWS_HIGHLIGHTS = 4
};
/* tone::ToneParams (include/tone/types.hpp:50-58): same members in the same order */
typedef struct {
    float gamma, contrast, shadows, highlights, black_point, white_point, mid_point;
} ImopToneParams;
/* Entries of a per-sample table: every value the frame's storage holds (256 for u8, bit depth
 * <= 8; 65536 for u16). */
size_t imop_tone_table_entries(int bit_depth);
/* The output sample of tone curve `algorithm` for every input sample value (host).  GAMMA,
 * S_CURVE, LEVELS and CURVES_3POINT map each sample on its own with one function for R, G and B
 * (src/tone/gamma.cpp:22-32, s_curve.cpp:21-39, levels.cpp:40-57, curves_3point.cpp:64-101), so
 * the table, evaluated with the reference's float expressions, gives its output exactly.
 * SHADOWS_HIGHLIGHTS couples the channels through a luminance and returns IMOP_ERR_UNSUPPORTED.
 * `entries` must be at least imop_tone_table_entries(bit_depth). */
int imop_tone_table(int algorithm, int bit_depth, const ImopToneParams* params, uint16_t* table, size_t entries);
/* Every sample of an interleaved RGB frame (u8 x 3 for bit depth <= 8, u16 x 3 otherwise) through
 * `table` (imop_tone_table_entries(bit_depth) host entries) on the device: host buffers in and out
 * (may alias), synchronous; the GPU form of tone::process_tone_cuda (src/gpu_dispatch.cpp:292-312). */
int imop_op_rgb_table(imop_isp_t ctx, int width, int height, int bit_depth, const uint16_t* table, const void* in,
                      void* out);

/* ---- differentiable pipeline (calibration) ------------------------------------------- */
/* No counterpart in the reference, which has no parameter gradients.  The differentiable
 * forward is the calibration chain
 *     unpack -> black level -> lens-shading grid -> Bayer WB -> demosaic -> CCM -> 33-knot tone
 * with every stage's formula and clamp kept and the integer rounding between stages dropped;
 * its output is the tone value t in FP32 (the RGB8 path would store (int)(255 t + 0.5)).
 * Demosaic HQLI or AMAZE (AMAZE's gradient weights are differentiated, |.| with sign(0) = 0);
 * clamps pass gradient strictly inside their range.  Defect correction has no parameters and is
 * not part of this chain.
 *
 * Parameter vector theta (FP32), in this order:
 *     bl[4]                 black level per CFA colour (R, Gr, Gb, B), in DN
 *     wb[3]                 Bayer WB gain R, G (both greens), B
 *     ccm[9]                row-major 3x3
 *     grid[grid_h][grid_w][4]  lens-shading gains per node and CFA colour
 *     knots[33]             tone curve at v/max = k/32, linear in between
 * 16 + 4*grid_w*grid_h + 33 values (933 for a 17x13 grid). */
typedef struct ImopAdjointDesc {
    int width, height, bit_depth, packed, pattern;
    int demosaic;          /* IMOP_DEMOSAIC_HQLI or IMOP_DEMOSAIC_AMAZE */
    int grid_w, grid_h;    /* 2..32 nodes per side, grid_w * grid_h <= 256 */
    int n_frames;          /* frames stored back to back (input bytes of one frame apart) */
} ImopAdjointDesc;

enum {
    IMOP_ADJ_TARGET = 0,   /* ref = target t (FP32 x 3 per pixel); loss = sum (t - target)^2 */
    IMOP_ADJ_UPSTREAM = 1  /* ref = dL/dt (FP32 x 3 per pixel); loss receives sum t * dL/dt */
};

int imop_adjoint_param_count(const ImopAdjointDesc* d);

/* Differentiable forward: t for every pixel of every frame (n_frames * h * w * 3 FP32). */
int imop_isp_render_device(imop_isp_t ctx, const ImopAdjointDesc* d, const float* d_theta, const void* d_raw,
                           float* d_rgb, void* stream);

/* Adjoint: recomputes the forward per tile, back-propagates dL/dt and writes dL/dtheta
 * (param_count FP32) and the loss (one FP32).  Per-CTA partial sums are added in a fixed order
 * by a second kernel. Asynchronous on `stream`. */
int imop_isp_backward_device(imop_isp_t ctx, const ImopAdjointDesc* d, const float* d_theta, const void* d_raw,
                             const float* d_ref, int mode, float* d_loss, float* d_grad, void* stream);

/* ---- no device allocation ----------------------------------------------------------- */
/* No counterpart in the reference: the reference's GPU glue allocates per call
 * (src/gpu_dispatch.cpp:433) or through per-thread workspaces.  This entry point is for callers
 * that cannot let a library allocate device memory - a loop that owns all device memory through
 * its own pool, or a real-time loop that cannot afford cudaMalloc / cudaFree stalling the device.
 * It runs the same fused pipeline as imop_isp_run_device on the caller's device frames and
 * allocates nothing: its parameter tables and defect-chain scratch live in one file-scope device
 * array of about 340 KB that every GPU loading the library keeps until exit.  The first call on
 * each device looks up that array's address (cudaGetSymbolAddress, with the device current); make
 * that first call before any stream capture begins.  Limits: bit depth <= 12, lens shading by an
 * explicit grid of at most 64x64 nodes or by polynomial, adaptive defect correction only (no
 * defect map), and at most 16384 defect-chain seeds per call (IMOP_ERR_CAPACITY beyond).  Other
 * parameters return IMOP_ERR_UNSUPPORTED before any work.  All calls share the array and each
 * call resets what must start at zero, so calls that overlap on the GPU (two streams or host
 * threads at once) race.  The call enqueues on `stream`, waits for it, and returns the device
 * status.  The array's address is kept from a device's first call on: do not use this entry point
 * across a cudaDeviceReset of that device. */
int imop_isp_run_device_noalloc(const ImopIspParams* p, const void* d_in, void* d_out, void* stream);

/* ---- synthetic scene (seeded, bit-identical on every host) --------------------------- */
/* Per CFA channel: 4 random 2-D sinusoids mapped to [lo, hi], shot noise (gain DN/e-) and
 * Gaussian read noise, rounded and clamped; written as u8 (bd <= 8) or u16 LSB-aligned. */
int imop_scene_render(int width, int height, int bit_depth, int pattern, uint64_t seed, float lo,
                      float hi, float gain_dn_per_e, float read_sigma_dn, void* out);
/* Seeded distinct defect positions inside [2,w-2)x[2,h-2): first half hot, second half dead. */
int imop_scene_defects(int width, int height, uint64_t seed, int count, ImopDefectPoint* out);
/* Write hot (max) / dead (0) values at the listed positions of an unpacked frame. */
int imop_scene_apply_defects(void* frame, int width, int height, int bit_depth,
                             const ImopDefectPoint* pts, int count);
/* Pack an unpacked u16 frame as the packed input of that bit depth (MIPI RAW10 / RAW12, other
 * depths an LSB-first bit stream); out must hold imop_packed_bytes(). */
size_t imop_packed_bytes(int width, int height, int bit_depth);
int imop_pack_mipi(const uint16_t* in, int width, int height, int bit_depth, uint8_t* out);

/* ---- format sniffing of raw blobs of unknown layout (host) ---------------------------- */
/* The reference's analyzer heuristics (imop::analyze_data, detect_bit_depth, suggest_dimensions,
 * guess_pattern in src/analyzer.cpp), with the same results: storage bit depth from the byte
 * count against known resolutions and from value statistics, packed detection, candidate
 * dimensions, Bayer phase from 2x2 votes and channel means. */
#define IMOP_ANALYZE_MAX_DIMS 16
typedef struct {
    int detected_bit_depth;
    int suggested_width, suggested_height;
    int pixel_count;
    int max_value, min_value;
    int is_likely_16bit;
    int is_packed;
    int n_dims;                          /* candidate dimensions held in dims */
    int dims[IMOP_ANALYZE_MAX_DIMS][2];  /* (width, height), most likely first */
} ImopDataInfo;
int imop_analyze_data(const void* data, size_t bytes, ImopDataInfo* info);
int imop_detect_bit_depth(const void* data, size_t bytes);
/* Candidate (width, height) pairs of a pixel count: writes up to cap of them to out, returns how
 * many there are (-1: bad arguments). */
int imop_suggest_dimensions(size_t pixel_count, int (*out)[2], int cap);
/* IMOP_RGGB ... of a frame of known size and storage (RGGB when undecided). */
int imop_guess_pattern(const void* data, int width, int height, int bit_depth, int packed);

/* ---- colour-correction matrix from patch measurements (host) ------------------------- */
/* The reference's least-squares CCM solve (color_calibration::process_solve_ccm): per output
 * channel the normal equations over the patches plus 1e-9 on the diagonal, in FP64, Gaussian
 * elimination with partial pivoting; same results.  Layouts of PatchColor / SolvedMatrix. */
enum { IMOP_CCM_LINEAR_3X3 = 0, IMOP_CCM_LINEAR_4X3 = 1, IMOP_CCM_POLY_3X9 = 2 };
typedef struct {
    float r, g, b;
} ImopPatchColor;
typedef struct {
    int type;     /* IMOP_CCM_* */
    float m[27];  /* row-major rows x cols, zeros past the used entries */
    int rows;     /* 3 */
    int cols;     /* 3, 4 or 9 */
} ImopSolvedMatrix;
int imop_solve_ccm(const ImopPatchColor* measured, const ImopPatchColor* reference, int n, int type,
                   ImopSolvedMatrix* out);

/* ---- baseline JPEG encode of RGB8 frames (device) ------------------------------------- */
/* Byte for byte the output of jpeg_codec::process_encode_baseline (src/jpeg_codec/
 * encode_baseline.cpp:222-376): JFIF 1.02 header, standard Annex K quantiser scaled by quality and
 * Huffman tables, 4:4:4 / 4:2:0 / 4:2:2 (subsample 0 / 1 / 2, clamped), the reference's float
 * colour conversion, DCT and quantisation, and its run-length coding.  Replaces
 * jpeg_codec::process_encode_cuda (src/jpeg_codec/cuda_dispatch.cpp:121-240) and, on a CUDA host,
 * process_encode_baseline.  Status codes of these entry points are jpeg_codec::JpegError
 * (include/jpeg_codec/types.hpp:15-29), checked in the reference's order. */
enum {
    IMOP_JPEG_OK = 0,
    IMOP_JPEG_NULL_INPUT = 1,
    IMOP_JPEG_NULL_OUTPUT = 2,
    IMOP_JPEG_INVALID_DIMENSIONS = 3,
    IMOP_JPEG_INVALID_BIT_DEPTH = 4, /* only 8 */
    IMOP_JPEG_INVALID_CHANNELS = 5,
    IMOP_JPEG_INVALID_QUALITY = 6,   /* 1..100 */
    IMOP_JPEG_IMAGE_TOO_SMALL = 7,   /* below 8x8 */
    IMOP_JPEG_ENCODE_FAILED = 8,
    IMOP_JPEG_DECODE_FAILED = 9,
    IMOP_JPEG_INVALID_DATA = 10,
    IMOP_JPEG_CUDA_NOT_AVAILABLE = 11,
    IMOP_JPEG_INTERNAL_ERROR = 12
};
typedef struct imop_jpeg_ctx* imop_jpeg_t;
/* A context owns the device scratch of two encodes in flight (grown on demand) and two internal
 * streams; it serves the device that was current when it was created.  Calls on one context are
 * ordered: do not run it on two caller streams at once. */
int imop_jpeg_create(imop_jpeg_t* out_ctx);
int imop_jpeg_destroy(imop_jpeg_t ctx);
/* jpeg_codec::get_max_jpeg_size (src/jpeg_codec/dispatch.cpp:35-41): w*h*9 + 65536 */
size_t imop_jpeg_max_bytes(int width, int height);
/* The header (SOI .. SOS) of an encode; copies up to cap bytes to out (when non-NULL) and
 * returns its full length. */
int imop_jpeg_header(int width, int height, int quality, int subsample, uint8_t* out, size_t cap);
/* Host RGB8 (h x w x 3, interleaved) in, JPEG bytes out.  *out_size: capacity on entry (0: the
 * default capacity), bytes written on return (min(JPEG size, capacity); the bytes past the
 * capacity are dropped, as the reference's writer drops them). */
int imop_jpeg_encode_host(imop_jpeg_t ctx, const uint8_t* rgb, int width, int height, int bit_depth, int quality,
                          int subsample, uint8_t* out, size_t* out_size);
/* Device RGB8 in, the whole JPEG written to device memory d_out[0 .. min(size, out_cap)) on
 * `stream` (a cudaStream_t; NULL = legacy default stream) without a host synchronisation.
 * d_out_size (device pointer, may be NULL) receives the bytes written when the stream reaches
 * it; imop_jpeg_last_size reads the sizes on the host (synchronising the stream). */
int imop_jpeg_encode_device(imop_jpeg_t ctx, const void* d_rgb, int width, int height, int bit_depth, int quality,
                            int subsample, void* d_out, size_t out_cap, size_t* d_out_size, void* stream);
/* Frames encoded back to back on two internal streams (the tail kernels of one frame overlap the
 * next frame's transform); they start when `stream` reaches the call and `stream` continues after
 * the last.  Every frame is validated first; nothing runs when one is invalid. */
typedef struct {
    const void* d_rgb;            /* h x w x 3 RGB8 in device memory */
    int width, height, quality, subsample;
    void* d_out;                  /* device output, out_cap bytes (0: the default capacity) */
    size_t out_cap;
    size_t* d_out_size;           /* device size_t receiving the bytes written, or NULL */
} ImopJpegFrame;
int imop_jpeg_encode_device_batch(imop_jpeg_t ctx, const ImopJpegFrame* frames, int n, void* stream);
/* Host frames with the copies overlapped: frame k's input copy and kernels run while frame k-1's
 * bytes come back.  Synchronous; each frame gets its own status and size; returns the first
 * non-zero status. */
typedef struct {
    const uint8_t* rgb;           /* h x w x 3 RGB8 (page-locked memory lets the copies overlap) */
    int width, height, quality, subsample;
    uint8_t* out;
    size_t out_cap;               /* 0: the default capacity */
    size_t out_size;              /* out: bytes written */
    int status;                   /* out: JpegError value */
} ImopJpegHostFrame;
int imop_jpeg_encode_host_batch(imop_jpeg_t ctx, ImopJpegHostFrame* frames, int n);
int imop_jpeg_last_size(imop_jpeg_t ctx, size_t* jpeg_bytes, size_t* written);
const char* imop_jpeg_last_error_string(void);

/* ---- RAW host frames to JPEG host bytes ----------------------------------------------- */
/* The two drop-ins chained without the RGB8 frame leaving the device: the bytes of
 * imop_isp_run_host followed by imop_jpeg_encode_host on its output, for every frame.  Frames
 * go in chunks (up to 4 frames, about 25 Mpix; the first half as large) through one fused
 * batch launch and one encoder device batch each; the raw copies of the next chunk and the JPEG
 * copies of the previous one overlap them.  The parameters must select IMOP_OUT_RGB8.  Every frame is validated first
 * (nothing runs when one is invalid); synchronous; returns an IMOP_ERR_* status, the device
 * status of the ISP (as imop_isp_sync_status) included. */
typedef struct {
    const ImopIspParams* params;  /* this frame's parameters; NULL = the ISP context's */
    const void* raw;              /* host input frame (page-locked memory lets the copies overlap) */
    int quality, subsample;       /* as imop_jpeg_encode_host */
    uint8_t* out;                 /* host JPEG bytes */
    size_t out_cap;               /* 0: the default capacity (imop_jpeg_max_bytes) */
    size_t out_size;              /* out: bytes written, min(JPEG size, capacity) */
} ImopRawJpegFrame;
int imop_isp_run_host_jpeg_batch(imop_isp_t isp, imop_jpeg_t jpeg, ImopRawJpegFrame* frames, int n);

/* ---- misc --------------------------------------------------------------------------- */
const char* imop_last_error_string(void);
int imop_abi_version(void);
/* 1 when a CUDA device is visible (cached, like has_cuda_shared in src/gpu_dispatch.cpp:37-43). */
int imop_has_cuda(void);
/* the current device's name ("" without a device) */
const char* imop_device_name(void);
/* Calls of the reference-named GPU glue (include/imop_ref_shims.hpp) that this process ran on the
 * device and that returned Ok: a reference dispatcher linked against this library falls back to
 * its CPU code silently on any other status, so this count tells an integrator which one ran. */
long long imop_shim_calls_served(void);
/* Fused-kernel launches this process enqueued, by kernel: the tile kernel (every chain, and the
 * border rows / columns of streamed frames), the light-chain kernel (HQLI without defect
 * correction or lens shading; both of its variants), the streaming kernel (the interior of AMAZE
 * frames) and, counted again on its own, the light-chain kernel's direct-read variant (frames
 * whose rows start on a 4-byte word).  A launch recorded into a CUDA graph counts once, when
 * it is recorded. */
enum { IMOP_KERNEL_TILE = 0, IMOP_KERNEL_LITE = 1, IMOP_KERNEL_STREAM = 2, IMOP_KERNEL_LITE_DIRECT = 3 };
long long imop_kernel_launches(int kernel);

/* ---- launch tuning ------------------------------------------------------------------ */
/* Launch parameters of the two streamed kernels per (kernel, input format, width class), measured
 * by the tuner (imop_gb300.tuning) and loaded by the caller.  For a launch the first entry whose
 * kernel matches, whose fmt matches (or is -1) and whose max_width is at least the widest frame of
 * the launch applies; with none, the built-in defaults (enabled, 16-row bands for the light-chain
 * kernel, 32-row bands and 100 % segments for the streaming kernel).  A launch recorded into a
 * graph keeps the parameters it was recorded with. */
typedef struct ImopTuneEntry {
    int kernel;      /* IMOP_KERNEL_LITE or IMOP_KERNEL_STREAM */
    int fmt;         /* input format: 0 u8, 1 u16, 2 MIPI RAW10, 3 MIPI RAW12; -1 any */
    int max_width;   /* frames up to this many columns */
    int enabled;     /* 0: frames of this class take the tile kernel instead */
    int band_rows;   /* rows of a band: the light-chain kernel's unit, the streaming kernel's claim */
    int seg_percent; /* streaming kernel: rows of a segment, in percent of the launch's strip rows
                        spread evenly over the resident warps */
} ImopTuneEntry;
/* replaces the table (n = 0 clears it); IMOP_ERR_INVALID_ARGUMENT for an entry out of range */
int imop_tuning_set(const ImopTuneEntry* entries, int n);
/* copies up to cap entries of the table to out; returns the table's length */
int imop_tuning_get(ImopTuneEntry* out, int cap);

#ifdef __cplusplus
}
#endif
#endif /* IMOP_ISP_H */
