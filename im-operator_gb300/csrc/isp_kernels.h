// isp_kernels.h - host-visible launchers of the CUDA kernels (no device code).
#pragma once

#include <cuda_runtime.h>

#include <mutex>

#include "isp_common.h"

namespace imop {

// nominal fused tile (the last tile of a row / column absorbs a remainder below 4)
constexpr int kTileW = 120;
constexpr int kTileH = 24;
// work-claim words of one streamed launch: a word per segment of its strips (at most kSegMax),
// then the count of segments taken; the last word counts the tiles of a streamed batch's
// border-column launch
constexpr int kStreamSegCap = 4096;
constexpr int kSegMax = kStreamSegCap - 2;
// narrow fused tile of the border columns of streamed frames (isp_fused_narrow.cu)
constexpr int kNarrowW = 16;
constexpr int kNarrowH = 128;

// Frames of one fused launch, passed by value as the kernel's parameter block.  The kernel walks
// the tiles of a list of rectangles (one per frame), rectangle after rectangle, tiles in raster
// order; CTAs claim tiles from a device counter, so border tiles (the general path) and
// partial tiles do not unbalance the CTAs.
constexpr int kBatchInline = 32;
constexpr int kMaxRects = 4 * kBatchInline;  // the border rectangles of a streamed batch
struct TileRect {
    int frame;
    int x0, y0, w, h;  // x0 even; w, h >= 4
    int tiles_x, tiles_y;
};
struct BatchLaunch {
    int n_frames;
    int n_items;
    int n_rects;
    int extra;                      // some frame reads a bit stream or applies a 3D LUT
    int demosaic;                   // the frames' common demosaic algorithm, 0 when they differ
    int fmt;                        // the frames' common input format, -1 when they differ
    int simple;                     // every frame has the common stage configuration (per-format kernels)
    int no_dpc_lsc;                 // no frame corrects defects or lens shading
    int* tile_counter;              // claims beyond the first gridDim.x items; zero at launch
    unsigned long long* seg_words;  // streaming kernel: per segment, bands claimed (front | back << 32)
    int band_h;                     // streamed kernels: rows of a band
    int owners = 0;                 // streamed kernels: segments below this start with band 0 claimed by their warp
    int dependent = 0;              // tile kernel: launched as a programmatic dependent, its counter already zero
    int rect_start[kMaxRects + 1];  // first item of each rectangle; rect_start[n_rects] = n_items
    TileRect rects[kMaxRects];
    FrameParams frames[kBatchInline];
};

// device scratch of the defect-chain fix-up
struct FixupScratch {
    int* heap;
    int* ov_idx;
    int* ov_val;
    int* n_ov;
    int cap;
};

// map-mode defect plan (built on the host from the defect list, uploaded once)
struct MapPlan {
    int n_comp;
    const int* comp_slot_ptr;  // n_comp + 1
    const int* comp_slots;     // unique slots of each component
    const int* comp_ent_ptr;   // n_comp + 1
    const int* comp_entries;   // slot of each map entry, in map order
    const int2* slot_xy;       // pixel of each slot
};

// guards the once-per-device kernel set-up (shared-memory opt-in, occupancy queries): the
// reference-named glue gives each host thread its own context, so first calls can come from
// several threads at once
std::mutex& device_setup_mutex();

// launches enqueued per fused kernel (IMOP_KERNEL_TILE / _LITE / _STREAM)
void count_launch(int kernel);

// launch parameters of a streamed kernel (1 light-chain, 2 streaming) for input format fmt and
// frames up to `width` columns, from the tuning table (imop_tuning_set) or the defaults
struct TuneParams {
    bool enabled;
    int band_rows;
    int seg_percent;
};
TuneParams tuning_for(int kernel, int fmt, int width);
// changes with every imop_tuning_set (part of the recorded-graph key)
int tuning_generation();

int fused_tile_grid(int w, int h, int& ntx, int& nty);
cudaError_t launch_tone_table(int mode, const float* d_lut, const float* d_knots, int bd, uint8_t* d_out,
                              cudaStream_t st);
// map-mode defect values of one frame (before the kernels that read them)
cudaError_t launch_map_resolve(const FrameParams& fp, const MapPlan& plan, cudaStream_t st);
// map resolve (map mode) + seed reset + fused tiles + fix-up, in stream order
// Optional second stream for the defect-chain fix-up of a single-frame launch: main_done is
// recorded after the tile kernel on the launch stream, and the fix-up kernels run on `st` after it,
// so the next frame's tile kernel can start while this frame's chains are resolved.  With
// defer_render only the chain resolution is enqueued; launch_fused_render enqueues the window
// re-rendering later (for example into a host frame, after the tile kernel's output was copied
// there).
struct SplitFixup {
    cudaStream_t st;
    cudaEvent_t main_done;
    bool defer_render;
};
cudaError_t launch_fused(const FrameParams& fp, const FixupScratch& fs, const MapPlan* plan, cudaStream_t st,
                         const SplitFixup* split = nullptr);
// the defect-chain window re-rendering of one frame (after launch_fused with defer_render), its
// windows written to `out`; nothing when the frame has no adaptive defect correction
cudaError_t launch_fused_render(const FrameParams& fp, const FixupScratch& fs, uint8_t* out, cudaStream_t st);
// Up to kBatchInline frames in one persistent launch plus the two fix-up launches (chain
// resolution, window re-rendering).  Each frame carries
// its own seed counter, seed list and fix-up scratch (FrameParams::fix_*); its seed counter must be
// zero and its map-mode values resolved when the launch runs.  tiles_x / tiles_y are filled in.
cudaError_t launch_fused_batch(FrameParams* frames, int n, cudaStream_t st);
// CTAs of the persistent fused kernel on the current device (SMs x resident CTAs per SM)
int fused_grid_limit(int out_bpc);

// light-chain kernel (isp_lite.cu): HQLI without defect correction, lens shading, CCM or 3D LUT,
// RGB8 out, bit depth <= 12, u8 / u16 / MIPI RAW10 / RAW12 input
bool lite_eligible(const FrameParams& fp);
// frames of one light-chain launch share this key (their output tables) and the input format
long long lite_table_key(const FrameParams& fp);
// units of work of a frame: strips across, bands down (a rectangle's tiles_x / tiles_y)
int lite_units_x(int w);
int lite_units_y(int h, int band_rows);
// one persistent launch over the units of bl's rectangles (bl.fmt: the frames' common format);
// frames 16-byte aligned with widths that are multiples of 8 and work-claim words take the
// direct-read variant, whose segments are chosen here
cudaError_t launch_lite(const BatchLaunch& bl, cudaStream_t st);
// Segments of the strips of bl's rectangles (tiles_x strips each): each strip cut into segments
// of seg_percent % of the rows that spread the launch's strip rows evenly over `warps` warps,
// at most kSegMax in all; bands of band_rows rows inside them (isp_segments.cuh).  False when
// the launch has more strips than kSegMax.
bool choose_segments(BatchLaunch& bl, int warps, int seg_percent, int band_rows);

// warp-streamed kernel for the AMAZE chains (isp_stream.cu): black level, adaptive defect
// correction, grid lens shading, Bayer-order white balance, AMAZE, CCM, tone -> RGB8 on the interior
// of each frame; u8 / u16 / MIPI RAW10 / RAW12 input, width a multiple of 8, bit depth <= 12
bool stream_eligible(const FrameParams& fp);
// frames of one streamed launch share this key (their tone table) and the input format
long long stream_table_key(const FrameParams& fp);
// the interior rectangle of a frame (tiles_x / tiles_y: strips and bands) and the four border
// rectangles (rows 0-6, rows h-7.., columns 0-7 and the right columns of the rows between) that the
// tile kernel takes
void stream_rects(const FrameParams& fp, TileRect& interior, TileRect (&border)[4]);
// the tile kernel over bl's rectangles in the narrow tile (AMAZE frames without a bit stream or
// 3D LUT; rectangles at most kNarrowW wide, tiles_x / tiles_y in that tile)
cudaError_t launch_fused_narrow(const BatchLaunch& bl, cudaStream_t st);
// one persistent launch over bl's interior rectangles (bl.fmt: the frames' common format); the
// band height, the same for every rectangle, is chosen here
cudaError_t launch_stream(const BatchLaunch& bl, cudaStream_t st);

// plain per-operator form: one kernel per stage over full frames in device memory.
// Buffers: bayer_a/bayer_b are w*h u16, rgb is w*h*3 u16.
struct PlainBuffers {
    uint16_t* bayer_a;
    uint16_t* bayer_b;
    uint16_t* rgb;
};
struct PlainDumps {  // device pointers, may be null
    uint16_t* unpacked;
    uint16_t* black_level;
    uint16_t* defect;
    uint16_t* lens_shading;
    uint16_t* white_balance;
    uint16_t* demosaic;
    uint16_t* ccm;
};
cudaError_t launch_plain(const FrameParams& fp, const FixupScratch& fs, const MapPlan* plan, const PlainBuffers& b,
                         const PlainDumps* dumps, cudaStream_t st);

// per-operator stages (the per-module drop-ins): u8 / u16-LE samples <-> u16 planes, one Bayer
// stage (1 black level, 2 defect correction, 4 lens shading) with its result back in `a`, one RGB
// stage (8 white balance, 16 CCM) in place
cudaError_t launch_widen(const uint8_t* in, uint16_t* out, size_t n, int bytes_per_sample, cudaStream_t st);
cudaError_t launch_narrow(const uint16_t* in, uint8_t* out, size_t n, int bytes_per_sample, cudaStream_t st);
cudaError_t launch_op_bayer(const FrameParams& fp, unsigned stage, const FixupScratch& fs, const MapPlan* plan,
                            uint16_t* a, uint16_t* b, cudaStream_t st);
cudaError_t launch_op_rgb(const FrameParams& fp, unsigned stage, uint16_t* rgb, cudaStream_t st);
// every one of n samples (u8 when bytes_per_sample is 1, u16 otherwise) through table, in -> out (may alias)
cudaError_t launch_table_map(const uint8_t* in, uint8_t* out, size_t n, int bytes_per_sample, const uint16_t* table,
                             cudaStream_t st);

}  // namespace imop
