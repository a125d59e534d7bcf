// isp_fused.cu - the fused RAW->RGB kernel for sm_103a, its defect-chain fix-up and the
// small set-up kernels it needs (tone table, map-mode defect resolution).
//
// Defect correction has raster-sequential, in-place semantics in the reference
// (src/defect_correct/adaptive.cpp:25-57): a pixel sees the corrected values of its four
// raster-earlier same-colour neighbours.  The fused kernel evaluates every pixel against the
// uncorrected mosaic (Jacobi) and flags the pixels where the difference matters: a pixel p is a
// seed when one of its earlier neighbours was corrected and re-evaluating p against those
// corrections changes p.  If no pixel is a seed the Jacobi result is the sequential result
// (the first raster pixel where they differ would be a seed).  Seeds are rare (two defects
// within one same-colour 5x5 window); the fix-up kernel re-resolves them in raster order with a
// min-heap, propagating to later neighbours while values keep changing, and re-renders the
// output windows around every pixel whose value differs from the Jacobi one.

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <vector>

#include "imop_isp.h"
#include "isp_kernels.h"
#include "isp_dpc.cuh"
#include "isp_fused_kernel.cuh"
#include "isp_tile.cuh"

namespace imop {

// ---------------------------------------------------------------------------------------------
// tone table: tone8[v] = clamp((int)(f(v)*255 + 0.5), 0, 255) for v in [0, 2^bd)
__global__ void tone_table_kernel(int mode, const float* lut, const float* knots, int bd, uint8_t* out) {
    int mvi = max_val_of(bd);
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v > mvi) return;
    float mv = (float)mvi;
    float t;
    if (mode == 1) {
        t = lut[v];
    } else if (mode == 2) {
        // curves_3point lerp rule (src/tone/curves_3point.cpp:128-134) over 33 knots
        float norm = __fdiv_rn((float)v, mv);
        float fi = dev::fmul(norm, 32.0f);
        int idx = dev::ftoi(fi);
        float frac = dev::fsub(fi, (float)idx);
        if (idx > 31) { idx = 31; frac = 1.0f; }
        t = dev::fadd(dev::fmul(knots[idx], dev::fsub(1.0f, frac)), dev::fmul(knots[idx + 1], frac));
    } else {
        t = __fdiv_rn((float)v, mv);
    }
    int q = dev::ftoi(dev::fadd(dev::fmul(t, 255.0f), 0.5f));
    out[v] = (uint8_t)dev::clampi(q, 0, 255);
}

// Defect-chain fix-up (adaptive mode) in two launches: the raster-order resolution, one warp
// per frame, then the re-rendering of the output windows around every changed pixel, spread
// over kRenderCtas CTAs per frame.  Windows may overlap; overlapping windows write identical
// values.
constexpr int kRenderCtas = 16;

constexpr int kResolveHeap = 6144, kResolveOv = 3072;  // shared-memory entries (48 KB)

__global__ void __launch_bounds__(32) dpc_resolve_kernel(const __grid_constant__ BatchLaunch bl) {
    __shared__ int heap[kResolveHeap], ov_idx[kResolveOv], ov_val[kResolveOv];
    const FrameParams& fp = bl.frames[blockIdx.x];
    if (!((fp.stages & 2u) && fp.dpc_mode == 0)) return;
    int n_ov = 0;
    if (*fp.seed_count > 0) {
        const FixupScratch fs{fp.fix_heap, fp.fix_ov_idx, fp.fix_ov_val, fp.fix_n_ov, fp.fix_cap};
        GlobalOrig orig{&fp, pattern_offsets(fp.pattern)};
        n_ov = resolve_chains_warp_smem(fp, orig, fs, heap, kResolveHeap, ov_idx, ov_val, kResolveOv);
        if (n_ov < 0) n_ov = resolve_chains_warp(fp, orig, fs);  // more chains than shared memory holds
    }
    if (threadIdx.x == 0) *fp.fix_n_ov = n_ov;
}

template <int TW, int TH, int OUTB>
__global__ void __launch_bounds__(kThreads) dpc_render_kernel(const __grid_constant__ BatchLaunch bl) {
    extern __shared__ __align__(16) uint8_t dsm[];
    auto& sm = *reinterpret_cast<TileSmem<TW, TH, OUTB>*>(dsm);
    const int f = blockIdx.x / kRenderCtas, part = blockIdx.x - f * kRenderCtas;
    const FrameParams& gfp = bl.frames[f];
    if (!((gfp.stages & 2u) && gfp.dpc_mode == 0)) return;
    const int n_ov = *gfp.fix_n_ov;
    if (part >= n_ov) return;
    tile_init(sm);
    if (threadIdx.x < 32) {
        const int* s = reinterpret_cast<const int*>(&gfp);
        int* d = reinterpret_cast<int*>(&sm.fp[0]);
        for (int k = threadIdx.x; k < (int)(sizeof(FrameParams) / 4); k += 32) d[k] = s[k];
    }
    __syncthreads();
    const Overrides ov{gfp.fix_ov_idx, gfp.fix_ov_val, n_ov};
    uint32_t parity = 0;
    // the output window around a changed pixel: radius 3 of demosaic support plus 2 of border
    // copies, started on an even column
    for (int k = part; k < n_ov; k += kRenderCtas) {
        const int p = gfp.fix_ov_idx[k];
        const int x = p % gfp.w, y = p / gfp.w;
        const int wx0 = max(0, (x - 5) & ~1), wx1 = min(gfp.w, x + 6);
        const int wy0 = max(0, y - 5), wy1 = min(gfp.h, y + 6);
        if (!process_tile_sync<TW, TH, OUTB>(sm, wx0, wy0, wx1 - wx0, wy1 - wy0, ov, parity)) return;
    }
}

// ---------------------------------------------------------------------------------------------
// map-mode defect resolution: one thread per component of mutually neighbouring map pixels,
// entries applied in map order (src/defect_correct/map_based.cpp:17-43)
__global__ void dpc_map_resolve_kernel(const __grid_constant__ FrameParams fp, MapPlan plan) {
    int comp = blockIdx.x * blockDim.x + threadIdx.x;
    if (comp >= plan.n_comp) return;
    PatternOffsets po = pattern_offsets(fp.pattern);
    int* val = const_cast<int*>(fp.map_val);
    for (int i = plan.comp_slot_ptr[comp]; i < plan.comp_slot_ptr[comp + 1]; i++) {
        int s = plan.comp_slots[i];
        int2 xy = plan.slot_xy[s];
        val[s] = dev::orig_value(fp, xy.x, xy.y, po);
    }
    for (int i = plan.comp_ent_ptr[comp]; i < plan.comp_ent_ptr[comp + 1]; i++) {
        int s = plan.comp_entries[i];
        int2 xy = plan.slot_xy[s];
        unsigned m = dev::dpc_valid_mask(xy.x, xy.y, fp.w, fp.h);
        int nb[8];
        for (int k = 0; k < 8; k++) {
            int dx, dy;
            nb_offsets(k, dx, dy);
            int v = 0;
            if ((m >> k) & 1u) {
                int nx = xy.x + dx, ny = xy.y + dy;
                int mvv = map_lookup(fp, nx, ny);
                v = mvv >= 0 ? mvv : dev::orig_value(fp, nx, ny, po);
            }
            nb[k] = v;
        }
        if (m) {
            int n;
            val[s] = dev::dpc_median8(nb, m, n);
        }
    }
}

// ---------------------------------------------------------------------------------------------
// host launchers

int fused_tile_grid(int w, int h, int& ntx, int& nty) {
    ntx = tiles_along(w, kTileW);
    nty = tiles_along(h, kTileH);
    return ntx * nty;
}

cudaError_t launch_tone_table(int mode, const float* d_lut, const float* d_knots, int bd, uint8_t* d_out,
                              cudaStream_t st) {
    int n = max_val_of(bd) + 1;
    tone_table_kernel<<<(n + 255) / 256, 256, 0, st>>>(mode, d_lut, d_knots, bd, d_out);
    return cudaGetLastError();
}

cudaError_t launch_map_resolve(const FrameParams& fp, const MapPlan& plan, cudaStream_t st) {
    if (!fp.in) return cudaErrorInvalidValue;  // the resolved values are read from the input frame
    if (plan.n_comp > 0) dpc_map_resolve_kernel<<<(plan.n_comp + 127) / 128, 128, 0, st>>>(fp, plan);
    return cudaGetLastError();
}

cudaError_t launch_fused_spec_u8(int dm, bool lite, const BatchLaunch& bl, int grid, size_t smem, cudaStream_t st);
cudaError_t launch_fused_spec_u16(int dm, bool lite, const BatchLaunch& bl, int grid, size_t smem, cudaStream_t st);
cudaError_t launch_fused_spec_p10(int dm, bool lite, const BatchLaunch& bl, int grid, size_t smem, cudaStream_t st);
cudaError_t launch_fused_spec_p12(int dm, bool lite, const BatchLaunch& bl, int grid, size_t smem, cudaStream_t st);

cudaError_t launch_fused_spec(int fmt, int dm, bool lite, const BatchLaunch& bl, int grid, size_t smem,
                              cudaStream_t st) {
    switch (fmt) {
        case FMT_U8: return launch_fused_spec_u8(dm, lite, bl, grid, smem, st);
        case FMT_U16: return launch_fused_spec_u16(dm, lite, bl, grid, smem, st);
        case FMT_P10: return launch_fused_spec_p10(dm, lite, bl, grid, smem, st);
        case FMT_P12: return launch_fused_spec_p12(dm, lite, bl, grid, smem, st);
        default: return cudaErrorInvalidValue;
    }
}

namespace {

constexpr int kMaxDevices = 64;

template <int OUTB>
struct FusedKernels {
    static constexpr size_t smem = sizeof(TileSmem<kTileW, kTileH, OUTB>);
    // 0: every format, stage and algorithm; 1..3: no bit stream / 3D LUT, one demosaic algorithm
    static void (*kernel(int k))(BatchLaunch) {
        switch (k) {
            case 1: return fused_batch_kernel<kTileW, kTileH, OUTB, false, DM_HQLI, 0>;
            case 2: return fused_batch_kernel<kTileW, kTileH, OUTB, false, DM_MG, 0>;
            case 3: return fused_batch_kernel<kTileW, kTileH, OUTB, false, DM_AMAZE, 0>;
            default: return fused_batch_kernel<kTileW, kTileH, OUTB, true, 0, 0>;
        }
    }
    static int variant(const BatchLaunch& bl) {
        if (bl.extra) return 0;
        return bl.demosaic == DM_HQLI ? 1 : bl.demosaic == DM_MG ? 2 : bl.demosaic == DM_AMAZE ? 3 : 0;
    }
    // dynamic shared memory opt-in and resident CTAs per SM, once per device
    static int ctas_per_sm[kMaxDevices];
    static int sms[kMaxDevices];
    static cudaError_t setup(int& grid_limit) {
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return e;
        if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
        std::lock_guard<std::mutex> lock(device_setup_mutex());
        if (!ctas_per_sm[dev]) {
            for (int k = 0; k < 4 && e == cudaSuccess; k++)
                e = cudaFuncSetAttribute(kernel(k), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e == cudaSuccess)
                e = cudaFuncSetAttribute(dpc_render_kernel<kTileW, kTileH, OUTB>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            int n = 0, m = 0;
            if (e == cudaSuccess)
                e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel(0), kThreads, smem);
            if (e == cudaSuccess) e = cudaDeviceGetAttribute(&m, cudaDevAttrMultiProcessorCount, dev);
            if (e != cudaSuccess) return e;
            sms[dev] = m;
            ctas_per_sm[dev] = n > 0 ? n : 1;
        }
        grid_limit = sms[dev] * ctas_per_sm[dev];
        return cudaSuccess;
    }
    static cudaError_t launch(const BatchLaunch& bl, bool fixup, cudaStream_t st, const SplitFixup* split) {
        int limit = 0;
        cudaError_t e = setup(limit);
        if (e != cudaSuccess) return e;
        if (bl.n_items > 0) {
            if (!bl.dependent && (e = cudaMemsetAsync(bl.tile_counter, 0, sizeof(int), st)) != cudaSuccess) return e;
            const int grid = bl.n_items < limit ? bl.n_items : limit;
            count_launch(0);
            if (OUTB == 3 && bl.simple && !bl.extra && bl.demosaic && bl.fmt >= FMT_U8 && bl.fmt <= FMT_P12) {
                if ((e = launch_fused_spec(bl.fmt, bl.demosaic, bl.no_dpc_lsc != 0, bl, grid, smem, st)) != cudaSuccess)
                    return e;
            } else if (bl.dependent) {
                if ((e = launch_dependent(kernel(variant(bl)), grid, kThreads, smem, st, bl)) != cudaSuccess) return e;
            } else {
                kernel(variant(bl))<<<grid, kThreads, smem, st>>>(bl);
            }
        }
        cudaStream_t fst = st;
        if (split) {
            // the fix-up follows the tile kernel on its own stream
            if ((e = cudaEventRecord(split->main_done, st)) != cudaSuccess ||
                (e = cudaStreamWaitEvent(split->st, split->main_done, 0)) != cudaSuccess)
                return e;
            fst = split->st;
        }
        if (fixup) {
            dpc_resolve_kernel<<<bl.n_frames, 32, 0, fst>>>(bl);
            if (!(split && split->defer_render))
                dpc_render_kernel<kTileW, kTileH, OUTB><<<bl.n_frames * kRenderCtas, kThreads, smem, fst>>>(bl);
        }
        return cudaGetLastError();
    }
    static cudaError_t render(const BatchLaunch& bl, cudaStream_t st) {
        int limit = 0;
        cudaError_t e = setup(limit);
        if (e != cudaSuccess) return e;
        dpc_render_kernel<kTileW, kTileH, OUTB><<<bl.n_frames * kRenderCtas, kThreads, smem, st>>>(bl);
        return cudaGetLastError();
    }
};
template <int OUTB> int FusedKernels<OUTB>::ctas_per_sm[kMaxDevices] = {};
template <int OUTB> int FusedKernels<OUTB>::sms[kMaxDevices] = {};

void add_rect(BatchLaunch& bl, int frame, int x0, int y0, int w, int h, int& items, int tw = kTileW, int th = kTileH) {
    TileRect& R = bl.rects[bl.n_rects];
    R.frame = frame;
    R.x0 = x0;
    R.y0 = y0;
    R.w = w;
    R.h = h;
    R.tiles_x = tiles_along(w, tw);
    R.tiles_y = tiles_along(h, th);
    bl.rect_start[bl.n_rects] = items;
    items += R.tiles_x * R.tiles_y;
    bl.n_rects++;
}

// the launch block of frames[0..n): tile counts, one rectangle per frame; false when the frames do
// not share one tile counter
bool make_launch(FrameParams* frames, int n, BatchLaunch& bl, bool& fixup) {
    bl.n_frames = n;
    bl.n_rects = 0;
    bl.extra = 0;
    bl.demosaic = 0;
    bl.fmt = -1;
    bl.simple = 1;
    bl.no_dpc_lsc = 1;
    // the frames of one launch come from one context and share its counter
    bl.tile_counter = frames[0].tile_counter;
    for (int f = 0; f < n; f++)
        if (!frames[f].tile_counter || frames[f].tile_counter != bl.tile_counter) return false;
    int items = 0;
    fixup = false;
    for (int f = 0; f < n; f++) {
        FrameParams& fp = frames[f];
        fp.tiles_x = tiles_along(fp.w, kTileW);
        fp.tiles_y = tiles_along(fp.h, kTileH);
        bl.frames[f] = fp;
        if (fp.fmt == FMT_PBITS || (fp.stages & 32u)) bl.extra = 1;
        if (f == 0) bl.demosaic = fp.demosaic, bl.fmt = fp.fmt;
        if (fp.demosaic != bl.demosaic) bl.demosaic = 0;
        if (fp.fmt != bl.fmt) bl.fmt = -1;
        // the stage configuration the per-format kernels fix at compile time
        const bool simple = (!(fp.stages & 2u) || fp.dpc_mode == 0) && (!(fp.stages & 4u) || fp.lsc_mode != 1) &&
                            fp.out_format == 0 && fp.out_bpc == 1;
        if (!simple) bl.simple = 0;
        if (fp.stages & 6u) bl.no_dpc_lsc = 0;
        fixup |= (fp.stages & 2u) && fp.dpc_mode == 0;
        add_rect(bl, f, 0, 0, fp.w, fp.h, items);
    }
    bl.rect_start[bl.n_rects] = items;
    bl.n_items = items;
    return true;
}

// the launch block of frames[0..n) for the light-chain kernel: one rectangle per frame in its units
bool make_lite_launch(FrameParams* frames, int n, BatchLaunch& bl, int band_rows) {
    bool fixup = false;
    if (!make_launch(frames, n, bl, fixup)) return false;
    bl.band_h = band_rows;
    int items = 0;
    for (int f = 0; f < n; f++) {
        TileRect& R = bl.rects[f];
        R.tiles_x = lite_units_x(R.w);
        R.tiles_y = lite_units_y(R.h, band_rows);
        bl.rect_start[f] = items;
        items += R.tiles_x * R.tiles_y;
    }
    bl.rect_start[bl.n_rects] = items;
    bl.n_items = items;
    return true;
}

cudaError_t launch_batch_group(FrameParams* frames, int n, cudaStream_t st, const SplitFixup* split = nullptr) {
    BatchLaunch bl;
    bool fixup = false;
    // the light-chain kernel takes frames of one input format that share their output tables
    int wmax = 0;
    for (int f = 0; f < n; f++) wmax = std::max(wmax, frames[f].w);
    const TuneParams tl = tuning_for(IMOP_KERNEL_LITE, frames[0].fmt, wmax);
    bool lite = tl.enabled;
    for (int f = 0; f < n; f++)
        lite = lite && lite_eligible(frames[f]) && frames[f].fmt == frames[0].fmt &&
               lite_table_key(frames[f]) == lite_table_key(frames[0]);
    if (lite) {
        if (!make_lite_launch(frames, n, bl, tl.band_rows)) return cudaErrorInvalidValue;
        cudaError_t e = launch_lite(bl, st);
        // no defect chains to resolve: a split caller's fix-up stream only waits for the tiles
        if (e == cudaSuccess && split) {
            if ((e = cudaEventRecord(split->main_done, st)) == cudaSuccess) e = cudaStreamWaitEvent(split->st, split->main_done, 0);
        }
        return e;
    }
    // the AMAZE chains: the interior of every frame by the streaming kernel, then the border rows
    // and columns by the tile kernel (its launch also runs the defect-chain fix-up of the frames)
    bool stream = tuning_for(IMOP_KERNEL_STREAM, frames[0].fmt, wmax).enabled;
    for (int f = 0; f < n; f++)
        stream = stream && stream_eligible(frames[f]) && frames[f].fmt == frames[0].fmt &&
                 frames[f].tone8 == frames[0].tone8 && frames[f].seg_words == frames[0].seg_words;
    if (!make_launch(frames, n, bl, fixup)) return cudaErrorInvalidValue;
    if (stream) {
        // interior: the streaming kernel; border columns: the narrow tile; border rows: the nominal
        // tile; then the fix-up
        BatchLaunch bs = bl, bn = bl;
        int items_s = 0, items_n = 0, items_b = 0;
        bs.n_rects = bn.n_rects = bl.n_rects = 0;
        for (int f = 0; f < n; f++) {
            TileRect in, border[4];
            stream_rects(frames[f], in, border);
            in.frame = f;
            bs.rects[bs.n_rects] = in;
            bs.rect_start[bs.n_rects++] = items_s;
            items_s += in.tiles_x * in.tiles_y;
            for (int k = 0; k < 2; k++) add_rect(bl, f, border[k].x0, border[k].y0, border[k].w, border[k].h, items_b);
            for (int k = 2; k < 4; k++)
                add_rect(bn, f, border[k].x0, border[k].y0, border[k].w, border[k].h, items_n, kNarrowW, kNarrowH);
        }
        bs.rect_start[bs.n_rects] = bs.n_items = items_s;
        bs.seg_words = frames[0].seg_words;
        bn.rect_start[bn.n_rects] = bn.n_items = items_n;
        bl.rect_start[bl.n_rects] = bl.n_items = items_b;
        // the column launch counts its tiles in the last claim word, which the streaming launch
        // leaves alone; the streaming launch's init kernel zeroes both border counters, and the
        // border launches are programmatic dependents in the same stream: they start beside the
        // streaming kernel once its CTAs run (and the init kernel is complete), on the SMs its
        // CTAs leave at the end.  The fix-up, launched the ordinary way, waits for all three.
        bn.tile_counter = reinterpret_cast<int*>(frames[0].seg_words + (kStreamSegCap - 1));
        bn.dependent = bl.dependent = 1;
        cudaError_t e = launch_stream(bs, st);
        if (e == cudaSuccess) e = launch_fused_narrow(bn, st);
        if (e == cudaSuccess)
            e = frames[0].out_bpc == 2 ? FusedKernels<6>::launch(bl, false, st, nullptr)
                                       : FusedKernels<3>::launch(bl, false, st, nullptr);
        if (e != cudaSuccess) return e;
        BatchLaunch bf = bl;
        bf.n_items = 0;
        bf.dependent = 0;
        return frames[0].out_bpc == 2 ? FusedKernels<6>::launch(bf, fixup, st, split)
                                      : FusedKernels<3>::launch(bf, fixup, st, split);
    }
    return frames[0].out_bpc == 2 ? FusedKernels<6>::launch(bl, fixup, st, split)
                                  : FusedKernels<3>::launch(bl, fixup, st, split);
}

FrameParams with_fixup(const FrameParams& fp_in, const FixupScratch& fs) {
    FrameParams fp = fp_in;
    fp.fix_heap = fs.heap;
    fp.fix_ov_idx = fs.ov_idx;
    fp.fix_ov_val = fs.ov_val;
    fp.fix_n_ov = fs.n_ov;
    fp.fix_cap = fs.cap;
    return fp;
}

}  // namespace

std::mutex& device_setup_mutex() {
    static std::mutex m;
    return m;
}

static std::atomic<long long> g_launches[4];
void count_launch(int kernel) { g_launches[kernel].fetch_add(1, std::memory_order_relaxed); }

extern "C" long long imop_kernel_launches(int kernel) {
    return (kernel >= 0 && kernel < 4) ? g_launches[kernel].load(std::memory_order_relaxed) : -1;
}

int fused_grid_limit(int out_bpc) {
    int limit = 0;
    cudaError_t e = out_bpc == 2 ? FusedKernels<6>::setup(limit) : FusedKernels<3>::setup(limit);
    return e == cudaSuccess ? limit : 0;
}

// which kernel instantiation a frame can use: frames with equal keys share the most specialised
// one (output channel width, bit-stream / 3D-LUT paths, demosaic algorithm, stage set, format)
static long long instantiation_key(const FrameParams& fp) {
    const bool extra = fp.fmt == FMT_PBITS || (fp.stages & 32u);
    const bool simple = (!(fp.stages & 2u) || fp.dpc_mode == 0) && (!(fp.stages & 4u) || fp.lsc_mode != 1) &&
                        fp.out_format == 0 && fp.out_bpc == 1;
    if (extra) return (long long)fp.out_bpc << 32;
    // the light-chain kernel: one launch per input format and output table set
    if (lite_eligible(fp) && tuning_for(IMOP_KERNEL_LITE, fp.fmt, fp.w).enabled)
        return (1LL << 62) | ((long long)fp.fmt << 56) | (lite_table_key(fp) & ((1LL << 56) - 1));
    // the streaming kernel: one launch per input format and tone table
    if (stream_eligible(fp) && tuning_for(IMOP_KERNEL_STREAM, fp.fmt, fp.w).enabled)
        return (1LL << 61) | ((long long)fp.fmt << 56) | (stream_table_key(fp) & ((1LL << 56) - 1));
    const bool lite = simple && !(fp.stages & 6u);
    return ((long long)fp.out_bpc << 32) | (1LL << 24) | ((long long)fp.demosaic << 16) | (simple ? (1 << 8) : 0) |
           (lite ? (1 << 12) : 0) | (simple ? fp.fmt + 1 : 0);
}

cudaError_t launch_fused_batch(FrameParams* frames, int n, cudaStream_t st) {
    // frames grouped by instantiation (stable: frames keep their order inside a group), then one
    // launch per run of at most kBatchInline frames of a group
    std::vector<int> order(n);
    for (int i = 0; i < n; i++) order[i] = i;
    std::vector<long long> key(n);
    for (int i = 0; i < n; i++) key[i] = instantiation_key(frames[i]);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return key[a] < key[b]; });
    std::vector<FrameParams> grouped(n);
    for (int i = 0; i < n; i++) grouped[i] = frames[order[i]];
    int i = 0;
    while (i < n) {
        int j = i + 1;
        while (j < n && j - i < kBatchInline && key[order[j]] == key[order[i]]) j++;
        cudaError_t e = launch_batch_group(grouped.data() + i, j - i, st);
        if (e != cudaSuccess) return e;
        i = j;
    }
    return cudaSuccess;
}

cudaError_t launch_fused(const FrameParams& fp_in, const FixupScratch& fs, const MapPlan* plan, cudaStream_t st,
                         const SplitFixup* split) {
    FrameParams fp = with_fixup(fp_in, fs);
    if ((fp.stages & 2u) && fp.dpc_mode == 1 && plan) {
        cudaError_t e = launch_map_resolve(fp, *plan, st);
        if (e != cudaSuccess) return e;
    }
    if ((fp.stages & 2u) && fp.dpc_mode == 0) {
        cudaError_t e = cudaMemsetAsync(fp.seed_count, 0, sizeof(int), st);
        if (e != cudaSuccess) return e;
    }
    return launch_batch_group(&fp, 1, st, split);
}

cudaError_t launch_fused_render(const FrameParams& fp_in, const FixupScratch& fs, uint8_t* out, cudaStream_t st) {
    FrameParams fp = with_fixup(fp_in, fs);
    fp.out = out;
    BatchLaunch bl;
    bool fixup = false;
    if (!make_launch(&fp, 1, bl, fixup)) return cudaErrorInvalidValue;
    if (!fixup) return cudaSuccess;
    return fp.out_bpc == 2 ? FusedKernels<6>::render(bl, st) : FusedKernels<3>::render(bl, st);
}

}  // namespace imop
