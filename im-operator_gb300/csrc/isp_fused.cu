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

#include "isp_kernels.h"
#include "isp_dpc.cuh"
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

// rtab[k] = 1 / (1 + k), correctly rounded (the AMAZE weights 1.0f / (1.0f + gradient))
__global__ void recip_table_kernel(float* out, int n) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] = __frcp_rn((float)(1 + k));
}

// ---------------------------------------------------------------------------------------------
// one CTA per tile, tiles in raster order
template <int TW, int TH, int OUTB>
__global__ void __launch_bounds__(kThreads) fused_frame_kernel(const __grid_constant__ FrameParams fp, int ntx,
                                                               int nty) {
    extern __shared__ __align__(16) uint8_t dsm[];
    auto& sm = *reinterpret_cast<TileSmem<TW, TH, OUTB>*>(dsm);
    tile_init(sm);
    uint32_t parity = 0;
    int t = blockIdx.x;
    int tx = t % ntx, ty = t / ntx;
    int x0, tw, y0, th;
    tile_span(fp.w, TW, ntx, tx, x0, tw);
    tile_span(fp.h, TH, nty, ty, y0, th);
    process_tile<TW, TH, OUTB>(fp, x0, y0, tw, th, sm, Overrides{nullptr, nullptr, 0}, true, parity);
}

// defect-chain fix-up (adaptive mode), one CTA per frame
template <int TW, int TH, int OUTB>
__global__ void __launch_bounds__(kThreads) dpc_fixup_kernel(const __grid_constant__ FrameParams fp,
                                                             FixupScratch fs) {
    extern __shared__ __align__(16) uint8_t dsm[];
    auto& sm = *reinterpret_cast<TileSmem<TW, TH, OUTB>*>(dsm);
    __shared__ int s_nov;
    if (*fp.seed_count == 0) return;
    tile_init(sm);
    if (threadIdx.x == 0) {
        GlobalOrig orig{&fp, pattern_offsets(fp.pattern)};
        s_nov = resolve_chains(fp, orig, fs);
        *fs.n_ov = s_nov;
    }
    __syncthreads();
    const int n_ov = s_nov;
    Overrides ov{fs.ov_idx, fs.ov_val, n_ov};
    uint32_t parity = 0;
    // re-render the output window around each changed pixel: radius 3 of demosaic support plus
    // 2 of border copies, started on an even column
    for (int k = 0; k < n_ov; k++) {
        int p = fs.ov_idx[k];
        int x = p % fp.w, y = p / fp.w;
        int wx0 = max(0, (x - 5) & ~1), wx1 = min(fp.w, x + 6);
        int wy0 = max(0, y - 5), wy1 = min(fp.h, y + 6);
        if (!process_tile<TW, TH, OUTB>(fp, wx0, wy0, wx1 - wx0, wy1 - wy0, sm, ov, false, parity)) return;
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

cudaError_t launch_recip_table(float* d_out, int n, cudaStream_t st) {
    recip_table_kernel<<<(n + 255) / 256, 256, 0, st>>>(d_out, n);
    return cudaGetLastError();
}

cudaError_t launch_map_resolve(const FrameParams& fp, const MapPlan& plan, cudaStream_t st) {
    if (plan.n_comp > 0) dpc_map_resolve_kernel<<<(plan.n_comp + 127) / 128, 128, 0, st>>>(fp, plan);
    return cudaGetLastError();
}

template <int OUTB>
static cudaError_t launch_fused_t(const FrameParams& fp, const FixupScratch& fs, cudaStream_t st) {
    constexpr size_t smem = sizeof(TileSmem<kTileW, kTileH, OUTB>);
    static bool attr_set = false;
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(fused_frame_kernel<kTileW, kTileH, OUTB>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(dpc_fixup_kernel<kTileW, kTileH, OUTB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    int ntx, nty;
    int n = fused_tile_grid(fp.w, fp.h, ntx, nty);
    fused_frame_kernel<kTileW, kTileH, OUTB><<<n, kThreads, smem, st>>>(fp, ntx, nty);
    if ((fp.stages & 2u) && fp.dpc_mode == 0) dpc_fixup_kernel<kTileW, kTileH, OUTB><<<1, kThreads, smem, st>>>(fp, fs);
    return cudaGetLastError();
}

cudaError_t launch_fused(const FrameParams& fp, const FixupScratch& fs, const MapPlan* plan, cudaStream_t st) {
    if ((fp.stages & 2u) && fp.dpc_mode == 1 && plan) launch_map_resolve(fp, *plan, st);
    if ((fp.stages & 2u) && fp.dpc_mode == 0) {
        cudaError_t e = cudaMemsetAsync(fp.seed_count, 0, sizeof(int), st);
        if (e != cudaSuccess) return e;
    }
    return fp.out_bpc == 2 ? launch_fused_t<6>(fp, fs, st) : launch_fused_t<3>(fp, fs, st);
}

}  // namespace imop
