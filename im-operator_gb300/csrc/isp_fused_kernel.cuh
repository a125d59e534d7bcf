// isp_fused_kernel.cuh - the persistent fused tile kernel and the launch of one of its
// instantiations.  Included by isp_fused.cu (the generic and per-algorithm instantiations) and
// by the isp_fused_spec_*.cu units (one input format each, for launches whose frames all share
// the format, the algorithm and the common stage configuration: see compute_tile's SPEC).
#pragma once

#include <cuda_runtime.h>

#include "isp_kernels.h"
#include "isp_segments.cuh"
#include "isp_tile.cuh"

namespace imop {

// ---------------------------------------------------------------------------------------------
// Persistent tile kernel: CTA c starts with item c of the launch's tile list (the tiles of each
// rectangle in raster order) and then claims items from the launch's counter, one item ahead of
// the one it stages.  Warp 0 stages the next item into the other raw buffer before the CTA
// computes the current one, so the copy of tile k+1 overlaps the arithmetic of tile k.

// rectangle of item `item`: the last rectangle starting at or before it
__device__ __forceinline__ int item_rect(const BatchLaunch& bl, int item) {
    int lo = 0, hi = bl.n_rects - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (bl.rect_start[mid] <= item) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// warp 0: copy the item's frame parameters into slot b and start staging its raw rows
template <int TW, int TH, int OUTB>
__device__ void stage_item(TileSmem<TW, TH, OUTB>& sm, const BatchLaunch& bl, int item, int b) {
    const int lane = threadIdx.x & 31;
    const int r = item_rect(bl, item);
    const TileRect& R = bl.rects[r];
    const FrameParams& src = bl.frames[R.frame];
    static_assert(sizeof(FrameParams) % 4 == 0, "frame parameters copy as words");
    const int* s = reinterpret_cast<const int*>(&src);
    int* d = reinterpret_cast<int*>(&sm.fp[b]);
    for (int k = lane; k < (int)(sizeof(FrameParams) / 4); k += 32) d[k] = s[k];
    int t = item - bl.rect_start[r];
    int ty = t / R.tiles_x, tx = t - ty * R.tiles_x;
    int x0, tw, y0, th;
    tile_span(R.w, TW, R.tiles_x, tx, x0, tw);
    tile_span(R.h, TH, R.tiles_y, ty, y0, th);
    __syncwarp();
    stage_tile(sm, b, R.x0 + x0, R.y0 + y0, tw, th);
}

template <int TW, int TH, int OUTB, bool EXTRA, int DM, int SPEC>
__global__ void __launch_bounds__(kThreads, 3) fused_batch_kernel(const __grid_constant__ BatchLaunch bl) {
    segs::release_dependents();  // a tile launch after this one may start beside it
    extern __shared__ __align__(16) uint8_t dsm[];
    auto& sm = *reinterpret_cast<TileSmem<TW, TH, OUTB>*>(dsm);
    const int n_items = bl.n_items;
    if ((int)blockIdx.x >= n_items) return;
    tile_init(sm);
    uint32_t par0 = 0, par1 = 0;
    const Overrides none{nullptr, nullptr, 0};
    // lane 0 of warp 0 holds the item claimed after the staged one (its counter read completes
    // while the CTA computes)
    int claimed = 0;
    if (threadIdx.x == 0) claimed = (int)gridDim.x + atomicAdd(bl.tile_counter, 1);
    if (threadIdx.x < 32) stage_item(sm, bl, blockIdx.x, 0);
    __syncthreads();
    int b = 0;
    while (true) {
        if (threadIdx.x < 32) {
            const int next = __shfl_sync(0xffffffffu, claimed, 0);
            if (next < n_items) {
                if (threadIdx.x == 0) claimed = (int)gridDim.x + atomicAdd(bl.tile_counter, 1);
                stage_item(sm, bl, next, b ^ 1);
            }
            if (threadIdx.x == 0) sm.next_item[b ^ 1] = next;
        }
        const FrameParams& fp = sm.fp[b];
        const bool full = tile_is_full<TW, TH>(fp, sm.tile[b][0], sm.tile[b][1], sm.tile[b][2], sm.tile[b][3]);
        uint32_t& par = b ? par1 : par0;
        bool ok = full ? compute_tile<TW, TH, OUTB, true, EXTRA, DM, SPEC>(sm, b, none, true, par)
                       : compute_tile<TW, TH, OUTB, false, EXTRA, DM, SPEC>(sm, b, none, true, par);
        // next_item[b ^ 1] was written before the barriers of compute_tile and is written again two
        // iterations on, after every thread has passed the barriers of the next compute_tile
        const bool more = sm.next_item[b ^ 1] < n_items;
        if (!ok) {
            // leave no bulk copy in flight into this CTA's shared memory
            if (more && (reinterpret_cast<uintptr_t>(sm.fp[b ^ 1].in) & 15) == 0)
                wait_bar(&sm.bar[b ^ 1], b ? par0 : par1);
            return;
        }
        if (!more) return;
        b ^= 1;
    }
}

// opts the instantiation into its dynamic shared memory (once per device) and launches it
template <int TW, int TH, int OUTB, bool EXTRA, int DM, int SPEC>
cudaError_t launch_fused_variant(const BatchLaunch& bl, int grid, size_t smem, cudaStream_t st) {
    static bool attr_done[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    {
        std::lock_guard<std::mutex> lock(device_setup_mutex());
        if (!attr_done[dev]) {
            e = cudaFuncSetAttribute(fused_batch_kernel<TW, TH, OUTB, EXTRA, DM, SPEC>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
            attr_done[dev] = true;
        }
    }
    if (bl.dependent) return launch_dependent(fused_batch_kernel<TW, TH, OUTB, EXTRA, DM, SPEC>, grid, kThreads, smem, st, bl);
    fused_batch_kernel<TW, TH, OUTB, EXTRA, DM, SPEC><<<grid, kThreads, smem, st>>>(bl);
    return cudaGetLastError();
}

// SPEC of the per-format units: the input format plus one, and the flag of the common stage
// configuration (adaptive or no defect correction, no polynomial shading, RGB8 output)
constexpr int spec_of_format(int fmt) { return (fmt + 1) | 8; }

// launch of the per-format instantiation for the frames' format and algorithm (isp_fused_spec_*.cu);
// lite: none of the frames corrects defects or lens shading
cudaError_t launch_fused_spec(int fmt, int dm, bool lite, const BatchLaunch& bl, int grid, size_t smem,
                              cudaStream_t st);

}  // namespace imop
