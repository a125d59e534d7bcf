// isp_lite.cu - persistent launch of the light-chain tile kernel (isp_lite.cuh) over the tiles of
// a batch of frames: CTAs claim tiles from a device counter, and warp 0 stages the next claimed
// tile into the second raw buffer while the CTA computes the current one.

#include <cuda_runtime.h>

#include "isp_fused_kernel.cuh"
#include "isp_kernels.h"
#include "isp_lite.cuh"

namespace imop {
namespace {

constexpr int kLiteTW = 256;
constexpr int kLiteTH = 16;
constexpr int kMaxDev = 64;

template <int TW, int TH>
__device__ void lite_stage_item(LiteSmem<TW, TH>& sm, const BatchLaunch& bl, int item, int b) {
    const int lane = threadIdx.x & 31;
    const int r = item_rect(bl, item);
    const TileRect& R = bl.rects[r];
    const FrameParams& src = bl.frames[R.frame];
    const int* s = reinterpret_cast<const int*>(&src);
    int* d = reinterpret_cast<int*>(&sm.fp[b]);
    for (int k = lane; k < (int)(sizeof(FrameParams) / 4); k += 32) d[k] = s[k];
    const int t = item - bl.rect_start[r];
    const int ty = t / R.tiles_x, tx = t - ty * R.tiles_x;
    int x0, tw, y0, th;
    tile_span(R.w, TW, R.tiles_x, tx, x0, tw);
    tile_span(R.h, TH, R.tiles_y, ty, y0, th);
    __syncwarp();
    lite_stage(sm, b, R.x0 + x0, R.y0 + y0, tw, th);
}

template <int TW, int TH>
__global__ void __launch_bounds__(kThreads, 3) lite_batch_kernel(const __grid_constant__ BatchLaunch bl) {
    extern __shared__ __align__(16) uint8_t dsm[];
    auto& sm = *reinterpret_cast<LiteSmem<TW, TH>*>(dsm);
    const int n_items = bl.n_items;
    if ((int)blockIdx.x >= n_items) return;
    if (threadIdx.x == 0) {
        ptx::mbar_init(&sm.bar[0], 1);
        ptx::mbar_init(&sm.bar[1], 1);
        ptx::fence_mbar_init();
        sm.tab_tone = nullptr;
        sm.tab_mode = -1;
    }
    __syncthreads();
    uint32_t par0 = 0, par1 = 0;
    int claimed = 0;
    if (threadIdx.x == 0) claimed = (int)gridDim.x + atomicAdd(bl.tile_counter, 1);
    if (threadIdx.x < 32) lite_stage_item(sm, bl, blockIdx.x, 0);
    __syncthreads();
    int b = 0;
    while (true) {
        if (threadIdx.x < 32) {
            const int next = __shfl_sync(0xffffffffu, claimed, 0);
            if (next < n_items) {
                if (threadIdx.x == 0) claimed = (int)gridDim.x + atomicAdd(bl.tile_counter, 1);
                lite_stage_item(sm, bl, next, b ^ 1);
            }
            if (threadIdx.x == 0) sm.next_item[b ^ 1] = next;
        }
        uint32_t& par = b ? par1 : par0;
        const bool ok = lite_compute(sm, b, par);
        const bool more = sm.next_item[b ^ 1] < n_items;
        if (!ok) {
            // leave no bulk copy in flight into this CTA's shared memory
            if (more && (reinterpret_cast<uintptr_t>(sm.fp[b ^ 1].in) & 15) == 0) wait_bar(&sm.bar[b ^ 1], b ? par0 : par1);
            return;
        }
        if (!more) return;
        b ^= 1;
    }
}

int g_lite_grid[kMaxDev];

}  // namespace

bool lite_eligible(const FrameParams& fp) {
    const bool fmt_ok = fp.fmt == FMT_U8 || fp.fmt == FMT_U16 || fp.fmt == FMT_P12 || fp.fmt == FMT_P10;
    return fmt_ok && fp.bd <= 12 && fp.demosaic == DM_HQLI && !(fp.stages & (2u | 4u | 16u | 32u)) &&
           fp.out_format == 0 && fp.out_bpc == 1 && fp.w >= 4 && fp.h >= 4;
}

int lite_tile_w() { return kLiteTW; }
int lite_tile_h() { return kLiteTH; }

cudaError_t launch_lite(const BatchLaunch& bl, cudaStream_t st) {
    using K = LiteSmem<kLiteTW, kLiteTH>;
    const size_t smem = sizeof(K);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDev) return cudaErrorInvalidDevice;
    int limit;
    {
        std::lock_guard<std::mutex> lock(device_setup_mutex());
        if (!g_lite_grid[dev]) {
            e = cudaFuncSetAttribute(lite_batch_kernel<kLiteTW, kLiteTH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem);
            int n = 0, m = 0;
            if (e == cudaSuccess)
                e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, lite_batch_kernel<kLiteTW, kLiteTH>, kThreads, smem);
            if (e == cudaSuccess) e = cudaDeviceGetAttribute(&m, cudaDevAttrMultiProcessorCount, dev);
            if (e != cudaSuccess) return e;
            g_lite_grid[dev] = m * (n > 0 ? n : 1);
        }
        limit = g_lite_grid[dev];
    }
    if (bl.n_items <= 0) return cudaSuccess;
    if ((e = cudaMemsetAsync(bl.tile_counter, 0, sizeof(int), st)) != cudaSuccess) return e;
    const int grid = bl.n_items < limit ? bl.n_items : limit;
    lite_batch_kernel<kLiteTW, kLiteTH><<<grid, kThreads, smem, st>>>(bl);
    return cudaGetLastError();
}

}  // namespace imop
