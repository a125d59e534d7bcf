// isp_fused_narrow.cu - the tile kernel in a narrow, tall tile (kNarrowW x kNarrowH) for the left
// and right border columns of streamed frames.  Those borders are 8 to 14 columns wide; in the
// nominal 120 x 24 tile a 3018-row border is 126 tiles that each pay the tile's staging and
// barrier latency for a sixteenth of its pixels, in this shape it is 24 tiles.

#include <cuda_runtime.h>

#include <mutex>

#include "isp_fused_kernel.cuh"
#include "isp_kernels.h"
#include "isp_tile.cuh"

namespace imop {
namespace {

constexpr int kMaxDev = 64;
int g_narrow_grid[kMaxDev];

void (*narrow_kernel())(BatchLaunch) { return fused_batch_kernel<kNarrowW, kNarrowH, 3, false, DM_AMAZE, 0>; }

}  // namespace

cudaError_t launch_fused_narrow(const BatchLaunch& bl, cudaStream_t st) {
    const size_t smem = sizeof(TileSmem<kNarrowW, kNarrowH, 3>);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDev) return cudaErrorInvalidDevice;
    int limit;
    {
        std::lock_guard<std::mutex> lock(device_setup_mutex());
        if (!g_narrow_grid[dev]) {
            e = cudaFuncSetAttribute(narrow_kernel(), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            int n = 0, m = 0;
            if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, narrow_kernel(), kThreads, smem);
            if (e == cudaSuccess) e = cudaDeviceGetAttribute(&m, cudaDevAttrMultiProcessorCount, dev);
            if (e != cudaSuccess) return e;
            g_narrow_grid[dev] = m * (n > 0 ? n : 1);
        }
        limit = g_narrow_grid[dev];
    }
    if (bl.n_items <= 0) return cudaSuccess;
    const int grid = bl.n_items < limit ? bl.n_items : limit;
    count_launch(0);
    if (bl.dependent) return launch_dependent(narrow_kernel(), grid, kThreads, smem, st, bl);
    if ((e = cudaMemsetAsync(bl.tile_counter, 0, sizeof(int), st)) != cudaSuccess) return e;
    narrow_kernel()<<<grid, kThreads, smem, st>>>(bl);
    return cudaGetLastError();
}

}  // namespace imop
