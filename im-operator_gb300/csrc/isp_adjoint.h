// isp_adjoint.h - host-visible launch interface of the differentiable chain (isp_adjoint.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace imop {

constexpr int kAdjMaxGridNodes = 256;  // lens-shading grid nodes (grid_w * grid_h)

// geometry and format of the frames of one launch (all frames alike)
struct AdjFrame {
    int w, h, bd, mv, fmt, pattern, demosaic, border_mode, gw, gh;
    int tiles_x, tiles_y;
    size_t in_bytes;  // bytes of one input frame (frames are back to back)
};

struct AdjLaunch {
    AdjFrame f;
    int n_frames;
    int n_items;      // n_frames * tiles_x * tiles_y
    int n_params;
    const float* theta;
    const uint8_t* raw;
    const float* ref;   // target or upstream gradient (backward)
    int mode;           // 0 target, 1 upstream gradient
    float* rgb_out;     // forward output
    float* partials;    // per CTA: n_params + 1 (loss last)
    unsigned* tile_counter;  // backward: [0] tiles claimed past the first wave, [1] CTAs done; zero at
                             // launch, cleared again by the launch's last CTA
};

int adj_tile_grid(int w, int h, int& tx, int& ty);
size_t adj_smem_bytes();
cudaError_t adj_grid_limit(int& limit);
cudaError_t launch_adjoint(const AdjLaunch& L, bool backward, int grid, float* d_grad, float* d_loss, cudaStream_t st);

}  // namespace imop
