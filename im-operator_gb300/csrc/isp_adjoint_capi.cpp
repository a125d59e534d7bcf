// isp_adjoint_capi.cpp - C ABI of the differentiable calibration chain (render and adjoint).

#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/imop_isp.h"
#include "isp_adjoint.h"
#include "isp_common.h"
#include "isp_context.h"

using namespace imop;

namespace {

int validate_desc(const ImopAdjointDesc* d) {
    if (!d) return set_error(IMOP_ERR_NULL_INPUT, "desc is null");
    if (d->width <= 0 || d->height <= 0) return set_error(IMOP_ERR_INVALID_DIMENSIONS, "invalid image dimensions");
    if (d->bit_depth < 1 || d->bit_depth > 16) return set_error(IMOP_ERR_INVALID_BIT_DEPTH, "bit depth must be 1-16");
    if (d->pattern < 0 || d->pattern > 3) return set_error(IMOP_ERR_INVALID_PATTERN, "invalid Bayer pattern");
    if (d->width < 6 || d->height < 6) return set_error(IMOP_ERR_IMAGE_TOO_SMALL, "image too small (min 6x6)");
    if (d->demosaic != IMOP_DEMOSAIC_HQLI && d->demosaic != IMOP_DEMOSAIC_AMAZE)
        return set_error(IMOP_ERR_UNSUPPORTED, "differentiable demosaic must be HQLI or AMAZE");
    if (d->grid_w < 2 || d->grid_h < 2 || d->grid_w > 32 || d->grid_h > 32 || d->grid_w * d->grid_h > kAdjMaxGridNodes)
        return set_error(IMOP_ERR_INVALID_ARGUMENT, "grid must be 2..32 nodes per side, at most 256 nodes");
    if (d->n_frames < 1) return set_error(IMOP_ERR_INVALID_ARGUMENT, "n_frames must be positive");
    if ((long long)d->width * d->height * d->n_frames * 3 >= (1LL << 40))
        return set_error(IMOP_ERR_UNSUPPORTED, "batch too large");
    return IMOP_OK;
}

int make_launch(const ImopAdjointDesc* d, AdjLaunch& L) {
    AdjFrame& f = L.f;
    f.w = d->width;
    f.h = d->height;
    f.bd = d->bit_depth;
    f.mv = max_val_of(d->bit_depth);
    f.fmt = input_format_of(d->packed, d->bit_depth);
    f.pattern = d->pattern;
    f.demosaic = d->demosaic;
    f.border_mode = (d->demosaic == IMOP_DEMOSAIC_AMAZE && d->bit_depth <= 8) ? BORDER_BOTH : BORDER_ROWS_THEN_COLS;
    f.gw = d->grid_w;
    f.gh = d->grid_h;
    f.in_bytes = input_bytes_of(f.fmt, d->bit_depth, f.w, f.h);
    int per = adj_tile_grid(f.w, f.h, f.tiles_x, f.tiles_y);
    L.n_frames = d->n_frames;
    L.n_items = per * d->n_frames;
    L.n_params = imop_adjoint_param_count(d);
    L.mode = 0;
    L.ref = nullptr;
    L.rgb_out = nullptr;
    L.partials = nullptr;
    L.tile_counter = nullptr;
    return IMOP_OK;
}

}  // namespace

extern "C" int imop_adjoint_param_count(const ImopAdjointDesc* d) {
    if (!d) return 0;
    return 16 + 4 * d->grid_w * d->grid_h + 33;
}

extern "C" int imop_isp_render_device(imop_isp_t ctx, const ImopAdjointDesc* d, const float* d_theta, const void* d_raw,
                                      float* d_rgb, void* stream) {
    if (!ctx) return set_error(IMOP_ERR_NULL_INPUT, "ctx is null");
    int rc = validate_desc(d);
    if (rc) return rc;
    if (!d_theta || !d_raw || !d_rgb) return set_error(IMOP_ERR_NULL_INPUT, "null device pointer");
    AdjLaunch L;
    make_launch(d, L);
    L.theta = d_theta;
    L.raw = static_cast<const uint8_t*>(d_raw);
    L.rgb_out = d_rgb;
    int limit = 0;
    cudaError_t e = adj_grid_limit(limit);
    if (e != cudaSuccess) return cuda_fail(e, "adjoint set-up");
    if ((e = launch_adjoint(L, false, std::min(limit, L.n_items), nullptr, nullptr, (cudaStream_t)stream)))
        return cuda_fail(e, "render launch");
    return IMOP_OK;
}

extern "C" int imop_isp_backward_device(imop_isp_t ctx, const ImopAdjointDesc* d, const float* d_theta,
                                        const void* d_raw, const float* d_ref, int mode, float* d_loss, float* d_grad,
                                        void* stream) {
    if (!ctx) return set_error(IMOP_ERR_NULL_INPUT, "ctx is null");
    int rc = validate_desc(d);
    if (rc) return rc;
    if (!d_theta || !d_raw || !d_ref || !d_grad) return set_error(IMOP_ERR_NULL_INPUT, "null device pointer");
    if (mode != IMOP_ADJ_TARGET && mode != IMOP_ADJ_UPSTREAM) return set_error(IMOP_ERR_INVALID_ARGUMENT, "mode");
    AdjLaunch L;
    make_launch(d, L);
    L.theta = d_theta;
    L.raw = static_cast<const uint8_t*>(d_raw);
    L.ref = d_ref;
    L.mode = mode;
    int limit = 0;
    cudaError_t e = adj_grid_limit(limit);
    if (e != cudaSuccess) return cuda_fail(e, "adjoint set-up");
    const int grid = std::min(limit, L.n_items);
    // the tile counter's two words (16 bytes kept), then the partial vectors; the counter is zeroed
    // when the buffer is made and each launch's last CTA clears it again
    const size_t need = 16 + (size_t)grid * (L.n_params + 1) * sizeof(float);
    if (ctx->adj_partials.size < need) {
        // the buffer may be read by an adjoint still running on another stream
        if ((e = cudaDeviceSynchronize())) return cuda_fail(e, "sync before partials growth");
        if ((e = ctx->adj_partials.ensure(need))) return cuda_fail(e, "alloc partials");
        if ((e = cudaMemset(ctx->adj_partials.ptr, 0, 16))) return cuda_fail(e, "tile counter");
    }
    L.tile_counter = static_cast<unsigned*>(ctx->adj_partials.ptr);
    L.partials = reinterpret_cast<float*>(static_cast<uint8_t*>(ctx->adj_partials.ptr) + 16);
    if ((e = launch_adjoint(L, true, grid, d_grad, d_loss, (cudaStream_t)stream))) return cuda_fail(e, "adjoint launch");
    return IMOP_OK;
}
