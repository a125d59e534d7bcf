// isp_fused_spec.inl - body of the per-format units isp_fused_spec_*.cu: the fused kernel
// instantiated for one input format (IMOP_SPEC_FMT) and each demosaic algorithm, with the common
// stage configuration fixed at compile time, with and without defect correction / lens shading.
#include "isp_fused_kernel.cuh"

namespace imop {

cudaError_t IMOP_SPEC_LAUNCH(int dm, bool lite, const BatchLaunch& bl, int grid, size_t smem, cudaStream_t st) {
    constexpr int S = spec_of_format(IMOP_SPEC_FMT), SL = S | 16;
    switch (dm) {
        case DM_HQLI:
            return lite ? launch_fused_variant<kTileW, kTileH, 3, false, DM_HQLI, SL>(bl, grid, smem, st)
                        : launch_fused_variant<kTileW, kTileH, 3, false, DM_HQLI, S>(bl, grid, smem, st);
        case DM_MG:
            return lite ? launch_fused_variant<kTileW, kTileH, 3, false, DM_MG, SL>(bl, grid, smem, st)
                        : launch_fused_variant<kTileW, kTileH, 3, false, DM_MG, S>(bl, grid, smem, st);
        default:
            return lite ? launch_fused_variant<kTileW, kTileH, 3, false, DM_AMAZE, SL>(bl, grid, smem, st)
                        : launch_fused_variant<kTileW, kTileH, 3, false, DM_AMAZE, S>(bl, grid, smem, st);
    }
}

}  // namespace imop
