// isp_context.h - host-side state behind an imop_isp_t handle.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "../../include/imop_isp.h"
#include "isp_common.h"
#include "isp_kernels.h"

namespace imop {

// an owned device allocation that only grows
struct DevBuf {
    void* ptr = nullptr;
    size_t size = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf();
    cudaError_t ensure(size_t bytes);
    void release();
};

// device copies of one frame's parameter tables
struct FrameTables {
    DevBuf grid, lut, knots, tone8, rtab;
    DevBuf map_row_ptr, map_ent, map_val, slot_xy, comp_slot_ptr, comp_slots, comp_ent_ptr, comp_entries;
    MapPlan plan{};
};

// defect-chain scratch (seeds, heap, overrides) and the sticky status word
struct FixupState {
    DevBuf seed_count, seeds, heap, ov_idx, ov_val, n_ov, status;
    int cap = 0;
};

int set_error(int code, const char* msg);
int cuda_fail(cudaError_t e, const char* what);
int validate_params(const ImopIspParams* p);
int device_ready();
void expand_frame_params(const ImopIspParams* p, FrameParams& fp);
int build_frame_params(const ImopIspParams* p, FrameTables& tabs, FrameParams& fp, cudaStream_t st);
int ensure_fixup(FixupState& fx, int cap);
void attach_fixup(FixupState& fx, FrameParams& fp, FixupScratch& fs);
int take_status(FixupState& fx);

}  // namespace imop

struct imop_isp_ctx {
    ImopIspParams params{};
    imop::FrameParams fp{};
    bool has_params = false;
    imop::FrameTables tabs;
    imop::FixupState fix;
    imop::DevBuf d_in, d_out;                      // run_host staging frames
    imop::DevBuf plain_a, plain_b, plain_rgb;      // plain per-operator intermediates
};
