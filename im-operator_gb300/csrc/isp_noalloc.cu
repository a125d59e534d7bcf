// isp_noalloc.cu - the fused pipeline for callers that cannot allocate device memory.
//
// Some callers cannot let a library call cudaMalloc: a camera or inference loop that owns every
// byte of device memory through its own pool and budgets it up front, or a real-time loop that
// must not stall, since cudaMalloc / cudaFree can synchronize the whole device and can fail under
// memory pressure at a moment the caller does not control.  imop_isp_run_device_noalloc() runs
// the same fused kernel and defect-chain fix-up as imop_isp_run_device(), but everything it needs
// beyond the caller's input and output frames - the parameter tables (lens-shading grid, tone
// LUT, the 8-bit tone table) and the fix-up scratch (seed list, heap,
// override list, counters, status word) - lives in the file-scope array g_noalloc_scratch below,
// which every GPU that loads the library holds until the process exits.
//
// Limits (checked before any work, IMOP_ERR_UNSUPPORTED otherwise): bit depth <= 12, an explicit
// lens-shading grid of at most 64 x 64 nodes (or polynomial / no lens shading), adaptive defect
// correction (no defect map), and at most kSeedCap defect-chain seeds per call (more is reported
// as IMOP_ERR_CAPACITY after the call).  The array is shared by every call on a device and keeps
// the last call's contents: each call re-uploads its tables and clears the counters that must
// start at zero, so calls that overlap on the GPU (two streams, two host threads) race on it.
// The array's device address, looked up on a device's first call, is kept for the life of the
// process: after a cudaDeviceReset of that device the module is loaded anew, so this entry point
// must not be used across a reset.

#include <cuda_runtime.h>

#include <mutex>

#include "../../include/imop_isp.h"
#include "isp_common.h"
#include "isp_context.h"
#include "isp_kernels.h"

namespace imop {
namespace {

constexpr int kSeedCap = 16384;          // defect-chain seeds (and heap / override entries) per call
constexpr int kGridMaxNodes = 64 * 64;   // lens-shading grid nodes
constexpr int kMaxBitDepth = 12;
constexpr int kToneMax = 1 << kMaxBitDepth;
constexpr int kMaxDevices = 64;

struct NoAllocScratch {
    int seed_count;
    int n_ov;
    int status;
    int tile_counter;
    int seeds[kSeedCap];
    int heap[kSeedCap];
    int ov_idx[kSeedCap];
    int ov_val[kSeedCap];
    float grid[kGridMaxNodes * 4];
    float lut[kToneMax];
    float knots[36];
    alignas(16) uint8_t tone8[kToneMax + 16];
};

// about 340 KB per device
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

std::mutex g_setup_mu;
NoAllocScratch* g_dev_scratch[kMaxDevices] = {};

// Device address of the array for the current device, looked up once per device (with that
// device current) on its first call.
int scratch_for_current_device(NoAllocScratch** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return set_error(IMOP_ERR_UNSUPPORTED, "device index beyond the no-alloc table");
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_dev_scratch[dev]) {
        void* ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_dev_scratch[dev] = static_cast<NoAllocScratch*>(ptr);
    }
    *out = g_dev_scratch[dev];
    return IMOP_OK;
}

}  // namespace
}  // namespace imop

using namespace imop;

extern "C" int imop_isp_run_device_noalloc(const ImopIspParams* p, const void* d_in, void* d_out, void* stream) {
    int rc = validate_params(p);
    if (rc) return rc;
    if (!d_in || !d_out) return set_error(IMOP_ERR_NULL_INPUT, "null frame pointer");
    if (p->bit_depth > kMaxBitDepth)
        return set_error(IMOP_ERR_UNSUPPORTED, "no-alloc entry point: bit depth above 12");
    if (p->stages & IMOP_STAGE_LUT3D)
        return set_error(IMOP_ERR_UNSUPPORTED, "no-alloc entry point: 3D LUTs need a device table");
    if ((p->stages & IMOP_STAGE_DEFECT) && p->dpc_mode != IMOP_DPC_ADAPTIVE)
        return set_error(IMOP_ERR_UNSUPPORTED, "no-alloc entry point: defect maps need device tables");
    const bool grid_lsc = (p->stages & IMOP_STAGE_LENS_SHADING) && p->lsc_mode != IMOP_LSC_POLYNOMIAL;
    if (grid_lsc && p->lsc_mode != IMOP_LSC_GRID)
        return set_error(IMOP_ERR_UNSUPPORTED, "no-alloc entry point: flat-field lens shading needs a host pass");
    if (grid_lsc && p->lsc_grid_w * p->lsc_grid_h > kGridMaxNodes)
        return set_error(IMOP_ERR_UNSUPPORTED, "no-alloc entry point: lens-shading grid above 64x64 nodes");
    if (!device_ready()) return set_error(IMOP_ERR_NO_DEVICE, "no CUDA device");

    NoAllocScratch* sc = nullptr;
    if ((rc = scratch_for_current_device(&sc))) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    FrameParams fp;
    expand_frame_params(p, fp);
    cudaError_t e;
    // parameter tables into the array (the caller's host tables are read synchronously)
    if (grid_lsc) {
        e = cudaMemcpyAsync(sc->grid, p->lsc_grid, sizeof(float) * 4 * p->lsc_grid_w * p->lsc_grid_h,
                            cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return cuda_fail(e, "upload grid");
        fp.gw = p->lsc_grid_w;
        fp.gh = p->lsc_grid_h;
        fp.grid = sc->grid;
    }
    fp.tone8 = sc->tone8;
    if (p->out_format == IMOP_OUT_RGB8) {
        const float* d_lut = nullptr;
        const float* d_knots = nullptr;
        if (p->tone_mode == IMOP_TONE_LUT) {
            if ((e = cudaMemcpyAsync(sc->lut, p->tone_lut, sizeof(float) * p->tone_lut_len, cudaMemcpyHostToDevice, st)))
                return cuda_fail(e, "upload tone lut");
            d_lut = sc->lut;
        } else if (p->tone_mode == IMOP_TONE_KNOTS) {
            if ((e = cudaMemcpyAsync(sc->knots, p->tone_knots, sizeof(float) * 33, cudaMemcpyHostToDevice, st)))
                return cuda_fail(e, "upload tone knots");
            d_knots = sc->knots;
        }
        if ((e = launch_tone_table(p->tone_mode, d_lut, d_knots, fp.bd, sc->tone8, st))) return cuda_fail(e, "tone table");
    }
    // counters that must start at zero (the array keeps the previous call's values)
    if ((e = cudaMemsetAsync(&sc->seed_count, 0, 3 * sizeof(int), st))) return cuda_fail(e, "clear counters");
    fp.in = static_cast<const uint8_t*>(d_in);
    fp.out = static_cast<uint8_t*>(d_out);
    fp.seed_count = &sc->seed_count;
    fp.seeds = sc->seeds;
    fp.seed_cap = kSeedCap;
    fp.status = &sc->status;
    fp.tile_counter = &sc->tile_counter;
    FixupScratch fs{sc->heap, sc->ov_idx, sc->ov_val, &sc->n_ov, kSeedCap};
    if ((e = launch_fused(fp, fs, nullptr, st))) return cuda_fail(e, "fused launch");
    // the status word is read on the caller's stream, so the call waits for its own work only
    // (a copy on the legacy default stream would also wait for unrelated blocking streams)
    int status = 0;
    if ((e = cudaMemcpyAsync(&status, &sc->status, sizeof(int), cudaMemcpyDeviceToHost, st)))
        return cuda_fail(e, "read status");
    if ((e = cudaStreamSynchronize(st))) return cuda_fail(e, "no-alloc run");
    if (status) return set_error(status, "device status after the no-alloc run (defect-chain capacity or wait limit)");
    return IMOP_OK;
}
