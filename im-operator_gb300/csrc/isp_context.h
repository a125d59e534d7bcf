// isp_context.h - host-side state behind an imop_isp_t handle.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <unordered_map>
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
    DevBuf grid, lut, knots, tone8, lut3d;
    DevBuf map_row_ptr, map_ent, map_val, slot_xy, comp_slot_ptr, comp_slots, comp_ent_ptr, comp_entries;
    MapPlan plan{};
    int n_slots = 0;  // unique map pixels (entries of map_val)
};

// map-mode plan built on the host from a defect list
struct HostMapPlan {
    std::vector<int> row_ptr;
    std::vector<int2> ent;  // (x, slot)
    std::vector<int2> slot_xy;
    std::vector<int> comp_slot_ptr, comp_slots, comp_ent_ptr, comp_entries;
};

template <class T>
cudaError_t upload(DevBuf& b, const std::vector<T>& v) {
    cudaError_t e = b.ensure((v.empty() ? 1 : v.size()) * sizeof(T));
    if (e != cudaSuccess || v.empty()) return e;
    return cudaMemcpy(b.ptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
}

// Parameter tables of many parameter sets, one device copy per distinct content (batches).  The
// maps are keyed by a hash of the content; each entry keeps the content bytes it was built from,
// so a hit is confirmed byte for byte.
template <class T>
struct CacheEntry {
    std::unique_ptr<T> obj;
    std::vector<uint8_t> key;
};
struct TableCache {
    std::unordered_map<uint64_t, CacheEntry<DevBuf>> grids, tones, lut3ds;
    std::unordered_map<uint64_t, CacheEntry<FrameTables>> maps;
    size_t entries() const { return grids.size() + tones.size() + lut3ds.size() + maps.size(); }
};

// per-frame defect-chain scratch and map values of a batch
struct BatchScratch {
    DevBuf seed_count, n_ov, seeds, heap, ov_idx, ov_val, map_val;
    int frames = 0, cap = 0, map_cap = 0;
};

// a recorded batch and its key (the stream, frame count and every frame's expanded parameters)
struct BatchGraph {
    uint64_t key = 0;
    std::vector<uint8_t> key_bytes;
    cudaGraphExec_t exec = nullptr;
    ~BatchGraph();
};

// defect-chain scratch (seeds, heap, overrides) and the sticky status word
struct FixupState {
    DevBuf seed_count, seeds, heap, ov_idx, ov_val, n_ov, status, tile_counter, seg;
    int cap = 0;
};

// Device slots, streams and events of the pipelined host batch.  Per frame: copy in (s_in), tile
// kernel (s_comp[frame & 1]: consecutive frames on two streams, so one frame's kernel fills the
// SMs that the previous one leaves at its end), defect-chain fix-up (s_fix, the highest stream
// priority, so its kernels take SMs as a tile kernel drains), copy out (s_out).  Each slot has its
// own fix-up scratch and tile counter, so frames of different slots never share device state.
struct HostPipeline {
    static constexpr int kSlots = 4;
    DevBuf d_in[kSlots], d_out[kSlots];
    FixupState fix[kSlots];
    cudaStream_t s_in = nullptr, s_comp[2] = {nullptr, nullptr}, s_fix = nullptr, s_out = nullptr;
    cudaEvent_t in_done[kSlots] = {}, main_done[kSlots] = {}, fix_done[kSlots] = {}, out_done[kSlots] = {};
    bool ready = false;
    ~HostPipeline();
};

// Device slots, streams and events of the RAW -> JPEG host batch.  Chunks of frames alternate
// between two slots; per chunk: raw copies in (s_in), one fused batch launch (s_isp), the
// encoder's device batch and the size read-back (s_jpg; the encoder runs on its own two lanes
// behind it), JPEG bytes out once their sizes are on the host (s_out).  A slot holds a chunk's
// frames back to back, each at a 256-byte aligned offset.
struct RawJpegPipe {
    static constexpr int kSlots = 2;
    static constexpr int kChunkFrames = 4;
    static constexpr long long kChunkPixels = 25000000;  // two 4024 x 3032 frames
    DevBuf raw[kSlots], rgb[kSlots], jpg[kSlots], size[kSlots];
    size_t* h_size[kSlots] = {nullptr, nullptr};  // page-locked copies of a chunk's JPEG sizes
    cudaStream_t s_in = nullptr, s_isp = nullptr, s_jpg = nullptr, s_out = nullptr;
    cudaEvent_t in_done[kSlots] = {}, isp_done[kSlots] = {}, jpg_done[kSlots] = {}, out_done[kSlots] = {};
    bool ready = false;
    ~RawJpegPipe();
};

int set_error(int code, const char* msg);
int cuda_fail(cudaError_t e, const char* what);
int validate_params(const ImopIspParams* p);
int device_ready();
void expand_frame_params(const ImopIspParams* p, FrameParams& fp);
int build_frame_params(const ImopIspParams* p, FrameTables& tabs, FrameParams& fp, cudaStream_t st);
int upload_map_plan(const ImopIspParams* p, FrameTables& tabs, FrameParams& fp);
void build_map_plan(const ImopDefectPoint* map, int n, int w, int h, HostMapPlan& P);
int flat_field_grid(const void* ff, int ffw, int ffh, int pattern, int bd, std::vector<float>& gm);
// 1 when every gain of an explicit lens-shading grid (ImopIspParams::lsc_grid) is finite and within
// [0, 15], the range the streaming kernel takes; 0 for the other shading modes
int lsc_grid_bounded(const ImopIspParams* p);
int ensure_fixup(FixupState& fx, int cap);
bool device_mapped_host(const void* p, size_t n);
void attach_fixup(FixupState& fx, FrameParams& fp, FixupScratch& fs);
int take_status(FixupState& fx);

}  // namespace imop

struct imop_isp_ctx {
    ImopIspParams params{};
    imop::FrameParams fp{};
    bool has_params = false;
    imop::FrameTables tabs;
    imop::FrameTables op_tabs;                     // tables of the per-operator entry points
    imop::DevBuf op_tone;                          // tone table of imop_op_rgb_table
    imop::FixupState fix;
    imop::DevBuf d_in, d_out;                      // run_host staging frames
    imop::DevBuf plain_a, plain_b, plain_rgb;      // plain per-operator intermediates
    imop::TableCache cache;                        // batch parameter tables
    imop::BatchScratch batch;                      // batch defect-chain scratch
    imop::HostPipeline pipe;                       // run_host_batch slots and streams
    imop::RawJpegPipe rawjpeg;                     // run_host_jpeg_batch slots and streams
    imop::BatchGraph graph;                        // last recorded batch
    cudaStream_t aux = nullptr;                    // table builds and graph capture
    imop::DevBuf adj_partials;                     // adjoint per-CTA partial sums
    ~imop_isp_ctx();
};
