// isp_capi.cpp - the C ABI (include/imop_isp.h): contexts, parameter upload, run entry points.
//
// Validation follows the reference dispatchers' order (null -> dimensions -> bit depth ->
// pattern -> too small) and returns the same codes, e.g. src/algorithms/dispatch.cpp:14-20,
// src/black_level/dispatch.cpp:7-15.  A context owns its device copies of every parameter
// table, the defect-chain scratch, and (for run_host) device staging frames; the caller owns
// every frame buffer it passes.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/imop_isp.h"
#include "isp_common.h"
#include "isp_context.h"
#include "isp_kernels.h"

using namespace imop;

namespace {

thread_local std::string t_last_error;

int fail(int code, const std::string& msg) {
    t_last_error = msg;
    return code;
}

}  // namespace

namespace imop {

int set_error(int code, const char* msg) { return fail(code, msg ? msg : ""); }

int cuda_fail(cudaError_t e, const char* what) {
    return fail(IMOP_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

DevBuf::~DevBuf() { release(); }
void DevBuf::release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    size = 0;
}
cudaError_t DevBuf::ensure(size_t bytes) {
    if (bytes <= size && ptr) return cudaSuccess;
    release();
    cudaError_t e = cudaMalloc(&ptr, bytes ? bytes : 1);
    if (e == cudaSuccess) size = bytes;
    return e;
}

// ---- map-mode plan ----------------------------------------------------------------------------
// Unique defect pixels inside [2,w-2)x[2,h-2) become slots (sorted by row, then column); slots
// that are same-colour neighbours at step 2 (or repeated entries) form components that the
// device resolves serially in map order.
void build_map_plan(const ImopDefectPoint* map, int n, int w, int h, HostMapPlan& P) {
    std::vector<std::pair<int, int>> keys;  // (y, x) of entries inside the interior
    std::vector<int> entry_key;             // per map entry: raster index or -1
    for (int i = 0; i < n; i++) {
        int x = map[i].x, y = map[i].y;
        if (x < 2 || x >= w - 2 || y < 2 || y >= h - 2) {
            entry_key.push_back(-1);
            continue;
        }
        keys.push_back({y, x});
        entry_key.push_back(y * w + x);
    }
    std::sort(keys.begin(), keys.end());
    keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
    const int ns = (int)keys.size();
    std::map<long long, int> slot_of;
    P.slot_xy.resize(ns);
    P.row_ptr.assign(h + 1, 0);
    P.ent.resize(ns);
    for (int s = 0; s < ns; s++) {
        P.slot_xy[s] = make_int2(keys[s].second, keys[s].first);
        slot_of[(long long)keys[s].first * w + keys[s].second] = s;
        P.ent[s] = make_int2(keys[s].second, s);
        P.row_ptr[keys[s].first + 1]++;
    }
    for (int y = 0; y < h; y++) P.row_ptr[y + 1] += P.row_ptr[y];
    // union-find over same-colour step-2 neighbours
    std::vector<int> parent(ns);
    std::iota(parent.begin(), parent.end(), 0);
    auto find = [&](int a) {
        while (parent[a] != a) a = parent[a] = parent[parent[a]];
        return a;
    };
    for (int s = 0; s < ns; s++) {
        int x = P.slot_xy[s].x, y = P.slot_xy[s].y;
        for (int dy = -2; dy <= 2; dy += 2)
            for (int dx = -2; dx <= 2; dx += 2) {
                if (!dx && !dy) continue;
                auto it = slot_of.find((long long)(y + dy) * w + (x + dx));
                if (it != slot_of.end()) parent[find(s)] = find(it->second);
            }
    }
    std::map<int, int> comp_of_root;
    std::vector<int> comp(ns);
    for (int s = 0; s < ns; s++) {
        int r = find(s);
        auto it = comp_of_root.find(r);
        if (it == comp_of_root.end()) it = comp_of_root.emplace(r, (int)comp_of_root.size()).first;
        comp[s] = it->second;
    }
    const int nc = (int)comp_of_root.size();
    std::vector<std::vector<int>> cs(nc), ce(nc);
    for (int s = 0; s < ns; s++) cs[comp[s]].push_back(s);
    for (int i = 0; i < n; i++) {
        if (entry_key[i] < 0) continue;
        int s = slot_of[entry_key[i]];
        ce[comp[s]].push_back(s);
    }
    P.comp_slot_ptr.assign(1, 0);
    P.comp_ent_ptr.assign(1, 0);
    P.comp_slots.clear();
    P.comp_entries.clear();
    for (int c = 0; c < nc; c++) {
        P.comp_slots.insert(P.comp_slots.end(), cs[c].begin(), cs[c].end());
        P.comp_entries.insert(P.comp_entries.end(), ce[c].begin(), ce[c].end());
        P.comp_slot_ptr.push_back((int)P.comp_slots.size());
        P.comp_ent_ptr.push_back((int)P.comp_entries.size());
    }
}

// Grid construction of lens_shading::process_flat_field (src/lens_shading/flat_field.cpp:30-76):
// a parameter derivation done once per set_params, 32 x 24 x 4 gains.
int lsc_grid_bounded(const ImopIspParams* p) {
    if (!(p->stages & IMOP_STAGE_LENS_SHADING) || p->lsc_mode != IMOP_LSC_GRID || !p->lsc_grid) return 0;
    const size_t n = (size_t)p->lsc_grid_w * p->lsc_grid_h * 4;
    for (size_t i = 0; i < n; i++)
        if (!(p->lsc_grid[i] >= 0.0f && p->lsc_grid[i] <= 15.0f)) return 0;
    return 1;
}

int flat_field_grid(const void* ff, int ffw, int ffh, int pattern, int bd, std::vector<float>& gm) {
    if (!ff) return fail(IMOP_ERR_NULL_INPUT, "flat-field frame is null");
    if (ffw <= 0 || ffh <= 0) return fail(IMOP_ERR_INVALID_DIMENSIONS, "flat-field dimensions");
    auto rd = [&](int x, int y) -> int {
        size_t i = (size_t)y * ffw + x;
        if (bd <= 8) return ((const uint8_t*)ff)[i];
        const uint8_t* b = (const uint8_t*)ff + 2 * i;
        return b[0] | (b[1] << 8);
    };
    PatternOffsets po = pattern_offsets(pattern);
    int mv = max_val_of(bd);
    float targets[4] = {0, 0, 0, 0};
    int counts[4] = {0, 0, 0, 0};
    int cx0 = ffw * 3 / 10, cx1 = ffw * 7 / 10, cy0 = ffh * 3 / 10, cy1 = ffh * 7 / 10;
    for (int y = cy0; y < cy1; y += 2)
        for (int x = cx0; x < cx1; x += 2) {
            int c = bayer_color(y, x, po);
            targets[c] += (float)rd(x, y);
            counts[c]++;
        }
    for (int c = 0; c < 4; c++) targets[c] = counts[c] > 0 ? targets[c] / (float)counts[c] : (float)mv;
    const int gw = 32, gh = 24;
    gm.assign(gw * gh * 4, 1.0f);
    for (int gy = 0; gy < gh; gy++)
        for (int gx = 0; gx < gw; gx++) {
            int fx0 = gx * ffw / gw, fx1 = (gx + 1) * ffw / gw, fy0 = gy * ffh / gh, fy1 = (gy + 1) * ffh / gh;
            float sum[4] = {0, 0, 0, 0};
            int cnt[4] = {0, 0, 0, 0};
            for (int y = fy0; y < fy1; y += 2)
                for (int x = fx0; x < fx1; x += 2) {
                    int c = bayer_color(y, x, po);
                    sum[c] += (float)rd(x, y);
                    cnt[c]++;
                }
            for (int c = 0; c < 4; c++) {
                float mean = cnt[c] > 0 ? sum[c] / (float)cnt[c] : targets[c];
                gm[(gy * gw + gx) * 4 + c] = targets[c] / std::max(1e-6f, mean);
            }
        }
    return IMOP_OK;
}

int validate_params(const ImopIspParams* p) {
    if (!p) return fail(IMOP_ERR_NULL_INPUT, "params is null");
    if (p->width <= 0 || p->height <= 0) return fail(IMOP_ERR_INVALID_DIMENSIONS, "invalid image dimensions");
    if (p->bit_depth < 1 || p->bit_depth > 16) return fail(IMOP_ERR_INVALID_BIT_DEPTH, "bit depth must be 1-16");
    if (p->pattern < 0 || p->pattern > 3) return fail(IMOP_ERR_INVALID_PATTERN, "invalid Bayer pattern");
    if (p->width < 6 || p->height < 6) return fail(IMOP_ERR_IMAGE_TOO_SMALL, "image too small for the pipeline (min 6x6)");
    if ((long long)p->width * p->height * 6 >= (1LL << 31))
        return fail(IMOP_ERR_UNSUPPORTED, "frame larger than 2^31 output bytes");
    if (p->demosaic != IMOP_DEMOSAIC_HQLI && p->demosaic != IMOP_DEMOSAIC_AMAZE && p->demosaic != IMOP_DEMOSAIC_MG)
        return fail(IMOP_ERR_UNSUPPORTED, "demosaic must be HQLI, MG or AMAZE");
    if (p->stages & ~(IMOP_STAGE_ALL | IMOP_STAGE_LUT3D)) return fail(IMOP_ERR_INVALID_ARGUMENT, "unknown stage bits");
    if (p->stages & IMOP_STAGE_LUT3D) {
        if (!p->lut3d) return fail(IMOP_ERR_NULL_INPUT, "lut3d is null");
        if (p->lut3d_size < 2 || p->lut3d_size > 65) return fail(IMOP_ERR_INVALID_ARGUMENT, "lut3d_size must be 2..65");
    }
    if (p->stage_order != IMOP_ORDER_BAYER_WB && p->stage_order != IMOP_ORDER_RGB_WB)
        return fail(IMOP_ERR_INVALID_ARGUMENT, "stage_order");
    if (p->stages & IMOP_STAGE_BLACK_LEVEL) {
        if (p->bl_mode != IMOP_BL_PER_CHANNEL && p->bl_mode != IMOP_BL_GLOBAL)
            return fail(IMOP_ERR_INVALID_ARGUMENT, "bl_mode");
    }
    if (p->stages & IMOP_STAGE_DEFECT) {
        if (p->dpc_mode != IMOP_DPC_ADAPTIVE && p->dpc_mode != IMOP_DPC_MAP_BASED)
            return fail(IMOP_ERR_INVALID_ARGUMENT, "dpc_mode");
        if (p->dpc_mode == IMOP_DPC_MAP_BASED && p->dpc_map_count > 0 && !p->dpc_map)
            return fail(IMOP_ERR_NULL_INPUT, "dpc_map is null");
    }
    if (p->stages & IMOP_STAGE_LENS_SHADING) {
        if (p->lsc_mode == IMOP_LSC_GRID) {
            if (!p->lsc_grid) return fail(IMOP_ERR_NULL_INPUT, "lsc_grid is null");
            if (p->lsc_grid_w < 2 || p->lsc_grid_h < 2 || p->lsc_grid_w > 1024 || p->lsc_grid_h > 1024)
                return fail(IMOP_ERR_INVALID_ARGUMENT, "lsc grid must be 2..1024 nodes per side");
        } else if (p->lsc_mode == IMOP_LSC_FLAT_FIELD) {
            if (!p->lsc_flat_field) return fail(IMOP_ERR_NULL_INPUT, "lsc_flat_field is null");
            if (p->lsc_flat_w <= 0 || p->lsc_flat_h <= 0) return fail(IMOP_ERR_INVALID_DIMENSIONS, "flat-field dims");
        } else if (p->lsc_mode != IMOP_LSC_POLYNOMIAL) {
            return fail(IMOP_ERR_INVALID_ARGUMENT, "lsc_mode");
        }
    }
    if (p->out_format != IMOP_OUT_RGB8 && p->out_format != IMOP_OUT_NATIVE)
        return fail(IMOP_ERR_INVALID_ARGUMENT, "out_format");
    if (p->out_format == IMOP_OUT_RGB8) {
        if (p->tone_mode == IMOP_TONE_LUT) {
            if (!p->tone_lut) return fail(IMOP_ERR_NULL_INPUT, "tone_lut is null");
            if (p->tone_lut_len != max_val_of(p->bit_depth) + 1)
                return fail(IMOP_ERR_INVALID_ARGUMENT, "tone_lut_len must be 2^bit_depth");
        } else if (p->tone_mode != IMOP_TONE_LINEAR && p->tone_mode != IMOP_TONE_KNOTS) {
            return fail(IMOP_ERR_INVALID_ARGUMENT, "tone_mode");
        }
    }
    return IMOP_OK;
}

int device_ready() {
    static int ready = -1;
    static std::once_flag once;
    std::call_once(once, [] {
        int n = 0;
        ready = (cudaGetDeviceCount(&n) == cudaSuccess && n > 0) ? 1 : 0;
    });
    return ready;
}

// Expand validated ImopIspParams into a FrameParams whose table pointers refer to `tabs`.
// Scalar expansion of validated parameters into FrameParams (no device or host allocation);
// table pointers are left null for the caller to fill.
void expand_frame_params(const ImopIspParams* p, FrameParams& fp) {
    std::memset(&fp, 0, sizeof(fp));
    fp.neg_zero = -0.0f;
    fp.w = p->width;
    fp.h = p->height;
    fp.bd = p->bit_depth;
    fp.mv = max_val_of(p->bit_depth);
    fp.fmt = input_format_of(p->packed, p->bit_depth);
    fp.pattern = p->pattern;
    fp.demosaic = p->demosaic;
    fp.border_mode = (p->demosaic == IMOP_DEMOSAIC_AMAZE && p->bit_depth <= 8) ? BORDER_BOTH : BORDER_ROWS_THEN_COLS;
    fp.stages = p->stages;
    if (p->stages & IMOP_STAGE_LUT3D) fp.lut3d_size = p->lut3d_size;  // the table pointer is the caller's to fill
    fp.stage_order = p->stage_order;
    fp.out_format = p->out_format;
    fp.out_bpc = (p->out_format == IMOP_OUT_NATIVE && p->bit_depth > 8) ? 2 : 1;
    fp.in_bytes = input_bytes_of(fp.fmt, fp.bd, fp.w, fp.h);
    for (int c = 0; c < 4; c++) {
        float v = (p->bl_mode == IMOP_BL_GLOBAL) ? p->bl_offset[0] : p->bl_offset[c];
        fp.bl[c] = std::max(0.0f, v);
    }
    // integral offsets: (int)((float)v - off) == v - off exactly, a saturating u16 subtract
    fp.bl_int = 1;
    for (int c = 0; c < 4; c++)
        if (!(fp.bl[c] == std::floor(fp.bl[c]) && fp.bl[c] <= 65535.0f)) fp.bl_int = 0;
    {
        PatternOffsets po = pattern_offsets(p->pattern);
        for (int par = 0; par < 2; par++) {
            uint32_t lo = (uint32_t)fp.bl[bayer_color(par, 0, po)], hi = (uint32_t)fp.bl[bayer_color(par, 1, po)];
            fp.bl2[par] = fp.bl_int ? (lo | (hi << 16)) : 0u;
            fp.bl_i[par][0] = fp.bl_int ? (int)lo : 0;
            fp.bl_i[par][1] = fp.bl_int ? (int)hi : 0;
        }
    }
    fp.mv2 = (uint32_t)fp.mv | ((uint32_t)fp.mv << 16);
    fp.dpc_mode = p->dpc_mode;
    {
        float t = std::max(0.05f, std::min(1.0f, p->dpc_threshold));
        fp.dpc_thr = (int)(t * (float)fp.mv);
        fp.thr2 = (uint32_t)fp.dpc_thr | ((uint32_t)fp.dpc_thr << 16);
    }
    fp.lsc_mode = (p->lsc_mode == IMOP_LSC_POLYNOMIAL) ? 1 : 0;
    if ((p->stages & IMOP_STAGE_LENS_SHADING) && p->lsc_mode == IMOP_LSC_POLYNOMIAL) {
        for (int c = 0; c < 4; c++)
            for (int k = 0; k < 3; k++) fp.poly[c][k] = p->lsc_poly[c][k];
        // src/lens_shading/polynomial.cpp:25-27
        fp.lsc_cx = p->lsc_center[0] * (float)fp.w;
        fp.lsc_cy = p->lsc_center[1] * (float)fp.h;
        fp.lsc_max_r = std::sqrt(fp.lsc_cx * fp.lsc_cx + fp.lsc_cy * fp.lsc_cy);
    }
    fp.wb_cfa[0] = p->wb_gain[0];
    fp.wb_cfa[1] = p->wb_gain[1];
    fp.wb_cfa[2] = p->wb_gain[1];
    fp.wb_cfa[3] = p->wb_gain[2];
    for (int i = 0; i < 3; i++) fp.wb_rgb[i] = p->wb_gain[i];
    for (int i = 0; i < 9; i++) fp.ccm[i] = p->ccm[i];
    fp.need_align = (fp.bd > 8 && fp.bd < 16 &&
                     !(p->stages & (IMOP_STAGE_BLACK_LEVEL | IMOP_STAGE_LENS_SHADING)) &&
                     !((p->stages & IMOP_STAGE_WHITE_BALANCE) && p->stage_order == IMOP_ORDER_BAYER_WB)) ? 1 : 0;
}

int upload_map_plan(const ImopIspParams* p, FrameTables& tabs, FrameParams& fp) {
    HostMapPlan P;
    build_map_plan(p->dpc_map, p->dpc_map_count, p->width, p->height, P);
    cudaError_t e;
    if ((e = upload(tabs.map_row_ptr, P.row_ptr)) || (e = upload(tabs.map_ent, P.ent)) ||
        (e = upload(tabs.slot_xy, P.slot_xy)) || (e = upload(tabs.comp_slot_ptr, P.comp_slot_ptr)) ||
        (e = upload(tabs.comp_slots, P.comp_slots)) || (e = upload(tabs.comp_ent_ptr, P.comp_ent_ptr)) ||
        (e = upload(tabs.comp_entries, P.comp_entries)) ||
        (e = tabs.map_val.ensure(std::max<size_t>(1, P.slot_xy.size()) * sizeof(int))))
        return cuda_fail(e, "upload defect map");
    fp.map_row_ptr = (const int*)tabs.map_row_ptr.ptr;
    fp.map_ent = (const int2*)tabs.map_ent.ptr;
    fp.map_val = (const int*)tabs.map_val.ptr;
    tabs.n_slots = (int)P.slot_xy.size();
    tabs.plan.n_comp = (int)P.comp_slot_ptr.size() - 1;
    tabs.plan.comp_slot_ptr = (const int*)tabs.comp_slot_ptr.ptr;
    tabs.plan.comp_slots = (const int*)tabs.comp_slots.ptr;
    tabs.plan.comp_ent_ptr = (const int*)tabs.comp_ent_ptr.ptr;
    tabs.plan.comp_entries = (const int*)tabs.comp_entries.ptr;
    tabs.plan.slot_xy = (const int2*)tabs.slot_xy.ptr;
    return IMOP_OK;
}

int build_frame_params(const ImopIspParams* p, FrameTables& tabs, FrameParams& fp, cudaStream_t st) {
    int rc = validate_params(p);
    if (rc) return rc;
    if (!device_ready()) return fail(IMOP_ERR_NO_DEVICE, "no CUDA device");
    expand_frame_params(p, fp);
    cudaError_t e;
    if ((p->stages & IMOP_STAGE_DEFECT) && p->dpc_mode == IMOP_DPC_MAP_BASED) {
        if ((rc = upload_map_plan(p, tabs, fp))) return rc;
    } else {
        tabs.plan.n_comp = 0;
    }
    if (p->stages & IMOP_STAGE_LENS_SHADING) {
        if (p->lsc_mode != IMOP_LSC_POLYNOMIAL) {
            std::vector<float> g;
            if (p->lsc_mode == IMOP_LSC_FLAT_FIELD) {
                rc = flat_field_grid(p->lsc_flat_field, p->lsc_flat_w, p->lsc_flat_h, p->pattern, p->bit_depth, g);
                if (rc) return rc;
                fp.gw = 32;
                fp.gh = 24;
            } else {
                g.assign(p->lsc_grid, p->lsc_grid + (size_t)p->lsc_grid_w * p->lsc_grid_h * 4);
                fp.gw = p->lsc_grid_w;
                fp.gh = p->lsc_grid_h;
            }
            if ((e = upload(tabs.grid, g))) return cuda_fail(e, "upload lens-shading grid");
            fp.grid = (const float*)tabs.grid.ptr;
            fp.lsc_bounded = lsc_grid_bounded(p);
        }
    }
    if (p->stages & IMOP_STAGE_LUT3D) {
        std::vector<float> l(p->lut3d, p->lut3d + (size_t)p->lut3d_size * p->lut3d_size * p->lut3d_size * 3);
        if ((e = upload(tabs.lut3d, l))) return cuda_fail(e, "upload 3D LUT");
        fp.lut3d = (const float*)tabs.lut3d.ptr;
    }
    // tone table (padded: the kernel reads it in 4-byte words)
    if ((e = tabs.tone8.ensure(std::max<size_t>((size_t)fp.mv + 1, 4096) + 16))) return cuda_fail(e, "alloc tone table");
    fp.tone8 = (const uint8_t*)tabs.tone8.ptr;
    if (p->out_format == IMOP_OUT_RGB8) {
        const float* d_lut = nullptr;
        const float* d_knots = nullptr;
        if (p->tone_mode == IMOP_TONE_LUT) {
            std::vector<float> l(p->tone_lut, p->tone_lut + p->tone_lut_len);
            if ((e = upload(tabs.lut, l))) return cuda_fail(e, "upload tone lut");
            d_lut = (const float*)tabs.lut.ptr;
        } else if (p->tone_mode == IMOP_TONE_KNOTS) {
            std::vector<float> k(p->tone_knots, p->tone_knots + 33);
            if ((e = upload(tabs.knots, k))) return cuda_fail(e, "upload tone knots");
            d_knots = (const float*)tabs.knots.ptr;
        }
        if ((e = launch_tone_table(p->tone_mode, d_lut, d_knots, fp.bd, (uint8_t*)tabs.tone8.ptr, st)))
            return cuda_fail(e, "tone table kernel");
    }
    return IMOP_OK;
}

int ensure_fixup(FixupState& fx, int cap) {
    cudaError_t e;
    if (fx.cap >= cap && fx.seed_count.ptr) return IMOP_OK;
    if ((e = fx.seed_count.ensure(sizeof(int))) || (e = fx.status.ensure(sizeof(int))) ||
        (e = fx.tile_counter.ensure(sizeof(int))) || (e = fx.seg.ensure(kStreamSegCap * sizeof(unsigned long long))) ||
        (e = fx.seeds.ensure((size_t)cap * sizeof(int))) || (e = fx.heap.ensure((size_t)cap * sizeof(int))) ||
        (e = fx.ov_idx.ensure((size_t)cap * sizeof(int))) || (e = fx.ov_val.ensure((size_t)cap * sizeof(int))) ||
        (e = fx.n_ov.ensure(sizeof(int))))
        return cuda_fail(e, "alloc defect-chain scratch");
    if ((e = cudaMemset(fx.status.ptr, 0, sizeof(int))) || (e = cudaMemset(fx.seed_count.ptr, 0, sizeof(int))) ||
        (e = cudaMemset(fx.n_ov.ptr, 0, sizeof(int))))
        return cuda_fail(e, "clear defect-chain scratch");
    fx.cap = cap;
    return IMOP_OK;
}

// [p, p + n) is page-locked host memory that the device addresses at the same pointer, so a kernel
// may store into it directly
bool device_mapped_host(const void* p, size_t n) {
    if (!p || n == 0) return false;
    const void* ends[2] = {p, static_cast<const char*>(p) + (n - 1)};
    for (const void* q : ends) {
        cudaPointerAttributes a{};
        if (cudaPointerGetAttributes(&a, q) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        if (a.type != cudaMemoryTypeHost || a.devicePointer != q) return false;
    }
    return true;
}

void attach_fixup(FixupState& fx, FrameParams& fp, FixupScratch& fs) {
    fp.seed_count = (int*)fx.seed_count.ptr;
    fp.seeds = (int*)fx.seeds.ptr;
    fp.seed_cap = fx.cap;
    fp.status = (int*)fx.status.ptr;
    fp.tile_counter = (int*)fx.tile_counter.ptr;
    fp.seg_words = (unsigned long long*)fx.seg.ptr;
    fp.seg_cap = kStreamSegCap;
    fs.heap = (int*)fx.heap.ptr;
    fs.ov_idx = (int*)fx.ov_idx.ptr;
    fs.ov_val = (int*)fx.ov_val.ptr;
    fs.n_ov = (int*)fx.n_ov.ptr;
    fs.cap = fx.cap;
}

// read and clear the sticky device status word
int take_status(FixupState& fx) {
    int s = 0;
    cudaError_t e = cudaMemcpy(&s, fx.status.ptr, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "read status");
    if (s) {
        cudaMemset(fx.status.ptr, 0, sizeof(int));
        return fail(s, s == IMOP_ERR_CAPACITY ? "defect-chain list capacity exceeded" : "device status error");
    }
    return IMOP_OK;
}

}  // namespace imop

// ==== C ABI ===================================================================================
extern "C" {

const char* imop_last_error_string(void) { return t_last_error.c_str(); }
int imop_abi_version(void) { return IMOP_ISP_ABI_VERSION; }
int imop_has_cuda(void) { return device_ready(); }

const char* imop_device_name(void) {
    thread_local char name[256];
    name[0] = 0;
    int dev = 0;
    cudaDeviceProp prop;
    if (device_ready() && cudaGetDevice(&dev) == cudaSuccess && cudaGetDeviceProperties(&prop, dev) == cudaSuccess) {
        std::strncpy(name, prop.name, sizeof(name) - 1);
        name[sizeof(name) - 1] = 0;
    }
    return name;
}

void imop_isp_params_default(ImopIspParams* p, int width, int height, int bit_depth, int packed) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->width = width;
    p->height = height;
    p->bit_depth = bit_depth;
    p->packed = packed;
    p->pattern = IMOP_RGGB;
    p->demosaic = IMOP_DEMOSAIC_HQLI;
    p->stages = 0;
    p->stage_order = IMOP_ORDER_BAYER_WB;
    p->dpc_threshold = 0.3f;
    p->lsc_center[0] = p->lsc_center[1] = 0.5f;
    p->wb_gain[0] = p->wb_gain[1] = p->wb_gain[2] = 1.0f;
    p->ccm[0] = p->ccm[4] = p->ccm[8] = 1.0f;
    p->tone_mode = IMOP_TONE_LINEAR;
    for (int i = 0; i < 33; i++) p->tone_knots[i] = (float)i / 32.0f;
    p->out_format = IMOP_OUT_RGB8;
}

size_t imop_isp_input_bytes(const ImopIspParams* p) {
    if (!p || p->width <= 0 || p->height <= 0) return 0;
    return input_bytes_of(input_format_of(p->packed, p->bit_depth), p->bit_depth, p->width, p->height);
}

size_t imop_isp_output_bytes(const ImopIspParams* p) {
    if (!p || p->width <= 0 || p->height <= 0) return 0;
    size_t n = (size_t)p->width * p->height * 3;
    return (p->out_format == IMOP_OUT_NATIVE && p->bit_depth > 8) ? 2 * n : n;
}

int imop_isp_create(imop_isp_t* out) {
    if (!out) return fail(IMOP_ERR_NULL_INPUT, "out_ctx is null");
    *out = nullptr;
    if (!device_ready()) return fail(IMOP_ERR_NO_DEVICE, "no CUDA device");
    imop_isp_ctx* c = new (std::nothrow) imop_isp_ctx();
    if (!c) return fail(IMOP_ERR_INTERNAL, "out of host memory");
    int rc = ensure_fixup(c->fix, 1 << 16);
    if (rc) {
        delete c;
        return rc;
    }
    *out = c;
    return IMOP_OK;
}

int imop_isp_destroy(imop_isp_t ctx) {
    if (!ctx) return fail(IMOP_ERR_NULL_INPUT, "ctx is null");
    cudaDeviceSynchronize();
    delete ctx;
    return IMOP_OK;
}

int imop_isp_set_params(imop_isp_t ctx, const ImopIspParams* p) {
    if (!ctx) return fail(IMOP_ERR_NULL_INPUT, "ctx is null");
    FrameParams fp;
    int rc = build_frame_params(p, ctx->tabs, fp, 0);
    if (rc) return rc;
    cudaError_t e = cudaStreamSynchronize(0);
    if (e != cudaSuccess) return cuda_fail(e, "set_params");
    ctx->params = *p;
    ctx->fp = fp;
    ctx->has_params = true;
    return IMOP_OK;
}

int imop_isp_set_tile(imop_isp_t ctx, int tile_w, int tile_h) {
    if (!ctx) return fail(IMOP_ERR_NULL_INPUT, "ctx is null");
    if (!((tile_w == 0 && tile_h == 0) || (tile_w == kTileW && tile_h == kTileH)))
        return fail(IMOP_ERR_UNSUPPORTED, "tile shape not compiled in");
    return IMOP_OK;
}

int imop_isp_run_device(imop_isp_t ctx, const void* d_in, void* d_out, void* stream) {
    if (!ctx) return fail(IMOP_ERR_NULL_INPUT, "ctx is null");
    if (!d_in || !d_out) return fail(IMOP_ERR_NULL_INPUT, "null frame pointer");
    if (!ctx->has_params) return fail(IMOP_ERR_INVALID_ARGUMENT, "set_params first");
    FrameParams fp = ctx->fp;
    fp.in = (const uint8_t*)d_in;
    fp.out = (uint8_t*)d_out;
    FixupScratch fs;
    attach_fixup(ctx->fix, fp, fs);
    cudaError_t e = launch_fused(fp, fs, &ctx->tabs.plan, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "fused launch");
    return IMOP_OK;
}

int imop_isp_run_device_plain(imop_isp_t ctx, const void* d_in, void* d_out, void* stream) {
    if (!ctx) return fail(IMOP_ERR_NULL_INPUT, "ctx is null");
    if (!d_in || !d_out) return fail(IMOP_ERR_NULL_INPUT, "null frame pointer");
    if (!ctx->has_params) return fail(IMOP_ERR_INVALID_ARGUMENT, "set_params first");
    FrameParams fp = ctx->fp;
    fp.in = (const uint8_t*)d_in;
    fp.out = (uint8_t*)d_out;
    size_t n = (size_t)fp.w * fp.h;
    cudaError_t e;
    if ((e = ctx->plain_a.ensure(n * 4)) || (e = ctx->plain_b.ensure(n * 4)) || (e = ctx->plain_rgb.ensure(n * 6)))
        return cuda_fail(e, "alloc plain buffers");
    FixupScratch fs;
    attach_fixup(ctx->fix, fp, fs);
    PlainBuffers b{(uint16_t*)ctx->plain_a.ptr, (uint16_t*)ctx->plain_b.ptr, (uint16_t*)ctx->plain_rgb.ptr};
    e = launch_plain(fp, fs, &ctx->tabs.plan, b, nullptr, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "plain launch");
    return IMOP_OK;
}

int imop_isp_run_host(imop_isp_t ctx, const void* in, size_t in_bytes, void* out, size_t out_bytes) {
    if (!ctx) return fail(IMOP_ERR_NULL_INPUT, "ctx is null");
    if (!in || !out) return fail(IMOP_ERR_NULL_INPUT, "null frame pointer");
    if (!ctx->has_params) return fail(IMOP_ERR_INVALID_ARGUMENT, "set_params first");
    size_t ib = imop_isp_input_bytes(&ctx->params), ob = imop_isp_output_bytes(&ctx->params);
    if (in_bytes < ib || out_bytes < ob) return fail(IMOP_ERR_INVALID_ARGUMENT, "buffer smaller than one frame");
    cudaError_t e;
    if ((e = ctx->d_in.ensure(ib)) || (e = ctx->d_out.ensure(ob))) return cuda_fail(e, "alloc staging frames");
    cudaStream_t st = 0;
    if ((e = cudaMemcpyAsync(ctx->d_in.ptr, in, ib, cudaMemcpyHostToDevice, st))) return cuda_fail(e, "H2D");
    int rc = imop_isp_run_device(ctx, ctx->d_in.ptr, ctx->d_out.ptr, st);
    if (rc) return rc;
    if ((e = cudaMemcpyAsync(out, ctx->d_out.ptr, ob, cudaMemcpyDeviceToHost, st))) return cuda_fail(e, "D2H");
    if ((e = cudaStreamSynchronize(st))) return cuda_fail(e, "run_host");
    return take_status(ctx->fix);
}

int imop_isp_dump_stages(imop_isp_t ctx, const void* in, size_t in_bytes, ImopStageDumps* dumps) {
    if (!ctx || !in || !dumps) return fail(IMOP_ERR_NULL_INPUT, "null argument");
    if (!ctx->has_params) return fail(IMOP_ERR_INVALID_ARGUMENT, "set_params first");
    FrameParams fp = ctx->fp;
    size_t ib = imop_isp_input_bytes(&ctx->params), ob = imop_isp_output_bytes(&ctx->params);
    if (in_bytes < ib) return fail(IMOP_ERR_INVALID_ARGUMENT, "input smaller than one frame");
    size_t n = (size_t)fp.w * fp.h;
    cudaError_t e;
    DevBuf dd[7];
    if ((e = ctx->d_in.ensure(ib)) || (e = ctx->d_out.ensure(ob)) || (e = ctx->plain_a.ensure(n * 4)) ||
        (e = ctx->plain_b.ensure(n * 4)) || (e = ctx->plain_rgb.ensure(n * 6)))
        return cuda_fail(e, "alloc dump buffers");
    const bool rgb_wb = fp.stage_order == 1;
    const size_t cnt[7] = {n, n, n, n, rgb_wb ? 3 * n : n, 3 * n, 3 * n};
    uint16_t* host[7] = {dumps->unpacked, dumps->black_level, dumps->defect, dumps->lens_shading,
                         dumps->white_balance, dumps->demosaic, dumps->ccm};
    uint16_t* dev[7] = {nullptr};
    for (int i = 0; i < 7; i++)
        if (host[i]) {
            if ((e = dd[i].ensure(cnt[i] * 2))) return cuda_fail(e, "alloc dump");
            dev[i] = (uint16_t*)dd[i].ptr;
        }
    if ((e = cudaMemcpy(ctx->d_in.ptr, in, ib, cudaMemcpyHostToDevice))) return cuda_fail(e, "H2D");
    fp.in = (const uint8_t*)ctx->d_in.ptr;
    fp.out = (uint8_t*)ctx->d_out.ptr;
    FixupScratch fs;
    attach_fixup(ctx->fix, fp, fs);
    PlainBuffers b{(uint16_t*)ctx->plain_a.ptr, (uint16_t*)ctx->plain_b.ptr, (uint16_t*)ctx->plain_rgb.ptr};
    PlainDumps pd{dev[0], dev[1], dev[2], dev[3], dev[4], dev[5], dev[6]};
    if ((e = launch_plain(fp, fs, &ctx->tabs.plan, b, &pd, 0))) return cuda_fail(e, "plain launch");
    if ((e = cudaDeviceSynchronize())) return cuda_fail(e, "dump_stages");
    for (int i = 0; i < 7; i++)
        if (host[i] && (e = cudaMemcpy(host[i], dev[i], cnt[i] * 2, cudaMemcpyDeviceToHost)))
            return cuda_fail(e, "D2H dump");
    if (dumps->output && (e = cudaMemcpy(dumps->output, ctx->d_out.ptr, ob, cudaMemcpyDeviceToHost)))
        return cuda_fail(e, "D2H output");
    return take_status(ctx->fix);
}

int imop_isp_last_stats(imop_isp_t ctx, int* dpc_seeds, int* dpc_overrides) {
    if (!ctx) return fail(IMOP_ERR_NULL_INPUT, "ctx is null");
    int s = 0, o = 0;
    cudaError_t e;
    if ((e = cudaDeviceSynchronize())) return cuda_fail(e, "sync");
    if ((e = cudaMemcpy(&s, ctx->fix.seed_count.ptr, sizeof(int), cudaMemcpyDeviceToHost))) return cuda_fail(e, "stats");
    if ((e = cudaMemcpy(&o, ctx->fix.n_ov.ptr, sizeof(int), cudaMemcpyDeviceToHost))) return cuda_fail(e, "stats");
    if (dpc_seeds) *dpc_seeds = s;
    if (dpc_overrides) *dpc_overrides = s ? o : 0;
    return IMOP_OK;
}

static int op_prepare(imop_isp_t ctx, const ImopIspParams* p, unsigned stage, ImopIspParams& q, FrameParams& fp) {
    if (!ctx) return fail(IMOP_ERR_NULL_INPUT, "ctx is null");
    if (!p) return fail(IMOP_ERR_NULL_INPUT, "params is null");
    q = *p;
    q.stages = stage;
    q.packed = 0;
    q.out_format = IMOP_OUT_NATIVE;
    q.stage_order = IMOP_ORDER_RGB_WB;
    // the operator tables are separate from the ones set_params built for run_device
    int rc = build_frame_params(&q, ctx->op_tabs, fp, 0);
    if (rc) return rc;
    return IMOP_OK;
}

int imop_op_bayer_stage(imop_isp_t ctx, const ImopIspParams* p, unsigned stage, void* data) {
    if (stage != IMOP_STAGE_BLACK_LEVEL && stage != IMOP_STAGE_DEFECT && stage != IMOP_STAGE_LENS_SHADING)
        return fail(IMOP_ERR_INVALID_ARGUMENT, "not a Bayer stage");
    if (!data) return fail(IMOP_ERR_NULL_INPUT, "null frame pointer");
    ImopIspParams q;
    FrameParams fp;
    int rc = op_prepare(ctx, p, stage, q, fp);
    if (rc) return rc;
    const size_t n = (size_t)fp.w * fp.h;
    const int bps = fp.bd <= 8 ? 1 : 2;
    cudaError_t e;
    if ((e = ctx->d_in.ensure(n * bps)) || (e = ctx->plain_a.ensure(n * 2)) || (e = ctx->plain_b.ensure(n * 2)))
        return cuda_fail(e, "alloc operator buffers");
    uint16_t* a = (uint16_t*)ctx->plain_a.ptr;
    FixupScratch fs;
    attach_fixup(ctx->fix, fp, fs);
    // the frame's own bytes are the input of the stage: map-mode defect values read them there
    fp.in = (const uint8_t*)ctx->d_in.ptr;
    fp.out = nullptr;
    if ((e = cudaMemcpy(ctx->d_in.ptr, data, n * bps, cudaMemcpyHostToDevice)) ||
        (e = launch_widen((const uint8_t*)ctx->d_in.ptr, a, n, bps, 0)) ||
        (e = launch_op_bayer(fp, stage, fs, &ctx->op_tabs.plan, a, (uint16_t*)ctx->plain_b.ptr, 0)) ||
        (e = launch_narrow(a, (uint8_t*)ctx->d_in.ptr, n, bps, 0)) ||
        (e = cudaMemcpy(data, ctx->d_in.ptr, n * bps, cudaMemcpyDeviceToHost)))
        return cuda_fail(e, "bayer stage");
    return take_status(ctx->fix);
}

int imop_op_rgb_stage(imop_isp_t ctx, const ImopIspParams* p, unsigned stage, const void* in, void* out) {
    if (stage != IMOP_STAGE_WHITE_BALANCE && stage != IMOP_STAGE_CCM && stage != IMOP_STAGE_LUT3D)
        return fail(IMOP_ERR_INVALID_ARGUMENT, "not an RGB stage");
    if (!in || !out) return fail(IMOP_ERR_NULL_INPUT, "null frame pointer");
    ImopIspParams q;
    FrameParams fp;
    int rc = op_prepare(ctx, p, stage, q, fp);
    if (rc) return rc;
    const size_t n = (size_t)fp.w * fp.h * 3;
    const int bps = fp.bd <= 8 ? 1 : 2;
    cudaError_t e;
    if ((e = ctx->d_in.ensure(n * bps)) || (e = ctx->plain_rgb.ensure(n * 2))) return cuda_fail(e, "alloc operator buffers");
    uint16_t* rgb = (uint16_t*)ctx->plain_rgb.ptr;
    if ((e = cudaMemcpy(ctx->d_in.ptr, in, n * bps, cudaMemcpyHostToDevice)) ||
        (e = launch_widen((const uint8_t*)ctx->d_in.ptr, rgb, n, bps, 0)) || (e = launch_op_rgb(fp, stage, rgb, 0)) ||
        (e = launch_narrow(rgb, (uint8_t*)ctx->d_in.ptr, n, bps, 0)) ||
        (e = cudaMemcpy(out, ctx->d_in.ptr, n * bps, cudaMemcpyDeviceToHost)))
        return cuda_fail(e, "rgb stage");
    return IMOP_OK;
}

}  // extern "C"
