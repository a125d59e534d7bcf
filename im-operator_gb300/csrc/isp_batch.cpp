// isp_batch.cpp - batches of frames with their own sizes, formats and parameter sets.
//
// imop_isp_batch_submit: every frame's parameters are expanded into a FrameParams whose table
// pointers come from the context's TableCache (one device copy per distinct grid / tone table /
// defect map / bit depth), each frame gets its own defect-chain scratch, and the frames go to the
// persistent fused kernels together: one launch walks the work of up to 32 frames.  With
// IMOP_BATCH_GRAPH the launches are recorded once into a CUDA graph and replayed while the
// descriptors stay the same.
//
// imop_isp_run_host_batch: the drop-in shape of imop::demosaic_cuda_batch
// (src/algorithms/cuda_dispatch.cpp:150-209), which double-buffers pinned staging copies around a
// graph per frame.  Here the caller's host frames are copied straight into one of four device
// slots on a copy-in stream, computed on two compute streams (consecutive frames alternate), their
// defect chains resolved on a fix-up stream, and copied back on a copy-out stream, with events
// between them, so frame k+1 is copied in and frame k-1 copied out while frame k runs.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <initializer_list>
#include <vector>

#include "../../include/imop_isp.h"
#include "isp_common.h"
#include "isp_context.h"
#include "isp_kernels.h"

namespace imop {
namespace {

constexpr int kBatchSeedCap = 16384;  // defect-chain entries per frame of a batch
constexpr size_t kCacheMaxEntries = 1024;

// Content key: the bytes that determine a table (or a recorded batch) and a hash of them.  The
// hash runs four independent multiply / xor-shift lanes over 8-byte words, so a 16 KB tone table
// hashes in a few microseconds; equality of the bytes themselves is what a cache hit requires.
struct Key {
    std::vector<uint8_t> b;
    void bytes(const void* p, size_t n) {
        const uint8_t* q = static_cast<const uint8_t*>(p);
        b.insert(b.end(), q, q + n);
    }
    template <class T>
    void val(const T& v) { bytes(&v, sizeof(T)); }
    uint64_t hash() const {
        const uint64_t M = 0xff51afd7ed558ccdull;
        uint64_t h[4] = {0x9e3779b97f4a7c15ull, 0xc2b2ae3d27d4eb4full, 0x165667b19e3779f9ull, 0x27d4eb2f165667c5ull};
        const size_t n = b.size();
        size_t i = 0;
        for (; i + 32 <= n; i += 32)
            for (int l = 0; l < 4; l++) {
                uint64_t w;
                std::memcpy(&w, b.data() + i + 8 * l, 8);
                h[l] = (h[l] ^ w) * M;
                h[l] ^= h[l] >> 32;
            }
        uint64_t r = n;
        for (; i < n; i++) r = (r ^ b[i]) * 0x100000001b3ull;
        for (int l = 0; l < 4; l++) {
            r ^= h[l] + 0x9e3779b97f4a7c15ull + (r << 6) + (r >> 2);
            r *= M;
            r ^= r >> 33;
        }
        return r;
    }
};

// the cache entry of `k`: an empty entry to build on a miss; an entry with other content under
// the same hash is emptied once the device has finished with it
template <class T>
int cache_entry(imop_isp_ctx* c, std::unordered_map<uint64_t, CacheEntry<T>>& m, Key& k, CacheEntry<T>*& out) {
    CacheEntry<T>& ent = m[k.hash()];
    if (ent.obj && ent.key != k.b) {
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) return cuda_fail(e, "sync before cache replacement");
        ent.obj.reset();
        c->graph.key = 0;
    }
    if (!ent.obj) ent.key = k.b;
    out = &ent;
    return IMOP_OK;
}

int ensure_aux(imop_isp_ctx* c) {
    if (c->aux) return IMOP_OK;
    cudaError_t e = cudaStreamCreateWithFlags(&c->aux, cudaStreamNonBlocking);
    return e == cudaSuccess ? IMOP_OK : cuda_fail(e, "create stream");
}

// Table pointers of one parameter set, built on a cache miss (synchronously, on the aux stream).
int resolve_tables(imop_isp_ctx* c, const ImopIspParams* p, FrameParams& fp, const FrameTables** map_tabs) {
    TableCache& tc = c->cache;
    cudaError_t e;
    int rc;
    *map_tabs = nullptr;
    if (tc.entries() > kCacheMaxEntries) {
        // drop everything once the cache is large; nothing enqueued may still read it
        if ((e = cudaDeviceSynchronize())) return cuda_fail(e, "sync before cache reset");
        tc.grids.clear();
        tc.tones.clear();
        tc.lut3ds.clear();
        tc.maps.clear();
        c->graph.key = 0;
    }
    if ((p->stages & IMOP_STAGE_DEFECT) && p->dpc_mode == IMOP_DPC_MAP_BASED) {
        Key k;
        k.val(p->width);
        k.val(p->height);
        k.bytes(p->dpc_map, sizeof(ImopDefectPoint) * (size_t)std::max(0, p->dpc_map_count));
        CacheEntry<FrameTables>* ent = nullptr;
        if ((rc = cache_entry(c, tc.maps, k, ent))) return rc;
        auto& slot = ent->obj;
        if (!slot) {
            slot.reset(new FrameTables());
            FrameParams tmp;
            if ((rc = upload_map_plan(p, *slot, tmp))) {
                tc.maps.erase(k.hash());
                return rc;
            }
        }
        fp.map_row_ptr = (const int*)slot->map_row_ptr.ptr;
        fp.map_ent = (const int2*)slot->map_ent.ptr;
        fp.map_val = (const int*)slot->map_val.ptr;
        *map_tabs = slot.get();
    }
    if ((p->stages & IMOP_STAGE_LENS_SHADING) && p->lsc_mode != IMOP_LSC_POLYNOMIAL) {
        Key k;
        k.val(p->lsc_mode);
        if (p->lsc_mode == IMOP_LSC_FLAT_FIELD) {
            k.val(p->lsc_flat_w);
            k.val(p->lsc_flat_h);
            k.val(p->pattern);
            k.val(p->bit_depth);
            k.bytes(p->lsc_flat_field, (size_t)p->lsc_flat_w * p->lsc_flat_h * (p->bit_depth <= 8 ? 1 : 2));
        } else {
            k.val(p->lsc_grid_w);
            k.val(p->lsc_grid_h);
            k.bytes(p->lsc_grid, sizeof(float) * 4 * (size_t)p->lsc_grid_w * p->lsc_grid_h);
        }
        CacheEntry<DevBuf>* ent = nullptr;
        if ((rc = cache_entry(c, tc.grids, k, ent))) return rc;
        auto& slot = ent->obj;
        if (!slot) {
            std::vector<float> g;
            if (p->lsc_mode == IMOP_LSC_FLAT_FIELD) {
                if ((rc = flat_field_grid(p->lsc_flat_field, p->lsc_flat_w, p->lsc_flat_h, p->pattern, p->bit_depth, g))) {
                    tc.grids.erase(k.hash());
                    return rc;
                }
            } else {
                g.assign(p->lsc_grid, p->lsc_grid + (size_t)p->lsc_grid_w * p->lsc_grid_h * 4);
            }
            slot.reset(new DevBuf());
            if ((e = upload(*slot, g))) {
                tc.grids.erase(k.hash());
                return cuda_fail(e, "upload lens-shading grid");
            }
        }
        fp.gw = p->lsc_mode == IMOP_LSC_FLAT_FIELD ? 32 : p->lsc_grid_w;
        fp.gh = p->lsc_mode == IMOP_LSC_FLAT_FIELD ? 24 : p->lsc_grid_h;
        fp.grid = (const float*)slot->ptr;
        fp.lsc_bounded = lsc_grid_bounded(p);
    }
    if (p->stages & IMOP_STAGE_LUT3D) {
        Key k;
        k.val(p->lut3d_size);
        k.bytes(p->lut3d, sizeof(float) * 3 * (size_t)p->lut3d_size * p->lut3d_size * p->lut3d_size);
        CacheEntry<DevBuf>* ent = nullptr;
        if ((rc = cache_entry(c, tc.lut3ds, k, ent))) return rc;
        if (!ent->obj) {
            std::vector<float> l(p->lut3d, p->lut3d + 3 * (size_t)p->lut3d_size * p->lut3d_size * p->lut3d_size);
            std::unique_ptr<DevBuf> d(new DevBuf());
            if ((e = upload(*d, l))) {
                tc.lut3ds.erase(k.hash());
                return cuda_fail(e, "upload 3D LUT");
            }
            ent->obj = std::move(d);
        }
        fp.lut3d = (const float*)ent->obj->ptr;
    }
    {
        Key k;
        k.val(p->out_format);
        k.val(p->bit_depth);
        if (p->out_format == IMOP_OUT_RGB8) {
            k.val(p->tone_mode);
            if (p->tone_mode == IMOP_TONE_LUT) k.bytes(p->tone_lut, sizeof(float) * (size_t)p->tone_lut_len);
            if (p->tone_mode == IMOP_TONE_KNOTS) k.bytes(p->tone_knots, sizeof(float) * 33);
        }
        CacheEntry<DevBuf>* ent = nullptr;
        if ((rc = cache_entry(c, tc.tones, k, ent))) return rc;
        auto& slot = ent->obj;
        if (!slot) {
            std::unique_ptr<DevBuf> t(new DevBuf());
            if ((e = t->ensure(std::max<size_t>((size_t)fp.mv + 1, 4096) + 16))) return cuda_fail(e, "alloc tone table");
            if ((e = cudaMemsetAsync(t->ptr, 0, t->size, c->aux))) return cuda_fail(e, "clear tone table");
            if (p->out_format == IMOP_OUT_RGB8) {
                DevBuf lut;
                const float* d_lut = nullptr;
                const float* d_knots = nullptr;
                if (p->tone_mode == IMOP_TONE_LUT) {
                    std::vector<float> l(p->tone_lut, p->tone_lut + p->tone_lut_len);
                    if ((e = upload(lut, l))) return cuda_fail(e, "upload tone lut");
                    d_lut = (const float*)lut.ptr;
                } else if (p->tone_mode == IMOP_TONE_KNOTS) {
                    std::vector<float> k(p->tone_knots, p->tone_knots + 33);
                    if ((e = upload(lut, k))) return cuda_fail(e, "upload tone knots");
                    d_knots = (const float*)lut.ptr;
                }
                if ((e = launch_tone_table(p->tone_mode, d_lut, d_knots, fp.bd, (uint8_t*)t->ptr, c->aux)))
                    return cuda_fail(e, "tone table kernel");
            }
            if ((e = cudaStreamSynchronize(c->aux))) return cuda_fail(e, "tone table");
            slot = std::move(t);
        }
        fp.tone8 = (const uint8_t*)slot->ptr;
    }
    return IMOP_OK;
}

int ensure_batch_scratch(imop_isp_ctx* c, int n, int map_slots) {
    BatchScratch& b = c->batch;
    if (b.frames >= n && b.map_cap >= map_slots && b.seed_count.ptr) return IMOP_OK;
    // buffers may be in use by enqueued batches
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_fail(e, "sync before batch scratch growth");
    int frames = std::max(n, b.frames), cap = kBatchSeedCap, mcap = std::max(map_slots, b.map_cap);
    size_t per = (size_t)frames * cap * sizeof(int);
    if ((e = b.seed_count.ensure(frames * sizeof(int))) || (e = b.n_ov.ensure(frames * sizeof(int))) ||
        (e = b.seeds.ensure(per)) || (e = b.heap.ensure(per)) || (e = b.ov_idx.ensure(per)) ||
        (e = b.ov_val.ensure(per)) || (e = b.map_val.ensure((size_t)frames * std::max(1, mcap) * sizeof(int))))
        return cuda_fail(e, "alloc batch scratch");
    if ((e = cudaMemset(b.seed_count.ptr, 0, frames * sizeof(int))) || (e = cudaMemset(b.n_ov.ptr, 0, frames * sizeof(int))))
        return cuda_fail(e, "clear batch scratch");
    b.frames = frames;
    b.cap = cap;
    b.map_cap = mcap;
    c->graph.key = 0;  // recorded graphs point at the old buffers
    return IMOP_OK;
}

struct PreparedFrame {
    FrameParams fp;
    const FrameTables* map_tabs;
};

// expand, validate and attach tables + scratch for every frame of a device batch
int prepare_batch(imop_isp_ctx* c, const ImopFrameDesc* frames, int n, std::vector<PreparedFrame>& out) {
    int map_slots = 0;
    out.resize(n);
    for (int i = 0; i < n; i++) {
        const ImopIspParams* p = frames[i].params ? frames[i].params : (c->has_params ? &c->params : nullptr);
        if (!p) return set_error(IMOP_ERR_INVALID_ARGUMENT, "frame without parameters and no set_params");
        int rc = validate_params(p);
        if (rc) return rc;
        if (!frames[i].in || !frames[i].out) return set_error(IMOP_ERR_NULL_INPUT, "null frame pointer");
        FrameParams& fp = out[i].fp;
        expand_frame_params(p, fp);
        if ((rc = resolve_tables(c, p, fp, &out[i].map_tabs))) return rc;
        if (out[i].map_tabs) map_slots = std::max(map_slots, out[i].map_tabs->n_slots);
        fp.in = (const uint8_t*)frames[i].in;
        fp.out = (uint8_t*)frames[i].out;
    }
    int rc = ensure_batch_scratch(c, n, map_slots);
    if (rc) return rc;
    BatchScratch& b = c->batch;
    for (int i = 0; i < n; i++) {
        FrameParams& fp = out[i].fp;
        size_t off = (size_t)i * b.cap;
        fp.seed_count = (int*)b.seed_count.ptr + i;
        fp.seeds = (int*)b.seeds.ptr + off;
        fp.seed_cap = b.cap;
        fp.status = (int*)c->fix.status.ptr;
        fp.tile_counter = (int*)c->fix.tile_counter.ptr;
        fp.seg_words = (unsigned long long*)c->fix.seg.ptr;
        fp.seg_cap = c->fix.seg.ptr ? kStreamSegCap : 0;
        fp.fix_heap = (int*)b.heap.ptr + off;
        fp.fix_ov_idx = (int*)b.ov_idx.ptr + off;
        fp.fix_ov_val = (int*)b.ov_val.ptr + off;
        fp.fix_n_ov = (int*)b.n_ov.ptr + i;
        fp.fix_cap = b.cap;
        if (out[i].map_tabs) fp.map_val = (const int*)b.map_val.ptr + (size_t)i * std::max(1, b.map_cap);
    }
    return IMOP_OK;
}

// the batch's device work, in stream order
cudaError_t enqueue_batch(imop_isp_ctx* c, std::vector<PreparedFrame>& pf, cudaStream_t st) {
    const int n = (int)pf.size();
    cudaError_t e = cudaSuccess;
    // the defect-chain seed counters, when a frame runs adaptive defect correction
    bool seeds = false;
    for (auto& f : pf) seeds = seeds || ((f.fp.stages & 2u) && f.fp.dpc_mode == 0);
    if (seeds && (e = cudaMemsetAsync(c->batch.seed_count.ptr, 0, n * sizeof(int), st)) != cudaSuccess) return e;
    for (auto& f : pf)
        if (f.map_tabs && (e = launch_map_resolve(f.fp, f.map_tabs->plan, st))) return e;
    std::vector<FrameParams> fps(n);
    for (int i = 0; i < n; i++) fps[i] = pf[i].fp;
    return launch_fused_batch(fps.data(), n, st);
}

Key batch_key(const std::vector<PreparedFrame>& pf, cudaStream_t st) {
    Key k;
    k.val(st);
    k.val(tuning_generation());  // a new tuning table records anew
    int n = (int)pf.size();
    k.val(n);
    for (auto& f : pf) k.bytes(&f.fp, sizeof(FrameParams));
    return k;
}

int submit_plain(imop_isp_ctx* c, std::vector<PreparedFrame>& pf, cudaStream_t st) {
    size_t maxn = 0;
    for (auto& f : pf) maxn = std::max(maxn, (size_t)f.fp.w * f.fp.h);
    cudaError_t e;
    if ((e = c->plain_a.ensure(maxn * 4)) || (e = c->plain_b.ensure(maxn * 4)) || (e = c->plain_rgb.ensure(maxn * 6)))
        return cuda_fail(e, "alloc plain buffers");
    PlainBuffers b{(uint16_t*)c->plain_a.ptr, (uint16_t*)c->plain_b.ptr, (uint16_t*)c->plain_rgb.ptr};
    for (auto& f : pf) {
        FrameParams fp = f.fp;
        FixupScratch fs{fp.fix_heap, fp.fix_ov_idx, fp.fix_ov_val, fp.fix_n_ov, fp.fix_cap};
        if ((e = launch_plain(fp, fs, f.map_tabs ? &f.map_tabs->plan : nullptr, b, nullptr, st)))
            return cuda_fail(e, "plain launch");
    }
    return IMOP_OK;
}

}  // namespace

HostPipeline::~HostPipeline() {  // also after a set-up that failed half way
    for (cudaStream_t st : {s_in, s_comp[0], s_comp[1], s_fix, s_out})
        if (st) cudaStreamDestroy(st);
    for (int i = 0; i < kSlots; i++)
        for (cudaEvent_t ev : {in_done[i], main_done[i], fix_done[i], out_done[i]})
            if (ev) cudaEventDestroy(ev);
}

BatchGraph::~BatchGraph() {
    if (exec) cudaGraphExecDestroy(exec);
}

}  // namespace imop

using namespace imop;

imop_isp_ctx::~imop_isp_ctx() {
    if (aux) cudaStreamDestroy(aux);
}

extern "C" int imop_isp_sync_status(imop_isp_t ctx, void* stream) {
    if (!ctx) return set_error(IMOP_ERR_NULL_INPUT, "ctx is null");
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "sync");
    return take_status(ctx->fix);
}

extern "C" int imop_isp_batch_submit(imop_isp_t ctx, const ImopFrameDesc* frames, int n, unsigned flags, void* stream) {
    if (!ctx) return set_error(IMOP_ERR_NULL_INPUT, "ctx is null");
    if (n < 0) return set_error(IMOP_ERR_INVALID_ARGUMENT, "negative frame count");
    if (n == 0) return IMOP_OK;
    if (!frames) return set_error(IMOP_ERR_NULL_INPUT, "frames is null");
    if ((flags & ~(unsigned)(IMOP_BATCH_GRAPH | IMOP_BATCH_PLAIN)) != 0) return set_error(IMOP_ERR_INVALID_ARGUMENT, "flags");
    int rc = ensure_aux(ctx);
    if (rc) return rc;
    std::vector<PreparedFrame> pf;
    if ((rc = prepare_batch(ctx, frames, n, pf))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    if (flags & IMOP_BATCH_PLAIN) return submit_plain(ctx, pf, st);
    cudaError_t e;
    if (!(flags & IMOP_BATCH_GRAPH)) {
        if ((e = enqueue_batch(ctx, pf, st))) return cuda_fail(e, "batch launch");
        return IMOP_OK;
    }
    Key bk = batch_key(pf, nullptr);
    const uint64_t key = bk.hash() | 1ull;  // 0 means "no graph"
    if (ctx->graph.key != key || ctx->graph.key_bytes != bk.b) {
        // record on the context's own stream (the legacy stream cannot be captured), replay on `st`
        if (fused_grid_limit(1) <= 0 || fused_grid_limit(2) <= 0) return set_error(IMOP_ERR_CUDA, "kernel set-up");
        if (ctx->graph.exec) {
            if ((e = cudaStreamSynchronize(st))) return cuda_fail(e, "sync before re-recording");
            cudaGraphExecDestroy(ctx->graph.exec);
            ctx->graph.exec = nullptr;
        }
        ctx->graph.key = 0;
        cudaGraph_t g = nullptr;
        if ((e = cudaStreamBeginCapture(ctx->aux, cudaStreamCaptureModeThreadLocal))) return cuda_fail(e, "begin capture");
        cudaError_t le = enqueue_batch(ctx, pf, ctx->aux);
        e = cudaStreamEndCapture(ctx->aux, &g);
        if (le != cudaSuccess || e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return cuda_fail(le != cudaSuccess ? le : e, "record batch");
        }
        e = cudaGraphInstantiate(&ctx->graph.exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_fail(e, "instantiate batch graph");
        ctx->graph.key = key;
        ctx->graph.key_bytes = std::move(bk.b);
    }
    if ((e = cudaGraphLaunch(ctx->graph.exec, st))) return cuda_fail(e, "graph launch");
    return IMOP_OK;
}

extern "C" int imop_isp_run_host_batch(imop_isp_t ctx, const ImopFrameDesc* frames, int n) {
    if (!ctx) return set_error(IMOP_ERR_NULL_INPUT, "ctx is null");
    if (n < 0) return set_error(IMOP_ERR_INVALID_ARGUMENT, "negative frame count");
    if (n == 0) return IMOP_OK;
    if (!frames) return set_error(IMOP_ERR_NULL_INPUT, "frames is null");
    int rc = ensure_aux(ctx);
    if (rc) return rc;
    HostPipeline& P = ctx->pipe;
    cudaError_t e;
    if (!P.ready) {
        // handles made by an earlier attempt that failed half way are kept, not made again
        int lo = 0, hi = 0;  // hi: the greatest priority (numerically lowest)
        if ((e = cudaDeviceGetStreamPriorityRange(&lo, &hi))) return cuda_fail(e, "create streams");
        for (cudaStream_t* st : {&P.s_in, &P.s_comp[0], &P.s_comp[1], &P.s_out})
            if (!*st && (e = cudaStreamCreateWithFlags(st, cudaStreamNonBlocking))) return cuda_fail(e, "create streams");
        if (!P.s_fix && (e = cudaStreamCreateWithPriority(&P.s_fix, cudaStreamNonBlocking, hi)))
            return cuda_fail(e, "create streams");
        for (int i = 0; i < HostPipeline::kSlots; i++) {
            for (cudaEvent_t* ev : {&P.in_done[i], &P.main_done[i], &P.fix_done[i], &P.out_done[i]})
                if (!*ev && (e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming))) return cuda_fail(e, "create events");
            if ((rc = ensure_fixup(P.fix[i], 1 << 16))) return rc;
        }
        P.ready = true;
    }
    // parameters, tables and sizes of every frame first (uploads are synchronous)
    std::vector<FrameParams> fps(n);
    std::vector<const FrameTables*> maps(n);
    std::vector<size_t> ib(n), ob(n);
    size_t max_in = 0, max_out = 0;
    for (int i = 0; i < n; i++) {
        const ImopIspParams* p = frames[i].params ? frames[i].params : (ctx->has_params ? &ctx->params : nullptr);
        if (!p) return set_error(IMOP_ERR_INVALID_ARGUMENT, "frame without parameters and no set_params");
        if ((rc = validate_params(p))) return rc;
        if (!frames[i].in || !frames[i].out) return set_error(IMOP_ERR_NULL_INPUT, "null frame pointer");
        expand_frame_params(p, fps[i]);
        if ((rc = resolve_tables(ctx, p, fps[i], &maps[i]))) return rc;
        ib[i] = imop_isp_input_bytes(p);
        ob[i] = imop_isp_output_bytes(p);
        max_in = std::max(max_in, ib[i]);
        max_out = std::max(max_out, ob[i]);
    }
    for (int s = 0; s < HostPipeline::kSlots; s++) {
        if (P.d_in[s].size < max_in || P.d_out[s].size < max_out) {
            if ((e = cudaDeviceSynchronize())) return cuda_fail(e, "sync before slot growth");
            if ((e = P.d_in[s].ensure(max_in)) || (e = P.d_out[s].ensure(max_out))) return cuda_fail(e, "alloc slots");
        }
    }
    // Once a copy is queued, an error return first waits for every stream of the pipeline: copies
    // from or to the caller's host frames may still be running, and the caller may free them as
    // soon as the call returns.
    auto fail = [&](cudaError_t err, const char* what) {
        for (cudaStream_t q : {P.s_in, P.s_comp[0], P.s_comp[1], P.s_fix, P.s_out}) cudaStreamSynchronize(q);
        return cuda_fail(err, what);
    };
    for (int i = 0; i < n; i++) {
        const int s = i % HostPipeline::kSlots;
        // the slot's own defect-chain scratch and tile counter; the context's sticky status word
        FixupScratch fs;
        FrameParams fp = fps[i];
        attach_fixup(P.fix[s], fp, fs);
        fp.status = (int*)ctx->fix.status.ptr;
        fp.in = (const uint8_t*)P.d_in[s].ptr;
        fp.out = (uint8_t*)P.d_out[s].ptr;
        // copy in once the slot's previous frame is fully computed (its fix-up reads the input)
        if ((e = cudaStreamWaitEvent(P.s_in, P.fix_done[s], 0)) ||
            (e = cudaMemcpyAsync(P.d_in[s].ptr, frames[i].in, ib[i], cudaMemcpyHostToDevice, P.s_in)) ||
            (e = cudaEventRecord(P.in_done[s], P.s_in)))
            return fail(e, "copy in");
        // tile kernel once the input arrived, the slot's previous output was copied out and its
        // fix-up scratch is free; the chain resolution follows on s_fix
        cudaStream_t sc = P.s_comp[i & 1];
        if ((e = cudaStreamWaitEvent(sc, P.in_done[s], 0)) || (e = cudaStreamWaitEvent(sc, P.out_done[s], 0)) ||
            (e = cudaStreamWaitEvent(sc, P.fix_done[s], 0)))
            return fail(e, "order compute");
        // map-mode frames resolve their map values into tables that frames with the same map share:
        // they follow the previous frame's tile kernel
        if (i > 0 && maps[i] && (e = cudaStreamWaitEvent(sc, P.main_done[(i - 1) % HostPipeline::kSlots], 0)))
            return fail(e, "order map frame");
        // A page-locked output frame is copied out right after the tile kernel and the fix-up then
        // writes its re-rendered windows into it; otherwise the copy waits for the whole fix-up.
        const bool direct_fix = device_mapped_host(frames[i].out, ob[i]);
        const SplitFixup split{P.s_fix, P.main_done[s], direct_fix};
        if ((e = launch_fused(fp, fs, maps[i] ? &maps[i]->plan : nullptr, sc, &split)))
            return fail(e, "fused launch");
        if (!direct_fix && (e = cudaEventRecord(P.fix_done[s], P.s_fix))) return fail(e, "fix-up done");
        if ((e = cudaStreamWaitEvent(P.s_out, direct_fix ? P.main_done[s] : P.fix_done[s], 0)) ||
            (e = cudaMemcpyAsync(frames[i].out, P.d_out[s].ptr, ob[i], cudaMemcpyDeviceToHost, P.s_out)) ||
            (e = cudaEventRecord(P.out_done[s], P.s_out)))
            return fail(e, "copy out");
        if (direct_fix) {
            if ((e = cudaStreamWaitEvent(P.s_fix, P.out_done[s], 0)) ||
                (e = launch_fused_render(fp, fs, (uint8_t*)frames[i].out, P.s_fix)) ||
                (e = cudaEventRecord(P.fix_done[s], P.s_fix)))
                return fail(e, "fix-up windows");
        }
    }
    if ((e = cudaStreamSynchronize(P.s_out)) || (e = cudaStreamSynchronize(P.s_fix)) ||
        (e = cudaStreamSynchronize(P.s_comp[0])) || (e = cudaStreamSynchronize(P.s_comp[1])) ||
        (e = cudaStreamSynchronize(P.s_in)))
        return fail(e, "run_host_batch");
    return take_status(ctx->fix);
}
