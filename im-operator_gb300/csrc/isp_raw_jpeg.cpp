// isp_raw_jpeg.cpp - RAW host frames to JPEG host bytes (imop_isp_run_host_jpeg_batch).
//
// The fused pipeline (the drop-in of the reference's per-stage *_cuda glue, src/gpu_dispatch.cpp)
// and the baseline encoder (the drop-in of jpeg_codec::process_encode_baseline,
// src/jpeg_codec/encode_baseline.cpp) chained on the device: the raw bytes go in and the JPEG
// bytes come out, the RGB8 frame between them stays in HBM.  Frames run in chunks, one fused
// batch launch and one encoder device batch per chunk, on two device slots, so that the raw
// copies of chunk c+1 and the JPEG copies of chunk c-1 overlap the kernels of chunk c.
#include <algorithm>
#include <initializer_list>
#include <string>
#include <vector>

#include "isp_context.h"
#include "isp_jpeg.h"

namespace imop {

RawJpegPipe::~RawJpegPipe() {
    for (int s = 0; s < kSlots; s++) {
        if (h_size[s]) cudaFreeHost(h_size[s]);
        for (cudaEvent_t ev : {in_done[s], isp_done[s], jpg_done[s], out_done[s]})
            if (ev) cudaEventDestroy(ev);
    }
    for (cudaStream_t st : {s_in, s_isp, s_jpg, s_out})
        if (st) cudaStreamDestroy(st);
}

namespace {

constexpr size_t kAlign = 256;
size_t align_up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

// one frame's sizes and its offsets within the slot of its chunk
struct RjFrame {
    const ImopIspParams* p;
    int ss;
    size_t in_bytes, rgb_bytes;
    size_t jpg_cap;  // device room for the JPEG: min(capacity, header + the encoder's worst case)
    size_t raw_off, rgb_off, jpg_off;
};

int setup(RawJpegPipe& P) {
    if (P.ready) return IMOP_OK;
    cudaError_t e;
    for (cudaStream_t* st : {&P.s_in, &P.s_isp, &P.s_jpg, &P.s_out})
        if (!*st && (e = cudaStreamCreateWithFlags(st, cudaStreamNonBlocking))) return cuda_fail(e, "create streams");
    for (int s = 0; s < RawJpegPipe::kSlots; s++) {
        for (cudaEvent_t* ev : {&P.in_done[s], &P.isp_done[s], &P.jpg_done[s], &P.out_done[s]})
            if (!*ev && (e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming))) return cuda_fail(e, "create events");
        if (!P.h_size[s] &&
            (e = cudaHostAlloc((void**)&P.h_size[s], RawJpegPipe::kChunkFrames * sizeof(size_t), cudaHostAllocDefault)))
            return cuda_fail(e, "alloc size records");
    }
    P.ready = true;
    return IMOP_OK;
}

// waits for everything the call enqueued (also after a failure, before the caller's buffers go)
cudaError_t drain(RawJpegPipe& P) {
    cudaError_t first = cudaSuccess;
    for (cudaStream_t st : {P.s_in, P.s_isp, P.s_jpg, P.s_out}) {
        const cudaError_t e = st ? cudaStreamSynchronize(st) : cudaSuccess;
        if (e != cudaSuccess && first == cudaSuccess) first = e;
    }
    return first;
}

int validate_frame(imop_isp_ctx* isp, const ImopRawJpegFrame& f, RjFrame& r) {
    const ImopIspParams* p = f.params ? f.params : (isp->has_params ? &isp->params : nullptr);
    if (!p) return set_error(IMOP_ERR_INVALID_ARGUMENT, "frame without parameters and no set_params");
    int rc = validate_params(p);
    if (rc) return rc;
    if (!f.raw || !f.out) return set_error(IMOP_ERR_NULL_INPUT, "null frame pointer");
    if (p->out_format != IMOP_OUT_RGB8) return set_error(IMOP_ERR_UNSUPPORTED, "the JPEG encoder takes RGB8 output");
    if (p->width < 8 || p->height < 8) return set_error(IMOP_ERR_IMAGE_TOO_SMALL, "image smaller than 8x8");
    if (f.quality < 1 || f.quality > 100) return set_error(IMOP_ERR_INVALID_ARGUMENT, "quality outside 1..100");
    const int w = p->width, h = p->height;
    r.p = p;
    r.ss = std::max(0, std::min(2, f.subsample));
    r.in_bytes = imop_isp_input_bytes(p);
    r.rgb_bytes = imop_isp_output_bytes(p);
    const size_t hdr = (size_t)imop_jpeg_header(w, h, f.quality, r.ss, nullptr, 0);
    const JpegGeom g = jpeg_geometry(w, h, r.ss);
    const size_t cap = f.out_cap > 0 ? f.out_cap : imop_jpeg_max_bytes(w, h);
    r.jpg_cap = std::min(cap, hdr + (size_t)g.words * 8 + 2);
    return IMOP_OK;
}

}  // namespace
}  // namespace imop

using namespace imop;

extern "C" int imop_isp_run_host_jpeg_batch(imop_isp_t isp, imop_jpeg_t jpeg, ImopRawJpegFrame* frames, int n) {
    if (!isp || !jpeg) return set_error(IMOP_ERR_NULL_INPUT, "null context");
    if (n < 0) return set_error(IMOP_ERR_INVALID_ARGUMENT, "negative frame count");
    if (n == 0) return IMOP_OK;
    if (!frames) return set_error(IMOP_ERR_NULL_INPUT, "frames is null");
    RawJpegPipe& P = isp->rawjpeg;
    constexpr int kSlots = RawJpegPipe::kSlots;
    // every frame validated, sized and placed in its chunk before anything runs
    std::vector<RjFrame> fr(n);
    std::vector<int> chunk_begin;
    size_t need_raw = 0, need_rgb = 0, need_jpg = 0;
    {
        size_t raw = 0, rgb = 0, jpg = 0;
        long long px = 0;
        for (int i = 0; i < n; i++) {
            frames[i].out_size = 0;
            int rc = validate_frame(isp, frames[i], fr[i]);
            if (rc) return rc;
            const long long fpx = (long long)fr[i].p->width * fr[i].p->height;
            const int in_chunk = chunk_begin.empty() ? 0 : i - chunk_begin.back();
            // the first chunk is half as large: less to copy before the first launch can start
            const long long limit = RawJpegPipe::kChunkPixels / (chunk_begin.size() == 1 ? 2 : 1);
            if (chunk_begin.empty() || in_chunk == RawJpegPipe::kChunkFrames || px + fpx > limit) {
                chunk_begin.push_back(i);
                raw = rgb = jpg = 0;
                px = 0;
            }
            fr[i].raw_off = raw, fr[i].rgb_off = rgb, fr[i].jpg_off = jpg;
            raw += align_up(fr[i].in_bytes);
            rgb += align_up(fr[i].rgb_bytes);
            jpg += align_up(fr[i].jpg_cap + 1);
            px += fpx;
            need_raw = std::max(need_raw, raw), need_rgb = std::max(need_rgb, rgb), need_jpg = std::max(need_jpg, jpg);
        }
    }
    chunk_begin.push_back(n);
    const int chunks = (int)chunk_begin.size() - 1;
    int rc = setup(P);
    if (rc) return rc;
    cudaError_t e;
    for (int s = 0; s < kSlots; s++) {
        if (P.raw[s].size < need_raw || P.rgb[s].size < need_rgb || P.jpg[s].size < need_jpg || !P.size[s].ptr) {
            if ((e = drain(P))) return cuda_fail(e, "sync before slot growth");
            if ((e = P.raw[s].ensure(need_raw)) || (e = P.rgb[s].ensure(need_rgb)) || (e = P.jpg[s].ensure(need_jpg)) ||
                (e = P.size[s].ensure(RawJpegPipe::kChunkFrames * sizeof(size_t))))
                return cuda_fail(e, "alloc slots");
        }
    }
    auto fail = [&](int code) {
        drain(P);
        return code;
    };
    // chunk c on slot c % 2: copies in, fused batch, encoder batch, sizes to the host
    auto enqueue = [&](int c) -> int {
        const int s = c % kSlots, b = chunk_begin[c], k = chunk_begin[c + 1] - b;
        uint8_t* raw = (uint8_t*)P.raw[s].ptr;
        uint8_t* rgb = (uint8_t*)P.rgb[s].ptr;
        uint8_t* jpg = (uint8_t*)P.jpg[s].ptr;
        size_t* d_size = (size_t*)P.size[s].ptr;
        cudaError_t e;
        // the slot's raw frames are free once its previous chunk's fused launch has run
        if ((e = cudaStreamWaitEvent(P.s_in, P.isp_done[s], 0))) return cuda_fail(e, "order copy in");
        for (int j = 0; j < k; j++) {
            const RjFrame& f = fr[b + j];
            if ((e = cudaMemcpyAsync(raw + f.raw_off, frames[b + j].raw, f.in_bytes, cudaMemcpyHostToDevice, P.s_in)))
                return cuda_fail(e, "copy in");
        }
        if ((e = cudaEventRecord(P.in_done[s], P.s_in))) return cuda_fail(e, "copy in");
        // the fused launch overwrites the slot's RGB8 frames once the encoder has read them
        if ((e = cudaStreamWaitEvent(P.s_isp, P.in_done[s], 0)) || (e = cudaStreamWaitEvent(P.s_isp, P.jpg_done[s], 0)))
            return cuda_fail(e, "order fused launch");
        ImopFrameDesc desc[RawJpegPipe::kChunkFrames];
        for (int j = 0; j < k; j++) desc[j] = {fr[b + j].p, raw + fr[b + j].raw_off, rgb + fr[b + j].rgb_off};
        int rc = imop_isp_batch_submit(isp, desc, k, 0, P.s_isp);
        if (rc) return rc;
        if ((e = cudaEventRecord(P.isp_done[s], P.s_isp))) return cuda_fail(e, "fused launch");
        // the encoder overwrites the slot's JPEG bytes once they were copied out
        if ((e = cudaStreamWaitEvent(P.s_jpg, P.isp_done[s], 0)) || (e = cudaStreamWaitEvent(P.s_jpg, P.out_done[s], 0)))
            return cuda_fail(e, "order encode");
        ImopJpegFrame jf[RawJpegPipe::kChunkFrames];
        for (int j = 0; j < k; j++) {
            const RjFrame& f = fr[b + j];
            jf[j] = {rgb + f.rgb_off, f.p->width, f.p->height, frames[b + j].quality, f.ss, jpg + f.jpg_off, f.jpg_cap,
                     d_size + j};
        }
        if ((rc = imop_jpeg_encode_device_batch(jpeg, jf, k, P.s_jpg)))
            return set_error(IMOP_ERR_CUDA, (std::string("jpeg encode: ") + imop_jpeg_last_error_string()).c_str());
        if ((e = cudaMemcpyAsync(P.h_size[s], d_size, k * sizeof(size_t), cudaMemcpyDeviceToHost, P.s_jpg)) ||
            (e = cudaEventRecord(P.jpg_done[s], P.s_jpg)))
            return cuda_fail(e, "size read-back");
        return IMOP_OK;
    };
    // chunk c's JPEG bytes to the host once their sizes are known
    auto finish = [&](int c) -> int {
        const int s = c % kSlots, b = chunk_begin[c], k = chunk_begin[c + 1] - b;
        cudaError_t e;
        if ((e = cudaEventSynchronize(P.jpg_done[s])) || (e = cudaStreamWaitEvent(P.s_out, P.jpg_done[s], 0)))
            return cuda_fail(e, "encode");
        const uint8_t* jpg = (const uint8_t*)P.jpg[s].ptr;
        for (int j = 0; j < k; j++) {
            const size_t bytes = std::min(P.h_size[s][j], fr[b + j].jpg_cap);
            frames[b + j].out_size = bytes;
            if (bytes && (e = cudaMemcpyAsync(frames[b + j].out, jpg + fr[b + j].jpg_off, bytes, cudaMemcpyDeviceToHost,
                                              P.s_out)))
                return cuda_fail(e, "copy out");
        }
        if ((e = cudaEventRecord(P.out_done[s], P.s_out))) return cuda_fail(e, "copy out");
        return IMOP_OK;
    };
    for (int c = 0; c <= chunks; c++) {
        if (c < chunks && (rc = enqueue(c))) return fail(rc);
        if (c > 0 && (rc = finish(c - 1))) return fail(rc);
    }
    if ((e = drain(P))) return cuda_fail(e, "run_host_jpeg_batch");
    return take_status(isp->fix);
}
