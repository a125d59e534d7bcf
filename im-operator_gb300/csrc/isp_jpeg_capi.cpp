// isp_jpeg_capi.cpp - C ABI of the device JPEG encoder: contexts, validation, the JFIF header,
// host and device entry points.
//
// Validation, clamping, capacity and truncation follow jpeg_codec::process_encode_baseline
// (src/jpeg_codec/encode_baseline.cpp:222-250) and validate_jpeg_encode_inputs
// (src/jpeg_codec/dispatch.cpp:11-29): null input, dimensions, bit depth (8 only), size >= 8x8,
// null output, quality 1..100, in that order; subsampling clamped to 0..2; a zero capacity means
// get_max_jpeg_size() = w*h*9 + 65536; bytes past the capacity are dropped and the reported size
// is min(JPEG size, capacity).  The header bytes are the reference's (encode_baseline.cpp:252-293
// with the writers at :108-220 and common.hpp:485-502).

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <array>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/imop_isp.h"
#include "isp_context.h"
#include "isp_jpeg.h"

using namespace imop;

namespace {

// ITU-T T.81 Annex K tables (also the reference's, common.hpp:57-93, :413-470)
const int kQLuma[64] = {16, 11, 10, 16, 24,  40,  51,  61,  12, 12, 14, 19, 26,  58,  60,  55,
                        14, 13, 16, 24, 40,  57,  69,  56,  14, 17, 22, 29, 51,  87,  80,  62,
                        18, 22, 37, 56, 68,  109, 103, 77,  24, 35, 55, 64, 81,  104, 113, 92,
                        49, 64, 78, 87, 103, 121, 120, 101, 72, 92, 95, 98, 112, 100, 103, 99};
const int kQChroma[64] = {17, 18, 24, 47, 99, 99, 99, 99, 18, 21, 26, 66, 99, 99, 99, 99,
                          24, 26, 56, 99, 99, 99, 99, 99, 47, 66, 99, 99, 99, 99, 99, 99,
                          99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99,
                          99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99};
const int kZigzag[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,
                         12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6,  7,  14, 21, 28,
                         35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
                         58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};
const uint8_t kDcLumaBits[16] = {0, 1, 5, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0};
const uint8_t kDcChromaBits[16] = {0, 3, 1, 1, 1, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0};
const uint8_t kDcVals[12] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11};
const uint8_t kAcLumaBits[16] = {0, 2, 1, 3, 3, 2, 4, 3, 5, 5, 4, 4, 0, 0, 1, 0x7d};
const uint8_t kAcLumaVals[162] = {
    0x01, 0x02, 0x03, 0x00, 0x04, 0x11, 0x05, 0x12, 0x21, 0x31, 0x41, 0x06, 0x13, 0x51, 0x61, 0x07, 0x22, 0x71,
    0x14, 0x32, 0x81, 0x91, 0xa1, 0x08, 0x23, 0x42, 0xb1, 0xc1, 0x15, 0x52, 0xd1, 0xf0, 0x24, 0x33, 0x62, 0x72,
    0x82, 0x09, 0x0a, 0x16, 0x17, 0x18, 0x19, 0x1a, 0x25, 0x26, 0x27, 0x28, 0x29, 0x2a, 0x34, 0x35, 0x36, 0x37,
    0x38, 0x39, 0x3a, 0x43, 0x44, 0x45, 0x46, 0x47, 0x48, 0x49, 0x4a, 0x53, 0x54, 0x55, 0x56, 0x57, 0x58, 0x59,
    0x5a, 0x63, 0x64, 0x65, 0x66, 0x67, 0x68, 0x69, 0x6a, 0x73, 0x74, 0x75, 0x76, 0x77, 0x78, 0x79, 0x7a, 0x83,
    0x84, 0x85, 0x86, 0x87, 0x88, 0x89, 0x8a, 0x92, 0x93, 0x94, 0x95, 0x96, 0x97, 0x98, 0x99, 0x9a, 0xa2, 0xa3,
    0xa4, 0xa5, 0xa6, 0xa7, 0xa8, 0xa9, 0xaa, 0xb2, 0xb3, 0xb4, 0xb5, 0xb6, 0xb7, 0xb8, 0xb9, 0xba, 0xc2, 0xc3,
    0xc4, 0xc5, 0xc6, 0xc7, 0xc8, 0xc9, 0xca, 0xd2, 0xd3, 0xd4, 0xd5, 0xd6, 0xd7, 0xd8, 0xd9, 0xda, 0xe1, 0xe2,
    0xe3, 0xe4, 0xe5, 0xe6, 0xe7, 0xe8, 0xe9, 0xea, 0xf1, 0xf2, 0xf3, 0xf4, 0xf5, 0xf6, 0xf7, 0xf8, 0xf9, 0xfa};
const uint8_t kAcChromaBits[16] = {0, 2, 1, 2, 4, 4, 3, 4, 7, 5, 4, 4, 0, 1, 2, 0x77};
const uint8_t kAcChromaVals[162] = {
    0x00, 0x01, 0x02, 0x03, 0x11, 0x04, 0x05, 0x21, 0x31, 0x06, 0x12, 0x41, 0x51, 0x07, 0x61, 0x71, 0x13, 0x22,
    0x32, 0x81, 0x08, 0x14, 0x42, 0x91, 0xa1, 0xb1, 0xc1, 0x09, 0x23, 0x33, 0x52, 0xf0, 0x15, 0x62, 0x72, 0xd1,
    0x0a, 0x16, 0x24, 0x34, 0xe1, 0x25, 0xf1, 0x17, 0x18, 0x19, 0x1a, 0x26, 0x27, 0x28, 0x29, 0x2a, 0x35, 0x36,
    0x37, 0x38, 0x39, 0x3a, 0x43, 0x44, 0x45, 0x46, 0x47, 0x48, 0x49, 0x4a, 0x53, 0x54, 0x55, 0x56, 0x57, 0x58,
    0x59, 0x5a, 0x63, 0x64, 0x65, 0x66, 0x67, 0x68, 0x69, 0x6a, 0x73, 0x74, 0x75, 0x76, 0x77, 0x78, 0x79, 0x7a,
    0x82, 0x83, 0x84, 0x85, 0x86, 0x87, 0x88, 0x89, 0x8a, 0x92, 0x93, 0x94, 0x95, 0x96, 0x97, 0x98, 0x99, 0x9a,
    0xa2, 0xa3, 0xa4, 0xa5, 0xa6, 0xa7, 0xa8, 0xa9, 0xaa, 0xb2, 0xb3, 0xb4, 0xb5, 0xb6, 0xb7, 0xb8, 0xb9, 0xba,
    0xc2, 0xc3, 0xc4, 0xc5, 0xc6, 0xc7, 0xc8, 0xc9, 0xca, 0xd2, 0xd3, 0xd4, 0xd5, 0xd6, 0xd7, 0xd8, 0xd9, 0xda,
    0xe2, 0xe3, 0xe4, 0xe5, 0xe6, 0xe7, 0xe8, 0xe9, 0xea, 0xf2, 0xf3, 0xf4, 0xf5, 0xf6, 0xf7, 0xf8, 0xf9, 0xfa};

thread_local std::string t_jpeg_error;

int jfail(int code, const std::string& msg) {
    t_jpeg_error = msg;
    set_error(code, msg.c_str());
    return code;
}

int jcuda(cudaError_t e, const char* what) {
    return jfail(IMOP_JPEG_INTERNAL_ERROR, std::string(what) + ": " + cudaGetErrorString(e));
}

void scale_qtable(int q[64], const int base[64], int quality) {
    const int qq = std::max(1, std::min(100, quality));
    const int s = qq < 50 ? 5000 / qq : 200 - qq * 2;
    for (int i = 0; i < 64; i++) q[i] = std::max(1, std::min(255, (base[i] * s + 50) / 100));
}

// canonical code assignment of a table into (size << 16) | code entries
void huff_lookup(const uint8_t bits[16], const uint8_t* vals, uint32_t* out, int n_out) {
    std::fill(out, out + n_out, 0u);
    int k = 0, code = 0;
    for (int len = 1; len <= 16; len++) {
        for (int j = 0; j < bits[len - 1]; j++, k++, code++)
            if (vals[k] < n_out) out[vals[k]] = ((uint32_t)len << 16) | (uint32_t)code;
        code <<= 1;
    }
}

struct Bytes {
    std::vector<uint8_t> v;
    void b(int x) { v.push_back((uint8_t)x); }
    void u16(int x) {
        b((x >> 8) & 0xFF);
        b(x & 0xFF);
    }
};

void dht(Bytes& o, int cls, int id, const uint8_t bits[16], const uint8_t* vals) {
    int n = 0;
    for (int i = 0; i < 16; i++) n += bits[i];
    o.b(0xFF), o.b(0xC4), o.u16(3 + 16 + n), o.b((cls << 4) | id);
    for (int i = 0; i < 16; i++) o.b(bits[i]);
    for (int i = 0; i < n; i++) o.b(vals[i]);
}

// SOI, JFIF APP0, DQT x2, SOF0, DHT x4, SOS
std::vector<uint8_t> jpeg_header(int w, int h, int quality, int ss) {
    int ql[64], qc[64];
    scale_qtable(ql, kQLuma, quality);
    scale_qtable(qc, kQChroma, quality);
    const int hy = ss == 0 ? 1 : 2, vy = ss == 1 ? 2 : 1;
    Bytes o;
    o.b(0xFF), o.b(0xD8);
    o.b(0xFF), o.b(0xE0), o.u16(16);
    for (char c : {'J', 'F', 'I', 'F'}) o.b(c);
    o.b(0), o.b(1), o.b(2), o.b(1), o.u16(72), o.u16(72), o.b(0), o.b(0);
    for (int t = 0; t < 2; t++) {
        o.b(0xFF), o.b(0xDB), o.u16(67), o.b(t);
        for (int i = 0; i < 64; i++) o.b((t ? qc : ql)[kZigzag[i]]);
    }
    o.b(0xFF), o.b(0xC0), o.u16(17), o.b(8), o.u16(h & 0xFFFF), o.u16(w & 0xFFFF), o.b(3);
    o.b(1), o.b((hy << 4) | vy), o.b(0);
    o.b(2), o.b(0x11), o.b(1);
    o.b(3), o.b(0x11), o.b(1);
    dht(o, 0, 0, kDcLumaBits, kDcVals);
    dht(o, 1, 0, kAcLumaBits, kAcLumaVals);
    dht(o, 0, 1, kDcChromaBits, kDcVals);
    dht(o, 1, 1, kAcChromaBits, kAcChromaVals);
    o.b(0xFF), o.b(0xDA), o.u16(12), o.b(3);
    o.b(1), o.b(0x00), o.b(2), o.b(0x11), o.b(3), o.b(0x11);
    o.b(0), o.b(63), o.b(0);
    return o.v;
}

int validate(const void* in, const void* out, int w, int h, int bd, int quality) {
    if (!in) return jfail(IMOP_JPEG_NULL_INPUT, "null input");
    if (w <= 0 || h <= 0) return jfail(IMOP_JPEG_INVALID_DIMENSIONS, "invalid dimensions");
    if (bd != 8) return jfail(IMOP_JPEG_INVALID_BIT_DEPTH, "bit depth must be 8");
    if (w < 8 || h < 8) return jfail(IMOP_JPEG_IMAGE_TOO_SMALL, "image smaller than 8x8");
    if (!out) return jfail(IMOP_JPEG_NULL_OUTPUT, "null output");
    if (quality < 1 || quality > 100) return jfail(IMOP_JPEG_INVALID_QUALITY, "quality outside 1..100");
    return IMOP_JPEG_OK;
}

}  // namespace

// device scratch of one encode in flight; a context has two, so that a batch runs consecutive
// frames on two streams and the latency-bound tail kernels of one frame overlap the next
// frame's transform
struct JpegLane {
    DevBuf acw, dc, acbits, blk_off, tile_sum, tile_off, words, chunk_ff, chunk_off, info, counters, rgb, out;
    bool dirty = true;             // the word stream and the counters must be zero before a launch
    cudaStream_t st = nullptr;     // batch stream of the lane
    cudaEvent_t ev = nullptr;      // join / info-ready marker
    cudaEvent_t ev_last = nullptr; // end of the lane's last use, on whichever stream it ran
    bool used = false;
    JpegInfo* h_info = nullptr;    // pinned
};

struct imop_jpeg_ctx {
    int device = 0;
    cudaEvent_t fork = nullptr;  // a device batch starts when the caller's stream reaches it
    JpegLane lane[2];
    DevBuf huff;
    // headers by (width, height, quality, subsample): host bytes and a device copy
    std::map<std::array<int, 4>, std::pair<std::vector<uint8_t>, std::unique_ptr<DevBuf>>> headers;
    JpegInfo last{};
    JpegLane* last_lane = nullptr;
    cudaStream_t last_stream = nullptr;
    bool last_pending = false;
    size_t last_base = 0;
};

namespace {

// a use of the lane's scratch on stream st starts after its previous use, whatever stream that
// ran on (the host calls use the lane's own stream, the device calls the caller's)
cudaError_t lane_acquire(JpegLane& l, cudaStream_t st) {
    return l.used ? cudaStreamWaitEvent(st, l.ev_last, 0) : cudaSuccess;
}
cudaError_t lane_release(JpegLane& l, cudaStream_t st) {
    l.used = true;
    return cudaEventRecord(l.ev_last, st);
}

// grows a lane's scratch to the geometry; clears its word stream and counters when (re)allocated
int prepare(JpegLane& l, const JpegGeom& g, cudaStream_t st) {
    cudaError_t e = cudaSuccess;
    const size_t nb = (size_t)g.nb;
    const size_t wbytes = (size_t)g.words * 4;
    const bool grow_words = l.words.size < wbytes;
    if ((e = l.acw.ensure(nb * kJpegAcWords * sizeof(uint32_t))) != cudaSuccess ||
        (e = l.dc.ensure(nb * sizeof(int))) != cudaSuccess || (e = l.acbits.ensure(nb * sizeof(int))) != cudaSuccess ||
        (e = l.blk_off.ensure(nb * sizeof(int))) != cudaSuccess ||
        (e = l.tile_sum.ensure((size_t)g.ntiles * sizeof(int))) != cudaSuccess ||
        (e = l.tile_off.ensure((size_t)g.ntiles * 8)) != cudaSuccess || (e = l.words.ensure(wbytes)) != cudaSuccess ||
        (e = l.chunk_ff.ensure((size_t)g.chunks * sizeof(int))) != cudaSuccess ||
        (e = l.chunk_off.ensure((size_t)g.chunks * 8)) != cudaSuccess ||
        (e = l.info.ensure(sizeof(JpegInfo))) != cudaSuccess)
        return jcuda(e, "jpeg scratch allocation");
    if (!l.counters.ptr) {
        if ((e = l.counters.ensure(2 * sizeof(unsigned))) != cudaSuccess) return jcuda(e, "jpeg scratch allocation");
        l.dirty = true;
    }
    if (grow_words || l.dirty) {
        if ((e = cudaMemsetAsync(l.words.ptr, 0, l.words.size, st)) != cudaSuccess ||
            (e = cudaMemsetAsync(l.counters.ptr, 0, l.counters.size, st)) != cudaSuccess)
            return jcuda(e, "jpeg clear");
        l.dirty = false;
    }
    return IMOP_JPEG_OK;
}

void fill_launch(imop_jpeg_ctx* c, JpegLane& l, const JpegGeom& g, int quality, JpegLaunch& L) {
    int ql[64], qc[64];
    scale_qtable(ql, kQLuma, quality);
    scale_qtable(qc, kQChroma, quality);
    std::memset(&L, 0, sizeof(L));
    L.g = g;
    for (int i = 0; i < 64; i++) {
        L.q[0][i] = (float)ql[i], L.q[1][i] = (float)qc[i];
        L.rq[0][i] = 1.0f / L.q[0][i], L.rq[1][i] = 1.0f / L.q[1][i];
    }
    L.huff = (const JpegHuff*)c->huff.ptr;
    L.acw = (uint32_t*)l.acw.ptr;
    L.dc = (int*)l.dc.ptr;
    L.acbits = (int*)l.acbits.ptr;
    L.blk_off = (int*)l.blk_off.ptr;
    L.tile_sum = (int*)l.tile_sum.ptr;
    L.tile_off = (unsigned long long*)l.tile_off.ptr;
    L.words = (uint32_t*)l.words.ptr;
    L.chunk_ff = (int*)l.chunk_ff.ptr;
    L.chunk_off = (unsigned long long*)l.chunk_off.ptr;
    L.info = (JpegInfo*)l.info.ptr;
    L.counters = (unsigned*)l.counters.ptr;
}

// the block count must index with 32-bit ints on the device
bool geometry_fits(const JpegGeom& g) { return g.nb < (1LL << 30); }

int launch(JpegLane& l, const JpegLaunch& L, cudaStream_t st) {
    const cudaError_t e = launch_jpeg_encode(L, st);
    if (e != cudaSuccess) {
        l.dirty = true;
        return jcuda(e, "jpeg kernels");
    }
    return IMOP_JPEG_OK;
}

// the header of (w, h, quality, subsample); its device copy is uploaded on first use
int header_for(imop_jpeg_ctx* c, int w, int h, int quality, int ss, cudaStream_t st,
               const std::pair<std::vector<uint8_t>, std::unique_ptr<DevBuf>>** out) {
    const std::array<int, 4> key = {w, h, quality, ss};
    auto it = c->headers.find(key);
    if (it == c->headers.end()) {
        if (c->headers.size() >= 64) c->headers.clear();  // cudaFree waits for copies still reading them
        auto& ent = c->headers[key];
        ent.first = jpeg_header(w, h, quality, ss);
        ent.second.reset(new DevBuf());
        cudaError_t e;
        if ((e = ent.second->ensure(ent.first.size())) != cudaSuccess ||
            (e = cudaMemcpyAsync(ent.second->ptr, ent.first.data(), ent.first.size(), cudaMemcpyHostToDevice, st)) !=
                cudaSuccess) {
            c->headers.erase(key);
            return jcuda(e, "jpeg header upload");
        }
        it = c->headers.find(key);
    }
    *out = &it->second;
    return IMOP_JPEG_OK;
}

// one frame, device in and out, on stream st with lane l (no host synchronisation)
int encode_device_on(imop_jpeg_ctx* c, JpegLane& l, const void* d_rgb, int w, int h, int quality, int ss, void* d_out,
                     size_t out_cap, size_t* d_out_size, cudaStream_t st) {
    const JpegGeom g = jpeg_geometry(w, h, ss);
    if (!geometry_fits(g)) return jfail(IMOP_JPEG_ENCODE_FAILED, "frame too large for one encode");
    const size_t cap = out_cap > 0 ? out_cap : imop_jpeg_max_bytes(w, h);
    int s;
    cudaError_t e;
    if ((e = lane_acquire(l, st)) != cudaSuccess) return jcuda(e, "jpeg lane");
    if ((s = prepare(l, g, st))) return s;
    const std::pair<std::vector<uint8_t>, std::unique_ptr<DevBuf>>* hd = nullptr;
    if ((s = header_for(c, w, h, quality, ss, st, &hd))) return s;
    if ((e = cudaMemcpyAsync(d_out, hd->second->ptr, std::min(cap, hd->first.size()), cudaMemcpyDeviceToDevice, st)) !=
        cudaSuccess)
        return jcuda(e, "jpeg header copy");
    JpegLaunch L;
    fill_launch(c, l, g, quality, L);
    L.rgb = (const uint8_t*)d_rgb;
    L.out = (uint8_t*)d_out;
    L.base = hd->first.size();
    L.out_cap = cap;
    L.size_out = (unsigned long long*)d_out_size;
    if ((s = launch(l, L, st))) return s;
    return (e = lane_release(l, st)) == cudaSuccess ? IMOP_JPEG_OK : jcuda(e, "jpeg lane");
}

}  // namespace

extern "C" {

int imop_jpeg_create(imop_jpeg_t* out_ctx) {
    if (!out_ctx) return jfail(IMOP_JPEG_NULL_OUTPUT, "null context pointer");
    *out_ctx = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        return jfail(IMOP_JPEG_CUDA_NOT_AVAILABLE, "no CUDA device");
    }
    auto* c = new imop_jpeg_ctx();
    cudaError_t e = cudaGetDevice(&c->device);
    float cs[64];
    for (int u = 0; u < 8; u++)
        for (int i = 0; i < 8; i++) cs[u * 8 + i] = std::cos((2.0f * i + 1.0f) * u * 3.14159265358979323846f / 16.0f);
    JpegHuff hf;
    huff_lookup(kDcLumaBits, kDcVals, hf.dc[0], 16);
    huff_lookup(kDcChromaBits, kDcVals, hf.dc[1], 16);
    huff_lookup(kAcLumaBits, kAcLumaVals, hf.ac[0], 256);
    huff_lookup(kAcChromaBits, kAcChromaVals, hf.ac[1], 256);
    if (e == cudaSuccess) e = jpeg_init_constants(cs);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->fork, cudaEventDisableTiming);
    for (int k = 0; k < 2 && e == cudaSuccess; k++) {
        JpegLane& l = c->lane[k];
        e = cudaStreamCreateWithFlags(&l.st, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&l.ev, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&l.ev_last, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaHostAlloc((void**)&l.h_info, sizeof(JpegInfo), cudaHostAllocDefault);
    }
    if (e == cudaSuccess) e = c->huff.ensure(sizeof(JpegHuff));
    if (e == cudaSuccess) e = cudaMemcpy(c->huff.ptr, &hf, sizeof(JpegHuff), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        imop_jpeg_destroy(c);
        return jcuda(e, "jpeg context");
    }
    *out_ctx = c;
    return IMOP_JPEG_OK;
}

int imop_jpeg_destroy(imop_jpeg_t c) {
    if (!c) return IMOP_JPEG_OK;
    cudaDeviceSynchronize();
    for (auto& l : c->lane) {
        if (l.h_info) cudaFreeHost(l.h_info);
        if (l.ev) cudaEventDestroy(l.ev);
        if (l.ev_last) cudaEventDestroy(l.ev_last);
        if (l.st) cudaStreamDestroy(l.st);
    }
    if (c->fork) cudaEventDestroy(c->fork);
    delete c;
    return IMOP_JPEG_OK;
}

size_t imop_jpeg_max_bytes(int width, int height) {
    return (size_t)width * (size_t)height * 3 * 3 + 65536;
}

int imop_jpeg_header(int width, int height, int quality, int subsample, uint8_t* out, size_t cap) {
    const int ss = std::max(0, std::min(2, subsample));
    const std::vector<uint8_t> h = jpeg_header(width, height, std::max(1, std::min(100, quality)), ss);
    if (out) std::memcpy(out, h.data(), std::min(cap, h.size()));
    return (int)h.size();
}

namespace {

// host frame -> lane: validation, input copy, kernels, size read-back queued on the lane's
// stream (lane.ev marks the size record); the bytes are fetched by host_finish
int host_enqueue(imop_jpeg_ctx* c, JpegLane& l, const uint8_t* rgb, int w, int h, int quality, int ss, size_t cap,
                 size_t hdr_bytes) {
    const JpegGeom g = jpeg_geometry(w, h, ss);
    if (!geometry_fits(g)) return jfail(IMOP_JPEG_ENCODE_FAILED, "frame too large for one encode");
    cudaStream_t st = l.st;
    int s;
    cudaError_t e;
    if ((e = lane_acquire(l, st)) != cudaSuccess) return jcuda(e, "jpeg lane");
    if ((s = prepare(l, g, st))) return s;
    const size_t seg_cap = cap > hdr_bytes ? cap - hdr_bytes : 0;
    const size_t stage = std::min(seg_cap, (size_t)g.words * 8 + 2);
    const size_t in_bytes = (size_t)w * h * 3;
    if ((e = l.rgb.ensure(in_bytes)) != cudaSuccess || (e = l.out.ensure(stage + 1)) != cudaSuccess)
        return jcuda(e, "jpeg staging allocation");
    if ((e = cudaMemcpyAsync(l.rgb.ptr, rgb, in_bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return jcuda(e, "jpeg input copy");
    JpegLaunch L;
    fill_launch(c, l, g, quality, L);
    L.rgb = (const uint8_t*)l.rgb.ptr;
    L.out = (uint8_t*)l.out.ptr;
    L.base = 0;
    L.out_cap = stage;
    L.size_out = nullptr;
    if ((s = launch(l, L, st))) return s;
    if ((e = cudaMemcpyAsync(l.h_info, l.info.ptr, sizeof(JpegInfo), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaEventRecord(l.ev, st)) != cudaSuccess) {
        l.dirty = true;
        return jcuda(e, "jpeg encode");
    }
    return IMOP_JPEG_OK;
}

// waits for the lane's size record, writes the header and queues the bytes' copy on the lane's
// stream; *out_size = min(JPEG size, cap)
int host_finish(imop_jpeg_ctx* c, JpegLane& l, const std::vector<uint8_t>& hdr, uint8_t* out, size_t cap,
                size_t* out_size) {
    cudaError_t e;
    if ((e = cudaEventSynchronize(l.ev)) != cudaSuccess) {
        l.dirty = true;
        return jcuda(e, "jpeg encode");
    }
    const JpegInfo info = *l.h_info;
    std::memcpy(out, hdr.data(), std::min(cap, hdr.size()));
    if (cap > hdr.size() && info.written > 0 &&
        (e = cudaMemcpyAsync(out + hdr.size(), l.out.ptr, (size_t)info.written, cudaMemcpyDeviceToHost, l.st)) !=
            cudaSuccess)
        return jcuda(e, "jpeg output copy");
    if ((e = lane_release(l, l.st)) != cudaSuccess) return jcuda(e, "jpeg lane");
    c->last = info;
    c->last.jpeg_bytes = hdr.size() + info.stuffed + 2;
    c->last.written = std::min((size_t)c->last.jpeg_bytes, cap);
    c->last_pending = false;
    *out_size = (size_t)c->last.written;
    return IMOP_JPEG_OK;
}

int ctx_check(imop_jpeg_ctx* c) {
    if (!c) return jfail(IMOP_JPEG_INTERNAL_ERROR, "null context");
    int dev = -1;
    if (cudaGetDevice(&dev) == cudaSuccess && dev != c->device) cudaSetDevice(c->device);
    return IMOP_JPEG_OK;
}

}  // namespace

int imop_jpeg_encode_host(imop_jpeg_t c, const uint8_t* rgb, int width, int height, int bit_depth, int quality,
                          int subsample, uint8_t* out, size_t* out_size) {
    int s;
    if ((s = ctx_check(c))) return s;
    if ((s = validate(rgb, out, width, height, bit_depth, quality))) return s;
    if (!out_size) return jfail(IMOP_JPEG_NULL_OUTPUT, "null output size");
    const int ss = std::max(0, std::min(2, subsample));
    const size_t cap = *out_size > 0 ? *out_size : imop_jpeg_max_bytes(width, height);
    const std::vector<uint8_t> hdr = jpeg_header(width, height, quality, ss);
    JpegLane& l = c->lane[0];
    if ((s = host_enqueue(c, l, rgb, width, height, quality, ss, cap, hdr.size()))) return s;
    if ((s = host_finish(c, l, hdr, out, cap, out_size))) return s;
    const cudaError_t e = cudaStreamSynchronize(l.st);
    return e == cudaSuccess ? IMOP_JPEG_OK : jcuda(e, "jpeg output copy");
}

int imop_jpeg_encode_host_batch(imop_jpeg_t c, ImopJpegHostFrame* frames, int n) {
    int s;
    if ((s = ctx_check(c))) return s;
    if (n < 0 || (n > 0 && !frames)) return jfail(IMOP_JPEG_NULL_INPUT, "null frame list");
    int first = IMOP_JPEG_OK;
    int prev = -1;  // frame whose bytes are still to be fetched
    std::vector<uint8_t> hdr_prev;
    int slot = 0;
    for (int k = 0; k <= n; k++) {
        int cur = -1;
        std::vector<uint8_t> hdr;
        if (k < n) {
            ImopJpegHostFrame& f = frames[k];
            f.out_size = 0;
            f.status = validate(f.rgb, f.out, f.width, f.height, 8, f.quality);
            if (f.status == IMOP_JPEG_OK) {
                const int ss = std::max(0, std::min(2, f.subsample));
                const size_t cap = f.out_cap > 0 ? f.out_cap : imop_jpeg_max_bytes(f.width, f.height);
                hdr = jpeg_header(f.width, f.height, f.quality, ss);
                f.status = host_enqueue(c, c->lane[slot], f.rgb, f.width, f.height, f.quality, ss, cap, hdr.size());
                if (f.status == IMOP_JPEG_OK) cur = k;
            }
            if (f.status != IMOP_JPEG_OK && first == IMOP_JPEG_OK) first = f.status;
        }
        if (prev >= 0) {  // the previous frame's bytes, while this frame's copy and kernels run
            ImopJpegHostFrame& f = frames[prev];
            const size_t cap = f.out_cap > 0 ? f.out_cap : imop_jpeg_max_bytes(f.width, f.height);
            f.status = host_finish(c, c->lane[slot ^ 1], hdr_prev, f.out, cap, &f.out_size);
            if (f.status != IMOP_JPEG_OK && first == IMOP_JPEG_OK) first = f.status;
        }
        prev = cur;
        if (cur >= 0) {
            hdr_prev.swap(hdr);
            slot ^= 1;
        }
    }
    for (auto& l : c->lane) {
        const cudaError_t e = cudaStreamSynchronize(l.st);
        if (e != cudaSuccess && first == IMOP_JPEG_OK) first = jcuda(e, "jpeg output copy");
    }
    return first;
}

int imop_jpeg_encode_device(imop_jpeg_t c, const void* d_rgb, int width, int height, int bit_depth, int quality,
                            int subsample, void* d_out, size_t out_cap, size_t* d_out_size, void* stream) {
    int s;
    if ((s = ctx_check(c))) return s;
    if ((s = validate(d_rgb, d_out, width, height, bit_depth, quality))) return s;
    const int ss = std::max(0, std::min(2, subsample));
    cudaStream_t st = (cudaStream_t)stream;
    if ((s = encode_device_on(c, c->lane[0], d_rgb, width, height, quality, ss, d_out, out_cap, d_out_size, st)))
        return s;
    c->last_lane = &c->lane[0];
    c->last_stream = st;
    c->last_pending = true;
    return IMOP_JPEG_OK;
}

int imop_jpeg_encode_device_batch(imop_jpeg_t c, const ImopJpegFrame* frames, int n, void* stream) {
    int s;
    if ((s = ctx_check(c))) return s;
    if (n < 0 || (n > 0 && !frames)) return jfail(IMOP_JPEG_NULL_INPUT, "null frame list");
    for (int k = 0; k < n; k++)
        if ((s = validate(frames[k].d_rgb, frames[k].d_out, frames[k].width, frames[k].height, 8, frames[k].quality)))
            return s;
    if (n == 0) return IMOP_JPEG_OK;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e;
    if ((e = cudaEventRecord(c->fork, st)) != cudaSuccess) return jcuda(e, "jpeg batch fork");
    for (auto& l : c->lane)
        if ((e = cudaStreamWaitEvent(l.st, c->fork, 0)) != cudaSuccess) return jcuda(e, "jpeg batch fork");
    int rc = IMOP_JPEG_OK;
    for (int k = 0; k < n && rc == IMOP_JPEG_OK; k++) {
        const ImopJpegFrame& f = frames[k];
        JpegLane& l = c->lane[k & 1];
        rc = encode_device_on(c, l, f.d_rgb, f.width, f.height, f.quality, std::max(0, std::min(2, f.subsample)),
                              f.d_out, f.out_cap, f.d_out_size, l.st);
    }
    for (auto& l : c->lane)  // the caller's stream continues after both lanes
        if ((e = cudaEventRecord(l.ev, l.st)) != cudaSuccess || (e = cudaStreamWaitEvent(st, l.ev, 0)) != cudaSuccess)
            return jcuda(e, "jpeg batch join");
    if (rc != IMOP_JPEG_OK) return rc;
    c->last_lane = &c->lane[(n - 1) & 1];
    c->last_stream = st;
    c->last_pending = true;
    return IMOP_JPEG_OK;
}

int imop_jpeg_last_size(imop_jpeg_t c, size_t* jpeg_bytes, size_t* written) {
    if (!c) return jfail(IMOP_JPEG_INTERNAL_ERROR, "null context");
    if (c->last_pending && c->last_lane) {
        cudaError_t e;
        if ((e = cudaMemcpyAsync(c->last_lane->h_info, c->last_lane->info.ptr, sizeof(JpegInfo), cudaMemcpyDeviceToHost,
                                 c->last_stream)) != cudaSuccess ||
            (e = cudaStreamSynchronize(c->last_stream)) != cudaSuccess)
            return jcuda(e, "jpeg size read-back");
        c->last = *c->last_lane->h_info;
        c->last_pending = false;
    }
    if (jpeg_bytes) *jpeg_bytes = (size_t)c->last.jpeg_bytes;
    if (written) *written = (size_t)c->last.written;
    return IMOP_JPEG_OK;
}

const char* imop_jpeg_last_error_string(void) { return t_jpeg_error.c_str(); }

}  // extern "C"
