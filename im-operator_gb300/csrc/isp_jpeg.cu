// isp_jpeg.cu - baseline JPEG encoder kernels (see isp_jpeg.h for the pipeline).
//
// Exactness: every float operation of the reference's encoder is one explicitly rounded IEEE
// operation here, in the reference's order (colour conversion common.hpp:196-201, DCT
// common.hpp:104-151 with the cosine factors the host evaluates with the same cosf, quantiser
// division and std::round encode_baseline.cpp:24-26).  The coefficient array is the reference's
// zz[kZigzag[i]] = round(block[i] / q[i]) (common.hpp:84-93), and the run-length / Huffman rules
// are those of encode_baseline.cpp:28-101, restated per 8-coefficient lane:
//   - a non-zero AC coefficient at p whose previous non-zero AC (or the DC slot) is at p' codes
//     floor((p - p' - 1) / 16) ZRL symbols, then symbol (((p - p' - 1) mod 16) << 4) | cat with
//     its cat value bits, or nothing at all when that symbol is absent from the table;
//   - EOB always follows the last non-zero AC coefficient, also at position 63, and a block
//     without AC coefficients codes EOB alone.

#include <cuda_runtime.h>
#include <stdint.h>

#include "isp_jpeg.h"

namespace imop {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kThreads = 256;
constexpr float kC0 = 0.5f * 0.70710678118654752440f;  // 0.5 * C(0), exact in float

__constant__ float c_cos[64];  // [u * 8 + i] = cosf((2i + 1) u pi / 16), from the host

// coefficient slot of natural index i: the standard zigzag table, which the reference uses as
// a natural -> slot map (zz[kZigzag[i]] = ...)
__constant__ uint8_t c_zz[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,
                                 12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6,  7,  14, 21, 28,
                                 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
                                 58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }

// where block b (coding order) samples the frame, its component and the previous block of the
// same component (DC prediction), following the MCU loop of encode_baseline.cpp:296-370
struct BlockPos {
    int comp;      // 0 Y, 1 Cb, 2 Cr
    int x0, y0;    // first sample
    int sx, sy;    // sample step (1 for luma, the luma sampling factors for chroma)
    int prev;      // previous block of the component, -1 for the first
};

__device__ __forceinline__ BlockPos block_pos(const JpegGeom& g, int b) {
    const unsigned m = (unsigned)b / (unsigned)g.bpm;
    const int k = b - (int)m * g.bpm;
    const unsigned my = m / (unsigned)g.mcus_x;
    const int mx = (int)(m - my * (unsigned)g.mcus_x) * g.mw;
    const int y = (int)my * g.mh;
    BlockPos p;
    if (k < g.ny) {
        p.comp = 0;
        p.x0 = mx + (k % g.hy) * 8;
        p.y0 = y + (k / g.hy) * 8;
        p.sx = 1;
        p.sy = 1;
        p.prev = k > 0 ? b - 1 : (m > 0 ? b - g.bpm + g.ny - 1 : -1);
    } else {
        p.comp = k - g.ny + 1;
        p.x0 = mx;
        p.y0 = y;
        p.sx = g.hy;
        p.sy = g.vy;
        p.prev = m > 0 ? b - g.bpm : -1;
    }
    return p;
}

// (int) of the reference's float YCbCr expressions
__device__ __forceinline__ int ycc(int r, int g, int b, int comp) {
    const float fr = (float)r, fg = (float)g, fb = (float)b;
    float v;
    if (comp == 0)
        v = fadd(fadd(fmul(0.299f, fr), fmul(0.587f, fg)), fmul(0.114f, fb));
    else if (comp == 1)
        v = fadd(fadd(fsub(fmul(-0.168736f, fr), fmul(0.331264f, fg)), fmul(0.5f, fb)), 128.0f);
    else
        v = fadd(fsub(fsub(fmul(0.5f, fr), fmul(0.418688f, fg)), fmul(0.081312f, fb)), 128.0f);
    return __float2int_rz(v);
}

__device__ __forceinline__ int category(int v) { return 32 - __clz(v < 0 ? -v : v); }

// value bits of a coefficient of category cat (negative values as v + 2^cat - 1)
__device__ __forceinline__ uint32_t value_bits(int v, int cat) {
    return (uint32_t)(v < 0 ? v + (1 << cat) - 1 : v);
}

// 8 int16 coefficients of one lane
struct Lane8 {
    int16_t z[8];
};

__device__ __forceinline__ Lane8 unpack8(uint4 v) {
    Lane8 l;
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int k = 0; k < 4; k++) {
        l.z[2 * k] = (int16_t)(w[k] & 0xFFFFu);
        l.z[2 * k + 1] = (int16_t)(w[k] >> 16);
    }
    return l;
}

// non-zero AC slots of the block (bit p = slot p, p >= 1), gathered over the 8 lanes of the block
__device__ __forceinline__ uint64_t block_mask(const Lane8& l, int r) {
    uint32_t byte = 0;
#pragma unroll
    for (int j = 0; j < 8; j++)
        if (l.z[j] != 0 && (r | j) != 0) byte |= 1u << j;
    uint64_t m = (uint64_t)byte << (8 * r);
    m |= __shfl_xor_sync(kFull, m, 1);
    m |= __shfl_xor_sync(kFull, m, 2);
    m |= __shfl_xor_sync(kFull, m, 4);
    return m;
}

// Walks the AC codes of lane r's slots [8r, 8r + 8) in order; emit(bits, len) receives each
// code with its value bits appended.  Returns the bits of the lane (EOB included when the lane
// holds the last non-zero coefficient, or is lane 0 of a block without any).
template <bool kEmit, class Emit>
__device__ __forceinline__ int lane_ac(const Lane8& l, int r, uint64_t mask, const uint32_t* ac, Emit&& emit) {
    const uint32_t zrl = ac[0xF0], eob = ac[0x00];
    int bits = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) {
        const int p = 8 * r + j;
        if (!((mask >> p) & 1)) continue;
        const uint64_t below = mask & ((1ull << p) - 1);
        const int prev = below ? 63 - __clzll((long long)below) : 0;
        const int run = p - prev - 1;
        const int v = l.z[j], cat = category(v);
        const uint32_t e = ac[((run & 15) << 4) | cat];
        const int size = (int)(e >> 16);
        bits += (run >> 4) * (int)(zrl >> 16) + (size ? size + cat : 0);
        if (kEmit) {
            for (int k = 0; k < (run >> 4); k++) emit(zrl & 0xFFFFu, (int)(zrl >> 16));
            if (size) emit(((e & 0xFFFFu) << cat) | value_bits(v, cat), size + cat);
        }
    }
    const int last = mask ? 63 - __clzll((long long)mask) : 0;
    if ((last >> 3) == r) {
        bits += (int)(eob >> 16);
        if (kEmit) emit(eob & 0xFFFFu, (int)(eob >> 16));
    }
    return bits;
}

// MSB-first writer into the zeroed big-endian word stream from an absolute bit position.  Only
// the first and the last word of a lane's span can hold other lanes' bits: those two are ORed
// atomically, the words in between belong to the lane alone and are stored.
struct BitSink {
    uint32_t* w;
    unsigned long long idx;
    uint64_t acc;
    int n;
    bool first;
    __device__ BitSink(uint32_t* words, unsigned long long start)
        : w(words), idx(start >> 5), acc(0), n((int)(start & 31)), first(true) {}
    __device__ __forceinline__ void operator()(uint32_t bits, int len) {
        acc = (acc << len) | bits;
        n += len;
        if (n >= 32) {
            n -= 32;
            const uint32_t word = (uint32_t)(acc >> n);
            if (first)
                atomicOr(w + idx, word);
            else
                w[idx] = word;
            first = false;
            idx++;
            acc &= (1ull << n) - 1;
        }
    }
    __device__ __forceinline__ void finish() {
        if (n > 0) atomicOr(w + idx, (uint32_t)(acc << (32 - n)));
    }
};

struct NoEmit {
    __device__ void operator()(uint32_t, int) const {}
};

// exclusive scan over the CTA; warp_sums holds NT / 32 entries
template <int NT, class T>
__device__ __forceinline__ T cta_excl_scan(T v, T* warp_sums, T& total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    T incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T nb = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += nb;
    }
    if (lane == 31) warp_sums[wid] = incl;
    __syncthreads();
    T pre = 0, tot = 0;
#pragma unroll
    for (int i = 0; i < NT / 32; i++) {
        const T s = warp_sums[i];
        if (i < wid) pre += s;
        tot += s;
    }
    __syncthreads();
    total = tot;
    return pre + incl - v;
}

// one CTA of 1024 threads: out[i] = sum(in[0..i)), returns the total
__device__ unsigned long long cta_scan_array(const int* in, unsigned long long* out, long long n) {
    __shared__ unsigned long long ws[32];
    unsigned long long carry = 0;
    for (long long base = 0; base < n; base += 1024) {
        const long long i = base + threadIdx.x;
        const unsigned long long v = i < n ? (unsigned long long)in[i] : 0ull;
        unsigned long long tot;
        const unsigned long long ex = cta_excl_scan<1024>(v, ws, tot);
        if (i < n) out[i] = carry + ex;
        carry += tot;
    }
    return carry;
}

// ---- transform: 8 threads per block; thread r owns sample row r, then coefficient column r ---
__global__ void __launch_bounds__(kThreads) jpeg_transform_kernel(JpegLaunch L) {
    __shared__ __align__(16) float T[kJpegBlocksPerCta][72];  // row-DCT output, [u * 8 + y]
    __shared__ __align__(16) int16_t Z[kJpegBlocksPerCta][64];
    __shared__ float sq[2][64];
    __shared__ uint8_t szz[64];
    __shared__ uint32_t sac[2][256];
    const int t = threadIdx.x;
    if (t < 128) sq[t >> 6][t & 63] = L.q[t >> 6][t & 63];
    if (t < 64) szz[t] = c_zz[t];
    for (int i = t; i < 512; i += kThreads) sac[i >> 8][i & 255] = L.huff->ac[i >> 8][i & 255];

    const int lb = t >> 3, r = t & 7;
    const long long bl = (long long)blockIdx.x * kJpegBlocksPerCta + lb;
    const bool live = bl < L.g.nb;
    const int b = (int)bl;
    BlockPos P;
    P.comp = 0;
    if (live) P = block_pos(L.g, b);

    // sample row r -> row DCT, written transposed
    float x[8];
    if (live) {
        const int py = min(P.y0 + r * P.sy, L.g.h - 1);
        const uint8_t* row = L.rgb + (size_t)py * (size_t)L.g.w * 3;
#pragma unroll
        for (int i = 0; i < 8; i++) {
            const int px = min(P.x0 + i * P.sx, L.g.w - 1);
            const uint8_t* s = row + (size_t)px * 3;
            x[i] = (float)(ycc(s[0], s[1], s[2], P.comp) - 128);
        }
    } else {
#pragma unroll
        for (int i = 0; i < 8; i++) x[i] = 0.0f;
    }
#pragma unroll
    for (int u = 0; u < 8; u++) {
        float s = 0.0f;
#pragma unroll
        for (int i = 0; i < 8; i++) s = fadd(s, fmul(x[i], c_cos[u * 8 + i]));
        T[lb][u * 8 + r] = fmul(u == 0 ? kC0 : 0.5f, s);
    }
    __syncthreads();

    // column u = r -> quantise into the coefficient slots
    {
        const float4 c0 = *reinterpret_cast<const float4*>(&T[lb][r * 8]);
        const float4 c1 = *reinterpret_cast<const float4*>(&T[lb][r * 8 + 4]);
        const float col[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
        const float* qt = sq[P.comp > 0 ? 1 : 0];
#pragma unroll
        for (int v = 0; v < 8; v++) {
            float s = 0.0f;
#pragma unroll
            for (int y = 0; y < 8; y++) s = fadd(s, fmul(col[y], c_cos[v * 8 + y]));
            const float X = fmul(v == 0 ? kC0 : 0.5f, s);
            const int i = v * 8 + r;
            Z[lb][szz[i]] = (int16_t)__float2int_rz(roundf(__fdiv_rn(X, qt[i])));
        }
    }
    __syncthreads();

    const uint4 raw = *reinterpret_cast<const uint4*>(&Z[lb][r * 8]);
    const Lane8 l = unpack8(raw);
    const uint64_t mask = block_mask(l, r);
    int bits = lane_ac<false>(l, r, mask, sac[P.comp > 0 ? 1 : 0], NoEmit{});
    bits += __shfl_xor_sync(kFull, bits, 1);
    bits += __shfl_xor_sync(kFull, bits, 2);
    bits += __shfl_xor_sync(kFull, bits, 4);
    if (!live) return;
    *reinterpret_cast<uint4*>(L.coef + (size_t)b * 64 + r * 8) = raw;
    if (r == 0) {
        L.acbits[b] = bits;
        L.dc[b] = l.z[0];
    }
}

// ---- offsets: per-block length with the DC difference; tile-local exclusive offsets ---------
__global__ void __launch_bounds__(kThreads) jpeg_offsets_kernel(JpegLaunch L) {
    __shared__ uint32_t sdc[2][16];
    __shared__ int ws[kThreads / 32];
    const int t = threadIdx.x;
    if (t < 32) sdc[t >> 4][t & 15] = L.huff->dc[t >> 4][t & 15];
    __syncthreads();
    const long long b0 = (long long)blockIdx.x * kJpegTileBlocks + t * 8;
    int len[8], sum = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) {
        len[j] = 0;
        if (b0 + j < L.g.nb) {
            const int b = (int)(b0 + j);
            const BlockPos P = block_pos(L.g, b);
            const int diff = L.dc[b] - (P.prev >= 0 ? L.dc[P.prev] : 0);
            const int cat = category(diff);
            len[j] = L.acbits[b] + (int)(sdc[P.comp > 0 ? 1 : 0][min(cat, 15)] >> 16) + cat;
        }
        sum += len[j];
    }
    int total;
    int off = cta_excl_scan<kThreads>(sum, ws, total);
#pragma unroll
    for (int j = 0; j < 8; j++) {
        if (b0 + j < L.g.nb) L.blk_off[b0 + j] = off;
        off += len[j];
    }
    if (t == 0) L.tile_sum[blockIdx.x] = total;
}

// ---- tiles: one CTA scans the tile sums -------------------------------------------------------
__global__ void __launch_bounds__(1024) jpeg_tiles_kernel(JpegLaunch L) {
    const unsigned long long total = cta_scan_array(L.tile_sum, L.tile_off, L.g.ntiles);
    if (threadIdx.x == 0) {
        L.info->total_bits = total;
        L.info->data_bytes = (total + 7) >> 3;
    }
}

// ---- emit: 8 threads per block write their codes at the block's offset ----------------------
__global__ void __launch_bounds__(kThreads) jpeg_emit_kernel(JpegLaunch L) {
    __shared__ uint32_t sac[2][256];
    __shared__ uint32_t sdc[2][16];
    const int t = threadIdx.x;
    for (int i = t; i < 512; i += kThreads) sac[i >> 8][i & 255] = L.huff->ac[i >> 8][i & 255];
    if (t < 32) sdc[t >> 4][t & 15] = L.huff->dc[t >> 4][t & 15];
    __syncthreads();

    const int lb = t >> 3, r = t & 7;
    const long long bl = (long long)blockIdx.x * kJpegBlocksPerCta + lb;
    const bool live = bl < L.g.nb;
    const int b = (int)bl;
    uint4 raw = make_uint4(0u, 0u, 0u, 0u);
    BlockPos P;
    P.comp = 0;
    P.prev = -1;
    if (live) {
        raw = *reinterpret_cast<const uint4*>(L.coef + (size_t)b * 64 + r * 8);
        P = block_pos(L.g, b);
    }
    const Lane8 l = unpack8(raw);
    const uint64_t mask = block_mask(l, r);
    const int tab = P.comp > 0 ? 1 : 0;
    int bits = lane_ac<false>(l, r, mask, sac[tab], NoEmit{});
    uint32_t dcode = 0;
    int dlen = 0;
    if (live && r == 0) {
        const int diff = l.z[0] - (P.prev >= 0 ? L.dc[P.prev] : 0);
        const int cat = category(diff);
        const uint32_t e = sdc[tab][min(cat, 15)];
        dlen = (int)(e >> 16) + cat;
        dcode = ((e & 0xFFFFu) << cat) | value_bits(diff, cat);
    }
    bits += dlen;
    int incl = bits;
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
        const int nb = __shfl_up_sync(kFull, incl, o, 8);
        if (r >= o) incl += nb;
    }
    if (!live || bits == 0) return;
    const unsigned long long start =
        L.tile_off[b / kJpegTileBlocks] + (unsigned long long)L.blk_off[b] + (unsigned long long)(incl - bits);
    BitSink sink(L.words, start);
    if (dlen) sink(dcode, dlen);
    lane_ac<true>(l, r, mask, sac[tab], sink);
    sink.finish();
}

// the 16 bytes of 4 big-endian words, most significant byte first
__device__ __forceinline__ uint8_t byte_of(const uint32_t w[4], int k) {
    return (uint8_t)(w[k >> 2] >> (24 - 8 * (k & 3)));
}

__device__ __forceinline__ int ff_count(const uint32_t w[4]) {
    int c = 0;
#pragma unroll
    for (int k = 0; k < 16; k++) c += byte_of(w, k) == 0xFF;
    return c;
}

// ---- ffcount: 0xFF bytes per 4 KB chunk (bytes past the stream are zero words) ---------------
__global__ void __launch_bounds__(kThreads) jpeg_ffcount_kernel(JpegLaunch L) {
    __shared__ int ws[kThreads / 32];
    const long long nch = (long long)((L.info->data_bytes + kJpegChunkBytes - 1) / kJpegChunkBytes);
    for (long long c = blockIdx.x; c < nch; c += gridDim.x) {
        const uint4 v = *reinterpret_cast<const uint4*>(L.words + (size_t)c * (kJpegChunkBytes / 4) + threadIdx.x * 4);
        const uint32_t w[4] = {v.x, v.y, v.z, v.w};
        int total;
        cta_excl_scan<kThreads>(ff_count(w), ws, total);
        if (threadIdx.x == 0) L.chunk_ff[c] = total;
    }
}

// ---- ffscan: chunk offsets, sizes and the EOI marker ---------------------------------------
__global__ void __launch_bounds__(1024) jpeg_ffscan_kernel(JpegLaunch L) {
    const unsigned long long nbytes = L.info->data_bytes;
    const long long nch = (long long)((nbytes + kJpegChunkBytes - 1) / kJpegChunkBytes);
    const unsigned long long nff = cta_scan_array(L.chunk_ff, L.chunk_off, nch);
    if (threadIdx.x == 0) {
        const unsigned long long stuffed = nbytes + nff, eoi = L.base + stuffed;
        if (eoi < L.out_cap) L.out[eoi] = 0xFF;
        if (eoi + 1 < L.out_cap) L.out[eoi + 1] = 0xD9;
        const unsigned long long jpeg = eoi + 2, written = jpeg < L.out_cap ? jpeg : L.out_cap;
        L.info->stuffed = stuffed;
        L.info->jpeg_bytes = jpeg;
        L.info->written = written;
        if (L.size_out) *L.size_out = written;
    }
}

// ---- stuff: bytes out with a 0x00 after each 0xFF; the consumed words are cleared -----------
__global__ void __launch_bounds__(kThreads) jpeg_stuff_kernel(JpegLaunch L) {
    __shared__ int ws[kThreads / 32];
    const unsigned long long nbytes = L.info->data_bytes;
    const long long nch = (long long)((nbytes + kJpegChunkBytes - 1) / kJpegChunkBytes);
    for (long long c = blockIdx.x; c < nch; c += gridDim.x) {
        uint4* src = reinterpret_cast<uint4*>(L.words + (size_t)c * (kJpegChunkBytes / 4) + threadIdx.x * 4);
        const uint4 v = *src;
        const uint32_t w[4] = {v.x, v.y, v.z, v.w};
        int total;
        const int before = cta_excl_scan<kThreads>(ff_count(w), ws, total);
        const unsigned long long byte0 = (unsigned long long)c * kJpegChunkBytes + threadIdx.x * 16ull;
        unsigned long long pos = L.base + byte0 + L.chunk_off[c] + (unsigned long long)before;
#pragma unroll
        for (int k = 0; k < 16; k++) {
            if (byte0 + k >= nbytes) break;
            const uint8_t bv = byte_of(w, k);
            if (pos < L.out_cap) L.out[pos] = bv;
            pos++;
            if (bv == 0xFF) {
                if (pos < L.out_cap) L.out[pos] = 0x00;
                pos++;
            }
        }
        *src = make_uint4(0u, 0u, 0u, 0u);
    }
}

}  // namespace

JpegGeom jpeg_geometry(int w, int h, int subsample) {
    JpegGeom g{};
    const int ss = subsample < 0 ? 0 : (subsample > 2 ? 2 : subsample);
    g.w = w;
    g.h = h;
    g.hy = ss == 0 ? 1 : 2;
    g.vy = ss == 1 ? 2 : 1;
    g.mw = 8 * g.hy;
    g.mh = 8 * g.vy;
    g.mcus_x = (w + g.mw - 1) / g.mw;
    g.mcus_y = (h + g.mh - 1) / g.mh;
    g.ny = g.hy * g.vy;
    g.bpm = g.ny + 2;
    g.nb = (long long)g.mcus_x * g.mcus_y * g.bpm;
    g.ntiles = (int)((g.nb + kJpegTileBlocks - 1) / kJpegTileBlocks);
    const long long bound_words = (g.nb * kJpegMaxBlockBits + 31) / 32 + 2;
    g.chunks = (bound_words + (kJpegChunkBytes / 4) - 1) / (kJpegChunkBytes / 4);
    g.words = g.chunks * (kJpegChunkBytes / 4);
    return g;
}

cudaError_t jpeg_init_constants(const float cos_table[64]) {
    return cudaMemcpyToSymbol(c_cos, cos_table, 64 * sizeof(float));
}

cudaError_t launch_jpeg_encode(const JpegLaunch& L, cudaStream_t st) {
    const unsigned grid_blocks = (unsigned)((L.g.nb + kJpegBlocksPerCta - 1) / kJpegBlocksPerCta);
    const unsigned grid_chunks = (unsigned)(L.g.chunks < 152 * 8 ? L.g.chunks : 152 * 8);
    jpeg_transform_kernel<<<grid_blocks, kThreads, 0, st>>>(L);
    jpeg_offsets_kernel<<<(unsigned)L.g.ntiles, kThreads, 0, st>>>(L);
    jpeg_tiles_kernel<<<1, 1024, 0, st>>>(L);
    jpeg_emit_kernel<<<grid_blocks, kThreads, 0, st>>>(L);
    jpeg_ffcount_kernel<<<grid_chunks, kThreads, 0, st>>>(L);
    jpeg_ffscan_kernel<<<1, 1024, 0, st>>>(L);
    jpeg_stuff_kernel<<<grid_chunks, kThreads, 0, st>>>(L);
    return cudaGetLastError();
}

}  // namespace imop
