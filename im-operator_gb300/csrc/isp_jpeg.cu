// isp_jpeg.cu - baseline JPEG encoder kernels (see isp_jpeg.h for the pipeline).
//
// Exactness: every float operation of the reference's encoder is one explicitly rounded IEEE
// operation here, in the reference's order (colour conversion common.hpp:196-201, DCT
// common.hpp:104-151 with the cosine factors the host evaluates with the same cosf, quantiser
// division and std::round encode_baseline.cpp:24-26; the division as a correctly rounded
// reciprocal product with one residual correction, equal to IEEE division).  The coefficient
// array is the reference's zz[kZigzag[i]] = round(block[i] / q[i]) (common.hpp:84-93), and the
// run-length / Huffman rules are those of encode_baseline.cpp:28-101, restated per slot:
//   - a non-zero AC coefficient at p whose previous non-zero AC (or the DC slot) is at p' codes
//     floor((p - p' - 1) / 16) ZRL symbols, then symbol (((p - p' - 1) mod 16) << 4) | cat with
//     its cat value bits, or nothing at all when that symbol is absent from the table;
//   - EOB always follows the last non-zero AC coefficient, also at position 63, and a block
//     without AC coefficients codes EOB alone.

#include <cuda_runtime.h>
#include <stdint.h>

#include "isp_device.cuh"
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

// OR len (<= 26) bits MSB-first at bit position pos of a shared word buffer
__device__ __forceinline__ void smem_put(uint32_t* buf, int pos, uint32_t bits, int len) {
    const int w = pos >> 5, end = (pos & 31) + len;
    if (end <= 32) {
        atomicOr(buf + w, bits << (32 - end));
    } else {
        atomicOr(buf + w, bits >> (end - 32));
        atomicOr(buf + w + 1, bits << (64 - end));
    }
}

// The AC codes of lane r's slots [8r, 8r + 8): per slot the ZRL count (bits 8..15 of cl) and the
// symbol code with its value bits appended (cw, length in bits 0..7 of cl; 0 when the symbol is
// absent from the table).  Returns the lane's bits, EOB included when the lane holds the last
// non-zero coefficient (lane 0 of a block without any).
struct LaneCodes {
    uint32_t cw[8];
    int cl[8];
    bool eob;
};

__device__ __forceinline__ int lane_codes(const Lane8& l, int r, uint64_t mask, const uint32_t* ac, LaneCodes& c) {
    const int zrl = (int)(ac[0xF0] >> 16), eob = (int)(ac[0x00] >> 16);
    // the previous non-zero AC slot before this lane's first one (0: the DC slot)
    const uint64_t below = mask & ((1ull << (8 * r)) - 1);
    int prev = below ? 63 - __clzll((long long)below) : 0;
    const uint32_t mine = (uint32_t)(mask >> (8 * r)) & 0xFFu;
    int bits = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) {
        c.cw[j] = 0u;
        c.cl[j] = 0;
        if (!((mine >> j) & 1)) continue;
        const int p = 8 * r + j;
        const int run = p - prev - 1, v = l.z[j], cat = category(v);
        prev = p;
        const uint32_t e = ac[((run & 15) << 4) | cat];
        const int size = (int)(e >> 16), len = size ? size + cat : 0;
        c.cw[j] = size ? ((e & 0xFFFFu) << cat) | value_bits(v, cat) : 0u;
        c.cl[j] = ((run >> 4) << 8) | len;
        bits += (run >> 4) * zrl + len;
    }
    c.eob = mine ? (r == 7 || (mask >> (8 * r + 8)) == 0) : (r == 0 && mask == 0);
    if (c.eob) bits += eob;
    return bits;
}

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

// one CTA of NT threads: out[i] = sum(in[0..i)), returns the total (in[] read past L1: other
// CTAs wrote it)
template <int NT>
__device__ unsigned long long cta_scan_array(const int* in, unsigned long long* out, long long n) {
    __shared__ unsigned long long ws[NT / 32];
    unsigned long long carry = 0;
    for (long long base = 0; base < n; base += NT) {
        const long long i = base + threadIdx.x;
        const unsigned long long v = i < n ? (unsigned long long)__ldcg(in + i) : 0ull;
        unsigned long long tot;
        const unsigned long long ex = cta_excl_scan<NT>(v, ws, tot);
        if (i < n) out[i] = carry + ex;
        carry += tot;
    }
    return carry;
}

// True in the CTA that finishes last (all CTAs' earlier global writes visible to it), which also
// rewinds the counter for the next launch on the stream.  No CTA waits for another.
__device__ __forceinline__ bool last_cta(unsigned* counter) {
    __shared__ int last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned done = atomicAdd(counter, 1u);
        last = done == gridDim.x - 1;
        if (last) *counter = 0u;
    }
    __syncthreads();
    if (last) __threadfence();
    return last != 0;
}

// ---- transform: 8 threads per block; thread r owns sample row r, then coefficient column r ---
__global__ void __launch_bounds__(kThreads) jpeg_transform_kernel(JpegLaunch L) {
    __shared__ __align__(16) float T[kJpegBlocksPerCta][72];  // row-DCT output, [u * 8 + y]
    __shared__ __align__(16) int16_t Z[kJpegBlocksPerCta][64];
    __shared__ uint32_t SB[kJpegBlocksPerCta][kJpegAcWords];  // each block's AC code, from bit 0
    __shared__ float sq[2][64], srq[2][64];
    __shared__ uint8_t szz[64];
    __shared__ uint32_t sac[2][256];
    const int t = threadIdx.x;
    if (t < 128) sq[t >> 6][t & 63] = L.q[t >> 6][t & 63], srq[t >> 6][t & 63] = L.rq[t >> 6][t & 63];
    if (t < 64) szz[t] = c_zz[t];
    for (int i = t; i < 512; i += kThreads) sac[i >> 8][i & 255] = L.huff->ac[i >> 8][i & 255];
    for (int i = t; i < kJpegBlocksPerCta * kJpegAcWords; i += kThreads) (&SB[0][0])[i] = 0u;

    const int lb = t >> 3, r = t & 7;
    const long long bl = (long long)blockIdx.x * kJpegBlocksPerCta + lb;
    const bool live = bl < L.g.nb;
    const int b = (int)bl;
    BlockPos P;
    P.comp = 0;
    if (live) P = block_pos(L.g, b);
    const int comp = P.comp;

    // sample row r -> row DCT, written transposed
    int xi[8];
#pragma unroll
    for (int i = 0; i < 8; i++) xi[i] = 0;
    if (live) {
        const int py = min(P.y0 + r * P.sy, L.g.h - 1);
        const uint8_t* row = L.rgb + ((size_t)py * (size_t)L.g.w + (size_t)P.x0) * 3;
        if (P.x0 + 7 * P.sx < L.g.w) {  // interior: fixed offsets from one base
            const int step = 3 * P.sx;
#pragma unroll
            for (int i = 0; i < 8; i++) xi[i] = ycc(row[i * step], row[i * step + 1], row[i * step + 2], comp) - 128;
        } else {
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const int dx = min(P.x0 + i * P.sx, L.g.w - 1) - P.x0;
                const uint8_t* s = row + dx * 3;
                xi[i] = ycc(s[0], s[1], s[2], comp) - 128;
            }
        }
    }
    float x[8];
#pragma unroll
    for (int i = 0; i < 8; i++) x[i] = (float)xi[i];
    // u = 0: every factor is cosf(0) = 1, so the products are the samples and the running sums are
    // integers of magnitude <= 1024, exact in float: the integer sum is the float sum
    T[lb][r] = fmul(kC0, (float)(((xi[0] + xi[1]) + (xi[2] + xi[3])) + ((xi[4] + xi[5]) + (xi[6] + xi[7]))));
#pragma unroll
    for (int u = 1; u < 8; u++) {
        float s = fmul(x[0], c_cos[u * 8]);
#pragma unroll
        for (int i = 1; i < 8; i++) s = fadd(s, fmul(x[i], c_cos[u * 8 + i]));
        T[lb][u * 8 + r] = fmul(0.5f, s);
    }
    __syncthreads();

    // column u = r -> quantise into the coefficient slots
    {
        const float4 c0 = *reinterpret_cast<const float4*>(&T[lb][r * 8]);
        const float4 c1 = *reinterpret_cast<const float4*>(&T[lb][r * 8 + 4]);
        const float col[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
        const float* qt = sq[comp > 0 ? 1 : 0];
        const float* rqt = srq[comp > 0 ? 1 : 0];
#pragma unroll
        for (int v = 0; v < 8; v++) {
            // the first product joins the running sum 0 exactly (a zero's sign cannot reach the
            // rounded integer); for v = 0 the factors are 1 and the products are the inputs
            float s = v == 0 ? col[0] : fmul(col[0], c_cos[v * 8]);
#pragma unroll
            for (int y = 1; y < 8; y++) s = fadd(s, v == 0 ? col[y] : fmul(col[y], c_cos[v * 8 + y]));
            const float X = fmul(v == 0 ? kC0 : 0.5f, s);
            const int i = v * 8 + r;
            Z[lb][szz[i]] = (int16_t)__float2int_rz(roundf(dev::quotient_by(X, qt[i], rqt[i])));
        }
    }
    __syncthreads();

    // AC codes: lane r codes slots [8r, 8r + 8) at its offset inside the block's code
    const Lane8 l = unpack8(*reinterpret_cast<const uint4*>(&Z[lb][r * 8]));
    const uint64_t mask = block_mask(l, r);
    const uint32_t* ac = sac[comp > 0 ? 1 : 0];
    LaneCodes c;
    const int bits = lane_codes(l, r, mask, ac, c);
    int incl = bits;
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
        const int nb = __shfl_up_sync(kFull, incl, o, 8);
        if (r >= o) incl += nb;
    }
    const int total = __shfl_sync(kFull, incl, 7, 8);
    if (!live) return;
    uint32_t* sb = SB[lb];
    int pos = incl - bits;
    const uint32_t zrl = ac[0xF0], eob = ac[0x00];
#pragma unroll
    for (int j = 0; j < 8; j++) {
        for (int k = 0; k < (c.cl[j] >> 8); k++, pos += (int)(zrl >> 16)) smem_put(sb, pos, zrl & 0xFFFFu, (int)(zrl >> 16));
        const int len = c.cl[j] & 0xFF;
        if (len) smem_put(sb, pos, c.cw[j], len), pos += len;
    }
    if (c.eob) smem_put(sb, pos, eob & 0xFFFFu, (int)(eob >> 16));
    __syncwarp(kFull & (0xFFu << (threadIdx.x & 24)));
    // the used words and one zero word after them
    const int nw = ((total + 31) >> 5) + 1;
    uint32_t* dst = L.acw + (size_t)b * kJpegAcWords;
    for (int k = r; k < nw; k += 8) dst[k] = sb[k];
    if (r == 0) {
        L.acbits[b] = total;
        L.dc[b] = l.z[0];
    }
}

// ---- offsets: per-block length with the DC difference, tile-local exclusive offsets; the last
// CTA turns the tile sums into tile offsets ---------------------------------------------------
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
    // the last CTA scans the tile sums into tile offsets and the total
    if (!last_cta(L.counters)) return;
    const unsigned long long bits = cta_scan_array<kThreads>(L.tile_sum, L.tile_off, L.g.ntiles);
    if (t == 0) {
        L.info->total_bits = bits;
        L.info->data_bytes = (bits + 7) >> 3;
    }
}

// ---- place: each block's DC code and AC code at its stream offset; 8 threads per block, thread
// r writes words r, r + 8, ... of the block's span.  The first and the last word, which the
// neighbouring blocks share, are ORed atomically into the zeroed stream. ----------------------
__global__ void __launch_bounds__(kThreads) jpeg_place_kernel(JpegLaunch L) {
    __shared__ uint32_t sdc[2][16];
    const int t = threadIdx.x;
    if (t < 32) sdc[t >> 4][t & 15] = L.huff->dc[t >> 4][t & 15];
    __syncthreads();
    const int lb = t >> 3, r = t & 7;
    const long long bl = (long long)blockIdx.x * kJpegBlocksPerCta + lb;
    if (bl >= L.g.nb) return;  // whole 8-thread groups
    const int b = (int)bl;
    const unsigned grp = 0xFFu << (t & 24);
    // thread 0 of the group works out the block's DC code and span; the others receive them
    uint32_t dcode = 0;
    int dlen = 0, pre = 0, end = 0;
    unsigned long long start = 0;
    if (r == 0) {
        const BlockPos P = block_pos(L.g, b);
        const int diff = L.dc[b] - (P.prev >= 0 ? L.dc[P.prev] : 0);
        const int cat = category(diff);
        const uint32_t e = sdc[P.comp > 0 ? 1 : 0][min(cat, 15)];
        dlen = (int)(e >> 16) + cat;
        dcode = ((e & 0xFFFFu) << cat) | value_bits(diff, cat);
        start = L.tile_off[b / kJpegTileBlocks] + (unsigned long long)L.blk_off[b];
        // the span as a virtual stream: (start mod 32) zero bits, the DC code, the AC code
        pre = (int)(start & 31) + dlen;  // 2 .. 53
        end = pre + L.acbits[b];
    }
    const int src = t & 24;
    dcode = __shfl_sync(grp, dcode, src);
    pre = __shfl_sync(grp, pre, src);
    end = __shfl_sync(grp, end, src);
    start = __shfl_sync(grp, start, src);
    const int nw = (end + 31) >> 5;
    const uint64_t pl = (uint64_t)dcode << (64 - pre);
    const uint32_t* A = L.acw + (size_t)b * kJpegAcWords;
    uint32_t* g = L.words + (start >> 5);
    for (int k = r; k < nw; k += 8) {
        const int lo = 32 * k;
        uint32_t v = lo < pre ? (uint32_t)((pl << lo) >> 32) : 0u;
        const int off = lo - pre;  // AC bit at the word's first position
        if (off >= 0) {
            const int j = off >> 5, s = off & 31;
            v |= (A[j] << s) | (s ? A[j + 1] >> (32 - s) : 0u);
        } else if (off > -32) {
            v |= A[0] >> (-off);
        }
        if (end - lo < 32) v &= ~0u << (32 - (end - lo));
        if (k == 0 || k == nw - 1)
            atomicOr(g + k, v);
        else
            g[k] = v;
    }
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

// ---- ffcount: 0xFF bytes per 4 KB chunk (bytes past the stream are zero words); the last CTA
// scans the counts into chunk offsets, sets the sizes and writes the EOI marker ---------------
__global__ void __launch_bounds__(kThreads) jpeg_ffcount_kernel(JpegLaunch L) {
    __shared__ int ws[kThreads / 32];
    const unsigned long long nbytes = L.info->data_bytes;
    const long long nch = (long long)((nbytes + kJpegChunkBytes - 1) / kJpegChunkBytes);
    for (long long c = blockIdx.x; c < nch; c += gridDim.x) {
        const uint4 v = *reinterpret_cast<const uint4*>(L.words + (size_t)c * (kJpegChunkBytes / 4) + threadIdx.x * 4);
        const uint32_t w[4] = {v.x, v.y, v.z, v.w};
        int total;
        cta_excl_scan<kThreads>(ff_count(w), ws, total);
        if (threadIdx.x == 0) L.chunk_ff[c] = total;
    }
    if (!last_cta(L.counters + 1)) return;
    const unsigned long long nff = cta_scan_array<kThreads>(L.chunk_ff, L.chunk_off, nch);
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

// ---- stuff: bytes out with a 0x00 after each 0xFF, staged per chunk in shared memory so the
// global writes are consecutive bytes per warp; the consumed words are cleared -----------------
__global__ void __launch_bounds__(kThreads) jpeg_stuff_kernel(JpegLaunch L) {
    __shared__ int ws[kThreads / 32];
    __shared__ uint8_t sb[2 * kJpegChunkBytes];
    const unsigned long long nbytes = L.info->data_bytes;
    const long long nch = (long long)((nbytes + kJpegChunkBytes - 1) / kJpegChunkBytes);
    for (long long c = blockIdx.x; c < nch; c += gridDim.x) {
        uint4* src = reinterpret_cast<uint4*>(L.words + (size_t)c * (kJpegChunkBytes / 4) + threadIdx.x * 4);
        const uint4 v = *src;
        *src = make_uint4(0u, 0u, 0u, 0u);
        const uint32_t w[4] = {v.x, v.y, v.z, v.w};
        int total;
        const int before = cta_excl_scan<kThreads>(ff_count(w), ws, total);
        const unsigned long long chunk0 = (unsigned long long)c * kJpegChunkBytes;
        const int in_chunk = (int)min((unsigned long long)kJpegChunkBytes, nbytes - chunk0);
        int pos = threadIdx.x * 16 + before;
#pragma unroll
        for (int k = 0; k < 16; k++) {
            if (threadIdx.x * 16 + k >= in_chunk) break;
            const uint8_t bv = byte_of(w, k);
            sb[pos++] = bv;
            if (bv == 0xFF) sb[pos++] = 0x00;
        }
        __syncthreads();
        const int n = in_chunk + total;
        const unsigned long long dst = L.base + chunk0 + L.chunk_off[c];
        for (int k = threadIdx.x; k < n; k += kThreads)
            if (dst + k < L.out_cap) L.out[dst + k] = sb[k];
        __syncthreads();
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
    jpeg_place_kernel<<<grid_blocks, kThreads, 0, st>>>(L);
    jpeg_ffcount_kernel<<<grid_chunks, kThreads, 0, st>>>(L);
    jpeg_stuff_kernel<<<grid_chunks, kThreads, 0, st>>>(L);
    return cudaGetLastError();
}

}  // namespace imop
