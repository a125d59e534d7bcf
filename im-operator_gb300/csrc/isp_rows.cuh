// isp_rows.cuh - raw rows read straight from the frame by the streamed kernels: each lane loads
// the words that hold its 8 samples of a row with plain coalesced loads (no staging through shared
// memory) and unpacks them as 4 packed u16 pairs, P[j] = sample 2j | sample 2j+1 << 16.
//
// The frames these kernels take are 16-byte aligned with a width that is a multiple of 8, so a
// lane's 8 samples start on a word: on the sample for u8 / u16 / RAW12, on the sample or two bytes
// before it for RAW10 (8 samples are two 5-byte groups).  The unpack follows the byte layouts of
// pixel::get_packed_raw (include/imop/pixel_utils.hpp:58-98), the same ones unpack12_pair and the
// tile kernel's staged reads implement.
#pragma once

#include <cstdint>

#include "isp_common.h"
#include "isp_ptx.cuh"
#include "isp_tile.cuh"

namespace imop {
namespace rows {

// bytes per sample as a fraction: u8 1/1, u16 2/1, RAW12 3/2, RAW10 5/4
template <int FMT>
__host__ __device__ constexpr int bytes_num() { return FMT == FMT_U8 ? 1 : FMT == FMT_U16 ? 2 : FMT == FMT_P12 ? 3 : 5; }
template <int FMT>
__host__ __device__ constexpr int bytes_den() { return FMT == FMT_P12 ? 2 : FMT == FMT_P10 ? 4 : 1; }

// the words holding the 8 samples that start at byte lane_byte of a row (zeros when !in); for
// RAW10 w[3] is the byte offset of the samples in the first word
template <int FMT>
__device__ __forceinline__ void load8(const uint8_t* row, int lane_byte, bool in, uint32_t (&w)[4]) {
    w[0] = w[1] = w[2] = w[3] = 0u;
    if (!in) return;
    const uint8_t* p = row + lane_byte;
    if (FMT == FMT_U8) {
        const uint2 v = __ldg(reinterpret_cast<const uint2*>(p));
        w[0] = v.x;
        w[1] = v.y;
    } else if (FMT == FMT_U16) {
        const uint4 v = __ldg(reinterpret_cast<const uint4*>(p));
        w[0] = v.x;
        w[1] = v.y;
        w[2] = v.z;
        w[3] = v.w;
    } else {
        const uint32_t* q = reinterpret_cast<const uint32_t*>(reinterpret_cast<uintptr_t>(p) & ~(uintptr_t)3);
        w[0] = __ldg(q);
        w[1] = __ldg(q + 1);
        w[2] = __ldg(q + 2);
        w[3] = (uint32_t)(reinterpret_cast<uintptr_t>(p) & 3);  // RAW10: byte offset in the first word
    }
}

// the 8 samples of load8's words as packed pairs
template <int FMT>
__device__ __forceinline__ void decode8(const uint32_t (&w)[4], uint32_t (&P)[4]) {
    if (FMT == FMT_U8) {
        P[0] = __byte_perm(w[0], 0u, 0x4140);
        P[1] = __byte_perm(w[0], 0u, 0x4342);
        P[2] = __byte_perm(w[1], 0u, 0x4140);
        P[3] = __byte_perm(w[1], 0u, 0x4342);
    } else if (FMT == FMT_U16) {
        P[0] = w[0];
        P[1] = w[1];
        P[2] = w[2];
        P[3] = w[3];
    } else if (FMT == FMT_P12) {
        P[0] = unpack12_pair(w[0]);
        P[1] = unpack12_pair(__funnelshift_r(w[0], w[1], 24));
        P[2] = unpack12_pair(__funnelshift_r(w[1], w[2], 16));
        P[3] = unpack12_pair(w[2] >> 8);
    } else {
        // RAW10: two 5-byte groups, each four high bytes then the four 2-bit remainders
        const int sh = 8 * (int)w[3];
        const uint32_t a = __funnelshift_r(w[0], w[1], sh), b = __funnelshift_r(w[1], w[2], sh), c = w[2] >> sh;
        const uint32_t hi[2] = {a, __funnelshift_r(b, c, 8)};
        const uint32_t lo[2] = {b & 0xFFu, (c >> 8) & 0xFFu};
#pragma unroll
        for (int g = 0; g < 2; g++)
#pragma unroll
            for (int s = 0; s < 2; s++) {
                const uint32_t h2 = __byte_perm(hi[g], 0u, s ? 0x4342 : 0x4140);  // two high bytes as halves
                const uint32_t l2 = ((lo[g] >> (4 * s)) & 3u) | (((lo[g] >> (4 * s + 2)) & 3u) << 16);
                P[2 * g + s] = (h2 << 2) | l2;
            }
    }
}

// The sample beside a strip: its last column's right neighbour or its first column's left one,
// in as few words as hold it (the strip's first column x0 is a multiple of 8; ring_load_edge
// brings them).  edge_byte is the byte of the row where the sample's bytes start:
//   LAST (the sample x0 - 1, the last of its group)     u8 x, u16 2x, RAW12 3(x >> 1), RAW10 5(x >> 2) + 3
//   first (the sample x0 + 256, the first of its group) u8 x, u16 2x, RAW12 3(x >> 1), RAW10 5(x >> 2)
template <int FMT>
struct Edge {
    static constexpr int N = FMT == FMT_P10 ? 3 : 1;  // RAW10: two words and the byte offset
    uint32_t g[N];
};
template <int FMT, bool LAST>
__host__ __device__ constexpr int edge_byte(int x) {
    return FMT == FMT_U8 ? x : FMT == FMT_U16 ? 2 * x : FMT == FMT_P12 ? 3 * (x >> 1) : 5 * (x >> 2) + (LAST ? 3 : 0);
}
template <int FMT, bool LAST>
__device__ __forceinline__ int decode_edge(const Edge<FMT>& e) {
    const uint32_t w = e.g[0];
    // u8 / u16 / RAW12 rows start on a word, so the sample's place in the word is fixed
    if (FMT == FMT_U8) return LAST ? (int)(w >> 24) : (int)(w & 0xFFu);
    if (FMT == FMT_U16) return LAST ? (int)(w >> 16) : (int)(w & 0xFFFFu);
    if (FMT == FMT_P12) return LAST ? (int)(unpack12_pair(w >> 8) >> 16) : (int)(unpack12_pair(w) & 0xFFFFu);
    // RAW10 rows start on an even byte: the high byte then (LAST) the remainder byte, bits 6-7, or
    // (first) the remainder byte four bytes on, bits 0-1
    const int sh = 8 * (int)e.g[2];
    if (LAST) {
        const uint32_t v = w >> sh;
        return (int)(((v & 0xFFu) << 2) | ((v >> 14) & 3u));
    }
    return (int)((((w >> sh) & 0xFFu) << 2) | ((e.g[1] >> sh) & 3u));
}

// The same words brought into shared memory by the lane itself (ptx::cp_async*), for a ring of
// rows: main = the lane's 16-byte slot, edge = its 8-byte slot for the sample beside the strip.
// Rows outside the frame (in false) fill the slots with zeros and read nothing; `any` stands in
// for the source address then.  The RAW10 byte offsets are not copied: ring_offset gives them.
template <int FMT>
__device__ __forceinline__ void ring_load8(uint32_t main, const uint8_t* row, int lane_byte, bool in, const void* any) {
    const uint8_t* p = row + lane_byte;
    if (FMT == FMT_U8) {
        ptx::cp_async8(main, in ? (const void*)p : any, in ? 8u : 0u);
    } else if (FMT == FMT_U16) {
        ptx::cp_async16(main, in ? (const void*)p : any, in ? 16u : 0u);
    } else {
        const uint8_t* q = reinterpret_cast<const uint8_t*>(reinterpret_cast<uintptr_t>(p) & ~(uintptr_t)3);
#pragma unroll
        for (int k = 0; k < 3; k++) ptx::cp_async4(main + 4 * k, in ? (const void*)(q + 4 * k) : any, in ? 4u : 0u);
    }
}
// the same for u8 / u16 rows that start on a word but not on the lane's 8- / 16-byte load:
// word copies, each limited to the `left` bytes of the row from the lane's first sample on (the
// samples past the row's end read as zeros)
template <int FMT>
__device__ __forceinline__ void ring_load8_words(uint32_t main, const uint8_t* row, int lane_byte, int left, bool in,
                                                 const void* any) {
    const uint8_t* p = row + lane_byte;
    constexpr int kWords = FMT == FMT_U8 ? 2 : 4;
#pragma unroll
    for (int k = 0; k < kWords; k++) {
        const int n = in ? min(max(left - 4 * k, 0), 4) : 0;
        ptx::cp_async4(main + 4 * k, n ? (const void*)(p + 4 * k) : any, (uint32_t)n);
    }
}
template <int FMT>
__device__ __forceinline__ void ring_load_edge(uint32_t edge, const uint8_t* row, int byte, bool in, const void* any) {
    const uint8_t* q =
        reinterpret_cast<const uint8_t*>(reinterpret_cast<uintptr_t>(row + byte) & ~(uintptr_t)3);
    ptx::cp_async4(edge, in ? (const void*)q : any, in ? 4u : 0u);
    if (FMT == FMT_P10) ptx::cp_async4(edge + 4, in ? (const void*)(q + 4) : any, in ? 4u : 0u);
}
// the byte offset of a RAW10 lane's samples (or edge sample) in its first copied word
__device__ __forceinline__ uint32_t ring_offset(const uint8_t* row, int byte) {
    return (uint32_t)(reinterpret_cast<uintptr_t>(row + byte) & 3);
}

}  // namespace rows
}  // namespace imop
