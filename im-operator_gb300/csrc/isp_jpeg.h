// isp_jpeg.h - baseline JPEG encoder of RGB8 frames on the device (internal interface).
//
// The output is byte for byte what jpeg_codec::process_encode_baseline writes
// (src/jpeg_codec/encode_baseline.cpp:222-376 of the reference): the same headers, the same
// float colour conversion and separable DCT, the same quantisation with the reference's
// coefficient permutation, and the same Huffman / run-length coding with its quirks.  The
// sequential bit writer is replaced by per-block code strings and lengths, a device prefix sum,
// parallel placement into a zeroed 32-bit word stream, and a parallel 0xFF byte-stuffing pass.
//
// Kernels (one stream, no host synchronisation between them):
//   transform  RGB8 -> Y/Cb/Cr sample blocks -> DCT -> quantise -> the block's DC and its AC
//              codes (ZRL / symbol / EOB) as a word-aligned bit string with its length
//   offsets    per-block bit length with the DC difference, tile-local exclusive offsets, tile
//              sums; the CTA that finishes last scans the tile sums -> tile offsets, total bits
//   place      each block's DC code and AC string at its offset in the word stream
//   ffcount    0xFF bytes per 4 KB chunk of the bit stream; the last CTA scans the counts ->
//              chunk offsets, sizes, EOI marker
//   stuff      bytes to the output with a 0x00 after every 0xFF; clears the words it consumed
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace imop {

constexpr int kJpegBlocksPerCta = 32;    // transform / place: 8 threads per block, 256 threads
constexpr int kJpegTileBlocks = 2048;    // offsets: 256 threads x 8 blocks
constexpr int kJpegChunkBytes = 4096;    // stuffing: 256 threads x 16 bytes
constexpr int kJpegMaxBlockBits = 1680;  // bound of one block's code (8-bit samples): DC <= 22,
                                         // 63 AC x (16 + 10), EOB <= 4
constexpr int kJpegAcWords = 53;         // per-block AC code slot: <= 1642 bits + one zero word

// Huffman lookup: (size << 16) | code per symbol; size 0 = symbol absent from the table
struct JpegHuff {
    uint32_t dc[2][16];   // [luma, chroma][category]
    uint32_t ac[2][256];  // [luma, chroma][(run << 4) | category]
};

// sizes the device reports (written by the last CTA of the ffcount kernel)
struct JpegInfo {
    unsigned long long total_bits;  // entropy-coded bits before stuffing
    unsigned long long data_bytes;  // ceil(total_bits / 8)
    unsigned long long stuffed;     // data bytes after stuffing
    unsigned long long jpeg_bytes;  // base + stuffed + 2 (EOI)
    unsigned long long written;     // min(jpeg_bytes, out_cap)
};

struct JpegGeom {
    int w, h;
    int hy, vy;        // luma sampling factors (chroma 1x1)
    int mw, mh;        // MCU size in pixels
    int mcus_x, mcus_y;
    int bpm, ny;       // blocks per MCU, luma blocks per MCU
    long long nb;      // blocks in coding order
    int ntiles;        // ceil(nb / kJpegTileBlocks)
    long long words;   // capacity of the bit stream in 32-bit words (multiple of 1024)
    long long chunks;  // capacity in stuffing chunks (words / 1024)
};

struct JpegLaunch {
    JpegGeom g;
    float q[2][64];   // quantiser (natural order) as float, [luma, chroma]
    float rq[2][64];  // 1 / q rounded to nearest (host IEEE division)
    const uint8_t* rgb;
    const JpegHuff* huff;
    uint32_t* acw;                   // nb x kJpegAcWords: each block's AC code from bit 0, big-endian
    int* dc;                         // nb: quantised DC
    int* acbits;                     // nb: bits of the AC code
    int* blk_off;                    // nb: offset of the block inside its tile (bits)
    int* tile_sum;                   // ntiles
    unsigned long long* tile_off;    // ntiles
    uint32_t* words;                 // bit stream, big-endian bit order inside each word; zero on entry
    int* chunk_ff;                   // chunks
    unsigned long long* chunk_off;   // chunks
    JpegInfo* info;
    unsigned* counters;              // 2 CTA-completion counters, zero between launches
    uint8_t* out;                    // stuffed bytes go to out[base ...], then FF D9
    unsigned long long base;         // bytes before the entropy-coded segment (header), 0 or its size
    unsigned long long out_cap;      // bytes of out that may be written
    unsigned long long* size_out;    // optional device copy of info->written
};

// the reference's geometry for (w, h, clamped subsample); words/chunks sized for the bound
JpegGeom jpeg_geometry(int w, int h, int subsample);
// uploads the cosine factors cosf((2i+1) u pi / 16) evaluated on the host (same libm as the
// reference's CPU encoder) to constant memory of the current device
cudaError_t jpeg_init_constants(const float cos_table[64]);
cudaError_t launch_jpeg_encode(const JpegLaunch& L, cudaStream_t st);

}  // namespace imop
