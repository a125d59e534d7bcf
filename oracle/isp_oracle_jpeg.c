/* isp_oracle_jpeg.c - TEST INFRASTRUCTURE ONLY: a plain-C restatement of the reference's baseline
 * JPEG encoder (jpeg_codec::process_encode_baseline, src/jpeg_codec/encode_baseline.cpp:222-376,
 * with the helpers of src/jpeg_codec/common.hpp), the checker of the GPU encoder.  Byte for byte
 * the reference's output, its quirks included:
 *  - zz[kZigzag[i]] = round(block[i] / q[i]) with kZigzag the natural index of each zigzag
 *    position (common.hpp:84-93), i.e. the coefficients are permuted by the inverse of the scan;
 *  - chroma is point-sampled at the MCU's top-left sample of each 2x1 / 2x2 group;
 *  - an EOB follows the last coefficient even when it is non-zero (encode_baseline.cpp:88-97);
 *  - a category missing from a Huffman table writes its value bits without a code (:40-47, :79-83);
 *  - the final partial byte is padded with 0 bits (common.hpp:245-253).
 * The cosine factors are cosf((2i+1) u pi / 16) in float as the reference evaluates them
 * (common.hpp:104-115), so both sides take them from the same libm. */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "isp_oracle.h"

/* ITU-T T.81 Annex K: quantisation tables K.1 / K.2 (natural order), zigzag scan (natural index of
 * each scan position), Huffman tables K.3 (code counts per length, symbol values) */
static const int kQLuma[64] = {16, 11, 10, 16, 24,  40,  51,  61,  12, 12, 14, 19, 26,  58,  60,  55,
                               14, 13, 16, 24, 40,  57,  69,  56,  14, 17, 22, 29, 51,  87,  80,  62,
                               18, 22, 37, 56, 68,  109, 103, 77,  24, 35, 55, 64, 81,  104, 113, 92,
                               49, 64, 78, 87, 103, 121, 120, 101, 72, 92, 95, 98, 112, 100, 103, 99};
static const int kQChroma[64] = {17, 18, 24, 47, 99, 99, 99, 99, 18, 21, 26, 66, 99, 99, 99, 99,
                                 24, 26, 56, 99, 99, 99, 99, 99, 47, 66, 99, 99, 99, 99, 99, 99,
                                 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99,
                                 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99};
static const int kScan[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,
                              12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6,  7,  14, 21, 28,
                              35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
                              58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};
static const uint8_t kDcLumaBits[16] = {0, 1, 5, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0};
static const uint8_t kDcChromaBits[16] = {0, 3, 1, 1, 1, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0};
static const uint8_t kDcVals[12] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11};
static const uint8_t kAcLumaBits[16] = {0, 2, 1, 3, 3, 2, 4, 3, 5, 5, 4, 4, 0, 0, 1, 0x7d};
static const uint8_t kAcLumaVals[162] = {
    0x01, 0x02, 0x03, 0x00, 0x04, 0x11, 0x05, 0x12, 0x21, 0x31, 0x41, 0x06, 0x13, 0x51, 0x61, 0x07, 0x22, 0x71,
    0x14, 0x32, 0x81, 0x91, 0xa1, 0x08, 0x23, 0x42, 0xb1, 0xc1, 0x15, 0x52, 0xd1, 0xf0, 0x24, 0x33, 0x62, 0x72,
    0x82, 0x09, 0x0a, 0x16, 0x17, 0x18, 0x19, 0x1a, 0x25, 0x26, 0x27, 0x28, 0x29, 0x2a, 0x34, 0x35, 0x36, 0x37,
    0x38, 0x39, 0x3a, 0x43, 0x44, 0x45, 0x46, 0x47, 0x48, 0x49, 0x4a, 0x53, 0x54, 0x55, 0x56, 0x57, 0x58, 0x59,
    0x5a, 0x63, 0x64, 0x65, 0x66, 0x67, 0x68, 0x69, 0x6a, 0x73, 0x74, 0x75, 0x76, 0x77, 0x78, 0x79, 0x7a, 0x83,
    0x84, 0x85, 0x86, 0x87, 0x88, 0x89, 0x8a, 0x92, 0x93, 0x94, 0x95, 0x96, 0x97, 0x98, 0x99, 0x9a, 0xa2, 0xa3,
    0xa4, 0xa5, 0xa6, 0xa7, 0xa8, 0xa9, 0xaa, 0xb2, 0xb3, 0xb4, 0xb5, 0xb6, 0xb7, 0xb8, 0xb9, 0xba, 0xc2, 0xc3,
    0xc4, 0xc5, 0xc6, 0xc7, 0xc8, 0xc9, 0xca, 0xd2, 0xd3, 0xd4, 0xd5, 0xd6, 0xd7, 0xd8, 0xd9, 0xda, 0xe1, 0xe2,
    0xe3, 0xe4, 0xe5, 0xe6, 0xe7, 0xe8, 0xe9, 0xea, 0xf1, 0xf2, 0xf3, 0xf4, 0xf5, 0xf6, 0xf7, 0xf8, 0xf9, 0xfa};
static const uint8_t kAcChromaBits[16] = {0, 2, 1, 2, 4, 4, 3, 4, 7, 5, 4, 4, 0, 1, 2, 0x77};
static const uint8_t kAcChromaVals[162] = {
    0x00, 0x01, 0x02, 0x03, 0x11, 0x04, 0x05, 0x21, 0x31, 0x06, 0x12, 0x41, 0x51, 0x07, 0x61, 0x71, 0x13, 0x22,
    0x32, 0x81, 0x08, 0x14, 0x42, 0x91, 0xa1, 0xb1, 0xc1, 0x09, 0x23, 0x33, 0x52, 0xf0, 0x15, 0x62, 0x72, 0xd1,
    0x0a, 0x16, 0x24, 0x34, 0xe1, 0x25, 0xf1, 0x17, 0x18, 0x19, 0x1a, 0x26, 0x27, 0x28, 0x29, 0x2a, 0x35, 0x36,
    0x37, 0x38, 0x39, 0x3a, 0x43, 0x44, 0x45, 0x46, 0x47, 0x48, 0x49, 0x4a, 0x53, 0x54, 0x55, 0x56, 0x57, 0x58,
    0x59, 0x5a, 0x63, 0x64, 0x65, 0x66, 0x67, 0x68, 0x69, 0x6a, 0x73, 0x74, 0x75, 0x76, 0x77, 0x78, 0x79, 0x7a,
    0x82, 0x83, 0x84, 0x85, 0x86, 0x87, 0x88, 0x89, 0x8a, 0x92, 0x93, 0x94, 0x95, 0x96, 0x97, 0x98, 0x99, 0x9a,
    0xa2, 0xa3, 0xa4, 0xa5, 0xa6, 0xa7, 0xa8, 0xa9, 0xaa, 0xb2, 0xb3, 0xb4, 0xb5, 0xb6, 0xb7, 0xb8, 0xb9, 0xba,
    0xc2, 0xc3, 0xc4, 0xc5, 0xc6, 0xc7, 0xc8, 0xc9, 0xca, 0xd2, 0xd3, 0xd4, 0xd5, 0xd6, 0xd7, 0xd8, 0xd9, 0xda,
    0xe2, 0xe3, 0xe4, 0xe5, 0xe6, 0xe7, 0xe8, 0xe9, 0xea, 0xf2, 0xf3, 0xf4, 0xf5, 0xf6, 0xf7, 0xf8, 0xf9, 0xfa};

typedef struct {
    int size[256], code[256];
} or_huff;

/* canonical codes: per length, consecutive codes, doubled between lengths (common.hpp:390-411) */
static void huff_build(or_huff* t, const uint8_t bits[16], const uint8_t* vals) {
    memset(t, 0, sizeof(*t));
    int k = 0, code = 0;
    for (int len = 1; len <= 16; len++) {
        for (int j = 0; j < bits[len - 1]; j++, k++, code++) {
            t->size[vals[k]] = len;
            t->code[vals[k]] = code;
        }
        code <<= 1;
    }
}

typedef struct {
    uint8_t* buf;
    size_t cap, pos;
    int acc, n;
} or_bits;

static void put_byte(or_bits* w, int b) {
    if (w->pos < w->cap) w->buf[w->pos++] = (uint8_t)b;
}
static void put_u16(or_bits* w, int v) {
    put_byte(w, (v >> 8) & 0xFF);
    put_byte(w, v & 0xFF);
}
/* MSB first; a completed 0xFF byte is followed by a stuffed 0x00 (common.hpp:231-243) */
static void put_bits(or_bits* w, int v, int n) {
    for (int i = n - 1; i >= 0; i--) {
        w->acc = (w->acc << 1) | ((v >> i) & 1);
        if (++w->n == 8) {
            put_byte(w, w->acc & 0xFF);
            if ((w->acc & 0xFF) == 0xFF) put_byte(w, 0);
            w->acc = 0;
            w->n = 0;
        }
    }
}

static int category(int v) {
    int a = v < 0 ? -v : v, c = 0;
    while (a) {
        c++;
        a >>= 1;
    }
    return c;
}

/* quantise + scan-permute + DPCM / run-length / Huffman of one block (encode_baseline.cpp:16-101) */
static void encode_block(or_bits* w, const float blk[64], int* prev_dc, const or_huff* dc, const or_huff* ac,
                         const int q[64]) {
    int zz[64];
    for (int i = 0; i < 64; i++) zz[kScan[i]] = (int)roundf(blk[i] / (float)q[i]);
    const int diff = zz[0] - *prev_dc;
    *prev_dc = zz[0];
    const int dcat = category(diff);
    if (dcat > 0) {
        put_bits(w, dc->code[dcat], dc->size[dcat]);
        put_bits(w, diff < 0 ? diff + (1 << dcat) - 1 : diff, dcat);
    } else {
        put_bits(w, dc->code[0], dc->size[0]);
    }
    int eob = 0, run = 0;
    for (int i = 1; i < 64; i++) {
        int rest_zero = 1;
        if (zz[i] == 0) {
            if (++run == 16) {
                for (int j = i + 1; j < 64; j++)
                    if (zz[j]) rest_zero = 0;
                if (rest_zero) {
                    put_bits(w, ac->code[0x00], ac->size[0x00]);
                    eob = 1;
                    break;
                }
                put_bits(w, ac->code[0xF0], ac->size[0xF0]);
                run = 0;
            }
        } else {
            const int v = zz[i], cat = category(v), sym = (run << 4) | cat;
            if (ac->size[sym] > 0) {
                put_bits(w, ac->code[sym], ac->size[sym]);
                put_bits(w, v < 0 ? v + (1 << cat) - 1 : v, cat);
            }
            run = 0;
        }
        rest_zero = 1;
        for (int j = i + 1; j < 64; j++)
            if (zz[j]) rest_zero = 0;
        if (rest_zero) {
            put_bits(w, ac->code[0x00], ac->size[0x00]);
            eob = 1;
            break;
        }
    }
    if (!eob) put_bits(w, ac->code[0x00], ac->size[0x00]);
}

/* separable DCT-II, rows then columns, each output 0.5 C(u) sum x[i] cos(...) (common.hpp:104-153) */
static void fdct(float b[64], const float cs[8][8]) {
    const float inv_sqrt2 = 0.70710678118654752440f;
    float t[64], col[8];
    for (int y = 0; y < 8; y++)
        for (int u = 0; u < 8; u++) {
            float s = 0.0f;
            for (int i = 0; i < 8; i++) s += b[y * 8 + i] * cs[u][i];
            t[y * 8 + u] = 0.5f * (u == 0 ? inv_sqrt2 : 1.0f) * s;
        }
    for (int u = 0; u < 8; u++) {
        for (int y = 0; y < 8; y++) col[y] = t[y * 8 + u];
        for (int v = 0; v < 8; v++) {
            float s = 0.0f;
            for (int i = 0; i < 8; i++) s += col[i] * cs[v][i];
            b[v * 8 + u] = 0.5f * (v == 0 ? inv_sqrt2 : 1.0f) * s;
        }
    }
}

static int sample(const uint8_t* in, int x, int y, int w, int c) {
    return in[((size_t)y * (size_t)w + (size_t)x) * 3 + (size_t)c];
}

/* component k (0 Y, 1 Cb, 2 Cr) of pixel (x, y), the reference's float expression and truncation
 * (common.hpp:196-201) */
static int ycc(const uint8_t* in, int x, int y, int w, int k) {
    const int r = sample(in, x, y, w, 0), g = sample(in, x, y, w, 1), b = sample(in, x, y, w, 2);
    if (k == 0) return (int)(0.299f * r + 0.587f * g + 0.114f * b);
    if (k == 1) return (int)(-0.168736f * r - 0.331264f * g + 0.5f * b + 128.0f);
    return (int)(0.5f * r - 0.418688f * g - 0.081312f * b + 128.0f);
}

void or_jpeg_scale_qtable(int q[64], const int base[64], int quality) {
    const int qq = quality < 1 ? 1 : (quality > 100 ? 100 : quality);
    const int s = qq < 50 ? 5000 / qq : 200 - 2 * qq;
    for (int i = 0; i < 64; i++) {
        const int v = (base[i] * s + 50) / 100;
        q[i] = v < 1 ? 1 : (v > 255 ? 255 : v);
    }
}

static void put_dht(or_bits* w, int cls, int id, const uint8_t bits[16], const uint8_t* vals) {
    int n = 0;
    for (int i = 0; i < 16; i++) n += bits[i];
    put_byte(w, 0xFF);
    put_byte(w, 0xC4);
    put_u16(w, 3 + 16 + n);
    put_byte(w, (cls << 4) | id);
    for (int i = 0; i < 16; i++) put_byte(w, bits[i]);
    for (int i = 0; i < n; i++) put_byte(w, vals[i]);
}

/* returns 0 (Ok) or the reference's JpegError value, checked in the reference's order
 * (validate_jpeg_encode_inputs, src/jpeg_codec/dispatch.cpp:11-29: only 8-bit input is valid) */
int or_jpeg_encode(const uint8_t* in, int w, int h, int bd, int quality, int subsample, uint8_t* out,
                   size_t* out_size) {
    if (!in) return 1;
    if (w <= 0 || h <= 0) return 3;
    if (bd != 8) return 4;
    if (w < 8 || h < 8) return 7;
    if (!out) return 2;
    if (quality < 1 || quality > 100) return 6;
    const int ss = subsample < 0 ? 0 : (subsample > 2 ? 2 : subsample);
    const int hy = ss == 0 ? 1 : 2, vy = ss == 1 ? 2 : 1;  /* luma sampling; chroma 1x1 */
    const int mw = 8 * hy, mh = 8 * vy;
    const int pw = (w + mw - 1) / mw * mw, ph = (h + mh - 1) / mh * mh;
    int ql[64], qc[64];
    or_jpeg_scale_qtable(ql, kQLuma, quality);
    or_jpeg_scale_qtable(qc, kQChroma, quality);
    float cs[8][8];
    for (int u = 0; u < 8; u++)
        for (int i = 0; i < 8; i++) cs[u][i] = cosf((2.0f * i + 1.0f) * u * 3.14159265358979323846f / 16.0f);
    or_huff dcl, dcc, acl, acc;
    huff_build(&dcl, kDcLumaBits, kDcVals);
    huff_build(&dcc, kDcChromaBits, kDcVals);
    huff_build(&acl, kAcLumaBits, kAcLumaVals);
    huff_build(&acc, kAcChromaBits, kAcChromaVals);
    or_bits wr = {out, *out_size ? *out_size : (size_t)w * h * 9 + 65536, 0, 0, 0};
    or_bits* W = &wr;
    /* SOI, JFIF APP0 (1.02, dpi 72x72), DQT luma / chroma in scan order, SOF0, DHT x4, SOS */
    put_byte(W, 0xFF), put_byte(W, 0xD8);
    put_byte(W, 0xFF), put_byte(W, 0xE0), put_u16(W, 16);
    put_byte(W, 'J'), put_byte(W, 'F'), put_byte(W, 'I'), put_byte(W, 'F'), put_byte(W, 0);
    put_byte(W, 1), put_byte(W, 2), put_byte(W, 1), put_u16(W, 72), put_u16(W, 72), put_byte(W, 0), put_byte(W, 0);
    for (int t = 0; t < 2; t++) {
        const int* q = t ? qc : ql;
        put_byte(W, 0xFF), put_byte(W, 0xDB), put_u16(W, 67), put_byte(W, t);
        for (int i = 0; i < 64; i++) put_byte(W, q[kScan[i]]);
    }
    put_byte(W, 0xFF), put_byte(W, 0xC0), put_u16(W, 17), put_byte(W, 8), put_u16(W, h), put_u16(W, w), put_byte(W, 3);
    put_byte(W, 1), put_byte(W, (hy << 4) | vy), put_byte(W, 0);
    put_byte(W, 2), put_byte(W, 0x11), put_byte(W, 1);
    put_byte(W, 3), put_byte(W, 0x11), put_byte(W, 1);
    put_dht(W, 0, 0, kDcLumaBits, kDcVals);
    put_dht(W, 1, 0, kAcLumaBits, kAcLumaVals);
    put_dht(W, 0, 1, kDcChromaBits, kDcVals);
    put_dht(W, 1, 1, kAcChromaBits, kAcChromaVals);
    put_byte(W, 0xFF), put_byte(W, 0xDA), put_u16(W, 12), put_byte(W, 3);
    put_byte(W, 1), put_byte(W, 0x00), put_byte(W, 2), put_byte(W, 0x11), put_byte(W, 3), put_byte(W, 0x11);
    put_byte(W, 0), put_byte(W, 63), put_byte(W, 0);
    /* MCUs in raster order: luma blocks (hy x vy), then one Cb and one Cr block */
    int pdc[3] = {0, 0, 0};
    float blk[64];
    for (int my = 0; my < ph; my += mh)
        for (int mx = 0; mx < pw; mx += mw) {
            for (int by = 0; by < vy; by++)
                for (int bx = 0; bx < hy; bx++) {
                    for (int j = 0; j < 8; j++)
                        for (int i = 0; i < 8; i++) {
                            int px = mx + bx * 8 + i, py = my + by * 8 + j;
                            if (px > w - 1) px = w - 1;
                            if (py > h - 1) py = h - 1;
                            blk[j * 8 + i] = (float)(ycc(in, px, py, w, 0) - 128);
                        }
                    fdct(blk, cs);
                    encode_block(W, blk, &pdc[0], &dcl, &acl, ql);
                }
            for (int k = 1; k <= 2; k++) {
                for (int j = 0; j < 8; j++)
                    for (int i = 0; i < 8; i++) {
                        int px = mx + i * hy, py = my + j * vy;
                        if (px > w - 1) px = w - 1;
                        if (py > h - 1) py = h - 1;
                        blk[j * 8 + i] = (float)(ycc(in, px, py, w, k) - 128);
                    }
                fdct(blk, cs);
                encode_block(W, blk, &pdc[k], &dcc, &acc, qc);
            }
        }
    if (W->n > 0) {
        const int b = (W->acc << (8 - W->n)) & 0xFF;
        put_byte(W, b);
        if (b == 0xFF) put_byte(W, 0);
        W->acc = W->n = 0;
    }
    put_byte(W, 0xFF), put_byte(W, 0xD9);
    *out_size = W->pos;
    return 0;
}
