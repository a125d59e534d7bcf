/* isp_oracle_scene.c - TEST INFRASTRUCTURE ONLY: the seeded synthetic frames of the workloads
 * (scene, defect positions, MIPI packing), restated in C so that the timed CPU baseline can render
 * the same frames without loading the product library.  Same model and arithmetic as the
 * product's generator (im-operator_gb300/csrc/scene.cpp): per CFA channel, 4 sinusoids with
 * amplitude U(0.5,1), frequency U(1,16) cycles per frame width, orientation U(0,pi) and phase
 * U(0,2pi) from a splitmix64 stream; sin/cos from a fixed Taylor polynomial after reduction by
 * pi/2 (no libm transcendental, so x86-64 and aarch64 agree); shot noise as the normal
 * approximation of Poisson and read noise, both from Irwin-Hall sums of twelve uniforms drawn
 * from a counter-based hash of (seed, pixel, draw); rounded and clamped.  Compiled with
 * -ffp-contract=off; tests/test_oracle_scene.py checks that the bytes equal the product's. */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "isp_oracle.h"

static const double kPi = 3.14159265358979323846;

static uint64_t splitmix64(uint64_t* s) {
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static uint64_t hash3(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t s = a * 0xD1B54A32D192ED03ull ^ (b + 0x9E3779B97F4A7C15ull) * 0x8CB92BA72F3D8DD7ull ^ c;
    return splitmix64(&s);
}
static double u01(uint64_t r) { return (double)(r >> 11) * (1.0 / 9007199254740992.0); }

static double sin_poly(double x) {
    double x2 = x * x, t = x, s = x;
    for (int k = 1; k <= 7; k++) {
        t = -t * x2 / (double)((2 * k) * (2 * k + 1));
        s = s + t;
    }
    return s;
}
static double cos_poly(double x) {
    double x2 = x * x, t = 1.0, s = 1.0;
    for (int k = 1; k <= 7; k++) {
        t = -t * x2 / (double)((2 * k - 1) * (2 * k));
        s = s + t;
    }
    return s;
}
static double sin_det(double x) {
    double q = floor(x / (kPi / 2.0) + 0.5);
    double r = x - q * (kPi / 2.0);
    int64_t qi = (int64_t)q;
    int m = (int)(((qi % 4) + 4) % 4);
    switch (m) {
        case 0: return sin_poly(r);
        case 1: return cos_poly(r);
        case 2: return -sin_poly(r);
        default: return -cos_poly(r);
    }
}
static double cos_det(double x) { return sin_det(x + kPi / 2.0); }

/* colour index 0=R 1=Gr 2=Gb 3=B of (row, col) for RGGB / BGGR / GRBG / GBRG */
static int cfa_color(int row, int col, int pattern) {
    static const int off[4][4] = {{0, 0, 1, 1}, {1, 1, 0, 0}, {0, 1, 1, 0}, {1, 0, 0, 1}};
    const int* o = off[pattern & 3];
    if ((row & 1) == o[0] && (col & 1) == o[1]) return 0;
    if ((row & 1) == o[2] && (col & 1) == o[3]) return 3;
    if ((row & 1) == o[0]) return 1;
    return 2;
}

int or_scene_render(int w, int h, int bd, int pattern, uint64_t seed, float lo, float hi, float gain,
                    float read_sigma, void* out) {
    if (!out || w <= 0 || h <= 0 || bd < 1 || bd > 16 || pattern < 0 || pattern > 3 || !(gain > 0.0f)) return 1;
    double amp[4][4], kx[4][4], ky[4][4], ph[4][4], ampsum[4];
    uint64_t st = seed;
    for (int c = 0; c < 4; c++) {
        ampsum[c] = 0.0;
        for (int k = 0; k < 4; k++) {
            double a = 0.5 + 0.5 * u01(splitmix64(&st));
            double freq = 1.0 + 15.0 * u01(splitmix64(&st));
            double theta = kPi * u01(splitmix64(&st));
            double phase = 2.0 * kPi * u01(splitmix64(&st));
            double k2 = 2.0 * kPi * freq / (double)w;
            amp[c][k] = a;
            kx[c][k] = k2 * cos_det(theta);
            ky[c][k] = k2 * sin_det(theta);
            ph[c][k] = phase;
            ampsum[c] += a;
        }
    }
    const int mv = (bd >= 16) ? 65535 : (1 << bd) - 1;
    const double dlo = lo, dhi = hi, g = gain, rs = read_sigma;
    double* cs = (double*)malloc(sizeof(double) * 16 * (size_t)w);
    double* ss = (double*)malloc(sizeof(double) * 16 * (size_t)w);
    if (!cs || !ss) {
        free(cs);
        free(ss);
        return 6;
    }
    for (int c = 0; c < 4; c++)
        for (int k = 0; k < 4; k++)
            for (int x = 0; x < w; x++) {
                double a = kx[c][k] * (double)x;
                cs[(size_t)(c * 4 + k) * w + x] = cos_det(a);
                ss[(size_t)(c * 4 + k) * w + x] = sin_det(a);
            }
    uint8_t* o8 = (uint8_t*)out;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; y++) {
        double rsn[16], rcs[16];
        for (int c = 0; c < 4; c++)
            for (int k = 0; k < 4; k++) {
                double b = ky[c][k] * (double)y + ph[c][k];
                rsn[c * 4 + k] = sin_det(b);
                rcs[c * 4 + k] = cos_det(b);
            }
        for (int x = 0; x < w; x++) {
            int c = cfa_color(y, x, pattern);
            double s = 0.0;
            for (int k = 0; k < 4; k++) {
                size_t ti = (size_t)(c * 4 + k) * w + x;
                double v = ss[ti] * rcs[c * 4 + k] + cs[ti] * rsn[c * 4 + k];
                s = s + amp[c][k] * v;
            }
            double f = (s + ampsum[c]) / (2.0 * ampsum[c]);
            double mean_dn = dlo + (dhi - dlo) * f;
            uint64_t pix = (uint64_t)y * (uint64_t)w + (uint64_t)x;
            double z1 = -6.0, z2 = -6.0;
            for (int i = 0; i < 12; i++) z1 = z1 + u01(hash3(seed, pix, (uint64_t)i));
            for (int i = 12; i < 24; i++) z2 = z2 + u01(hash3(seed, pix, (uint64_t)i));
            double e = mean_dn / g;
            double shot = e + sqrt(e > 0.0 ? e : 0.0) * z1;
            double dn = shot * g + rs * z2;
            double r = floor(dn + 0.5);
            int v = r < 0.0 ? 0 : (r > (double)mv ? mv : (int)r);
            size_t i = (size_t)pix;
            if (bd <= 8) {
                o8[i] = (uint8_t)v;
            } else {
                o8[2 * i] = (uint8_t)(v & 0xFF);
                o8[2 * i + 1] = (uint8_t)(v >> 8);
            }
        }
    }
    free(cs);
    free(ss);
    return 0;
}

/* distinct positions in [2,w-2)x[2,h-2) from a splitmix64 stream, first half hot, second dead;
 * written as (x, y) int pairs */
int or_scene_defects(int w, int h, uint64_t seed, int count, int* xy) {
    if ((!xy && count > 0) || w < 5 || h < 5) return 1;
    long long avail = (long long)(w - 4) * (long long)(h - 4);
    if (count < 0 || count > avail) return 1;
    uint8_t* seen = (uint8_t*)calloc(((size_t)w * h + 7) / 8, 1);
    if (!seen) return 6;
    uint64_t st = seed ^ 0xDEFEC7ull;
    int n = 0;
    while (n < count) {
        int x = 2 + (int)(splitmix64(&st) % (uint64_t)(w - 4));
        int y = 2 + (int)(splitmix64(&st) % (uint64_t)(h - 4));
        size_t key = (size_t)y * (size_t)w + (size_t)x;
        if (seen[key >> 3] & (1u << (key & 7))) continue;
        seen[key >> 3] |= (uint8_t)(1u << (key & 7));
        xy[2 * n] = x;
        xy[2 * n + 1] = y;
        n++;
    }
    free(seen);
    return 0;
}

void or_scene_apply_defects(uint16_t* frame, int w, int bd, const int* xy, int count) {
    const int mv = (bd >= 16) ? 65535 : (1 << bd) - 1;
    for (int i = 0; i < count; i++) frame[(size_t)xy[2 * i + 1] * w + xy[2 * i]] = (uint16_t)((i < count / 2) ? mv : 0);
}

/* MIPI RAW12 (2 px / 3 B) or RAW10 (4 px / 5 B) of n u16 samples, as pixel::get_packed_raw reads them */
void or_pack_mipi(const uint16_t* in, size_t n, int bd, uint8_t* out) {
    const size_t size = (n * (size_t)bd + 7) / 8;
    memset(out, 0, size);
    if (bd == 12) {
        for (size_t k = 0; 2 * k < n; k++) {
            unsigned p0 = in[2 * k] & 0xFFF, p1 = (2 * k + 1 < n) ? (in[2 * k + 1] & 0xFFF) : 0;
            uint8_t b[3] = {(uint8_t)(p0 >> 4), (uint8_t)((p0 & 0xF) | ((p1 & 0xF) << 4)), (uint8_t)(p1 >> 4)};
            for (int j = 0; j < 3; j++)
                if (3 * k + j < size) out[3 * k + j] = b[j];
        }
    } else if (bd == 10) {
        for (size_t k = 0; 4 * k < n; k++) {
            uint8_t b[5] = {0, 0, 0, 0, 0};
            for (int s = 0; s < 4; s++) {
                unsigned p = (4 * k + s < n) ? (in[4 * k + s] & 0x3FF) : 0;
                b[s] = (uint8_t)(p >> 2);
                b[4] |= (uint8_t)((p & 3) << (2 * s));
            }
            for (int j = 0; j < 5; j++)
                if (5 * k + j < size) out[5 * k + j] = b[j];
        }
    }
}
