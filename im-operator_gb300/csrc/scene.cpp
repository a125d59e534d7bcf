// scene.cpp - seeded synthetic Bayer frames, MIPI packers and defect maps.
//
// The generator must give the same bytes on an x86-64 build host and on an aarch64 GPU host,
// so it avoids libm transcendental functions (their last bit differs between libm builds):
// sin/cos are evaluated here with a fixed polynomial, Gaussian noise is the Irwin-Hall sum of
// twelve uniforms, Poisson shot noise is its normal approximation (every scene sample is at
// least 128 electrons, where the approximation is tight), and the file is compiled with
// -ffp-contract=off.  Per-pixel noise comes from a counter-based hash of (seed, pixel, draw),
// so the result does not depend on how many threads render it.
//
// Scene model: per CFA channel, the sum of 4 sinusoids with amplitude U(0.5,1), frequency
// U(1,16) cycles per frame width, orientation U(0,pi) and phase U(0,2pi), normalised by its
// amplitude bound to [0,1], mapped linearly to [lo,hi] DN; shot noise at gain DN/e-, read noise
// sigma DN; rounded and clamped to [0, 2^bd-1].

#include <cmath>
#include <cstdint>
#include <cstring>
#include <unordered_set>
#include <vector>

#include "../../include/imop_isp.h"
#include "isp_common.h"

namespace {

constexpr double kPi = 3.14159265358979323846;

inline uint64_t splitmix64(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline uint64_t hash3(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t s = a * 0xD1B54A32D192ED03ull ^ (b + 0x9E3779B97F4A7C15ull) * 0x8CB92BA72F3D8DD7ull ^ c;
    return splitmix64(s);
}
inline double u01(uint64_t r) { return (double)(r >> 11) * (1.0 / 9007199254740992.0); }

// sin on [-pi/4, pi/4] and cos on the same range: Taylor series to x^15 / x^14
double sin_poly(double x) {
    double x2 = x * x;
    double t = x, s = x;
    for (int k = 1; k <= 7; k++) {
        t = -t * x2 / (double)((2 * k) * (2 * k + 1));
        s = s + t;
    }
    return s;
}
double cos_poly(double x) {
    double x2 = x * x;
    double t = 1.0, s = 1.0;
    for (int k = 1; k <= 7; k++) {
        t = -t * x2 / (double)((2 * k - 1) * (2 * k));
        s = s + t;
    }
    return s;
}
// sin(x) for any finite x: reduce by multiples of pi/2
double sin_det(double x) {
    double q = std::floor(x / (kPi / 2.0) + 0.5);
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
double cos_det(double x) { return sin_det(x + kPi / 2.0); }

struct Wave {
    double amp, kx, ky, phase;
};

}  // namespace

extern "C" int imop_scene_render(int w, int h, int bd, int pattern, uint64_t seed, float lo, float hi,
                                 float gain, float read_sigma, void* out) {
    if (!out) return IMOP_ERR_NULL_INPUT;
    if (w <= 0 || h <= 0) return IMOP_ERR_INVALID_DIMENSIONS;
    if (bd < 1 || bd > 16) return IMOP_ERR_INVALID_BIT_DEPTH;
    if (pattern < 0 || pattern > 3) return IMOP_ERR_INVALID_PATTERN;
    if (!(gain > 0.0f)) return IMOP_ERR_INVALID_ARGUMENT;
    Wave waves[4][4];
    double ampsum[4];
    uint64_t st = seed;
    for (int c = 0; c < 4; c++) {
        ampsum[c] = 0.0;
        for (int k = 0; k < 4; k++) {
            double amp = 0.5 + 0.5 * u01(splitmix64(st));
            double freq = 1.0 + 15.0 * u01(splitmix64(st));
            double theta = kPi * u01(splitmix64(st));
            double phase = 2.0 * kPi * u01(splitmix64(st));
            double k2 = 2.0 * kPi * freq / (double)w;
            waves[c][k] = {amp, k2 * cos_det(theta), k2 * sin_det(theta), phase};
            ampsum[c] += amp;
        }
    }
    const int mv = (bd >= 16) ? 65535 : (1 << bd) - 1;
    const double dlo = lo, dhi = hi, g = gain, rs = read_sigma;
    // separable angles: sin(kx*x + ky*y + p) from per-column and per-row sin/cos tables
    std::vector<double> cs((size_t)16 * w), ss((size_t)16 * w);
    for (int c = 0; c < 4; c++)
        for (int k = 0; k < 4; k++)
            for (int x = 0; x < w; x++) {
                double a = waves[c][k].kx * (double)x;
                cs[(size_t)(c * 4 + k) * w + x] = cos_det(a);
                ss[(size_t)(c * 4 + k) * w + x] = sin_det(a);
            }
    uint8_t* o8 = (uint8_t*)out;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; y++) {
        double rsn[16], rcs[16];
        for (int c = 0; c < 4; c++)
            for (int k = 0; k < 4; k++) {
                double b = waves[c][k].ky * (double)y + waves[c][k].phase;
                rsn[c * 4 + k] = sin_det(b);
                rcs[c * 4 + k] = cos_det(b);
            }
        for (int x = 0; x < w; x++) {
            int c = imop::bayer_color_host(y, x, pattern);
            double s = 0.0;
            for (int k = 0; k < 4; k++) {
                size_t ti = (size_t)(c * 4 + k) * w + x;
                // sin(a + b) = sin a cos b + cos a sin b
                double v = ss[ti] * rcs[c * 4 + k] + cs[ti] * rsn[c * 4 + k];
                s = s + waves[c][k].amp * v;
            }
            double f = (s + ampsum[c]) / (2.0 * ampsum[c]);
            double mean_dn = dlo + (dhi - dlo) * f;
            uint64_t pix = (uint64_t)y * (uint64_t)w + (uint64_t)x;
            double z1 = -6.0, z2 = -6.0;
            for (int i = 0; i < 12; i++) z1 = z1 + u01(hash3(seed, pix, (uint64_t)i));
            for (int i = 12; i < 24; i++) z2 = z2 + u01(hash3(seed, pix, (uint64_t)i));
            double e = mean_dn / g;
            double shot = e + std::sqrt(e > 0.0 ? e : 0.0) * z1;
            double dn = shot * g + rs * z2;
            double r = std::floor(dn + 0.5);
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
    return IMOP_OK;
}

extern "C" int imop_scene_defects(int w, int h, uint64_t seed, int count, ImopDefectPoint* out) {
    if (!out && count > 0) return IMOP_ERR_NULL_INPUT;
    if (w < 5 || h < 5) return IMOP_ERR_IMAGE_TOO_SMALL;
    long long avail = (long long)(w - 4) * (long long)(h - 4);
    if (count < 0 || count > avail) return IMOP_ERR_INVALID_ARGUMENT;
    std::unordered_set<uint64_t> seen;
    uint64_t st = seed ^ 0xDEFEC7ull;
    int n = 0;
    while (n < count) {
        int x = 2 + (int)(splitmix64(st) % (uint64_t)(w - 4));
        int y = 2 + (int)(splitmix64(st) % (uint64_t)(h - 4));
        uint64_t key = (uint64_t)y * (uint64_t)w + (uint64_t)x;
        if (!seen.insert(key).second) continue;
        out[n].x = x;
        out[n].y = y;
        n++;
    }
    return IMOP_OK;
}

extern "C" int imop_scene_apply_defects(void* frame, int w, int h, int bd, const ImopDefectPoint* pts,
                                        int count) {
    if (!frame || (!pts && count > 0)) return IMOP_ERR_NULL_INPUT;
    if (bd < 1 || bd > 16) return IMOP_ERR_INVALID_BIT_DEPTH;
    const int mv = (bd >= 16) ? 65535 : (1 << bd) - 1;
    uint8_t* o8 = (uint8_t*)frame;
    for (int i = 0; i < count; i++) {
        int x = pts[i].x, y = pts[i].y;
        if (x < 0 || y < 0 || x >= w || y >= h) return IMOP_ERR_INVALID_ARGUMENT;
        int v = (i < count / 2) ? mv : 0;
        size_t idx = (size_t)y * w + x;
        if (bd <= 8) {
            o8[idx] = (uint8_t)v;
        } else {
            o8[2 * idx] = (uint8_t)(v & 0xFF);
            o8[2 * idx + 1] = (uint8_t)(v >> 8);
        }
    }
    return IMOP_OK;
}

extern "C" size_t imop_packed_bytes(int w, int h, int bd) {
    if (w <= 0 || h <= 0 || bd <= 0) return 0;
    return ((size_t)w * (size_t)h * (size_t)bd + 7) / 8;
}

// Inverse of the MIPI readers (include/imop/pixel_utils.hpp:69-98 of the reference).  Pixels of a
// trailing incomplete group are packed as far as the buffer reaches; the reader returns 0 there.
extern "C" int imop_pack_mipi(const uint16_t* in, int w, int h, int bd, uint8_t* out) {
    if (!in || !out) return IMOP_ERR_NULL_INPUT;
    if (w <= 0 || h <= 0) return IMOP_ERR_INVALID_DIMENSIONS;
    if (bd < 1 || bd > 16) return IMOP_ERR_INVALID_BIT_DEPTH;
    size_t n = (size_t)w * h, size = imop_packed_bytes(w, h, bd);
    std::memset(out, 0, size);
    if (bd != 10 && bd != 12) {
        // other depths: one LSB-first bit stream, sample i at bits [i bd, (i + 1) bd)
        const unsigned mv = bd >= 16 ? 0xFFFFu : (1u << bd) - 1;
        for (size_t i = 0; i < n; i++) {
            const size_t bit = i * (size_t)bd;
            const uint32_t v = (uint32_t)(in[i] & mv) << (bit & 7);
            for (size_t j = bit >> 3, k = 0; k < 3 && j < size; j++, k++) out[j] |= (uint8_t)(v >> (8 * k));
        }
    } else if (bd == 12) {
        for (size_t k = 0; 2 * k < n; k++) {
            unsigned p0 = in[2 * k] & 0xFFF, p1 = (2 * k + 1 < n) ? (in[2 * k + 1] & 0xFFF) : 0;
            uint8_t b[3] = {(uint8_t)(p0 >> 4), (uint8_t)((p0 & 0xF) | ((p1 & 0xF) << 4)), (uint8_t)(p1 >> 4)};
            for (int j = 0; j < 3; j++)
                if (3 * k + j < size) out[3 * k + j] = b[j];
        }
    } else {
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
    return IMOP_OK;
}
