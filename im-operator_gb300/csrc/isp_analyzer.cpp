// isp_analyzer.cpp - format sniffing of raw blobs of unknown layout (host code).
//
// The same heuristics as the reference's analyzer (src/analyzer.cpp), so that an ingest path fed
// by this library classifies a blob exactly as im-operator does: storage bit depth from the byte
// count against a table of known resolutions and from the value statistics, packed detection,
// candidate dimensions, and the Bayer phase from 2x2 diagonal votes and channel means.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>

#include "../../include/imop_isp.h"

namespace {

// pixel counts of known sensor / video resolutions (src/analyzer.cpp:13-24); the table's
// contents decide the classification, so it lists the same resolutions
constexpr size_t kKnownPixels[] = {
    640 * 480,   720 * 480,   720 * 576,   800 * 600,   1024 * 768,  1280 * 720,  1280 * 800,  1280 * 1024,
    1440 * 900,  1920 * 1080, 1920 * 1200, 2048 * 1536, 2560 * 1440, 2560 * 1600, 3840 * 2160, 4096 * 2160,
    4096 * 3072, 5120 * 2880, 5320 * 4600, 7680 * 4320, 1006 * 758,  4024 * 3032,
};

bool known_pixels(size_t n) {
    for (size_t k : kKnownPixels)
        if (n == k) return true;
    return false;
}

uint16_t u16_at(const uint8_t* d, size_t i) {
    uint16_t v;
    std::memcpy(&v, d + 2 * i, 2);
    return v;
}

// largest u16 value of the first 100000 samples -> the smallest depth holding it (:27-42)
int depth_from_u16_values(const uint8_t* d, size_t bytes) {
    const size_t n = std::min(bytes / 2, (size_t)100000);
    unsigned mx = 0;
    for (size_t i = 0; i < n; i++) mx = std::max(mx, (unsigned)u16_at(d, i));
    if (mx <= 255) return 8;
    if (mx <= 1023) return 10;
    if (mx <= 4095) return 12;
    if (mx <= 16383) return 14;
    return 16;
}

// Packed bits read as u16 words nearly always have a non-zero high byte and are almost never
// zero (:47-70): > 85 % high bytes and < 1 % zero words among the first 10000 words.
bool packed_like(const uint8_t* d, size_t bytes) {
    if (bytes < 8) return false;
    const size_t n = std::min(bytes / 2, (size_t)10000);
    size_t high = 0, zero = 0;
    for (size_t i = 0; i < n; i++) {
        const uint16_t v = u16_at(d, i);
        high += (v >> 8) != 0;
        zero += v == 0;
    }
    return (double)high / (double)n > 0.85 && (double)zero / (double)n < 0.01;
}

int detect_depth(const uint8_t* d, size_t bytes) {
    if (!d || bytes == 0) return 0;
    if (known_pixels(bytes)) return 8;
    if (bytes % 2 == 0 && known_pixels(bytes / 2)) return depth_from_u16_values(d, bytes);
    if (packed_like(d, bytes)) {
        for (int bd : {10, 12, 14, 16}) {
            const size_t n = bytes * 8 / (size_t)bd;
            if (known_pixels(n) || known_pixels(n + 1)) return bd;
        }
    }
    if (bytes % 2 == 0 && bytes >= 4) {
        // unpacked 16-bit storage of an unknown size: many high bytes and values above 255
        const size_t n = std::min(bytes / 2, (size_t)10000);
        size_t high = 0;
        unsigned mx = 0;
        for (size_t i = 0; i < n; i++) {
            const uint16_t v = u16_at(d, i);
            high += (v >> 8) > 0;
            mx = std::max(mx, (unsigned)v);
        }
        if ((double)high / (double)n > 0.3 && mx > 255) return 16;
    }
    return 8;
}

// candidate (w, h): common widths x common heights, else divisors within 100 of sqrt(n), both
// sides >= 64, at most 5 (:121-151)
int dimensions(size_t n, int (*out)[2], int cap) {
    static const int kWidths[] = {640, 720, 800, 1024, 1280, 1440, 1920, 2048, 2560, 3840, 4096, 5120, 7680};
    static const int kHeights[] = {480, 576, 600, 720, 768, 800, 1024, 1080, 1200, 1440, 1536, 2048, 2160, 3072, 4320};
    int k = 0;
    if (n == 0) return 0;
    for (int w : kWidths) {
        if (n % (size_t)w) continue;
        const size_t h = n / (size_t)w;
        for (int ch : kHeights)
            if (h == (size_t)ch) {
                if (k < cap) out[k][0] = w, out[k][1] = ch;
                k++;
                break;
            }
    }
    if (k > 0) return k;
    const int r = (int)std::sqrt((double)n);
    for (int w = r - 100; w <= r + 100; w++) {
        if (w <= 0 || n % (size_t)w) continue;
        const int h = (int)(n / (size_t)w);
        if (w >= 64 && h >= 64) {
            if (k < cap) out[k][0] = w, out[k][1] = h;
            k++;
            if (k >= 5) break;
        }
    }
    return k;
}

}  // namespace

extern "C" int imop_detect_bit_depth(const void* data, size_t bytes) {
    return detect_depth(static_cast<const uint8_t*>(data), bytes);
}

extern "C" int imop_suggest_dimensions(size_t pixel_count, int (*out)[2], int cap) {
    if (cap < 0 || (cap > 0 && !out)) return -1;
    return dimensions(pixel_count, out, cap);
}

extern "C" int imop_analyze_data(const void* data_v, size_t bytes, ImopDataInfo* info) {
    if (!info) return IMOP_ERR_NULL_INPUT;
    std::memset(info, 0, sizeof(*info));
    const uint8_t* d = static_cast<const uint8_t*>(data_v);
    if (!d || bytes == 0) return IMOP_OK;
    const int bd = detect_depth(d, bytes);
    info->detected_bit_depth = bd;
    info->is_likely_16bit = bd > 8;
    if (bd > 8) {
        if (known_pixels(bytes / 2)) {
            // u16 storage: extremes over every sample (:174-183)
            const size_t n = bytes / 2;
            info->pixel_count = (int)n;
            int mn = 65535, mx = 0;
            for (size_t i = 0; i < n; i++) {
                const int v = u16_at(d, i);
                mn = std::min(mn, v);
                mx = std::max(mx, v);
            }
            info->min_value = mn;
            info->max_value = mx;
        } else {
            // packed: the pixel count the bits allow (one more when that is a known size), and
            // extremes of the first 10000 samples read from two bytes each, as the reference
            // does (:184-203; samples spanning three bytes lose their top bits there too)
            info->is_packed = 1;
            int n = (int)(bytes * 8 / (size_t)bd);
            if (!known_pixels((size_t)n) && known_pixels((size_t)n + 1)) n++;
            info->pixel_count = n;
            int mn = bd >= 16 ? 65535 : (1 << bd) - 1, mx = 0;
            const int mask = (int)((1u << bd) - 1);
            const int m = std::min(n, 10000);
            for (int i = 0; i < m; i++) {
                const int bo = i * bd / 8, bs = i * bd % 8;
                if ((size_t)bo + 1 < bytes) {
                    const int v = ((d[bo] | (d[bo + 1] << 8)) >> bs) & mask;
                    mn = std::min(mn, v);
                    mx = std::max(mx, v);
                }
            }
            info->min_value = mn;
            info->max_value = mx;
        }
    } else {
        info->pixel_count = (int)bytes;
        int mn = 255, mx = 0;
        for (size_t i = 0; i < bytes; i++) {
            mn = std::min(mn, (int)d[i]);
            mx = std::max(mx, (int)d[i]);
        }
        info->min_value = mn;
        info->max_value = mx;
    }
    const int k = dimensions((size_t)info->pixel_count, info->dims, IMOP_ANALYZE_MAX_DIMS);
    info->n_dims = std::min(k, IMOP_ANALYZE_MAX_DIMS);
    if (k > 0) {
        info->suggested_width = info->dims[0][0];
        info->suggested_height = info->dims[0][1];
    }
    return IMOP_OK;
}

namespace {

// one sample of a frame in the given storage (pixel::get_packed_raw for packed input; u16
// samples above the depth's maximum were MSB-aligned and shift down, align_raw_value)
int sample_at(const uint8_t* d, int x, int y, int w, int h, int bd, bool packed, size_t bytes) {
    if (x < 0 || x >= w || y < 0 || y >= h) return 0;
    const size_t i = (size_t)y * (size_t)w + (size_t)x;
    if (bd <= 8) return d[i];
    if (packed) {
        const int mv = bd >= 16 ? 65535 : (1 << bd) - 1;
        if (bd == 12) {
            const size_t off = i / 2 * 3;
            if (off + 2 >= bytes) return 0;
            return (i & 1) ? ((d[off + 2] << 4) | (d[off + 1] >> 4)) & mv : ((d[off] << 4) | (d[off + 1] & 0xF)) & mv;
        }
        if (bd == 10) {
            const size_t off = i / 4 * 5;
            const int s = (int)(i & 3);
            if (off + 4 >= bytes) return 0;
            return ((d[off + (size_t)s] << 2) | ((d[off + 4] >> (2 * s)) & 3)) & mv;
        }
        const size_t bit = i * (size_t)bd, off = bit / 8;
        const int shift = (int)(bit % 8);
        if (off >= bytes) return 0;
        const int nb = (int)std::min((size_t)((bd + shift + 7) / 8), bytes - off);
        uint32_t v = 0;
        for (int k = 0; k < nb; k++) v |= (uint32_t)d[off + (size_t)k] << (8 * k);
        return (int)((v >> shift) & (uint32_t)mv);
    }
    int v = u16_at(d, i);
    const int mv = bd >= 16 ? 65535 : (1 << bd) - 1;
    if (bd < 16 && v > mv) v >>= (16 - bd);
    return v;
}

}  // namespace

// Bayer phase (src/analyzer.cpp:206-319): 2x2 blocks of low local contrast vote for the diagonal
// that holds the two greens (the flatter one); the channel means of the winning family's two
// non-green sites then tell red from blue (a ratio above 1.15 flips the default).
extern "C" int imop_guess_pattern(const void* data_v, int w, int h, int bd, int packed) {
    const uint8_t* d = static_cast<const uint8_t*>(data_v);
    if (!d || w < 4 || h < 4) return IMOP_RGGB;
    const size_t bytes = packed ? ((size_t)w * h * (size_t)bd + 7) / 8 : (size_t)w * h * (bd <= 8 ? 1 : 2);
    auto val = [&](int x, int y) { return sample_at(d, x, y, w, h, bd, packed != 0, bytes); };

    const int n_px = (int)((long long)w * h);
    const int n_sample = std::min(20000, n_px);
    int lo = val(0, 0), hi = lo;
    for (int i = 0; i < n_sample; i++) {
        const int p = (int)((long long)i * 10007 % n_px);
        const int v = val(p % w, p / w);
        lo = std::min(lo, v);
        hi = std::max(hi, v);
    }
    const int range = std::max(1, hi - lo);
    int step = std::max(1, (int)std::sqrt((double)w * h / 5000.0));
    step = std::max(2, step / 2 * 2);
    const double conf = std::max(1.0, range * 0.02);
    int vote_diag = 0, vote_anti = 0;  // greens on the anti-diagonal (RGGB / BGGR) or the diagonal
    for (int y = 0; y < h - 1; y += step) {
        for (int x = 0; x < w - 1; x += step) {
            const double tl = val(x, y), tr = val(x + 1, y), bl = val(x, y + 1), br = val(x + 1, y + 1);
            const double d1 = std::abs(tl - br), d2 = std::abs(tr - bl);
            if (std::abs(d1 - d2) < conf) continue;
            const double local = std::max({tl, tr, bl, br}) - std::min({tl, tr, bl, br});
            if (local > range * 0.15) continue;
            const double hd = std::abs(tl - tr) + std::abs(bl - br), vd = std::abs(tl - bl) + std::abs(tr - br);
            if (std::max(hd, vd) / std::max(1.0, std::min(hd, vd)) > 4.0) continue;
            if (d2 < d1) vote_anti++;
            else vote_diag++;
        }
    }
    const int gstep = std::max(1, std::min(w, h) / 256) | 1;
    double sum[4] = {0, 0, 0, 0};  // sites (even, even) (odd, odd) (even row, odd col) (odd row, even col)
    int cnt[4] = {0, 0, 0, 0};
    for (int y = 0; y < h; y += gstep)
        for (int x = 0; x < w; x += gstep) {
            const int k = ((y & 1) == 0 && (x & 1) == 0) ? 0 : ((y & 1) && (x & 1)) ? 1 : ((y & 1) == 0) ? 2 : 3;
            sum[k] += val(x, y);
            cnt[k]++;
        }
    if (std::abs(vote_anti - vote_diag) <= 2 && vote_anti + vote_diag < 10) return IMOP_RGGB;
    if (vote_anti >= vote_diag) {
        const double a = cnt[0] ? sum[0] / cnt[0] : 0, b = cnt[1] ? sum[1] / cnt[1] : 0;
        return (a > 0 ? b / a : 0) > 1.15 ? IMOP_BGGR : IMOP_RGGB;
    }
    const double a = cnt[2] ? sum[2] / cnt[2] : 0, b = cnt[3] ? sum[3] / cnt[3] : 0;
    return (a > 0 ? b / a : 0) > 1.15 ? IMOP_GBRG : IMOP_GRBG;
}
