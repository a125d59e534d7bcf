// The reference-compatible C++ entry points (include/imop_ref_shims.hpp) against the CPU oracle:
// every shim on seeded frames of several sizes, bit depths and patterns, outputs compared byte for
// byte.  Built and run by tests/test_gpu_shims.py; prints one line per case and exits non-zero on
// any mismatch.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "../../include/imop_isp.h"
#include "../../include/imop_ref_shims.hpp"
extern "C" {
#include "../../oracle/isp_oracle.h"
}

static int failures = 0;

static void report(const char* what, int w, int h, int bd, bool ok) {
    std::printf("%-28s %5dx%-5d bd %2d : %s\n", what, w, h, bd, ok ? "ok" : "MISMATCH");
    if (!ok) failures++;
}

// seeded frame in the reference's storage (u8 for bd <= 8, u16 otherwise): a smooth scene with
// noise and 0.1 % hot / dead pixels, as a camera delivers (uniform noise would make most pixels
// defect candidates and overflow the defect-chain list, which the library reports as an error)
static std::vector<uint8_t> frame(int w, int h, int bd, int seed, int channels = 1) {
    std::mt19937 rng(seed);
    std::normal_distribution<float> noise(0.0f, 0.01f);
    const int mv = (1 << bd) - 1;
    const float fx = 0.02f + 0.01f * (seed % 5), fy = 0.03f + 0.01f * (seed % 3);
    size_t n = (size_t)w * h * channels;
    std::vector<uint8_t> f(n * (bd <= 8 ? 1 : 2));
    for (size_t i = 0; i < n; i++) {
        const int px = (int)(i / channels), x = px % w, y = px / w, c = (int)(i % channels);
        float t = 0.45f + 0.3f * std::sin(fx * x + c) * std::cos(fy * y) + noise(rng);
        int v = (int)(t * mv);
        v = v < 0 ? 0 : (v > mv ? mv : v);
        if (rng() % 997 == 0) v = (rng() & 1) ? mv : 0;
        if (bd <= 8) f[i] = (uint8_t)v;
        else { f[2 * i] = (uint8_t)v; f[2 * i + 1] = (uint8_t)(v >> 8); }
    }
    return f;
}

static std::vector<uint16_t> widen(const std::vector<uint8_t>& f, int bd) {
    size_t n = bd <= 8 ? f.size() : f.size() / 2;
    std::vector<uint16_t> o(n);
    for (size_t i = 0; i < n; i++) o[i] = bd <= 8 ? f[i] : (uint16_t)(f[2 * i] | (f[2 * i + 1] << 8));
    return o;
}

int main() {
    const int sizes[][2] = {{64, 48}, {131, 70}, {1006, 758}};
    const int depths[] = {8, 10, 12};
    int seed = 1;
    for (auto& s : sizes)
        for (int bd : depths) {
            const int w = s[0], h = s[1], pat = seed % 4, mv = (1 << bd) - 1;
            const auto P = static_cast<imop::BayerPattern>(pat);
            // black level, per channel and global
            for (int mode = 0; mode < 2; mode++) {
                auto f = frame(w, h, bd, seed++);
                auto ref = widen(f, bd);
                black_level::BlackLevelParams bp;
                bp.r_offset = 0.031f * mv; bp.gr_offset = 0.05f * mv; bp.gb_offset = 0.04f * mv; bp.b_offset = 17.5f;
                float off[4] = {bp.r_offset, bp.gr_offset, bp.gb_offset, bp.b_offset};
                auto st = black_level::process_black_level_cuda(f.data(), w, h, P,
                    mode ? black_level::BlackLevelAlgorithm::GLOBAL : black_level::BlackLevelAlgorithm::PER_CHANNEL, bd, bp);
                or_black_level(ref.data(), w, h, pat, bd, mode, off);
                report(mode ? "black_level GLOBAL" : "black_level PER_CHANNEL", w, h, bd,
                       st == black_level::BlackLevelError::Ok && widen(f, bd) == ref);
            }
            // defect correction, adaptive and map-based
            {
                auto f = frame(w, h, bd, seed++);
                auto ref = widen(f, bd);
                defect_correct::DefectCorrectParams dp;
                dp.threshold = 0.2f;
                auto st = defect_correct::process_defect_correct_cuda(f.data(), w, h, P,
                    defect_correct::DefectCorrectAlgorithm::ADAPTIVE, bd, dp);
                or_dpc_adaptive(ref.data(), w, h, pat, bd, dp.threshold);
                report("defect_correct ADAPTIVE", w, h, bd, st == defect_correct::DefectCorrectError::Ok && widen(f, bd) == ref);
                auto g = frame(w, h, bd, seed++);
                auto ref2 = widen(g, bd);
                std::vector<defect_correct::DefectPoint> map;
                std::mt19937 rng(seed);
                for (int k = 0; k < 40; k++) map.push_back({(int)(rng() % w), (int)(rng() % h)});
                map.push_back({map[0].x + 2, map[0].y});
                map.push_back(map[1]);
                dp.map = map.data();
                dp.map_count = (int)map.size();
                st = defect_correct::process_defect_correct_cuda(g.data(), w, h, P,
                    defect_correct::DefectCorrectAlgorithm::MAP_BASED, bd, dp);
                or_dpc_map(ref2.data(), w, h, pat, bd, reinterpret_cast<const ImopDefectPoint*>(map.data()), dp.map_count);
                report("defect_correct MAP_BASED", w, h, bd, st == defect_correct::DefectCorrectError::Ok && widen(g, bd) == ref2);
            }
            // lens shading, polynomial and flat field
            {
                auto f = frame(w, h, bd, seed++);
                auto ref = widen(f, bd);
                lens_shading::LensShadingParams lp;
                lp.r_coef = {0.4f, 0.1f, -0.05f}; lp.gr_coef = {0.3f, 0.05f, 0.0f};
                lp.gb_coef = {0.31f, 0.04f, 0.01f}; lp.b_coef = {0.5f, -0.1f, 0.2f};
                lp.center_x = 0.48f; lp.center_y = 0.53f;
                auto st = lens_shading::process_lens_shading_cuda(f.data(), w, h, P,
                    lens_shading::LensShadingAlgorithm::POLYNOMIAL, bd, lp);
                float coef[4][3] = {{0.4f, 0.1f, -0.05f}, {0.3f, 0.05f, 0.0f}, {0.31f, 0.04f, 0.01f}, {0.5f, -0.1f, 0.2f}};
                or_lsc_poly(ref.data(), w, h, pat, bd, coef, lp.center_x, lp.center_y);
                report("lens_shading POLYNOMIAL", w, h, bd, st == lens_shading::LensShadingError::Ok && widen(f, bd) == ref);
                auto g = frame(w, h, bd, seed++);
                auto ref2 = widen(g, bd);
                auto ff = frame(w, h, bd, seed++);
                lp.flat_field = ff.data();
                lp.flat_field_width = w;
                lp.flat_field_height = h;
                st = lens_shading::process_lens_shading_cuda(g.data(), w, h, P,
                    lens_shading::LensShadingAlgorithm::FLAT_FIELD, bd, lp);
                std::vector<float> grid(32 * 24 * 4);
                bool ok = or_lsc_flat_field_grid(ff.data(), w, h, pat, bd, grid.data()) == 0;
                or_lsc_grid(ref2.data(), w, h, pat, bd, grid.data(), 32, 24);
                report("lens_shading FLAT_FIELD", w, h, bd, ok && st == lens_shading::LensShadingError::Ok && widen(g, bd) == ref2);
            }
            // white balance and CCM on RGB
            {
                auto f = frame(w, h, bd, seed++, 3);
                auto ref = widen(f, bd);
                std::vector<uint8_t> out(f.size());
                auto st = white_balance::process_white_balance_cuda(f.data(), out.data(), w, h, 3, bd, 1.9f, 1.0f, 1.6f);
                float gains[3] = {1.9f, 1.0f, 1.6f};
                or_wb_rgb(ref.data(), w, h, bd, gains);
                report("white_balance MANUAL", w, h, bd, st == white_balance::WhiteBalanceError::Ok && widen(out, bd) == ref);
                auto g = frame(w, h, bd, seed++, 3);
                auto ref2 = widen(g, bd);
                float m[9] = {1.6f, -0.4f, -0.2f, -0.25f, 1.5f, -0.25f, -0.1f, -0.5f, 1.6f};
                auto st2 = ccm::process_ccm_cuda(g.data(), out.data(), w, h, 3, bd, m);
                or_ccm(ref2.data(), w, h, bd, m);
                report("ccm LINEAR_3X3", w, h, bd, st2 == ccm::CCMError::Ok && widen(out, bd) == ref2);
                // custom 3D LUT (a seeded 9^3 cube around the identity)
                lut::LUT3D cube;
                cube.size = 9;
                uint32_t s = (uint32_t)seed * 2654435761u + 7u;
                for (int r = 0; r < 9; r++)
                    for (int gg = 0; gg < 9; gg++)
                        for (int b = 0; b < 9; b++) {
                            const float idv[3] = {r / 8.0f, gg / 8.0f, b / 8.0f};
                            for (int c = 0; c < 3; c++) {
                                s = s * 1664525u + 1013904223u;
                                cube.data.push_back(idv[c] + ((float)(s >> 8) / 16777216.0f - 0.5f) * 0.2f);
                            }
                        }
                auto q = frame(w, h, bd, seed++, 3);
                auto ref3 = widen(q, bd);
                auto st3 = lut::process_lut_cuda(q.data(), out.data(), w, h, 3, bd, cube);
                or_lut3d(ref3.data(), w, h, bd, cube.data.data(), cube.size);
                report("lut CUSTOM_3D", w, h, bd, st3 == lut::LUTError::Ok && widen(out, bd) == ref3);
            }
            // demosaic
            {
                auto f = frame(w, h, bd, seed++);
                auto bay = widen(f, bd);
                const imop::DemosaicAlgorithm algos[3] = {imop::DemosaicAlgorithm::HQLI, imop::DemosaicAlgorithm::MG,
                                                          imop::DemosaicAlgorithm::AMAZE};
                for (auto a : algos) {
                    std::vector<uint8_t> out((size_t)w * h * 3 * (bd <= 8 ? 1 : 2));
                    auto st = imop::demosaic_cuda(f.data(), out.data(), w, h, P, a, bd, false);
                    std::vector<uint16_t> ref((size_t)w * h * 3);
                    if (a == imop::DemosaicAlgorithm::HQLI) or_demosaic_hqli(bay.data(), ref.data(), w, h, pat, bd);
                    else if (a == imop::DemosaicAlgorithm::MG) or_demosaic_mg(bay.data(), ref.data(), w, h, pat, bd);
                    else or_demosaic_amaze(bay.data(), ref.data(), w, h, pat, bd);
                    report("demosaic_cuda", w, h, bd, st == imop::DemosaicError::Ok && widen(out, bd) == ref);
                }
                // unsupported algorithm -> InternalError (the dispatcher falls back to the CPU)
                std::vector<uint8_t> out((size_t)w * h * 3 * (bd <= 8 ? 1 : 2));
                report("demosaic_cuda RCD fallback", w, h, bd,
                       imop::demosaic_cuda(f.data(), out.data(), w, h, P, imop::DemosaicAlgorithm::RCD, bd, false) ==
                           imop::DemosaicError::InternalError);
                // batch of three frames
                std::vector<std::vector<uint8_t>> ins, outs;
                std::vector<const uint8_t*> ip;
                std::vector<uint8_t*> op;
                for (int k = 0; k < 3; k++) {
                    ins.push_back(frame(w, h, bd, seed++));
                    outs.emplace_back((size_t)w * h * 3 * (bd <= 8 ? 1 : 2));
                }
                for (int k = 0; k < 3; k++) { ip.push_back(ins[k].data()); op.push_back(outs[k].data()); }
                auto st = imop::demosaic_cuda_batch(ip.data(), op.data(), 3, w, h, P, imop::DemosaicAlgorithm::AMAZE, bd);
                bool ok = st == imop::DemosaicError::Ok;
                for (int k = 0; k < 3; k++) {
                    std::vector<uint16_t> ref((size_t)w * h * 3);
                    auto b = widen(ins[k], bd);
                    or_demosaic_amaze(b.data(), ref.data(), w, h, pat, bd);
                    ok = ok && widen(outs[k], bd) == ref;
                }
                report("demosaic_cuda_batch", w, h, bd, ok);
            }
        }
    // tone curves: GAMMA, S_CURVE, LEVELS and CURVES_3POINT on the device, every sample equal to the
    // per-sample table of the reference's expression (imop_tone_table, pinned against the reference
    // on the CPU); SHADOWS_HIGHLIGHTS couples the channels and falls back to the CPU
    {
        const long long served0 = imop_shim_calls_served();
        int tone_calls = 0;
        const int tsz[2][2] = {{64, 48}, {1006, 758}};
        for (int bd : {8, 10, 12, 16})
            for (int ti = 0; ti < 2; ti++)
                for (int a = 0; a < 4; a++) {
                    const int w = tsz[ti][0], h = tsz[ti][1];
                    auto f = frame(w, h, bd == 16 ? 15 : bd, 900 + bd * 10 + a, 3);
                    std::vector<uint8_t> out(f.size());
                    tone::ToneParams tp;
                    tp.gamma = 2.2f + 0.3f * a; tp.contrast = 0.35f * a - 0.2f; tp.shadows = 0.4f - 0.3f * a;
                    tp.highlights = 0.1f * a; tp.black_point = 0.04f * a; tp.white_point = 0.97f - 0.05f * a;
                    tp.mid_point = 0.4f + 0.05f * a;
                    const auto algo = static_cast<tone::ToneAlgorithm>(a);
                    const auto st = tone::process_tone_cuda(f.data(), out.data(), w, h, 3, algo, bd, tp);
                    std::vector<uint16_t> table(imop_tone_table_entries(bd));
                    ImopToneParams ip;
                    std::memcpy(&ip, &tp, sizeof(ip));
                    bool ok = st == tone::ToneError::Ok &&
                              imop_tone_table(a, bd, &ip, table.data(), table.size()) == IMOP_OK;
                    const auto in16 = widen(f, bd), out16 = widen(out, bd);
                    for (size_t i = 0; ok && i < in16.size(); i++) ok = out16[i] == table[in16[i]];
                    tone_calls++;
                    static const char* names[4] = {"tone GAMMA", "tone S_CURVE", "tone LEVELS", "tone CURVES_3POINT"};
                    report(names[a], w, h, bd, ok);
                }
        report("tone calls served on the device", tone_calls, 1, 0,
               imop_shim_calls_served() - served0 == tone_calls);
        tone::ToneParams tp;
        uint8_t px[3] = {1, 2, 3}, po[3];
        report("tone SHADOWS_HIGHLIGHTS fallback", 1, 1, 8,
               tone::process_tone_cuda(px, po, 1, 1, 3, tone::ToneAlgorithm::SHADOWS_HIGHLIGHTS, 8, tp) ==
                   tone::ToneError::InternalError);
    }
    // jpeg_codec::process_encode_cuda: the oracle's bytes (the reference's baseline encoder) for
    // every subsampling, a range of qualities and sizes; the reference's status codes
    {
        std::mt19937 rng(77);
        const int sizes[4][2] = {{8, 8}, {37, 29}, {640, 480}, {1001, 333}};
        for (int si = 0; si < 4; si++)
            for (int ss = 0; ss < 3; ss++) {
                const int w = sizes[si][0], h = sizes[si][1], q = 10 + 30 * ss + 7 * si;
                std::vector<uint8_t> rgb((size_t)w * h * 3);
                for (size_t i = 0; i < rgb.size(); i++) rgb[i] = (uint8_t)((i * 37 + 127 + (rng() & 15)) % 256);
                const size_t cap = (size_t)w * h * 9 + 65536;
                std::vector<uint8_t> a(cap), b(cap);
                size_t na = 0, nb = 0;
                jpeg_codec::JpegParams jp;
                jp.quality = q;
                jp.chroma_subsample = ss;
                const auto st = jpeg_codec::process_encode_cuda(rgb.data(), a.data(), &na, w, h, 3, 8, jp);
                const int so = or_jpeg_encode(rgb.data(), w, h, 8, q, ss, b.data(), &nb);
                report("jpeg process_encode_cuda", w, h, 8,
                       st == jpeg_codec::JpegError::Ok && so == 0 && na == nb && std::memcmp(a.data(), b.data(), na) == 0);
            }
        std::vector<uint8_t> z(8 * 8 * 3), o(1 << 16);
        size_t n = 0;
        jpeg_codec::JpegParams jp;
        report("jpeg null input", 8, 8, 8,
               jpeg_codec::process_encode_cuda(nullptr, o.data(), &n, 8, 8, 3, 8, jp) == jpeg_codec::JpegError::NullInput);
        report("jpeg bit depth", 8, 8, 16,
               jpeg_codec::process_encode_cuda(z.data(), o.data(), &n, 8, 8, 3, 16, jp) ==
                   jpeg_codec::JpegError::InvalidBitDepth);
        report("jpeg too small", 4, 4, 8,
               jpeg_codec::process_encode_cuda(z.data(), o.data(), &n, 4, 4, 3, 8, jp) == jpeg_codec::JpegError::ImageTooSmall);
        jp.quality = 0;
        report("jpeg quality", 8, 8, 8,
               jpeg_codec::process_encode_cuda(z.data(), o.data(), &n, 8, 8, 3, 8, jp) == jpeg_codec::JpegError::InvalidQuality);
        int dw = 0, dh = 0, dc = 0;
        const uint8_t junk[4] = {0x12, 0x34, 0x56, 0x78};
        report("jpeg decode invalid data", 1, 1, 8,
               jpeg_codec::process_decode_cuda(junk, 4, o.data(), &dw, &dh, &dc) == jpeg_codec::JpegError::InvalidJpegData);
        // without the reference's CPU decoder linked in, decoding is not served here
        const uint8_t soi[4] = {0xFF, 0xD8, 0xFF, 0xD9};
        report("jpeg decode without the CPU decoder", 1, 1, 8,
               jpeg_codec::process_decode_cuda(soi, 4, o.data(), &dw, &dh, &dc) == jpeg_codec::JpegError::InternalError);
    }
    std::printf("%s\n", failures ? "FAILED" : "ALL OK");
    return failures ? 1 : 0;
}
