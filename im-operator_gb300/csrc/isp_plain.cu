// isp_plain.cu - the same pipeline as one kernel per stage over full frames kept in device
// memory: the per-operator form that the fused kernel is measured against, and the source of
// the per-stage dumps used by the parity tests.  Each stage kernel has the arithmetic of the
// fused path (isp_device.cuh) and reads / writes whole frames.

#include <cuda_runtime.h>

#include <algorithm>

#include "isp_kernels.h"
#include "isp_dpc.cuh"
#include "isp_tile.cuh"

namespace imop {

namespace {

constexpr int kPlainThreads = 256;

inline int plain_blocks(size_t n) {
    size_t b = (n + kPlainThreads - 1) / kPlainThreads;
    return (int)(b < 152 * 16 ? b : 152 * 16);
}

#define GRID_STRIDE(i, n) for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < (n); i += (size_t)gridDim.x * blockDim.x)

// every pixel (x, y) of a W x H plane, i = y * W + x: rows over the grid's y blocks, columns over
// its x threads (no division per pixel)
#define FOR_PIXELS(x, y, i, W, H)                                                                  \
    for (int y = blockIdx.y; y < (H); y += gridDim.y)                                               \
        for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < (W); x += gridDim.x * blockDim.x) \
            if (const size_t i = (size_t)y * (W) + x; true)

// 2-D grid of those loops: enough column blocks for a row, rows up to about 16 CTAs per SM
inline dim3 pixel_grid(int w, int h) {
    const int gx = (w + kPlainThreads - 1) / kPlainThreads;
    const int gy = std::max(1, std::min(h, 152 * 16 / std::max(1, gx)));
    return dim3((unsigned)gx, (unsigned)gy);
}

__global__ void unpack_kernel(const __grid_constant__ FrameParams fp, uint16_t* out) {
    FOR_PIXELS(x, y, i, fp.w, fp.h) {
        out[i] = (uint16_t)dev::load_raw(fp, x, y);
    }
}

__global__ void black_level_kernel(const __grid_constant__ FrameParams fp, uint16_t* d) {
    PatternOffsets po = pattern_offsets(fp.pattern);
    FOR_PIXELS(x, y, i, fp.w, fp.h) {
        d[i] = (uint16_t)dev::black_level(fp, d[i], bayer_color(y, x, po));
    }
}

// Jacobi defect pass: out = F(in) (adaptive) / in (other pixels)
__global__ void dpc_jacobi_kernel(const __grid_constant__ FrameParams fp, const uint16_t* in, uint16_t* out) {
    const int W = fp.w, H = fp.h;
    FOR_PIXELS(x, y, i, W, H) {
        int v = in[i];
        if (x >= 2 && x < W - 2 && y >= 2 && y < H - 2) {
            int nb[8] = {in[i - 2 * W - 2], in[i - 2 * W], in[i - 2 * W + 2], in[i - 2],
                         in[i + 2], in[i + 2 * W - 2], in[i + 2 * W], in[i + 2 * W + 2]};
            v = dev::dpc_apply(v, nb, dev::dpc_valid_mask(x, y, W, H), fp.dpc_thr);
        }
        out[i] = (uint16_t)v;
    }
}

__global__ void dpc_seed_kernel(const __grid_constant__ FrameParams fp, const uint16_t* orig, const uint16_t* jac) {
    const int W = fp.w, H = fp.h;
    FOR_PIXELS(x, y, i, W, H) {
        if (x < 2 || x >= W - 2 || y < 2 || y >= H - 2) continue;
        unsigned m = dev::dpc_valid_mask(x, y, W, H);
        const size_t e[4] = {i - 2 * W - 2, i - 2 * W, i - 2 * W + 2, i - 2};
        bool any = false;
        for (int k = 0; k < 4; k++)
            if ((m >> k) & 1u) any |= jac[e[k]] != orig[e[k]];
        if (!any) continue;
        int nb[8] = {jac[e[0]], jac[e[1]], jac[e[2]], jac[e[3]],
                     orig[i + 2], orig[i + 2 * W - 2], orig[i + 2 * W], orig[i + 2 * W + 2]};
        int s1 = dev::dpc_apply(orig[i], nb, m, fp.dpc_thr);
        if (s1 != jac[i]) {
            int slot = atomicAdd(fp.seed_count, 1);
            if (slot < fp.seed_cap) fp.seeds[slot] = (int)i;
            else atomicExch(fp.status, 104);
        }
    }
}

struct BufOrig {
    const uint16_t* d;
    int w;
    __device__ int operator()(int x, int y) const { return d[(size_t)y * w + x]; }
};

__global__ void dpc_fixup_plain_kernel(const __grid_constant__ FrameParams fp, FixupScratch fs, const uint16_t* orig,
                                       uint16_t* jac) {
    if (*fp.seed_count == 0) return;
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        int n = resolve_chains(fp, BufOrig{orig, fp.w}, fs);
        *fs.n_ov = n;
        for (int k = 0; k < n; k++) jac[fs.ov_idx[k]] = (uint16_t)fs.ov_val[k];
    }
}

__global__ void dpc_map_apply_kernel(const __grid_constant__ FrameParams fp, const uint16_t* in, uint16_t* out) {
    const int W = fp.w, H = fp.h;
    FOR_PIXELS(x, y, i, W, H) {
        int v = in[i];
        if (x >= 2 && x < W - 2 && y >= 2 && y < H - 2) {
            int s = map_lookup(fp, x, y);
            if (s >= 0) v = s;
        }
        out[i] = (uint16_t)v;
    }
}

__global__ void lens_shading_kernel(const __grid_constant__ FrameParams fp, uint16_t* d) {
    PatternOffsets po = pattern_offsets(fp.pattern);
    FOR_PIXELS(x, y, i, fp.w, fp.h) {
        int c = bayer_color(y, x, po);
        d[i] = (uint16_t)((fp.lsc_mode == 1) ? dev::lsc_poly(fp, d[i], x, y, c) : dev::lsc_grid(fp, d[i], x, y, c));
    }
}

// Bayer WB (spec order) and the demosaic's align_raw_value read
__global__ void bayer_wb_kernel(const __grid_constant__ FrameParams fp, uint16_t* d, int do_wb) {
    PatternOffsets po = pattern_offsets(fp.pattern);
    FOR_PIXELS(x, y, i, fp.w, fp.h) {
        int v = d[i];
        if (do_wb) v = dev::gain_round(v, fp.wb_cfa[bayer_color(y, x, po)], fp.mv);
        if (fp.bd > 8 && fp.bd < 16 && v > fp.mv) v >>= (16 - fp.bd);
        d[i] = (uint16_t)v;
    }
}

__global__ void green_kernel(const __grid_constant__ FrameParams fp, const uint16_t* bay, float* green) {
    const int W = fp.w, H = fp.h;
    PatternOffsets po = pattern_offsets(fp.pattern);
    FOR_PIXELS(x, y, i, W, H) {
        bool at_r = ((y & 1) == po.r_row) && ((x & 1) == po.r_col);
        bool at_b = ((y & 1) == po.b_row) && ((x & 1) == po.b_col);
        bool interior = x >= 2 && x < W - 2 && y >= 2 && y < H - 2;
        float g = -1.0f;
        if (!at_r && !at_b) {
            if (interior || fp.demosaic == DM_MG) g = (float)bay[i];
        } else if (interior) {
            int c = bay[i];
            if (fp.demosaic == DM_AMAZE) {
                g = dev::amaze_green(c, bay[i - 1], bay[i + 1], bay[i - 2], bay[i + 2], bay[i - W], bay[i + W],
                                     bay[i - 2 * W], bay[i + 2 * W]);
            } else {
                int n1 = bay[i - W] + bay[i + W] + bay[i + 1] + bay[i - 1];
                int n2 = bay[i - 2 * W] + bay[i + 2 * W] + bay[i + 2] + bay[i - 2];
                if (fp.bd <= 8) {
                    g = (float)dev::clampi((4 * c + 2 * n1 - n2 + 4) >> 3, 0, fp.mv);
                } else {
                    float t = dev::fsub(dev::fadd(dev::fmul(4.0f, (float)c), dev::fmul(2.0f, (float)n1)), (float)n2);
                    g = __fdiv_rn(t, 8.0f);
                }
            }
        }
        green[i] = g;
    }
}

__global__ void demosaic_rgb_kernel(const __grid_constant__ FrameParams fp, const uint16_t* bay, const float* green,
                                    uint16_t* rgb) {
    const int W = fp.w, H = fp.h, mv = fp.mv;
    PatternOffsets po = pattern_offsets(fp.pattern);
    auto B_ = [&](int x, int y) -> int { return bay[(size_t)y * W + x]; };
    auto G_ = [&](int x, int y) -> float { return green[(size_t)y * W + x]; };
    FOR_PIXELS(x, y, i, W, H) {
        int sx, sy;
        dev::border_source(x, y, W, H, fp.border_mode, sx, sy);
        bool at_r = ((sy & 1) == po.r_row) && ((sx & 1) == po.r_col);
        bool at_b = ((sy & 1) == po.b_row) && ((sx & 1) == po.b_col);
        int R = 0, Gv = 0, Bv = 0;
        if (fp.demosaic == DM_HQLI) {
            if (sx >= 2 && sx < W - 2 && sy >= 2 && sy < H - 2) {
                int n4 = B_(sx - 1, sy) + B_(sx + 1, sy) + B_(sx, sy - 1) + B_(sx, sy + 1);
                int d4 = B_(sx - 1, sy - 1) + B_(sx + 1, sy - 1) + B_(sx - 1, sy + 1) + B_(sx + 1, sy + 1);
                if (at_r) { R = B_(sx, sy); Gv = (n4 + 2) / 4; Bv = (d4 + 2) / 4; }
                else if (at_b) { R = (d4 + 2) / 4; Gv = (n4 + 2) / 4; Bv = B_(sx, sy); }
                else {
                    Gv = B_(sx, sy);
                    int hz = (B_(sx - 1, sy) + B_(sx + 1, sy) + 1) / 2;
                    int vt = (B_(sx, sy - 1) + B_(sx, sy + 1) + 1) / 2;
                    if ((sy & 1) == po.r_row) { R = hz; Bv = vt; } else { Bv = hz; R = vt; }
                }
                R = min(R, mv); Gv = min(Gv, mv); Bv = min(Bv, mv);
            }
        } else if (fp.demosaic == DM_MG && fp.bd <= 8) {
            int g = (int)G_(sx, sy);
            int Ri = 0, Bi = 0;
            if (sx >= 1 && sx < W - 1 && sy >= 1 && sy < H - 1) {
                auto cdi = [&](int xx, int yy) { return B_(xx, yy) - (int)G_(xx, yy); };
                if (at_r || at_b) {
                    int s = cdi(sx - 1, sy - 1) + cdi(sx + 1, sy - 1) + cdi(sx - 1, sy + 1) + cdi(sx + 1, sy + 1);
                    int other = g + (s + 2) / 4;
                    if (at_r) { Ri = B_(sx, sy); Bi = other; } else { Bi = B_(sx, sy); Ri = other; }
                } else {
                    int hz = cdi(sx - 1, sy) + cdi(sx + 1, sy), vt = cdi(sx, sy - 1) + cdi(sx, sy + 1);
                    int rc = ((sy & 1) == po.r_row) ? hz : vt, bc = ((sy & 1) == po.r_row) ? vt : hz;
                    Ri = g + (rc + 1) / 2;
                    Bi = g + (bc + 1) / 2;
                }
            }
            R = dev::clampi(Ri, 0, mv); Gv = dev::clampi(g, 0, mv); Bv = dev::clampi(Bi, 0, mv);
        } else {
            float g = G_(sx, sy), Rf = 0.0f, Bf = 0.0f;
            if (sx >= 1 && sx < W - 1 && sy >= 1 && sy < H - 1) {
                auto cd = [&](int xx, int yy) { return dev::fsub((float)B_(xx, yy), G_(xx, yy)); };
                if (at_r || at_b) {
                    float s = dev::fadd(dev::fadd(dev::fadd(cd(sx - 1, sy - 1), cd(sx + 1, sy - 1)), cd(sx - 1, sy + 1)),
                                        cd(sx + 1, sy + 1));
                    float other = dev::fadd(g, dev::fmul(s, 0.25f));
                    if (at_r) { Rf = (float)B_(sx, sy); Bf = other; } else { Bf = (float)B_(sx, sy); Rf = other; }
                } else {
                    float hz = dev::fadd(cd(sx - 1, sy), cd(sx + 1, sy));
                    float vt = dev::fadd(cd(sx, sy - 1), cd(sx, sy + 1));
                    bool rrow = (sy & 1) == po.r_row;
                    Rf = dev::fadd(g, dev::fmul(rrow ? hz : vt, 0.5f));
                    Bf = dev::fadd(g, dev::fmul(rrow ? vt : hz, 0.5f));
                }
            }
            R = dev::round_plane(Rf, mv); Gv = dev::round_plane(g, mv); Bv = dev::round_plane(Bf, mv);
        }
        rgb[3 * i] = (uint16_t)R;
        rgb[3 * i + 1] = (uint16_t)Gv;
        rgb[3 * i + 2] = (uint16_t)Bv;
    }
}

__global__ void rgb_wb_kernel(const __grid_constant__ FrameParams fp, uint16_t* rgb) {
    size_t n = (size_t)fp.w * fp.h * 3;
    GRID_STRIDE(i, n) rgb[i] = (uint16_t)dev::gain_round(rgb[i], fp.wb_rgb[i % 3], fp.mv);
}

__global__ void ccm_kernel(const __grid_constant__ FrameParams fp, uint16_t* rgb) {
    size_t n = (size_t)fp.w * fp.h;
    FrameParams f = fp;
    f.stages = 16u;  // CCM only
    GRID_STRIDE(i, n) {
        int r = rgb[3 * i], g = rgb[3 * i + 1], b = rgb[3 * i + 2];
        dev::rgb_tail(f, r, g, b);
        rgb[3 * i] = (uint16_t)r;
        rgb[3 * i + 1] = (uint16_t)g;
        rgb[3 * i + 2] = (uint16_t)b;
    }
}

__global__ void lut3d_kernel(const __grid_constant__ FrameParams fp, uint16_t* rgb) {
    size_t n = (size_t)fp.w * fp.h;
    GRID_STRIDE(i, n) {
        int r = rgb[3 * i], g = rgb[3 * i + 1], b = rgb[3 * i + 2];
        dev::lut3d_apply(fp.lut3d, fp.lut3d_size, fp.mv, r, g, b);
        rgb[3 * i] = (uint16_t)r;
        rgb[3 * i + 1] = (uint16_t)g;
        rgb[3 * i + 2] = (uint16_t)b;
    }
}

__global__ void output_kernel(const __grid_constant__ FrameParams fp, const uint16_t* rgb) {
    size_t n = (size_t)fp.w * fp.h * 3;
    GRID_STRIDE(i, n) {
        int v = rgb[i];
        if (fp.out_format == 0) fp.out[i] = __ldg(fp.tone8 + v);
        else if (fp.out_bpc == 1) fp.out[i] = (uint8_t)v;
        else reinterpret_cast<uint16_t*>(fp.out)[i] = (uint16_t)v;
    }
}

// u8 / u16-LE samples <-> u16 plane
__global__ void widen_kernel(const uint8_t* in, uint16_t* out, size_t n, int bps) {
    GRID_STRIDE(i, n) out[i] = bps == 1 ? (uint16_t)in[i] : (uint16_t)(in[2 * i] | (in[2 * i + 1] << 8));
}
__global__ void narrow_kernel(const uint16_t* in, uint8_t* out, size_t n, int bps) {
    GRID_STRIDE(i, n) {
        if (bps == 1) {
            out[i] = (uint8_t)in[i];
        } else {
            out[2 * i] = (uint8_t)in[i];
            out[2 * i + 1] = (uint8_t)(in[i] >> 8);
        }
    }
}

}  // namespace

cudaError_t launch_plain(const FrameParams& fp, const FixupScratch& fs, const MapPlan* plan, const PlainBuffers& b,
                         const PlainDumps* dumps, cudaStream_t st) {
    const size_t n = (size_t)fp.w * fp.h;
    const int nb = plain_blocks(n), nb3 = plain_blocks(3 * n);
    const dim3 pg = pixel_grid(fp.w, fp.h);
    auto dump = [&](uint16_t* dst, const uint16_t* src, size_t cnt) -> cudaError_t {
        if (!dst) return cudaSuccess;
        return cudaMemcpyAsync(dst, src, cnt * sizeof(uint16_t), cudaMemcpyDeviceToDevice, st);
    };
    PlainDumps none{};
    if (!dumps) dumps = &none;
    uint16_t* A = b.bayer_a;
    uint16_t* B = b.bayer_b;
    unpack_kernel<<<pg, kPlainThreads, 0, st>>>(fp, A);
    dump(dumps->unpacked, A, n);
    if (fp.stages & 1u) black_level_kernel<<<pg, kPlainThreads, 0, st>>>(fp, A);
    dump(dumps->black_level, A, n);
    if (fp.stages & 2u) {
        if (fp.dpc_mode == 0) {
            cudaMemsetAsync(fp.seed_count, 0, sizeof(int), st);
            dpc_jacobi_kernel<<<pg, kPlainThreads, 0, st>>>(fp, A, B);
            dpc_seed_kernel<<<pg, kPlainThreads, 0, st>>>(fp, A, B);
            dpc_fixup_plain_kernel<<<1, 32, 0, st>>>(fp, fs, A, B);
        } else {
            if (plan) launch_map_resolve(fp, *plan, st);
            dpc_map_apply_kernel<<<pg, kPlainThreads, 0, st>>>(fp, A, B);
        }
        uint16_t* t = A; A = B; B = t;
    }
    dump(dumps->defect, A, n);
    if (fp.stages & 4u) lens_shading_kernel<<<pg, kPlainThreads, 0, st>>>(fp, A);
    dump(dumps->lens_shading, A, n);
    bool wb = (fp.stages & 8u) != 0;
    bayer_wb_kernel<<<pg, kPlainThreads, 0, st>>>(fp, A, (wb && fp.stage_order == 0) ? 1 : 0);
    if (wb && fp.stage_order == 0) dump(dumps->white_balance, A, n);
    float* green = reinterpret_cast<float*>(B);  // bayer_b is sized for w*h floats
    if (fp.demosaic != DM_HQLI) green_kernel<<<pg, kPlainThreads, 0, st>>>(fp, A, green);
    demosaic_rgb_kernel<<<pg, kPlainThreads, 0, st>>>(fp, A, green, b.rgb);
    dump(dumps->demosaic, b.rgb, 3 * n);
    if (wb && fp.stage_order == 1) {
        rgb_wb_kernel<<<nb3, kPlainThreads, 0, st>>>(fp, b.rgb);
        dump(dumps->white_balance, b.rgb, 3 * n);
    }
    if (fp.stages & 16u) ccm_kernel<<<nb, kPlainThreads, 0, st>>>(fp, b.rgb);
    dump(dumps->ccm, b.rgb, 3 * n);
    if (fp.stages & 32u) lut3d_kernel<<<nb, kPlainThreads, 0, st>>>(fp, b.rgb);
    output_kernel<<<nb3, kPlainThreads, 0, st>>>(fp, b.rgb);
    return cudaGetLastError();
}

cudaError_t launch_widen(const uint8_t* in, uint16_t* out, size_t n, int bytes_per_sample, cudaStream_t st) {
    widen_kernel<<<plain_blocks(n), kPlainThreads, 0, st>>>(in, out, n, bytes_per_sample);
    return cudaGetLastError();
}

cudaError_t launch_narrow(const uint16_t* in, uint8_t* out, size_t n, int bytes_per_sample, cudaStream_t st) {
    narrow_kernel<<<plain_blocks(n), kPlainThreads, 0, st>>>(in, out, n, bytes_per_sample);
    return cudaGetLastError();
}

// One Bayer stage on plane a (result back in a; b is scratch of the same size).
cudaError_t launch_op_bayer(const FrameParams& fp, unsigned stage, const FixupScratch& fs, const MapPlan* plan,
                            uint16_t* a, uint16_t* b, cudaStream_t st) {
    const size_t n = (size_t)fp.w * fp.h;
    const dim3 pg = pixel_grid(fp.w, fp.h);
    cudaError_t e = cudaSuccess;
    if (stage == 1u) {
        black_level_kernel<<<pg, kPlainThreads, 0, st>>>(fp, a);
    } else if (stage == 2u) {
        if (fp.dpc_mode == 0) {
            if ((e = cudaMemsetAsync(fp.seed_count, 0, sizeof(int), st))) return e;
            dpc_jacobi_kernel<<<pg, kPlainThreads, 0, st>>>(fp, a, b);
            dpc_seed_kernel<<<pg, kPlainThreads, 0, st>>>(fp, a, b);
            dpc_fixup_plain_kernel<<<1, 32, 0, st>>>(fp, fs, a, b);
        } else {
            if (plan && (e = launch_map_resolve(fp, *plan, st))) return e;
            dpc_map_apply_kernel<<<pg, kPlainThreads, 0, st>>>(fp, a, b);
        }
        if ((e = cudaGetLastError())) return e;
        return cudaMemcpyAsync(a, b, n * sizeof(uint16_t), cudaMemcpyDeviceToDevice, st);
    } else if (stage == 4u) {
        lens_shading_kernel<<<pg, kPlainThreads, 0, st>>>(fp, a);
    } else {
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// One RGB stage (white balance or CCM) on an RGB u16 x 3 plane, in place.
// per-sample table map (tone curves): each thread maps 8 consecutive samples, the tail one by one
template <typename T>
__global__ void table_map_kernel(const T* in, T* out, size_t n, const uint16_t* __restrict__ table) {
    const size_t groups = n / 8;
    for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < groups; g += (size_t)gridDim.x * blockDim.x) {
        T v[8];
#pragma unroll
        for (int k = 0; k < 8; k++) v[k] = in[8 * g + k];
#pragma unroll
        for (int k = 0; k < 8; k++) out[8 * g + k] = (T)__ldg(table + v[k]);
    }
    if (blockIdx.x == 0 && threadIdx.x < n - 8 * groups) {
        const size_t i = 8 * groups + threadIdx.x;
        out[i] = (T)__ldg(table + in[i]);
    }
}

cudaError_t launch_table_map(const uint8_t* in, uint8_t* out, size_t n, int bytes_per_sample, const uint16_t* table,
                             cudaStream_t st) {
    const int nb = plain_blocks((n + 7) / 8);
    if (bytes_per_sample == 1) table_map_kernel<uint8_t><<<nb, kPlainThreads, 0, st>>>(in, out, n, table);
    else
        table_map_kernel<uint16_t><<<nb, kPlainThreads, 0, st>>>(reinterpret_cast<const uint16_t*>(in),
                                                                 reinterpret_cast<uint16_t*>(out), n, table);
    return cudaGetLastError();
}

cudaError_t launch_op_rgb(const FrameParams& fp, unsigned stage, uint16_t* rgb, cudaStream_t st) {
    const size_t n = (size_t)fp.w * fp.h;
    if (stage == 8u) rgb_wb_kernel<<<plain_blocks(3 * n), kPlainThreads, 0, st>>>(fp, rgb);
    else if (stage == 16u) ccm_kernel<<<plain_blocks(n), kPlainThreads, 0, st>>>(fp, rgb);
    else if (stage == 32u) lut3d_kernel<<<plain_blocks(n), kPlainThreads, 0, st>>>(fp, rgb);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

}  // namespace imop
