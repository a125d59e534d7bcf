// isp_dpc.cuh - raster-order re-resolution of defect-correction chains.
//
// The reference corrects defects in raster order, in place (src/defect_correct/adaptive.cpp:25-57).
// Kernels evaluate every pixel against the uncorrected mosaic (Jacobi) and collect "seeds":
// pixels with a corrected raster-earlier neighbour whose value changes when that correction is
// seen.  resolve_chains() replays only those pixels, in raster order via a min-heap, pushing the
// raster-later neighbours of every pixel whose value differs from its Jacobi value, and returns
// the sorted list of such pixels with their sequential values.  Every pixel it does not visit
// keeps its Jacobi value, which then equals the sequential one.
#pragma once

#include "isp_kernels.h"
#include "isp_tile.cuh"

namespace imop {

namespace {

__device__ __forceinline__ void nb_offsets(int k, int& dx, int& dy) {
    const int DX[8] = {-2, 0, 2, -2, 2, -2, 0, 2};
    const int DY[8] = {-2, -2, -2, 0, 0, 2, 2, 2};
    dx = DX[k];
    dy = DY[k];
}

// Jacobi value of (x,y): every neighbour uncorrected
template <class Orig>
__device__ int jacobi_at(const FrameParams& fp, Orig orig, int x, int y) {
    unsigned m = dev::dpc_valid_mask(x, y, fp.w, fp.h);
    int nb[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
        int dx, dy;
        nb_offsets(k, dx, dy);
        nb[k] = ((m >> k) & 1u) ? orig(x + dx, y + dy) : 0;
    }
    return dev::dpc_apply(orig(x, y), nb, m, fp.dpc_thr);
}

__device__ void heap_push(int* h, int& n, int v) {
    int i = n++;
    while (i > 0) {
        int p = (i - 1) >> 1;
        if (h[p] <= v) break;
        h[i] = h[p];
        i = p;
    }
    h[i] = v;
}
__device__ int heap_pop(int* h, int& n) {
    int top = h[0];
    int v = h[--n];
    int i = 0;
    while (true) {
        int l = 2 * i + 1;
        if (l >= n) break;
        int r = l + 1;
        int c = (r < n && h[r] < h[l]) ? r : l;
        if (h[c] >= v) break;
        h[i] = h[c];
        i = c;
    }
    if (n > 0) h[i] = v;
    return top;
}

}  // namespace

// Serial raster-order resolution of the seeds (one thread).  `orig(x,y)` gives the uncorrected
// black-levelled sample.  Writes the sorted override list and returns its length.
template <class Orig>
__device__ int resolve_chains(const FrameParams& fp, Orig orig, const FixupScratch& fs) {
    int n_seed = min(*fp.seed_count, fp.seed_cap);
    int* heap = fs.heap;
    int hn = 0;
    for (int i = 0; i < n_seed; i++) heap_push(heap, hn, fp.seeds[i]);
    int n_ov = 0, last = -1;
    const int W = fp.w, H = fp.h;
    while (hn > 0) {
        int p = heap_pop(heap, hn);
        if (p == last) continue;
        last = p;
        int x = p % W, y = p / W;
        unsigned m = dev::dpc_valid_mask(x, y, W, H);
        int nb[8];
#pragma unroll
        for (int k = 0; k < 8; k++) {
            int dx, dy;
            nb_offsets(k, dx, dy);
            int v = 0;
            if ((m >> k) & 1u) {
                int nx = x + dx, ny = y + dy;
                if (k < 4) {
                    int s = find_override(fs.ov_idx, fs.ov_val, n_ov, ny * W + nx);
                    v = s >= 0 ? s : jacobi_at(fp, orig, nx, ny);
                } else {
                    v = orig(nx, ny);
                }
            }
            nb[k] = v;
        }
        int s = dev::dpc_apply(orig(x, y), nb, m, fp.dpc_thr);
        if (s != jacobi_at(fp, orig, x, y)) {
            if (n_ov >= fs.cap) {
                atomicExch(fp.status, 104 /* IMOP_ERR_CAPACITY */);
                break;
            }
            fs.ov_idx[n_ov] = p;
            fs.ov_val[n_ov] = s;
            n_ov++;
            for (int k = 4; k < 8; k++) {
                if (!((m >> k) & 1u)) continue;
                int dx, dy;
                nb_offsets(k, dx, dy);
                if (hn >= fs.cap) {
                    atomicExch(fp.status, 104);
                    break;
                }
                heap_push(heap, hn, (y + dy) * W + (x + dx));
            }
        }
    }
    return n_ov;
}

// The same resolution by one warp, for the fix-up launch: lane 0 owns the heap and the override
// list; for every popped pixel, lanes 0..3 evaluate its earlier neighbours (override or Jacobi
// value), lanes 4..7 read its later neighbours, lane 8 its own sample and lane 9 its Jacobi
// value, all at once, so the serial chain waits on one round of loads per pixel instead of six.
template <class Orig>
__device__ int resolve_chains_warp(const FrameParams& fp, Orig orig, const FixupScratch& fs) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int W = fp.w, H = fp.h;
    int* heap = fs.heap;
    int hn = 0, n_ov = 0, last = -1;
    if (lane == 0) {
        const int n_seed = min(*fp.seed_count, fp.seed_cap);
        for (int i = 0; i < n_seed; i++) heap_push(heap, hn, fp.seeds[i]);
    }
    hn = __shfl_sync(full, hn, 0);
    while (hn > 0) {
        int p = 0;
        if (lane == 0) p = heap_pop(heap, hn);
        p = __shfl_sync(full, p, 0);
        hn = __shfl_sync(full, hn, 0);
        if (p == last) continue;
        last = p;
        const int x = p % W, y = p / W;
        const unsigned m = dev::dpc_valid_mask(x, y, W, H);
        __syncwarp();  // lane 0's override writes are visible to the lanes that search them
        int v = 0;
        if (lane < 8) {
            if ((m >> lane) & 1u) {
                int dx, dy;
                nb_offsets(lane, dx, dy);
                const int nx = x + dx, ny = y + dy;
                if (lane < 4) {
                    const int s = find_override(fs.ov_idx, fs.ov_val, n_ov, ny * W + nx);
                    v = s >= 0 ? s : jacobi_at(fp, orig, nx, ny);
                } else {
                    v = orig(nx, ny);
                }
            }
        } else if (lane == 8) {
            v = orig(x, y);
        } else if (lane == 9) {
            v = jacobi_at(fp, orig, x, y);
        }
        int nb[8];
#pragma unroll
        for (int k = 0; k < 8; k++) nb[k] = __shfl_sync(full, v, k);
        const int c = __shfl_sync(full, v, 8), jac = __shfl_sync(full, v, 9);
        int stop = 0;
        if (lane == 0) {
            const int s = dev::dpc_apply(c, nb, m, fp.dpc_thr);
            if (s != jac) {
                if (n_ov >= fs.cap) {
                    atomicExch(fp.status, 104 /* IMOP_ERR_CAPACITY */);
                    stop = 1;
                } else {
                    fs.ov_idx[n_ov] = p;
                    fs.ov_val[n_ov] = s;
                    n_ov++;
                    for (int k = 4; k < 8; k++) {
                        if (!((m >> k) & 1u)) continue;
                        int dx, dy;
                        nb_offsets(k, dx, dy);
                        if (hn >= fs.cap) {
                            atomicExch(fp.status, 104);
                            break;
                        }
                        heap_push(heap, hn, (y + dy) * W + (x + dx));
                    }
                }
            }
        }
        n_ov = __shfl_sync(full, n_ov, 0);
        hn = __shfl_sync(full, hn, 0);
        if (__shfl_sync(full, stop, 0)) break;
    }
    return n_ov;
}

struct GlobalOrig {
    const FrameParams* fp;
    PatternOffsets po;
    __device__ int operator()(int x, int y) const { return dev::orig_value(*fp, x, y, po); }
};

}  // namespace imop
