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

// The warp resolution below with its heap and override list in shared memory (hcap / ocap
// entries): the pops, pushes and override searches of the serial chain then wait on shared
// memory instead of on global memory, and the seeds load in parallel.  Returns -1, having written
// nothing, when the chains need more entries than that; the caller then runs the global version.
template <class Orig>
__device__ int resolve_chains_warp_smem(const FrameParams& fp, Orig orig, const FixupScratch& fs, int* heap, int hcap,
                                        int* ov_idx, int* ov_val, int ocap) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int W = fp.w, H = fp.h;
    const int n_seed = min(*fp.seed_count, fp.seed_cap);
    if (n_seed > hcap) return -1;
    for (int i = lane; i < n_seed; i += 32) heap[i] = fp.seeds[i];
    __syncwarp();
    int hn = 0, n_ov = 0, last = -1, bad = 0;
    if (lane == 0) {
        // heapify in place (sift-down from the last parent)
        hn = n_seed;
        for (int i = hn / 2 - 1; i >= 0; i--) {
            const int v = heap[i];
            int j = i;
            while (true) {
                const int l = 2 * j + 1;
                if (l >= hn) break;
                const int r = l + 1;
                const int c = (r < hn && heap[r] < heap[l]) ? r : l;
                if (heap[c] >= v) break;
                heap[j] = heap[c];
                j = c;
            }
            heap[j] = v;
        }
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
        __syncwarp();  // lane 0's writes of the override list are visible to the lanes that search it
        // the 20 same-colour samples every value of this pixel depends on, one load per lane in one
        // round: rows y-4, y-2, y, y+2 by columns x-4 .. x+4 (step 2); outside the frame 0 (the
        // valid masks leave those out)
        int win = 0;
        if (lane < 20) {
            const int wx = x - 4 + 2 * (lane % 5), wy = y - 4 + 2 * (lane / 5);
            if (wx >= 0 && wx < W && wy >= 0 && wy < H) win = orig(wx, wy);
        }
        // lanes 0-3: the Jacobi value of earlier neighbour k (override first), 4-7: later neighbour
        // k's sample, 8: the pixel's sample, 9: its Jacobi value
        int cx = x, cy = y;  // the pixel whose Jacobi value this lane evaluates
        if (lane < 4) {
            int dx, dy;
            nb_offsets(lane, dx, dy);
            cx = x + dx;
            cy = y + dy;
        }
        const unsigned cm = dev::dpc_valid_mask(cx, cy, W, H);
        int jn[8];
#pragma unroll
        for (int k = 0; k < 8; k++) {
            int dx, dy;
            nb_offsets(k, dx, dy);
            // window slot of (cx + dx, cy + dy) (inside it for every lane that uses the value)
            const int col = (cx + dx - x + 4) >> 1, row = (cy + dy - y + 4) >> 1;
            const int src = min(max(row, 0), 3) * 5 + min(max(col, 0), 4);
            jn[k] = __shfl_sync(full, win, src);
        }
        const int own = __shfl_sync(full, win, ((cy - y + 4) >> 1) * 5 + ((cx - x + 4) >> 1));
        // lanes 4-7: later neighbour k, lane 8 (and the others): the pixel itself
        int dxl = 0, dyl = 0;
        if (lane >= 4 && lane < 8) nb_offsets(lane, dxl, dyl);
        const int sample = __shfl_sync(full, win, ((dyl + 4) >> 1) * 5 + ((dxl + 4) >> 1));
        int v = 0;
        if (lane < 4) {
            if ((m >> lane) & 1u) {
                const int s = find_override(ov_idx, ov_val, n_ov, cy * W + cx);
                v = s >= 0 ? s : dev::dpc_apply(own, jn, cm, fp.dpc_thr);
            }
        } else if (lane < 8) {
            if ((m >> lane) & 1u) v = sample;
        } else if (lane == 8) {
            v = sample;
        } else if (lane == 9) {
            v = dev::dpc_apply(own, jn, cm, fp.dpc_thr);
        }
        int nb[8];
#pragma unroll
        for (int k = 0; k < 8; k++) nb[k] = __shfl_sync(full, v, k);
        const int c = __shfl_sync(full, v, 8), jac = __shfl_sync(full, v, 9);
        if (lane == 0) {
            const int s = dev::dpc_apply(c, nb, m, fp.dpc_thr);
            if (s != jac) {
                if (n_ov >= ocap) {
                    bad = 1;
                } else {
                    ov_idx[n_ov] = p;
                    ov_val[n_ov] = s;
                    n_ov++;
                    for (int k = 4; k < 8 && !bad; k++) {
                        if (!((m >> k) & 1u)) continue;
                        int dx, dy;
                        nb_offsets(k, dx, dy);
                        if (hn >= hcap) bad = 1;
                        else heap_push(heap, hn, (y + dy) * W + (x + dx));
                    }
                }
            }
        }
        n_ov = __shfl_sync(full, n_ov, 0);
        hn = __shfl_sync(full, hn, 0);
        if (__shfl_sync(full, bad, 0)) return -1;
    }
    if (n_ov > fs.cap) {
        if (lane == 0) atomicExch(fp.status, 104 /* IMOP_ERR_CAPACITY */);
        return 0;
    }
    __syncwarp();
    for (int i = lane; i < n_ov; i += 32) {
        fs.ov_idx[i] = ov_idx[i];
        fs.ov_val[i] = ov_val[i];
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
