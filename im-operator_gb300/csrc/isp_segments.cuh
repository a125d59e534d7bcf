// isp_segments.cuh - work claiming of the streamed kernels.  Each strip of a frame is cut into
// segments (about one per resident warp), each segment into bands.  A warp streams its own
// segment's bands from the front, one after the other without re-reading warm-up rows; a warp
// whose segment is done takes single bands from the back of other segments.
//
// Per segment one 64-bit word: the claims made from the front (bits 0-22) and from the back
// (bits 23-45), whether a warp adopted the segment (bit 46) and the segment's band count (bits
// 48-63), written by the launch's init kernel before the streamed kernel runs: zero claims, or
// band 0 already claimed for the segment's warp (which then starts on it with no atomic).
// A claim is valid while the two counts before it sum to less than the band count, so a warp
// looking for work reads everything it needs from the word.  Segments beyond the launch's warps
// start without an owner: the first warp that finds one sets its adopted bit and streams it from
// the front like an owner.  The claim that takes a segment's last band counts the segment in the
// word after the launch's last segment word; a warp looking for work stops once that count
// reaches the number of segments.
#pragma once

#include <cuda_runtime.h>

namespace imop {
namespace segs {

constexpr unsigned long long kFrontOne = 1ull;
constexpr unsigned long long kBackOne = 1ull << 23;
constexpr unsigned long long kAdopted = 1ull << 46;
constexpr int kMaxBands = 65535;

__host__ __device__ inline unsigned long long initial_word(int nb) { return (unsigned long long)nb << 48; }
__device__ __forceinline__ unsigned front_of(unsigned long long w) { return (unsigned)w & 0x7FFFFFu; }
__device__ __forceinline__ unsigned back_of(unsigned long long w) { return (unsigned)(w >> 23) & 0x7FFFFFu; }
__device__ __forceinline__ unsigned bands_of(unsigned long long w) { return (unsigned)(w >> 48); }
__device__ __forceinline__ bool open(unsigned long long w) { return front_of(w) + back_of(w) < bands_of(w); }

// The streamed kernels are launched as programmatic dependents of their init kernel: they may
// start while it runs (their table prologue overlaps it) and wait for its writes before the
// first claim.  Both are no-ops for a kernel launched the ordinary way.
__device__ __forceinline__ void release_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void wait_init() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// rows [s0, s0 + len) of a segment in nb bands: band i
__device__ __forceinline__ void band_of(int s0, int len, int nb, int i, int& y0, int& bh) {
    const int q = len / nb, rem = len - q * nb;
    y0 = s0 + i * q + min(i, rem);
    bh = q + (i < rem ? 1 : 0);
}
// rows [y0, y0 + h) in n segments, the first h % n of them one row taller: segment t
__device__ __forceinline__ void split_rows(int y0, int h, int n, int t, int& s0, int& len) {
    const int q = h / n, rem = h - q * n;
    s0 = y0 + t * q + min(t, rem);
    len = q + (t < rem ? 1 : 0);
}

// A front claim whose atomic returned `old` (it may be settled later, when its band is needed):
// the band, or -1 when the segment had none left; the claim of the last band counts the segment
// in `taken`
__device__ __forceinline__ int settle_front(unsigned long long old, unsigned long long* taken) {
    const unsigned f = front_of(old), b = back_of(old), nb = bands_of(old);
    if (f + b >= nb) return -1;
    if (f + b + 1 == nb) atomicAdd(taken, 1ull);
    return (int)f;
}
// one lane: the next band from the front (the segment's own warp) / back (another warp), or -1
__device__ __forceinline__ int claim_front(unsigned long long* w, unsigned long long* taken) {
    return settle_front(atomicAdd(w, kFrontOne), taken);
}
// up to k bands from the back in one claim: the first of them (-1 if none was left) and, in n,
// how many (contiguous; fewer than k when the front claims reached them)
__device__ __forceinline__ int claim_back(unsigned long long* w, unsigned long long* taken, unsigned k, int& n) {
    const unsigned long long old = atomicAdd(w, kBackOne * k);
    const unsigned f = front_of(old), b = back_of(old), nb = bands_of(old);
    n = 0;
    if (f + b >= nb) return -1;
    if (f + b + k >= nb) atomicAdd(taken, 1ull);
    // bands [f, nb - b) were unclaimed; this claim took the last k of them (k may exceed their
    // number when other claims came between the read that chose k and this one)
    const int last = (int)nb - 1 - (int)b, first = max((int)f, (int)nb - (int)b - (int)k);
    n = last - first + 1;
    return first;
}

// The work of one warp gw of nwarps over the nseg segments of `words` (the taken count at
// words[nseg]): first its own segments from the front (the caller continues each band after
// band): segment gw, then gw + nwarps, gw + 2 nwarps, ... (those beyond the launch's warps are
// adopted first, so that a warp looking for work may take one over); then, 128 segments tested
// per pass from the last one that held work on, one still open: adopted and streamed from the
// front if no warp has begun it, else its last unclaimed band.  next() gives the
// segment, its first band and band count to do and whether the warp streams on from them; it
// returns false when every segment is taken, or when a whole pass finds none open.
struct Walk {
    int base, scanned, nwarps, next_own, owners;
    // owners: segments below it start with band 0 claimed for their warp by the init kernel
    __device__ __forceinline__ Walk(int gw, int nseg, int nw, int own_claimed)
        : base(gw % nseg), scanned(0), nwarps(nw), next_own(gw), owners(own_claimed) {}

    __device__ __forceinline__ bool next(unsigned long long* words, int nseg, int gw, int lane, int& seg, int& band,
                                         int& nbands, bool& own) {
        nbands = 1;
        const unsigned full = 0xffffffffu;
        while (next_own < nseg) {
            const int s = next_own;
            next_own += nwarps;
            if (s < owners) {
                seg = s;
                band = 0;
                own = true;
                return true;
            }
            int i = -1;
            if (lane == 0 && (s < nwarps || !(atomicOr(words + s, kAdopted) & kAdopted)))
                i = claim_front(words + s, words + nseg);
            i = __shfl_sync(full, i, 0);
            if (i >= 0) {
                seg = s;
                band = i;
                own = true;
                return true;
            }
        }
        own = false;
        const volatile unsigned long long* vw = words;
        while (scanned < nseg) {
            unsigned long long wv[4];  // segment base + lane + 32 i (wrapped), or nothing open
#pragma unroll
            for (int i = 0; i < 4; i++) {
                int c = base + lane + 32 * i;  // base < nseg
                if (c >= nseg) c -= nseg;
                if (c >= nseg) c %= nseg;  // fewer than 128 segments
                wv[i] = lane + 32 * i < nseg ? vw[c] : 0ull;
            }
            if (vw[nseg] >= (unsigned long long)nseg) return false;  // every segment taken
            unsigned m[4];
#pragma unroll
            for (int i = 0; i < 4; i++) m[i] = __ballot_sync(full, open(wv[i]));
            // an open segment of the window, chosen from a place that depends on the warp, so the
            // warps looking for work spread over the open segments instead of all claiming the
            // first one
            const int rot = gw & 31, grot = (gw >> 5) & 3;
            int s = -1;
#pragma unroll
            for (int t = 0; t < 4; t++) {
                const int i = (t + grot) & 3;
                const unsigned mm = i == 0 ? m[0] : i == 1 ? m[1] : i == 2 ? m[2] : m[3];
                if (s < 0 && mm) {
                    const int bit = (__ffs(__funnelshift_r(mm, mm, rot)) - 1 + rot) & 31;
                    int c = base + bit + 32 * i;
                    if (c >= nseg) c -= nseg;
                    if (c >= nseg) c %= nseg;
                    s = c;
                }
            }
            if (s < 0) {
                base += 128;
                if (base >= nseg) base %= nseg;
                scanned += 128;
                continue;
            }
            int j = 0, n = 1;
            bool adopt = false;
            if (lane == 0) {
                if (s >= nwarps && !(atomicOr(words + s, kAdopted) & kAdopted)) {
                    adopt = true;
                    j = claim_front(words + s, words + nseg);
                } else {
                    // one band: a range taken from the back could not be taken over in turn
                    j = claim_back(words + s, words + nseg, 1u, n);
                }
            }
            j = __shfl_sync(full, j, 0);
            n = __shfl_sync(full, n, 0);
            adopt = __shfl_sync(full, adopt, 0);
            base = s;  // the segment may hold more
            scanned = 0;
            if (j >= 0) {
                seg = s;
                band = j;
                nbands = adopt ? 1 : n;
                own = adopt;
                return true;
            }
        }
        return false;
    }
};

// host: launch kernel k as a programmatic dependent of the kernel before it in stream st
inline cudaError_t launch_dependent_impl(const void* k, dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                                         void** args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelExC(&cfg, k, args);
}

}  // namespace segs

template <class Arg>
inline cudaError_t launch_dependent(void (*k)(Arg), int grid, int block, size_t smem, cudaStream_t st, const Arg& a) {
    void* args[1] = {const_cast<Arg*>(&a)};
    return segs::launch_dependent_impl(reinterpret_cast<const void*>(k), dim3(grid), dim3(block), smem, st, args);
}

}  // namespace imop
