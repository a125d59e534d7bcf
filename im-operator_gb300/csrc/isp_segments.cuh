// isp_segments.cuh - work claiming of the streamed kernels.  Each strip of a frame is cut into
// segments (about one per resident warp), each segment into bands.  A warp streams its own
// segment's bands from the front, one after the other without re-reading warm-up rows; a warp
// whose segment is done takes single bands from the back of other segments.
//
// Per segment one 64-bit word: the claims made from the front (bits 0-23) and from the back
// (bits 24-47) and the segment's band count (bits 48-63, written with zero counts by the launch's
// init kernel before the streamed kernel runs).  A claim is valid while the two counts before it
// sum to less than the band count, so a warp looking for work reads everything it needs from the
// word.  The claim that takes a segment's last band counts the segment in the word after the
// launch's last segment word; a warp looking for work stops once that count reaches the number of
// segments.
#pragma once

namespace imop {
namespace segs {

constexpr unsigned long long kFrontOne = 1ull;
constexpr unsigned long long kBackOne = 1ull << 24;
constexpr int kMaxBands = 65535;

__host__ __device__ inline unsigned long long initial_word(int nb) { return (unsigned long long)nb << 48; }
__device__ __forceinline__ unsigned front_of(unsigned long long w) { return (unsigned)w & 0xFFFFFFu; }
__device__ __forceinline__ unsigned back_of(unsigned long long w) { return (unsigned)(w >> 24) & 0xFFFFFFu; }
__device__ __forceinline__ unsigned bands_of(unsigned long long w) { return (unsigned)(w >> 48); }
__device__ __forceinline__ bool open(unsigned long long w) { return front_of(w) + back_of(w) < bands_of(w); }

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
__device__ __forceinline__ int claim_back(unsigned long long* w, unsigned long long* taken) {
    const unsigned long long old = atomicAdd(w, kBackOne);
    const unsigned f = front_of(old), b = back_of(old), nb = bands_of(old);
    if (f + b >= nb) return -1;
    if (f + b + 1 == nb) atomicAdd(taken, 1ull);
    return (int)(nb - 1 - b);
}

// The work of one warp over the nseg segments of `words` (the taken count at words[nseg]): first
// its own segment gw from the front (the caller continues it band after band), then single bands
// from the back of others: 128 segments tested per pass, from the last one that held work on, a
// band taken from the first one still open.  next() gives the segment and band to do and whether
// it is the warp's own; it returns false when every segment is taken, or when a whole pass finds
// none open.
struct Walk {
    int base, scanned;
    bool own_pending;
    __device__ __forceinline__ Walk(int gw, int nseg) : base(gw % nseg), scanned(0), own_pending(gw < nseg) {}

    __device__ __forceinline__ bool next(unsigned long long* words, int nseg, int gw, int lane, int& seg, int& band,
                                         bool& own) {
        const unsigned full = 0xffffffffu;
        if (own_pending) {
            own_pending = false;
            int i = 0;
            if (lane == 0) i = claim_front(words + gw, words + nseg);
            i = __shfl_sync(full, i, 0);
            if (i >= 0) {
                seg = gw;
                band = i;
                own = true;
                return true;
            }
        }
        own = false;
        const volatile unsigned long long* vw = words;
        while (scanned < nseg) {
            unsigned long long wv[4];
            int cand[4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                int c = base + lane + 32 * i;  // base < nseg
                if (c >= nseg) c -= nseg;
                if (c >= nseg) c %= nseg;  // fewer than 128 segments
                cand[i] = c;
                wv[i] = lane + 32 * i < nseg ? vw[c] : 0ull;
            }
            if (vw[nseg] >= (unsigned long long)nseg) return false;  // every segment taken
            int s = -1;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const unsigned m = __ballot_sync(full, open(wv[i]));
                if (s < 0 && m) s = __shfl_sync(full, cand[i], __ffs(m) - 1);
            }
            if (s < 0) {
                base += 128;
                if (base >= nseg) base %= nseg;
                scanned += 128;
                continue;
            }
            int j = 0;
            if (lane == 0) j = claim_back(words + s, words + nseg);
            j = __shfl_sync(full, j, 0);
            base = s;  // the segment may hold more
            scanned = 0;
            if (j >= 0) {
                seg = s;
                band = j;
                return true;
            }
        }
        return false;
    }
};

}  // namespace segs
}  // namespace imop
