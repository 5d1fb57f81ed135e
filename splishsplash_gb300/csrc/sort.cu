// Stable LSD radix sort of (uint32 key, uint32 value) pairs with 8-bit digits.
// Used to order particles by the Morton code of their cell every step.
//
// Per pass: (1) per-tile digit histograms, stored digit-major; (2) an exclusive scan
// of each digit's row over the tiles, one block per digit, with the row totals; (3) a
// stable scatter whose tiles add the scan of the digit totals to their row offsets, and
// rank the items of a tile with warp match masks and per-warp digit counts.
// The histogram buffer holds 256 x (tiles + 1) words: the rows, then the digit totals.
#include "sph_ctx.h"

namespace sphgb {

namespace {

constexpr int kSortThreads = 256;
constexpr int kItems = kSortTile / kSortThreads;   // 8
constexpr int kRadix = 256;
constexpr int kWarps = kSortThreads / 32;

__global__ void __launch_bounds__(kSortThreads) k_hist(const uint32_t *__restrict__ keys, uint32_t n, int shift,
                                                      uint32_t *__restrict__ hist, uint32_t num_tiles, unsigned *lc)
{
    count_launch(lc);
    __shared__ uint32_t h[kRadix];
    h[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * kSortTile;
#pragma unroll
    for (int r = 0; r < kItems; r++) {
        const uint32_t idx = base + r * kSortThreads + threadIdx.x;
        if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & 0xffu], 1u);
    }
    __syncthreads();
    hist[(size_t)threadIdx.x * num_tiles + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of each digit's row of tile counts, one block per digit: row d of the
// digit-major histogram (num_tiles entries) becomes the per-tile offsets within digit d,
// and dtot[d] receives the row total.  Each thread scans a contiguous chunk serially; a
// block scan of the chunk totals gives each chunk its base.
__global__ void __launch_bounds__(kSortThreads) k_scan_rows(uint32_t *__restrict__ hist, uint32_t num_tiles,
                                                           uint32_t *__restrict__ dtot, unsigned *lc)
{
    count_launch(lc);
    __shared__ uint32_t wsum[kWarps];
    uint32_t *row = hist + (size_t)blockIdx.x * num_tiles;
    const uint32_t per = (num_tiles + kSortThreads - 1) / kSortThreads;
    const uint32_t lo = min(threadIdx.x * per, num_tiles), hi = min(lo + per, num_tiles);
    uint32_t s = 0;
    for (uint32_t i = lo; i < hi; i++) s += row[i];
    // block-wide exclusive scan of the chunk totals
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t v = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    if (lane == 31) wsum[warp] = v;
    __syncthreads();
    uint32_t wbase = 0;
    for (int w = 0; w < warp; w++) wbase += wsum[w];
    uint32_t run = wbase + v - s;
    for (uint32_t i = lo; i < hi; i++) {
        const uint32_t x = row[i];
        row[i] = run;
        run += x;
    }
    if (threadIdx.x == kSortThreads - 1) dtot[blockIdx.x] = wbase + v;
}

__global__ void __launch_bounds__(kSortThreads) k_scatter(const uint32_t *__restrict__ kin, const uint32_t *__restrict__ vin,
                                                         uint32_t *__restrict__ kout, uint32_t *__restrict__ vout,
                                                         uint32_t n, int shift, const uint32_t *__restrict__ scanned,
                                                         const uint32_t *__restrict__ dtot, uint32_t num_tiles,
                                                         unsigned *lc)
{
    count_launch(lc);
    __shared__ uint32_t base[kRadix];
    __shared__ uint32_t run[kRadix];
    __shared__ uint32_t wcnt[kWarps][kRadix];
    __shared__ uint32_t wsum[kWarps];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    // digit base: exclusive scan of the digit totals, then this tile's offset within the digit
    {
        const uint32_t x = dtot[t];
        uint32_t v = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += u;
        }
        if (lane == 31) wsum[warp] = v;
        __syncthreads();
        uint32_t wb = 0;
        for (int w = 0; w < warp; w++) wb += wsum[w];
        base[t] = wb + v - x + scanned[(size_t)t * num_tiles + blockIdx.x];
    }
    run[t] = 0;
#pragma unroll
    for (int w = 0; w < kWarps; w++) wcnt[w][t] = 0;
    __syncthreads();
    const uint32_t lt_mask = (1u << lane) - 1u;
    const uint32_t tile0 = blockIdx.x * kSortTile;
    for (int r = 0; r < kItems; r++) {
        const uint32_t idx = tile0 + r * kSortThreads + t;
        const bool valid = idx < n;
        const uint32_t key = valid ? kin[idx] : 0u;
        const uint32_t val = valid ? vin[idx] : 0u;
        const uint32_t d = valid ? ((key >> shift) & 0xffu) : 0x100u;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const uint32_t lrank = __popc(peers & lt_mask);
        const bool leader = lane == (__ffs(peers) - 1);
        if (valid && leader) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t pre = run[d];
            for (int w = 0; w < warp; w++) pre += wcnt[w][d];
            const uint32_t dst = base[d] + pre + lrank;
            kout[dst] = key;
            vout[dst] = val;
        }
        __syncthreads();
        uint32_t s = 0;
#pragma unroll
        for (int w = 0; w < kWarps; w++) {
            s += wcnt[w][t];
            wcnt[w][t] = 0;
        }
        run[t] += s;
        __syncthreads();
    }
}

}  // namespace

bool radix_sort_pairs(uint32_t *keys, uint32_t *vals, uint32_t *keys2, uint32_t *vals2, uint32_t n, int key_bits,
                      uint32_t *hist, uint32_t num_tiles, cudaStream_t s, unsigned *lc)
{
    if (n == 0) return false;
    const uint32_t tiles = (n + kSortTile - 1) / kSortTile;
    (void)num_tiles;
    uint32_t *dtot = hist + (size_t)kRadix * tiles;   // digit totals after the tile histograms
    bool swapped = false;
    uint32_t *ki = keys, *vi = vals, *ko = keys2, *vo = vals2;
    for (int shift = 0; shift < key_bits; shift += 8) {
        k_hist<<<tiles, kSortThreads, 0, s>>>(ki, n, shift, hist, tiles, lc);
        k_scan_rows<<<kRadix, kSortThreads, 0, s>>>(hist, tiles, dtot, lc);
        k_scatter<<<tiles, kSortThreads, 0, s>>>(ki, vi, ko, vo, n, shift, hist, dtot, tiles, lc);
        uint32_t *tk = ki, *tv = vi;
        ki = ko; vi = vo; ko = tk; vo = tv;
        swapped = !swapped;
    }
    return swapped;
}

}  // namespace sphgb
