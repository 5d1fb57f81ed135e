// Stable LSD radix sort of (uint32 key, uint32 value) pairs with 8-bit digits.
// Used to order particles by the Morton code of their cell every step.
//
// Per pass: (1) per-tile digit histograms, stored digit-major so that one
// exclusive scan over [digit][tile] yields every tile's global base per digit
// in stable order; (2) a single-block scan; (3) a stable scatter that ranks the
// items of a tile with warp match masks and per-warp digit counts.
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

// Exclusive scan of m entries by one block of 32 warps.  Warp w owns the
// contiguous chunk [w*C, (w+1)*C) and walks it 32 entries at a time with
// coalesced loads and warp shuffles; a scan of the 32 chunk totals gives each
// warp its base.
__global__ void __launch_bounds__(1024) k_scan(uint32_t *__restrict__ data, uint32_t m, unsigned *lc)
{
    count_launch(lc);
    __shared__ uint32_t tot[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t C = ((m + 31) / 32 + 31) / 32 * 32;   // chunk per warp, multiple of 32
    const uint32_t lo = min((uint32_t)warp * C, m), hi = min(lo + C, m);
    uint32_t s = 0;
    for (uint32_t i = lo + lane; i < hi; i += 32) s += data[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) tot[warp] = s;
    __syncthreads();
    if (warp == 0) {
        uint32_t v = tot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += u;
        }
        tot[lane] = v - tot[lane];   // exclusive
    }
    __syncthreads();
    uint32_t run = tot[warp];
    for (uint32_t base = lo; base < hi; base += 32) {
        const uint32_t i = base + lane;
        const uint32_t x = i < hi ? data[i] : 0u;
        uint32_t v = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += u;
        }
        if (i < hi) data[i] = run + v - x;
        run += __shfl_sync(0xffffffffu, v, 31);
    }
}

__global__ void __launch_bounds__(kSortThreads) k_scatter(const uint32_t *__restrict__ kin, const uint32_t *__restrict__ vin,
                                                         uint32_t *__restrict__ kout, uint32_t *__restrict__ vout,
                                                         uint32_t n, int shift, const uint32_t *__restrict__ scanned,
                                                         uint32_t num_tiles, unsigned *lc)
{
    count_launch(lc);
    __shared__ uint32_t base[kRadix];
    __shared__ uint32_t run[kRadix];
    __shared__ uint32_t wcnt[kWarps][kRadix];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    base[t] = scanned[(size_t)t * num_tiles + blockIdx.x];
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
    bool swapped = false;
    uint32_t *ki = keys, *vi = vals, *ko = keys2, *vo = vals2;
    for (int shift = 0; shift < key_bits; shift += 8) {
        k_hist<<<tiles, kSortThreads, 0, s>>>(ki, n, shift, hist, tiles, lc);
        k_scan<<<1, 1024, 0, s>>>(hist, kRadix * tiles, lc);
        k_scatter<<<tiles, kSortThreads, 0, s>>>(ki, vi, ko, vo, n, shift, hist, tiles, lc);
        uint32_t *tk = ki, *tv = vi;
        ki = ko; vi = vo; ko = tk; vo = tv;
        swapped = !swapped;
    }
    return swapped;
}

}  // namespace sphgb
